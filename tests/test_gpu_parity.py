"""GPU parity: the CUDA step (through the C ABI) against BETSE's own results.

Golden fixtures hold BETSE's state after selected step counts on seeded
clusters (``tests/golden/make_golden.py``). Tolerances:

* plain FP64 form: concentrations within 1e-10 relative (max|a-b| / max|b|);
  Vmem within 1e-10 relative plus the FP64 cancellation floor of the charge
  sum (``golden_io.vm_floor``: 4 ulp of the largest ionic charge term, in
  volts), because Vmem is a small difference of ~1e7 C/m3 charges and BETSE's
  own dense-BLAS summation order is one of many equally rounded orders;
* FP32/FP64-split form: |Vmem - Vmem_ref| < 1e-6 V.
"""
import numpy as np
import pytest

import golden_io as gi

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-10
TOL_SPLIT_V = 1e-6


def _engine(d, precision):
    from betse_gb300.engine import ClusterEngine
    cg, sp, Dm, st, D_env = gi.engine_inputs(d)
    eng = ClusterEngine(cg, sp, precision)
    eng.set_membrane_diffusivity(Dm)
    if sp.is_ecm:
        eng.set_env_diffusivity(D_env)
    eng.upload(**st)
    return eng


def _cmp_env(eng_env, ref_env, ecm):
    if ecm:
        return gi.rel_err(eng_env, ref_env)
    return gi.rel_err(eng_env, ref_env[:, 0])


@pytest.mark.parametrize('name', gi.CASES)
def test_state_fp64_matches_betse(name):
    d = gi.load(name)
    ecm = bool(d['par_is_ecm'])
    with _engine(d, 'fp64') as eng:
        done = 0
        for cp in d['meta_checkpoints']:
            eng.step(int(cp - done))
            done = int(cp)
            st = eng.check_stable()
            s = eng.download()
            ok, e_vm, bound = gi.vm_err_ok(d, s['vm'], d[f's{cp}_vm'], d[f's{cp}_cc_cells'])
            e_cc = gi.rel_err(s['cc_cells'], d[f's{cp}_cc_cells'])
            e_cm = gi.rel_err(s['cc_at_mem'], d[f's{cp}_cc_at_mem'])
            e_env = _cmp_env(s['cc_env'], d[f's{cp}_cc_env'], ecm)
            assert ok, (cp, e_vm, bound)
            assert e_cc < TOL_FP64, (cp, e_cc)
            assert e_cm < TOL_FP64, (cp, e_cm)
            assert e_env < TOL_FP64, (cp, e_env)
            if 'gjopen' in s:
                # voltage-gated gap junctions: the open fraction is state
                e_go = gi.rel_err(s['gjopen'], d[f's{cp}_gjopen'])
                assert e_go < TOL_FP64, (cp, e_go)
            assert st['steps_done'] == done


@pytest.mark.parametrize('name', gi.CASES)
def test_outputs_fp64_match_betse(name):
    d = gi.load(name)
    cp = int(d['meta_checkpoints'][1])
    ecm = bool(d['par_is_ecm'])
    with _engine(d, 'fp64') as eng:
        eng.step(cp, outputs=True)
        o = eng.outputs()
    keys = ['fluxes_mem', 'fluxes_gj', 'rate_NaKATP', 'rho_cells', 'Jn', 'I_mem', 'J_cell_x',
            'J_cell_y', 'Jc', 'vm_ave', 'dvm', 'E_cell_x', 'E_cell_y', 'Emc', 'E_gj_x',
            'E_gj_y', 'gjopen', 'sigma_cell']
    floors = gi.output_floors(d, d[f's{cp}_cc_cells'], o)
    for k in keys:
        ref = d[f's{cp}_{k}']
        got = o[k]
        err = np.max(np.abs(got - ref))
        floor = floors.get(k, 0.0)
        assert err <= TOL_FP64 * np.max(np.abs(ref)) + floor, (k, err, floor)
    if ecm:
        for k in ('v_env',):
            assert gi.rel_err(o[k], d[f's{cp}_{k}']) < 1e-9, k


@pytest.mark.parametrize('name', gi.CASES)
def test_split_precision_vmem_error(name):
    d = gi.load(name)
    if gi.polar(d):
        from betse_gb300._lib import BxLibraryError
        with pytest.raises(BxLibraryError, match='per-membrane'):
            _engine(d, 'split')
        return
    with _engine(d, 'split') as eng:
        done = 0
        for cp in d['meta_checkpoints']:
            eng.step(int(cp - done))
            done = int(cp)
            eng.check_stable()
            s = eng.download()
            err = np.max(np.abs(s['vm'] - d[f's{cp}_vm']))
            assert err < TOL_SPLIT_V, (cp, err)
            assert gi.rel_err(s['cc_cells'], d[f's{cp}_cc_cells']) < 1e-5
            if 'gjopen' in s:
                # FP32 open fraction (values in [gj_min, 1])
                assert np.max(np.abs(s['gjopen'] - d[f's{cp}_gjopen'])) < 1e-5


@pytest.mark.parametrize('name', ['noecm_r50_s7', 'ecm_r40_s13_ca'])
@pytest.mark.parametrize('precision', ['fp64', 'split'])
def test_graph_chunks_equal_eager_steps(precision, name):
    """CUDA-graph-replayed steps give bit-identical state to eager steps
    (also through the extracellular pipeline the Ca-ATPase reorders)."""
    d = gi.load(name)
    with _engine(d, precision) as a, _engine(d, precision) as b:
        a.step(70)                 # graph chunks of 32 + eager tail
        for _ in range(70):
            b.step(1)              # eager only
        sa, sb = a.download(), b.download()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


@pytest.mark.parametrize('precision', ['fp64', 'split'])
def test_deterministic_repeat(precision):
    d = gi.load('noecm_r80_s1')
    res = []
    for _ in range(2):
        with _engine(d, precision) as e:
            e.step(100)
            res.append(e.download())
    for k in res[0]:
        assert np.array_equal(res[0][k], res[1][k]), k


@pytest.mark.parametrize('precision', ['fp64', 'split'])
def test_nan_input_raises_unstable(precision):
    from betse_gb300.exceptions import BetseSimUnstableException
    d = gi.load('noecm_r20_s2')
    cg, sp, Dm, st, _ = gi.engine_inputs(d)
    from betse_gb300.engine import ClusterEngine
    with ClusterEngine(cg, sp, precision) as eng:
        eng.set_membrane_diffusivity(Dm)
        st = dict(st)
        cc = st['cc_cells'].copy()
        cc[0, 3] = np.nan            # poisoned host input, not a device fault
        st['cc_cells'] = cc
        eng.upload(**st)
        eng.step(2)
        with pytest.raises(BetseSimUnstableException):
            eng.check_stable()


def test_split_outputs_close_to_betse():
    """The split form's sampled-step outputs (FP32 fluxes) against BETSE's FP64."""
    d = gi.load('noecm_r80_s1')
    cp = int(d['meta_checkpoints'][1])
    with _engine(d, 'split') as eng:
        eng.step(cp, outputs=True)
        o = eng.outputs()
    for k in ('fluxes_mem', 'fluxes_gj', 'rate_NaKATP', 'Jn', 'I_mem', 'J_cell_x', 'J_cell_y',
              'vm_ave', 'sigma_cell', 'E_gj_x', 'E_gj_y', 'gjopen'):
        ref = d[f's{cp}_{k}']
        assert np.max(np.abs(o[k] - ref)) <= 2e-3 * np.max(np.abs(ref)) + 1e-30, k


@pytest.mark.parametrize('precision', ['fp64', 'split'])
def test_autotune_keeps_state_and_results(precision):
    """Autotuning changes the CTA partition, not the simulation: the state is
    restored and the result after stepping matches an untuned engine."""
    d = gi.load('noecm_r80_s1')
    with _engine(d, precision) as a, _engine(d, precision) as b:
        tpb, ms = a.autotune(5)
        assert tpb in (8, 16, 32, 64, 128, 192, 256) and ms > 0
        s0 = a.download()
        assert np.array_equal(s0['vm'], b.download()['vm'])
        a.step(40)
        b.step(40)
        sa, sb = a.download(), b.download()
    # the well-mixed environment adds the CTAs' partial sums in partition
    # order, so a different CTA size rounds differently (FP64: ~1e-16)
    tol = 1e-13 if precision == 'fp64' else 1e-12
    for k in sa:
        assert gi.rel_err(sa[k], sb[k]) <= tol, k


@pytest.mark.parametrize('tpb,kernel', [(16, 0), (32, 0), (64, 0), (128, 0), (256, 0), (16, 5), (32, 5),
                                        (64, 5)])
def test_fp64_cta_sizes_match_betse(tpb, kernel):
    """Every CTA size of the plain FP64 kernel, and the small-cluster kernel
    (5: lanes per ion, the environment mixed by the last CTA), reproduces
    BETSE's state at every checkpoint."""
    d = gi.load('noecm_r80_s1')
    with _engine(d, 'fp64') as eng:
        eng.set_launch_config(tpb, kernel)
        done = 0
        for cp in d['meta_checkpoints']:
            eng.step(int(cp - done))
            done = int(cp)
            eng.check_stable()
            s = eng.download()
            ok, e_vm, bound = gi.vm_err_ok(d, s['vm'], d[f's{cp}_vm'], d[f's{cp}_cc_cells'])
            assert ok, (tpb, cp, e_vm, bound)
            assert gi.rel_err(s['cc_cells'], d[f's{cp}_cc_cells']) < TOL_FP64, (tpb, cp)
            assert _cmp_env(s['cc_env'], d[f's{cp}_cc_env'], False) < TOL_FP64, (tpb, cp)
        assert eng.launch_config() == (tpb, kernel)


@pytest.mark.parametrize('tpb', [192, 256])
def test_split_launch_configs_bit_identical(tpb):
    """Tile-per-CTA and persistent pipelined split kernels, and both CTA sizes,
    give bit-identical state: the same arithmetic in the same order."""
    d = gi.load('noecm_r80_s1')
    res = []
    for persist in (False, True):
        with _engine(d, 'split') as e:
            e.set_launch_config(tpb, persist)
            e.step(75)
            e.check_stable()
            res.append(e.download())
    with _engine(d, 'split') as e:
        e.step(75)
        ref = e.download()
    for k in ref:
        assert np.array_equal(res[0][k], res[1][k]), k
        assert np.array_equal(res[0][k], ref[k]), k


@pytest.mark.parametrize('precision', ['fp64', 'split'])
def test_voltage_gated_gj_state_round_trip_and_autotune(precision):
    """The gap-junction open fraction survives download/upload and the
    autotuner's re-partitioning; the persistent kernel is refused with gating."""
    d = gi.load('noecm_r50_s9_vgj')
    with _engine(d, precision) as a, _engine(d, precision) as b:
        a.step(5)
        b.step(5)
        s = a.download()
        assert 'gjopen' in s and np.all(s['gjopen'] <= 1.0)
        a.upload(**s)
        a.autotune(3)
        a.step(7)
        b.step(7)
        sa, sb = a.download(), b.download()
        if precision == 'split':
            with pytest.raises(Exception):
                a.set_launch_config(256, True)
    # the well-mixed environment adds the CTAs' partial sums in partition
    # order, so a different CTA size rounds differently (FP64: ~1e-16)
    tol = 1e-13 if precision == 'fp64' else 1e-12
    for k in sa:
        assert gi.rel_err(sa[k], sb[k]) <= tol, k


@pytest.mark.parametrize('precision', ['fp64', 'split'])
def test_upload_checks_and_download_into_given_arrays(precision):
    """The device-side upload checks refuse what BETSE's layouts cannot hold
    (and leave no state behind); downloads fill caller-given arrays."""
    from betse_gb300._lib import BxLibraryError
    from betse_gb300.engine import ClusterEngine
    d = gi.load('noecm_r50_s7')
    cg, sp, Dm, st, _ = gi.engine_inputs(d)
    with ClusterEngine(cg, sp, precision) as eng:
        eng.set_membrane_diffusivity(Dm)
        bad = dict(st)
        cam = st['cc_at_mem'].copy()
        cam[0, 1] += 1.0                     # membrane 1 of cell 0 differs from membrane 0
        bad['cc_at_mem'] = cam
        with pytest.raises(BxLibraryError, match='cc_at_mem must be constant'):
            eng.upload(**bad)
        with pytest.raises(BxLibraryError):
            eng.step(1)                      # no state after a failed upload
        with pytest.raises(ValueError, match='vm: expected'):
            eng.upload(**dict(st, vm=st['vm'][:-1]))   # refused before the C library reads it
        if precision == 'split':
            bad = dict(st)
            vm = st['vm'].copy()
            vm[1] += 1e-3
            bad['vm'] = vm
            with pytest.raises(BxLibraryError, match='uniform'):
                eng.upload(**bad)
        eng.upload(**st)
        eng.step(5)
        ref = eng.download()
        out = {k: np.full_like(v, np.nan) for k, v in ref.items()}
        got = eng.download(out=out)
        for k in ref:
            assert got[k] is out[k]
            assert np.array_equal(out[k], ref[k]), k


@pytest.mark.parametrize('name', ['noecm_r80_s1', 'noecm_r50_s7'])
def test_ion_lane_kernel_equals_tile_kernel(name):
    """The small-cluster kernel does k_cell_step's arithmetic per ion and per
    (cell, ion) in the same order; only the environment's partial sums add
    in another order, so the two agree to rounding after 300 steps."""
    d = gi.load(name)
    with _engine(d, 'fp64') as a, _engine(d, 'fp64') as b:
        a.set_launch_config(32, 0)
        b.set_launch_config(32, 5)
        a.step(300)
        b.step(300)
        b.check_stable()
        sa, sb = a.download(), b.download()
    for k in sa:
        assert gi.rel_err(sb[k], sa[k]) < 1e-13, k
