"""GPU parity of the split form's factored kernels (one thread per cell; the
transmembrane flux and the pump once per cell from the static sum of
Dm * mem_sa; gap-junction fluxes per paired membrane).

* against BETSE's own states (golden fixtures): |Vmem - Vmem_BETSE| < 1e-6 V
  and concentrations within 1e-5 relative, the split form's bar;
* against the per-membrane split kernel: the same bar (they differ only by
  FP32 rounding of the flux sums);
* resident (cooperative, shared-memory) against streaming factored: the same
  per-cell arithmetic; only the order of the environment sum differs, so the
  double-float concentrations agree to 1e-9 relative and the FP32 records
  (cc_at_mem, Vmem) to a couple of FP32 ulps;
* the resident kernel's grid barrier: a wait that cannot complete is
  reported as a timeout and leaves the state unchanged (no GPU fault).
"""
import numpy as np
import pytest

import golden_io as gi
import oracle
import synthetic

pytestmark = pytest.mark.gpu

TOL_SPLIT_V = 1e-6
NOECM = ['noecm_r80_s1', 'noecm_r50_s7', 'noecm_r20_s2']


def _engine(d, kernel, tpb=256, variant=0):
    from betse_gb300.engine import ClusterEngine
    cg, sp, Dm, st, _ = gi.engine_inputs(d)
    eng = ClusterEngine(cg, sp, 'split')
    eng.set_membrane_diffusivity(Dm)
    eng.upload(**st)
    eng.set_launch_config(tpb, kernel, variant)
    return eng


@pytest.mark.parametrize('kernel', ['factored', 'resident'])
@pytest.mark.parametrize('name', NOECM)
def test_factored_state_matches_betse(name, kernel):
    d = gi.load(name)
    with _engine(d, kernel) as eng:
        if kernel == 'resident':
            assert eng.resident_info()['fits']
        done = 0
        for cp in d['meta_checkpoints']:
            eng.step(int(cp - done))
            done = int(cp)
            eng.check_stable()
            s = eng.download()
            err = np.max(np.abs(s['vm'] - d[f's{cp}_vm']))
            assert err < TOL_SPLIT_V, (cp, err)
            assert gi.rel_err(s['cc_cells'], d[f's{cp}_cc_cells']) < 1e-5, cp
            assert gi.rel_err(s['cc_env'], d[f's{cp}_cc_env'][:, 0]) < 1e-5, cp


@pytest.mark.parametrize('tpb', [192, 256])
def test_factored_close_to_per_membrane_kernel(tpb):
    d = gi.load('noecm_r80_s1')
    res = {}
    for kernel in ('tile', 'factored', 'resident'):
        with _engine(d, kernel, tpb) as e:
            e.step(300)
            e.check_stable()
            res[kernel] = e.download()
    for kernel in ('factored', 'resident'):
        assert np.max(np.abs(res[kernel]['vm'] - res['tile']['vm'])) < TOL_SPLIT_V, kernel
        assert gi.rel_err(res[kernel]['cc_cells'], res['tile']['cc_cells']) < 1e-6, kernel
    # double-float concentrations agree closely; the FP32 record (cc_at_mem,
    # Vmem) may round one or two FP32 ulps apart
    for k in ('cc_cells', 'cc_env'):
        assert gi.rel_err(res['resident'][k], res['factored'][k]) < 1e-9, k
    assert gi.rel_err(res['resident']['cc_at_mem'], res['factored']['cc_at_mem']) < 2.5e-7
    assert np.max(np.abs(res['resident']['vm'] - res['factored']['vm'])) < 2e-8


def test_factored_ragged_cells_against_oracle():
    """Cells of 1 to 20 membranes, random partners, boundary membranes."""
    d = synthetic.ragged_fixture()
    g, p, s = gi.geometry(d), gi.params(d), gi.state(d)
    n = 30
    oracle.run(g, p, s, n)
    for kernel in ('factored', 'resident'):
        with _engine(d, kernel) as e:
            e.step(n)
            e.check_stable()
            got = e.download()
        assert np.max(np.abs(got['vm'] - s.vm)) < TOL_SPLIT_V, kernel
        assert gi.rel_err(got['cc_cells'], s.cc_cells) < 1e-5, kernel


def test_factored_batch_equals_alone():
    """A sweep on the factored kernel: each cluster as if stepped alone, bit
    for bit (tiles never straddle clusters; each cluster's environment is
    reduced on its own)."""
    from betse_gb300.engine import BatchEngine, ClusterEngine
    ds = [synthetic.ragged_fixture(), gi.load('noecm_r50_s7'), gi.load('noecm_r80_s1')]
    ins = [gi.engine_inputs(d) for d in ds]
    with BatchEngine([x[0] for x in ins], [x[1] for x in ins], 'split') as b:
        b.set_membrane_diffusivity([x[2] for x in ins])
        b.upload_states([x[3] for x in ins])
        b.set_launch_config(256, 'factored')
        b.step(45)
        got = b.download_states()
    for (cg, sp, Dm, st, _), s in zip(ins, got):
        with ClusterEngine(cg, sp, 'split') as e:
            e.set_membrane_diffusivity(Dm)
            e.upload(**st)
            e.set_launch_config(256, 'factored')
            e.step(45)
            ref = e.download()
        for k in ('vm', 'cc_cells', 'cc_at_mem', 'cc_env'):
            assert np.array_equal(s[k], ref[k]), k


def test_resident_runs_hand_over_to_output_steps():
    """A run with outputs: the resident launch does all steps but the last,
    which the tile kernel computes with its outputs; the state continues
    where the resident run left it."""
    d = gi.load('noecm_r80_s1')
    with _engine(d, 'resident') as a, _engine(d, 'factored') as b:
        a.step(71, outputs=True)
        b.step(70)
        b.set_launch_config(256, 'tile')
        b.step(1, outputs=True)
        sa, sb = a.download(), b.download()
        oa, ob = a.outputs(), b.outputs()
    for k in ('cc_cells', 'cc_env'):
        assert gi.rel_err(sa[k], sb[k]) < 1e-9, k
    assert gi.rel_err(sa['cc_at_mem'], sb['cc_at_mem']) < 2.5e-7
    for k in ('fluxes_mem', 'fluxes_gj', 'rho_cells', 'vm_ave', 'Jn'):
        assert gi.rel_err(oa[k], ob[k]) < 1e-6, k


def test_resident_barrier_timeout_is_reported_and_harmless():
    """Failure detection without a fault: the barrier self-check makes every
    CTA's bounded wait run out; the timeout is reported, the state is the one
    before the launch, and stepping continues normally."""
    d = gi.load('noecm_r50_s7')
    with _engine(d, 'resident') as e:
        e.step(10)
        before = e.download()
        assert e.resident_barrier_check(0.05) is True
        after = e.download()
        for k in before:
            assert np.array_equal(before[k], after[k]), k
        e.step(10)
        e.check_stable()
        got = e.download()
    with _engine(d, 'factored') as f:
        f.step(20)
        ref = f.download()
    for k in ('cc_cells', 'cc_env'):
        assert gi.rel_err(got[k], ref[k]) < 1e-9, k
    assert gi.rel_err(got['cc_at_mem'], ref['cc_at_mem']) < 2.5e-7


def test_pipelined_equals_factored_bit_for_bit():
    """The persistent pipelined factored kernel computes k_split_fact's
    arithmetic on staged copies of the same data: the same state, bit for
    bit, on a golden cluster, ragged cells and a batch of clusters."""
    from betse_gb300.engine import BatchEngine
    for d in (gi.load('noecm_r80_s1'), synthetic.ragged_fixture()):
        res = []
        for kernel in ('factored', 'pipelined'):
            with _engine(d, kernel) as e:
                e.step(45)
                e.check_stable()
                res.append(e.download())
        for k in res[0]:
            assert np.array_equal(res[0][k], res[1][k]), k
    ds = [synthetic.ragged_fixture(), gi.load('noecm_r50_s7'), gi.load('noecm_r80_s1')]
    ins = [gi.engine_inputs(d) for d in ds]
    got = []
    for kernel in ('factored', 'pipelined'):
        with BatchEngine([x[0] for x in ins], [x[1] for x in ins], 'split') as b:
            b.set_membrane_diffusivity([x[2] for x in ins])
            b.upload_states([x[3] for x in ins])
            b.set_launch_config(256, kernel)
            b.step(70)
            got.append(b.download_states())
    for a, c in zip(*got):
        for k in a:
            assert np.array_equal(a[k], c[k]), k


@pytest.mark.parametrize('variant', [2, 12, 13, 14, 16])
def test_factored_variants_equal_bit_for_bit(variant):
    """The factored kernel's variants (junctions per load round; entries
    prefetched before the dependency wait) order the same arithmetic the same
    way: the state matches the default variant bit for bit, on a golden
    cluster and on ragged cells (cells with more junctions than prefetched)."""
    for d in (gi.load('noecm_r80_s1'), synthetic.ragged_fixture()):
        res = []
        for v in (4, variant):
            with _engine(d, 'factored', variant=v) as e:
                e.step(45)
                e.check_stable()
                res.append(e.download())
        for k in res[0]:
            assert np.array_equal(res[0][k], res[1][k]), (variant, k)
