"""Pin the CPU oracle against BETSE's own results (golden fixtures).

The oracle restates ``Simulator._run_sim_core_loop`` with CSR segment sums; it
must reproduce BETSE's state to 1e-12 relative (Vmem 1e-10 after 2000 steps,
where the dense-GEMV summation order of the reference shows).  Vmem and the
quantities built on it are small differences of large charges, so each check
also allows the FP64 cancellation floor of that difference
(``golden_io.vm_floor`` / ``output_floors``): NumPy builds differ in the order
they sum a dot product, and the floor is what such a change can move.
"""
import numpy as np
import pytest

import golden_io as gi
import oracle


@pytest.mark.parametrize('name', gi.CASES)
def test_oracle_state_matches_betse(name):
    d = gi.load(name)
    g, p, s = gi.geometry(d), gi.params(d), gi.state(d)
    ok, err, bound = gi.vm_err_ok(d, oracle.init_vm(g, p, s), d['init_vm'], d['init_cc_cells'], rel=1e-13)
    assert ok, (err, bound)
    done = 0
    for cp in d['meta_checkpoints']:
        oracle.run(g, p, s, int(cp - done))
        done = int(cp)
        tol_v = 1e-10 if cp > 500 else 1e-12
        ok, err, bound = gi.vm_err_ok(d, s.vm, d[f's{cp}_vm'], d[f's{cp}_cc_cells'], rel=tol_v)
        assert ok, (cp, err, bound)
        assert gi.rel_err(s.cc_cells, d[f's{cp}_cc_cells']) < 1e-12
        assert gi.rel_err(s.cc_at_mem, d[f's{cp}_cc_at_mem']) < 1e-12
        assert gi.rel_err(s.cc_env, d[f's{cp}_cc_env']) < 1e-12


@pytest.mark.parametrize('name', gi.CASES)
def test_oracle_outputs_match_betse(name):
    d = gi.load(name)
    g, p, s = gi.geometry(d), gi.params(d), gi.state(d)
    g.lap_inv = np.linalg.pinv(oracle.fields.make_laplacian(*g.grid_shape, g.delta))
    cps = [int(c) for c in d['meta_checkpoints'][:2]]
    done = 0
    for cp in cps:
        out = oracle.run(g, p, s, cp - done, outputs_last=True)
        done = cp
        floors = gi.output_floors(d, d[f's{cp}_cc_cells'], out)
        vfl = gi.vm_floor(d, d[f's{cp}_cc_cells'])
        # the environment potential carries the Vmem floor, its gradient that
        # floor over one grid spacing
        floors.update(v_env=vfl, E_env_x=2 * vfl / float(d['geom_delta']), E_env_y=2 * vfl / float(d['geom_delta']))
        for k in ('fluxes_mem', 'fluxes_gj', 'rate_NaKATP', 'rho_cells', 'Jn', 'I_mem',
                  'J_cell_x', 'J_cell_y', 'Jc', 'vm_ave', 'dvm', 'E_cell_x', 'E_cell_y', 'Emc',
                  'E_gj_x', 'E_gj_y', 'gjopen', 'sigma_cell', 'E_env_x', 'E_env_y', 'v_env'):
            ref = np.asarray(d[f's{cp}_{k}'])
            err = np.max(np.abs(np.asarray(out[k]) - ref))
            # quantities without a derived floor (fields built on Vmem) get 1e-10
            rel = 1e-12 if k in floors else 1e-10
            assert err <= rel * np.max(np.abs(ref)) + floors.get(k, 0.0), (k, err)
        if bool(p.is_ecm):
            # divergence-free current via two dense lapENVinv products
            for k in ('J_env_x', 'J_env_y', 'B_field'):
                assert gi.rel_err(out[k], d[f's{cp}_{k}']) < 1e-6, k
        else:
            # without ECM the field is a pure gradient: its divergence-free part is
            # zero and both codes return round-off; bound it by the input scale
            scale = g.sigma * np.max(np.abs(out['E_env_x']))
            for k in ('J_env_x', 'J_env_y'):
                assert np.max(np.abs(out[k])) < 1e-12 * scale
                assert np.max(np.abs(d[f's{cp}_{k}'])) < 1e-12 * scale


def test_laplacian_inverse_matches_pinv():
    A = oracle.fields.make_laplacian(12, 13, 2e-6)
    assert np.allclose(np.linalg.inv(A), np.linalg.pinv(A), rtol=1e-10, atol=1e-22)


def test_gaussian_matches_scipy():
    ndi = pytest.importorskip('scipy.ndimage')
    rng = np.random.default_rng(0)
    a = rng.standard_normal((17, 23))
    for mode in ('reflect', 'constant'):
        ref = ndi.gaussian_filter(a, 1.0, mode=mode)
        got = oracle.gaussian_filter(a, 1.0, mode=mode)
        assert np.max(np.abs(ref - got)) < 1e-14


def test_electroflux_limits():
    # no voltage: pure diffusion D/d (cA - cB) (sim_toolbox.py:24 docstring)
    f = oracle.electroflux(np.array([10.0]), np.array([4.0]), 1e-18, 7.5e-9, 1.0,
                           np.array([0.0]), 310.0, 96485.0, 8.314)
    assert np.isclose(f[0], 1e-18 / 7.5e-9 * (10.0 - 4.0), rtol=1e-12)
    # Nernst potential: zero flux
    cA, cB, z, T = 145.0, 12.0, 1.0, 310.0
    v = (8.314 * T / (z * 96485.0)) * np.log(cA / cB)
    f = oracle.electroflux(np.array([cA]), np.array([cB]), 1e-18, 7.5e-9, z,
                           np.array([v]), T, 96485.0, 8.314)
    assert abs(f[0]) < 1e-10 * 1e-18 / 7.5e-9 * cA
