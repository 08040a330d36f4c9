"""GPU environment fields (``bx_env_fields``) against BETSE's get_current.

The golden fixtures hold BETSE's v_env, E_env_x/y, J_env_x/y and B_field after
the second checkpoint (``physics/ion_current.py:50-171``).  The dense operator
is ``pinv(makeLaplacian)`` as BETSE builds it (``finitediff.py:252-431``).

Tolerances, plain FP64 step:
* v_env: 1e-10 of max|v_env| plus the Vmem cancellation floor (v_env is -vm/2
  smoothed without ECM; with ECM it is the environment charge potential);
* E_env: 1e-8 relative (a difference of neighbouring v_env values);
* J_env, B_field with ECM: 1e-6 relative, the bound the NumPy oracle itself
  meets against BETSE (the divergence-free part of a mostly irrotational
  current cancels);
* J_env without ECM: the field is a pure gradient, so its divergence-free part
  is round-off; bounded by 1e-11 of sigma*max|E_env|.
Split step (no ECM): |v_env - ref| < 1e-6 V, as Vmem.
"""
import numpy as np
import pytest

import golden_io as gi
import oracle

pytestmark = pytest.mark.gpu


def _run(d, precision):
    from betse_gb300.engine import ClusterEngine
    cg, sp, Dm, st, D_env = gi.engine_inputs(d)
    g = gi.geometry(d)
    cp = int(d['meta_checkpoints'][1])
    lap_inv = np.linalg.pinv(oracle.fields.make_laplacian(*g.grid_shape, g.delta))
    with ClusterEngine(cg, sp, precision) as eng:
        eng.set_membrane_diffusivity(Dm)
        if sp.is_ecm:
            eng.set_env_diffusivity(D_env)
        eng.upload(**st)
        eng.set_lap_env_inv(lap_inv)
        eng.step(cp, outputs=True)
        f = eng.env_fields(g.D_env_weight)
        f2 = eng.env_fields(g.D_env_weight)
    return f, f2, cp, g


@pytest.mark.parametrize('name', gi.CASES)
def test_env_fields_fp64_match_betse(name):
    d = gi.load(name)
    ecm = bool(d['par_is_ecm'])
    f, f2, cp, g = _run(d, 'fp64')
    for k in f:
        assert np.array_equal(f[k], f2[k]), k  # deterministic, no state change
    ref = {k: np.asarray(d[f's{cp}_{k}']).ravel() for k in f}
    vfl = gi.vm_floor(d, d[f's{cp}_cc_cells'])
    err_v = np.max(np.abs(f['v_env'] - ref['v_env']))
    assert err_v <= 1e-10 * np.max(np.abs(ref['v_env'])) + vfl, (err_v, vfl)
    for k in ('E_env_x', 'E_env_y'):
        assert gi.rel_err(f[k], ref[k]) < 1e-8, (k, gi.rel_err(f[k], ref[k]))
    if ecm:
        for k in ('J_env_x', 'J_env_y', 'B_field'):
            assert gi.rel_err(f[k], ref[k]) < 1e-6, (k, gi.rel_err(f[k], ref[k]))
    else:
        scale = g.sigma * np.max(np.abs(ref['E_env_x']))
        for k in ('J_env_x', 'J_env_y'):
            assert np.max(np.abs(f[k])) < 1e-11 * scale, (k, np.max(np.abs(f[k])), scale)


@pytest.mark.parametrize('name', [c for c in gi.CASES if c.startswith('noecm')])
def test_env_fields_split_match_betse(name):
    d = gi.load(name)
    if gi.polar(d):
        pytest.skip('the split form refuses cell polarizability (tested in the step parity tests)')
    f, _, cp, g = _run(d, 'split')
    ref = np.asarray(d[f's{cp}_v_env']).ravel()
    assert np.max(np.abs(f['v_env'] - ref)) < 1e-6
    for k in ('E_env_x', 'E_env_y'):
        r = np.asarray(d[f's{cp}_{k}']).ravel()
        assert gi.rel_err(f[k], r) < 1e-3, (k, gi.rel_err(f[k], r))


def test_env_fields_match_oracle_on_perturbed_weights():
    """A non-uniform D_env_weight gives a current with a divergence-free part;
    the GPU chain (double-float products) follows the oracle's FP64 chain."""
    d = gi.load('noecm_r50_s7')
    from betse_gb300.engine import ClusterEngine
    cg, sp, Dm, _, _ = gi.engine_inputs(d)
    g, p = gi.geometry(d), gi.params(d)
    # start from a checkpoint: the initial state is near-neutral (Vmem ~ 0)
    pre = f"s{int(d['meta_checkpoints'][1])}"
    s = gi.state(d, prefix=pre)
    st = dict(vm=s.vm, cc_cells=s.cc_cells, cc_at_mem=s.cc_at_mem, cc_env=s.cc_env)
    rng = np.random.default_rng(5)
    w = rng.uniform(0.2, 1.0, size=int(np.prod(g.grid_shape)))
    lap_inv = np.linalg.pinv(oracle.fields.make_laplacian(*g.grid_shape, g.delta))
    with ClusterEngine(cg, sp, 'fp64') as eng:
        eng.set_membrane_diffusivity(Dm)
        eng.upload(**st)
        eng.set_lap_env_inv(lap_inv)
        eng.step(1, outputs=True)
        f = eng.env_fields(w)
    g.lap_inv = lap_inv
    g.D_env_weight = w
    ref = oracle.step(g, p, gi.state(d, prefix=pre), outputs=True)
    for k in ('v_env', 'E_env_x', 'E_env_y', 'J_env_x', 'J_env_y', 'B_field'):
        r = np.asarray(ref[k]).ravel()
        assert gi.rel_err(f[k], r) < 1e-8, (k, gi.rel_err(f[k], r))


def test_env_fields_need_output_step():
    from betse_gb300 import _lib
    from betse_gb300.engine import ClusterEngine
    d = gi.load('noecm_r20_s2')
    cg, sp, Dm, st, _ = gi.engine_inputs(d)
    g = gi.geometry(d)
    with ClusterEngine(cg, sp, 'fp64') as eng:
        eng.set_membrane_diffusivity(Dm)
        eng.upload(**st)
        with pytest.raises(_lib.BxLibraryError):
            eng.env_fields()  # no operator yet
        eng.set_lap_env_inv(np.linalg.pinv(oracle.fields.make_laplacian(*g.grid_shape, g.delta)))
        eng.step(2, outputs=False)
        with pytest.raises(_lib.BxLibraryError):
            eng.env_fields()  # last step computed no outputs
