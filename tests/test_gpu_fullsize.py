"""Parity at the benchmark sizes: the CUDA step against the oracle.

The oracle (checked against BETSE's own results in test_oracle_golden.py) runs
a few time steps of the full benchmark clusters: ~100k cells without
extracellular spaces and ~20k cells with a 199x200 environment grid.
Tolerances as in test_gpu_parity.py: FP64 concentrations 1e-10 relative, Vmem
1e-10 relative plus the FP64 cancellation floor of the charge sum; split form
|Vmem - Vmem_oracle| < 1e-6 V.
"""
import numpy as np
import pytest

import golden_io as gi
import oracle
from oracle.adapt import from_workload

pytestmark = pytest.mark.gpu

CASES = {
    'cluster100k': dict(radius=1450e-6, seed=3, is_ecm=False, dt=5e-3, dm_range=(1e-19, 1e-16),
                        grid_size=20),
    'ecm20k': dict(radius=662e-6, seed=11, is_ecm=True, dt=5e-3, dm_range=(1e-19, 1e-17),
                   grid_size=200, cell_space=25e-9),
}


def _vm_floor(p, g, cc):
    charge = (np.abs(p.zs * p.F)[:, None] * np.abs(cc)).sum(axis=0)
    return 4 * np.finfo(np.float64).eps * np.max(charge * g.diviterm) / p.cm


def _engine(g, p, Dm, st, D_env, precision):
    from betse_gb300.engine import ClusterEngine
    e = ClusterEngine(g, p, precision)
    e.set_membrane_diffusivity(Dm)
    if D_env is not None:
        e.set_env_diffusivity(D_env)
    e.upload(**st)
    return e


@pytest.fixture(scope='module', params=sorted(CASES))
def case(request):
    from betse_gb300 import generator as gen
    kw = dict(CASES[request.param])
    radius, seed = kw.pop('radius'), kw.pop('seed')
    g, p, Dm, st, D_env = gen.workload(radius, seed, **kw)
    return request.param, g, p, Dm, st, D_env


def test_fp64_matches_oracle_at_full_size(case):
    name, g, p, Dm, st, D_env = case
    n = 4
    geo, par, s = from_workload(g, p, Dm, st, D_env)
    for _ in range(n):
        oracle.step(geo, par, s)
    with _engine(g, p, Dm, st, D_env, 'fp64') as e:
        e.step(n)
        e.check_stable()
        out = e.download()
    err = np.max(np.abs(out['vm'] - s.vm))
    bound = 1e-10 * np.max(np.abs(s.vm)) + _vm_floor(p, g, s.cc_cells)
    assert err <= bound, (name, err, bound)
    assert gi.rel_err(out['cc_cells'], s.cc_cells) < 1e-10
    if p.is_ecm:
        assert gi.rel_err(out['cc_env'], s.cc_env) < 1e-10
        assert gi.rel_err(out['E_env_x'], np.ravel(s.E_env_x)) < 1e-8
    else:
        assert gi.rel_err(out['cc_env'], s.cc_env[:, 0]) < 1e-10


def test_split_matches_oracle_at_full_size(case):
    name, g, p, Dm, st, D_env = case
    n = 10
    geo, par, s = from_workload(g, p, Dm, st, D_env)
    for _ in range(n):
        oracle.step(geo, par, s)
    with _engine(g, p, Dm, st, D_env, 'split') as e:
        e.step(n)
        e.check_stable()
        out = e.download()
    err = np.max(np.abs(out['vm'] - s.vm))
    assert err < 1e-6, (name, err)
    assert gi.rel_err(out['cc_cells'], s.cc_cells) < 1e-6


# ---- the full run length of each workload against the C restatement of the
# oracle (OpenMP; the same step, pinned to BETSE in test_oracle_c.py)
HORIZON = {'cluster100k': 1000, 'ecm20k': 500}
CHECKPOINTS = (1, 10, 100, 500, 1000)


def _c_stepper(g, p, Dm, st, D_env):
    cstep = pytest.importorskip('oracle.cstep')
    try:
        cstep.build()
    except Exception as e:          # no C compiler on this host
        pytest.skip(f'C restatement not built: {e}')
    geo, par, s = from_workload(g, p, Dm, st, D_env)
    return cstep.Stepper(geo, par, s)


@pytest.mark.parametrize('precision', ['fp64', 'split'])
def test_full_horizon_matches_c_oracle(case, precision):
    """FP64: concentrations within 1e-10 relative and Vmem within 1e-10
    relative plus the FP64 cancellation floor at every checkpoint of the
    run; split form (the kernel the autotuner picks): |Vmem - Vmem_oracle| <
    1e-6 V at every checkpoint.  The per-checkpoint errors are printed (run
    with -s to see config 3's error curve)."""
    name, g, p, Dm, st, D_env = case
    n_total = HORIZON[name]
    ref = _c_stepper(g, p, Dm, st, D_env)
    curve = []
    with _engine(g, p, Dm, st, D_env, precision) as e:
        if precision == 'split':
            e.autotune(20)
        done = 0
        for cp in [c for c in CHECKPOINTS if c <= n_total]:
            e.step(cp - done)
            ref.step(cp - done)
            done = cp
            e.check_stable()
            out = e.download()
            r = ref.state()
            err = float(np.max(np.abs(out['vm'] - r['vm'])))
            e_cc = gi.rel_err(out['cc_cells'], r['cc_cells'])
            e_env = gi.rel_err(out['cc_env'], r['cc_env'] if p.is_ecm else r['cc_env'][:, 0])
            curve.append((cp, err, e_cc, e_env))
            if precision == 'fp64':
                bound = 1e-10 * np.max(np.abs(r['vm'])) + _vm_floor(p, g, r['cc_cells'])
                assert err <= bound, (name, cp, err, bound)
                assert e_cc < 1e-10, (name, cp, e_cc)
                assert e_env < 1e-10, (name, cp, e_env)
                if p.is_ecm:
                    assert gi.rel_err(out['E_env_x'], np.ravel(r['E_env_x'])) < 1e-8, (name, cp)
                    assert gi.rel_err(out['E_env_y'], np.ravel(r['E_env_y'])) < 1e-8, (name, cp)
            else:
                assert err < 1e-6, (name, cp, err)
                assert e_cc < 1e-5, (name, cp, e_cc)
        kernel = e.launch_config()
    print(f'\n{name} {precision} launch {kernel}: step, max|dVm| (V), cc rel, env rel')
    for row in curve:
        print('  %5d  %.3e  %.3e  %.3e' % row)
