"""Size-independent properties of the step on the full 100k-cell benchmark
cluster, where the oracle is too slow to follow many steps.

* Gap junctions only exchange ions between cells: with the transmembrane
  fluxes and the pump switched off, each ion's amount in the cells,
  sum_c vol_c c_c, stays put. BETSE's GHK flux is antisymmetric under swapping
  the two cells, and partners share area and weight. The total moves only by
  rounding.
* With every flux switched off the step is a fixed point: after one step
  (which recomputes Vmem from the charge) the state no longer changes, bit
  for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def cluster():
    from betse_gb300 import generator as gen
    g, p, Dm, st, _ = gen.workload(1450e-6, 3, is_ecm=False, dt=5e-3, dm_range=(1e-19, 1e-16), grid_size=20)
    # cells start apart (each scaled by its own factor, so each stays near
    # neutral), otherwise the junctions between identical cells carry nothing
    rng = np.random.default_rng(4)
    f = 1.0 + 0.02 * rng.uniform(-1.0, 1.0, size=g.n_cells)
    cc = np.asarray(st['cc_cells']) * f[None, :]
    m2c = np.asarray(g.mem_to_cells)
    st = dict(st, cc_cells=cc, cc_at_mem=cc[:, m2c].copy())
    return g, p, Dm, st


def _amounts(g, cc):
    return np.asarray(cc) @ np.asarray(g.cell_vol)


@pytest.mark.parametrize('precision,tol', [('fp64', 1e-12), ('split', 1e-10)])
def test_gap_junctions_conserve_cell_amounts(cluster, precision, tol):
    from betse_gb300.engine import ClusterEngine
    g, p, Dm, st = cluster
    with ClusterEngine(g, p.replace(alpha_NaK=0.0), precision) as e:
        e.set_membrane_diffusivity(np.zeros_like(Dm))
        e.upload(**st)
        e.step(20)
        e.check_stable()
        s = e.download()
    a0, a1 = _amounts(g, st['cc_cells']), _amounts(g, s['cc_cells'])
    moved = np.max(np.abs(np.asarray(s['cc_cells']) - np.asarray(st['cc_cells'])))
    assert moved > 0.0                       # the junctions did move ions between cells
    assert np.all(np.abs(a1 - a0) <= tol * np.abs(a0)), np.abs(a1 - a0) / np.abs(a0)
    # the environment saw no membrane flux
    assert np.array_equal(s['cc_env'], np.asarray(st['cc_env']).reshape(s['cc_env'].shape))


@pytest.mark.parametrize('precision', ['fp64', 'split'])
def test_no_flux_step_is_a_fixed_point(cluster, precision):
    from betse_gb300.engine import ClusterEngine
    g, p, Dm, st = cluster
    with ClusterEngine(g, p.replace(alpha_NaK=0.0, gj_surface=0.0), precision) as e:
        e.set_membrane_diffusivity(np.zeros_like(Dm))
        e.upload(**st)
        e.step(1)
        s1 = e.download()
        e.step(40)                           # graph-replayed chunks and eager steps
        s2 = e.download()
    for k in s1:
        assert np.array_equal(s1[k], s2[k]), k
    # the concentrations never moved (the split form keeps ~48 bits of them)
    tol = 0.0 if precision == 'fp64' else 1e-14
    c0 = np.asarray(st['cc_cells'])
    assert np.max(np.abs(s1['cc_cells'] - c0)) <= tol * np.max(np.abs(c0))
