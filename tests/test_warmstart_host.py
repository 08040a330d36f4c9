"""Host logic of the learned warm start (no GPU)."""
import numpy as np

from betse_gb300 import generator as gen
from betse_gb300 import warmstart as ws
from oracle import generator as ogen


def _cluster():
    # the NumPy restatement of the generator stands in for the GPU one here
    R = np.sqrt(300 / 0.0456) * 1e-6
    return gen.workload(R, 21, dt=1e-2, cluster=ogen.make_cluster(R, 21))


def test_identity_prediction_reproduces_initial_state():
    g, p, Dm, st, _ = _cluster()
    y = ws.cell_targets(g, st, st)
    s = ws.warm_state(g, p, st, y)
    assert np.allclose(s['cc_cells'], st['cc_cells'], rtol=1e-12, atol=0)
    assert np.allclose(s['vm'], st['vm'], rtol=0, atol=1e-12)
    assert np.allclose(s['cc_env'], st['cc_env'], rtol=1e-14)


def test_warm_state_is_consistent():
    g, p, Dm, st, _ = _cluster()
    rng = np.random.default_rng(0)
    y = ws.cell_targets(g, st, st)
    y[:, :5] += rng.normal(0, 0.05, (g.n_cells, 5))
    y[:, 5] = rng.uniform(-0.06, -0.02, g.n_cells)
    s = ws.warm_state(g, p, st, y)
    # Vmem is the predicted one, through BETSE's charge relation (sim.py:2027-2029)
    vm_cell = s['vm'][np.asarray(g.cell_mem_ptr)[:-1]]
    assert np.allclose(vm_cell, y[:, 5], rtol=1e-6, atol=1e-9)
    # every ion's total amount (cells + well-mixed environment) is kept
    tot0 = st['cc_cells'] @ g.cell_vol + np.asarray(st['cc_env']) * g.n_mems * p.vol_env
    tot1 = s['cc_cells'] @ g.cell_vol + s['cc_env'] * g.n_mems * p.vol_env
    assert np.allclose(tot0, tot1, rtol=1e-12)
    assert np.all(s['cc_cells'] > 0)
    assert np.array_equal(s['cc_at_mem'], s['cc_cells'][:, g.mem_to_cells])


def test_features_and_graph_shapes():
    g, p, Dm, st, _ = _cluster()
    x = ws.cell_features(g, p, Dm)
    assert x.shape == (g.n_cells, 10) and np.all(np.isfinite(x))
    ptr, nbr = ws.graph_of([g, g])
    assert len(ptr) == 2 * g.n_cells + 1 and nbr.max() < 2 * g.n_cells
    assert np.all(nbr[ptr[g.n_cells]:] >= g.n_cells)


def test_unusable_prediction_returns_none():
    g, p, Dm, st, _ = _cluster()
    y = ws.cell_targets(g, st, st)
    y[3, 5] = 2.0            # far outside any membrane potential
    assert ws.warm_state(g, p, st, y) is None
    y = ws.cell_targets(g, st, st)
    y[0, 0] = np.nan
    assert ws.warm_state(g, p, st, y) is None
