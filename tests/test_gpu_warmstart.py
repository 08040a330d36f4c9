"""The learned warm start against the plain init (same stepping, same residual test).

Fresh clusters (seeds outside the training set) step from the uniform initial
profile and from the committed network's prediction until max |dVm/dt| < 1e-6
V/s.  The warm start must reach the test on every cluster the plain method
settles (one whose explicit step diverges is left out of both arms) and cut the mean
number of steps per cluster at least 3x on this small sample (bench.py
reports the same measurement on a larger sample of fresh 5000-cell clusters)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_warm_start_reaches_steady_state_faster():
    from betse_gb300 import warmstart as ws
    w = ws.WarmStart()
    r = ws.evaluate(w, n_clusters=8, n_cells=2000, seed=4242, max_steps=1_500_000, log=lambda s: None)
    warm = r['warm'][0]
    assert r['cold']['passed'] >= 6          # the plain method settles these clusters
    assert warm['passed'] == r['cold']['passed'] and warm['unstable'] == 0
    assert warm['speedup_mean_steps'] >= 3.0, warm


def test_prediction_is_a_consistent_state():
    from betse_gb300 import generator as gen
    from betse_gb300 import warmstart as ws
    w = ws.WarmStart()
    gs, ps, Dms, sts = gen.sweep_workload(4, 777, cells_range=(800, 1200), dt=ws.DT,
                                          mult_range=ws.MULT_RANGE, pump_range=ws.PUMP_RANGE)
    pred, _ = w.predict(gs, ps, Dms)
    for g, p, s, y in zip(gs, ps, sts, pred):
        assert y.shape == (g.n_cells, ws.N_OUT) and np.all(np.isfinite(y))
        st = ws.warm_state(g, p, s, y)
        if st is None:
            continue
        vm_cell = st['vm'][np.asarray(g.cell_mem_ptr)[:-1]]
        assert np.allclose(vm_cell, y[:, -1], rtol=1e-6, atol=1e-9)
