"""Batched sweep: clusters stepped together in one launch give the same state
as each cluster stepped alone (bit-identical: a CTA never spans two clusters),
and per-cluster pump rates and diffusivities take effect."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _clusters():
    from betse_gb300 import generator as gen
    out = []
    for k, (R, mult, pm) in enumerate([(60e-6, 1.0, 1.0), (90e-6, 3.0, 0.2), (45e-6, 0.3, 5.0)]):
        g, p, Dm, st, _ = gen.workload(R, 10 + k, dt=5e-3, na_k_dm_mult=mult, pump_mult=pm)
        out.append((g, p, Dm, st))
    return out


@pytest.mark.parametrize('precision,persist', [('split', False), ('split', True), ('fp64', False)])
def test_batch_equals_individual_runs(precision, persist):
    from betse_gb300.engine import BatchEngine, ClusterEngine
    cl = _clusters()
    n = 150
    with BatchEngine([c[0] for c in cl], [c[1] for c in cl], precision) as b:
        if persist:
            b.set_launch_config(256, True)
        b.set_membrane_diffusivity([c[2] for c in cl])
        b.upload_states([c[3] for c in cl])
        b.step(n)
        b.check_stable()
        got = b.download_states()
    for (g, p, Dm, st), s in zip(cl, got):
        with ClusterEngine(g, p, precision) as e:
            e.set_membrane_diffusivity(Dm)
            e.upload(**st)
            e.step(n)
            ref = e.download()
        for k in ('vm', 'cc_cells', 'cc_at_mem', 'cc_env'):
            assert np.array_equal(s[k], ref[k]), k


def test_batch_pump_rates_differ():
    from betse_gb300.engine import BatchEngine
    cl = _clusters()
    same = [(cl[0][0], cl[0][1], cl[0][2], cl[0][3]),
            (cl[0][0], cl[0][1].replace(alpha_NaK=cl[0][1].alpha_NaK * 4), cl[0][2], cl[0][3])]
    with BatchEngine([c[0] for c in same], [c[1] for c in same], 'split') as b:
        b.set_membrane_diffusivity([c[2] for c in same])
        b.upload_states([c[3] for c in same])
        b.step(100)
        a, c = b.download_states()
    assert not np.array_equal(a['vm'], c['vm'])
    # a faster Na/K pump leaves less Na inside
    assert c['cc_cells'][0].mean() < a['cc_cells'][0].mean()
