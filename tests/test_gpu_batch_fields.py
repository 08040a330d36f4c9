"""Batched environment fields (one tcgen05 GEMM per grid shape) against each
cluster's own field chain (double-float products, bx_env_fields).

Clusters of several grid shapes and spacings step together; each
cluster's fields must match the single-cluster path: v_env to 1e-12 relative
(same stencils), E_env and the divergence-free current to 1e-6 of their
maximum (BF16x3 products with one FP64 refinement against double-float
products), B_field to 1e-6 of its maximum."""
import numpy as np
import pytest

import golden_io as gi
import oracle

pytestmark = pytest.mark.gpu


def _clusters():
    from betse_gb300 import generator as gen
    out = []
    for k, (n, grid) in enumerate(((260, 12), (400, 16), (330, 12), (500, 16), (300, 12))):
        R = np.sqrt(n / 0.0456) * 1e-6
        out.append(gen.workload(R, 50 + k, dt=1e-2, grid_size=grid))
    return out


def test_batch_fields_match_single_cluster_fields():
    from betse_gb300.engine import BatchEngine, ClusterEngine
    cl = _clusters()
    rng = np.random.default_rng(1)
    ws = [rng.uniform(0.3, 1.0, g.n_grid) for g, *_ in cl]
    n = 30
    singles = []
    for (g, p, Dm, st, _), w in zip(cl, ws):
        with ClusterEngine(g, p, 'fp64') as e:
            e.set_membrane_diffusivity(Dm)
            e.upload(**st)
            e.set_lap_env_inv(np.linalg.inv(oracle.fields.make_laplacian(*g.grid_shape, g.delta)))
            e.step(n, outputs=True)
            singles.append(e.env_fields(w))
    geoms = [c[0] for c in cl]
    assert len({tuple(g.grid_shape) for g in geoms}) >= 2
    b = BatchEngine(geoms, [c[1] for c in cl], 'fp64')
    b.set_membrane_diffusivity([c[2] for c in cl])
    b.upload_states([c[3] for c in cl])
    b.step(n, outputs=True)
    from betse_gb300 import _lib
    with pytest.raises(_lib.BxLibraryError):
        b.env_fields(ws)          # no operator for the shapes yet
    done = set()
    for g in geoms:
        if tuple(g.grid_shape) not in done:
            done.add(tuple(g.grid_shape))
            b.set_lap_env_inv_shape(np.linalg.inv(oracle.fields.make_laplacian(*g.grid_shape, g.delta)),
                                    g.grid_shape, g.delta)
    fb = b.env_fields(ws)
    b.close()
    for one, bat in zip(singles, fb):
        assert gi.rel_err(bat['v_env'], one['v_env']) < 1e-12
        for k in ('E_env_x', 'E_env_y', 'J_env_x', 'J_env_y', 'B_field'):
            assert gi.rel_err(bat[k], one[k]) < 1e-6, (k, gi.rel_err(bat[k], one[k]))
