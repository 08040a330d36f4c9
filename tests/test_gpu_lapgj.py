"""cells.lapGJinv at any size: the multigrid-preconditioned CG solver
(bx_graph_*, csrc/bx_graph.cu) against BETSE's own operator and against the
dense FP64 construction.

* BETSE's lapGJinv (tests/golden/lapgj_r80_s1.npz, made by BETSE's
  Cells.graphLaplacian on its own DEC mesh): LapGJ.apply on a block of
  right-hand sides within 1e-10 relative, and the pressures.py:59 product
  sim.PP = lapGJinv @ (-div_u_osmo rho dt) within 1e-10; L+ against
  numpy's pinv of the graph Laplacian;
* a generated 4000-cell cluster: apply against lap_gj_operators (dense FP64
  on the host) within 1e-10, and the dense operator built on the GPU from
  the solver (BF16x3 tensor-core tiles) within the BF16x3 bound 1e-4;
* the 100k-cell cluster of the benchmark: every column converges to 1e-12
  relative residual, the result is orthogonal to the constants, and one
  column applied alone equals the same column applied in a block (columns
  are independent; the two stop at different iterations, so within 1e-6).
Solves for the 1e-10 comparisons run to 1e-14 relative residual: the error
of a CG iterate is bounded by the residual times the condition number of L
(~400 at 267 cells, ~6e3 at 4000).
"""
import os

import numpy as np
import pytest

import golden_io as gi

pytestmark = pytest.mark.gpu


def _fixture():
    return dict(np.load(os.path.join(gi.GOLDEN, 'lapgj_r80_s1.npz')))


def _args(d):
    return d['mesh_tri_edges'], d['mesh_tri_edge_len'], d['mesh_vor_edge_len'], d['mesh_vor_sa']


def test_apply_matches_betse_lapgjinv():
    from betse_gb300.dense import LapGJ
    d = _fixture()
    A = d['lapGJinv']
    rhs = -d['press_div_u_osmo'] * d['press_rho'] * d['press_dt']
    rng = np.random.default_rng(5)
    X = np.concatenate([rhs[:, None], rng.standard_normal((len(rhs), 40))], axis=1)
    with LapGJ(*_args(d), max_rhs=64) as op:
        Y = op.apply(X, tol=1e-14)
        print(f'\nlapGJinv ({len(A)} cells), levels {op.level_sizes}: {op.last_iters} CG iterations, '
              f'residual {op.last_rel_res:.1e}')
    assert gi.rel_err(Y, A @ X) < 1e-10
    assert gi.rel_err(Y[:, 0], d['press_PP']) < 1e-10


def test_solve_matches_pinv_of_the_graph_laplacian():
    from betse_gb300.dense import LapGJ, _incidence
    d = _fixture()
    n = len(d['mesh_vor_sa'])
    D = _incidence(d['mesh_tri_edges'], n).toarray()
    Lp = np.linalg.pinv(D.T @ D)
    B = np.random.default_rng(6).standard_normal((n, 7))
    with LapGJ(*_args(d), max_rhs=8) as op:
        X = op.solve(B, tol=1e-14)
    assert gi.rel_err(X, Lp @ B) < 1e-10


@pytest.fixture(scope='module')
def cluster4k():
    from betse_gb300.dense import lap_gj_inputs
    from betse_gb300.generator import make_cluster
    gc = make_cluster(300e-6, 5)
    return lap_gj_inputs(gc.geom, gc.cell_centres)


def test_apply_matches_dense_construction(cluster4k):
    from betse_gb300.dense import LapGJ, lap_gj_operators
    inv, _ = lap_gj_operators(*cluster4k)
    X = np.random.default_rng(7).standard_normal((len(inv), 96))
    with LapGJ(*cluster4k, max_rhs=64) as op:
        Y = op.apply(X, tol=1e-14)
        print(f'\n{len(inv)} cells, levels {op.level_sizes}: {op.last_iters} CG iterations')
    assert gi.rel_err(Y, inv @ X) < 1e-10


def test_dense_build_on_the_gpu(cluster4k):
    from betse_gb300.dense import LapGJ, lap_gj_operators
    inv, _ = lap_gj_operators(*cluster4k)
    X = np.random.default_rng(8).standard_normal((len(inv), 128))
    with LapGJ(*cluster4k, max_rhs=256) as op:
        dense = op.dense()
        try:
            Y = dense.apply(X)
        finally:
            dense.close()
    e = gi.rel_err(Y, inv @ X)
    print(f'\ndense lapGJinv built on the GPU ({len(inv)} cells), BF16x3 products: rel err {e:.2e}')
    assert e < 1e-4


def test_full_size_apply_converges():
    import torch
    from betse_gb300.dense import LapGJ, lap_gj_inputs
    from betse_gb300.generator import make_cluster
    gc = make_cluster(1450e-6, 3)
    args = lap_gj_inputs(gc.geom, gc.cell_centres)
    n = len(args[3])
    X = torch.randn(n, 32, dtype=torch.float64, device='cuda', generator=torch.Generator('cuda').manual_seed(1))
    with LapGJ(*args, max_rhs=32) as op:
        Y = op.apply(X, tol=1e-12)
        it = op.last_iters
        y0 = op.apply(X[:, 5:6].contiguous(), tol=1e-12)
    print(f'\n{n} cells: {it} CG iterations to 1e-12')
    assert it < 200
    assert float(Y.sum(dim=0).abs().max()) <= 1e-9 * float(Y.abs().max()) * n ** 0.5
    assert gi.rel_err(y0[:, 0].cpu().numpy(), Y[:, 5].cpu().numpy()) < 1e-6
