"""tcgen05 BF16x3 dense-operator products against FP64 NumPy.

Tolerances (max|Y - Y_ref| / max|Y_ref|):
* one BF16x3 GEMM: 1e-4 -- the split keeps ~16 significand bits of each
  operand and drops lo*lo (2^-16 relative), accumulation is FP32;
* with one refinement step against the forward operator L (A = L^-1): 1e-6,
  and at least 20x below the unrefined error (the step multiplies the error
  by ||(A_bf16x3 - A) L||, small for a well-conditioned grid Laplacian).
"""
import numpy as np
import pytest

import golden_io as gi
import oracle

pytestmark = pytest.mark.gpu


def _op(A, forward=None):
    from betse_gb300.dense import DenseOperator
    return DenseOperator(A, forward)


@pytest.mark.parametrize('n,nrhs', [(300, 40), (2500, 300), (128, 128), (64, 1)])
def test_bf16x3_gemm_matches_fp64(n, nrhs):
    rng = np.random.default_rng(n + nrhs)
    A = rng.standard_normal((n, n))
    X = rng.standard_normal((n, nrhs))
    with _op(A) as op:
        Y = op.apply(X)
    ref = A @ X
    assert gi.rel_err(Y, ref) < 1e-4, gi.rel_err(Y, ref)
    assert gi.rel_err(Y, ref) > 0  # the tensor-core path, not an FP64 copy


def test_refinement_with_grid_laplacian():
    """lapENVinv = inverse of the Dirichlet 5-point Laplacian (finitediff.py:252-431)."""
    import scipy.sparse as sp
    L = oracle.fields.make_laplacian(17, 23, 2.5e-6)
    A = np.linalg.inv(L)
    rng = np.random.default_rng(3)
    X = rng.standard_normal((L.shape[0], 70))
    ref = A @ X
    with _op(A, sp.csr_matrix(L)) as op:
        y0 = op.apply(X)
        y1 = op.apply(X, refine=True)
    e0, e1 = gi.rel_err(y0, ref), gi.rel_err(y1, ref)
    assert e0 < 1e-4, e0
    assert e1 < 1e-6 and e1 < e0 / 20, (e0, e1)


def test_column_scale_and_cluster_batch():
    """Clusters sharing a grid shape share lapENVinv = delta^2 K(shape): one GEMM
    with a per-column delta^2 reproduces each cluster's own product."""
    import scipy.sparse as sp
    shape = (19, 20)
    K = np.linalg.inv(oracle.fields.make_laplacian(*shape, 1.0))
    deltas = np.array([2.1e-6, 3.3e-6, 4.0e-6])
    rng = np.random.default_rng(11)
    X = rng.standard_normal((K.shape[0], 2 * len(deltas)))
    scale = np.repeat(deltas ** 2, 2)
    with _op(K, sp.csr_matrix(oracle.fields.make_laplacian(*shape, 1.0))) as op:
        Y = op.apply(X, refine=True, col_scale=scale)
    for c, d in enumerate(deltas):
        Ac = np.linalg.inv(oracle.fields.make_laplacian(*shape, d))
        ref = Ac @ X[:, 2 * c:2 * c + 2]
        assert gi.rel_err(Y[:, 2 * c:2 * c + 2], ref) < 1e-6


def test_repeat_is_deterministic():
    rng = np.random.default_rng(9)
    A = rng.standard_normal((700, 700))
    X = rng.standard_normal((700, 130))
    with _op(A) as op:
        assert np.array_equal(op.apply(X), op.apply(X))


def test_lapgj_inverse_products_match_betse():
    """BETSE's own cells.lapGJinv (graphLaplacian, cells.py:1845-1894) applied
    on the tensor cores: the pressures.py:59 product sim.PP = lapGJinv @
    (-div_u_osmo rho dt) against BETSE's, and a block of 64 right-hand sides
    against FP64, within the BF16x3 bound (no refinement: BETSE's lapGJ is not
    the inverse of its lapGJinv, so the forward-operator step does not apply).
    The errors are printed."""
    import os
    d = dict(np.load(os.path.join(gi.GOLDEN, 'lapgj_r80_s1.npz')))
    A = d['lapGJinv']
    rhs = -d['press_div_u_osmo'] * d['press_rho'] * d['press_dt']
    rng = np.random.default_rng(3)
    X = np.concatenate([rhs[:, None], rng.standard_normal((len(rhs), 63))], axis=1)
    with _op(A) as op:
        Y = op.apply(X)
    e_pp = gi.rel_err(Y[:, 0], d['press_PP'])
    e_blk = gi.rel_err(Y, A @ X)
    print(f'\nlapGJinv ({len(A)} cells) on tcgen05 BF16x3: pressures product rel err {e_pp:.2e}, '
          f'64-column block {e_blk:.2e}')
    assert e_pp < 1e-4 and e_blk < 1e-4
