"""Dense inverse-Laplacian products with batched right-hand sides (tcgen05).

``DenseOperator(A)`` keeps ``A`` (``cells.lapGJinv`` or ``cells.lapENVinv``,
FP64 ``[n, n]``) on the GPU as BF16 hi/lo tiles; ``apply(X)`` returns
``A @ X`` for a block of right-hand sides ``X [n, nrhs]`` -- what BETSE
computes one column at a time with ``np.dot(cells.lapGJinv, rhs)``
(``betse/science/physics/pressures.py:59``) or ``np.dot(cells.lapENVinv, rhs)``
(``physics/ion_current.py:90,170``).  With the forward operator ``L`` that
``A`` inverts (``set_forward``), ``apply(X, refine=True)`` adds one FP64
refinement step ``Y += A (X - L Y)``.

Device memory for X and Y comes from PyTorch (CUDA tensors); numpy inputs are
copied to the current device and the result is returned as numpy.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib


def lap_gj_operators(tri_edges, tri_edge_len, vor_edge_len, vor_sa):
    """``cells.lapGJinv`` and ``cells.lapGJ`` (``Cells.graphLaplacian``,
    ``betse/science/cells.py:1845-1894``) from the DEC mesh of the cluster
    (``cells.mesh.tri_edges``, ``tri_edge_len``, ``vor_edge_len``, ``vor_sa``).

    BETSE forms ``pinv(D) W (-pinv(D)^T) A`` with ``D`` the edge-vertex
    incidence matrix (``-1`` at ``tri_edges[:, 0]``, ``+1`` at
    ``tri_edges[:, 1]``), ``W = diag(tri_len / vor_len)``, ``A = diag(vor_sa)``
    and ``pinv(D)`` from a dense SVD of the ``[edges, cells]`` matrix.  For a
    connected graph ``pinv(D) = L+ D^T`` with ``L = D^T D`` the (sparse,
    unweighted) graph Laplacian and ``L+ = (L + J/n)^-1 - J/n``, so

        lapGJinv = -L+ (D^T W D) L+ A,

    one dense solve of size ``n`` instead of the SVD of an ``[edges, n]``
    matrix (FP64, on the host: a set-up step, O(n^3)).  Note that ``lapGJ`` is
    not the inverse of ``lapGJinv`` (their product differs from the identity
    by ~0.25 on BETSE's own clusters): BETSE pairs a pseudo-inverse of the
    unweighted incidence with a weighted forward operator."""
    import scipy.sparse as sp
    e = np.asarray(tri_edges, np.int64)
    A = np.asarray(vor_sa, np.float64)
    n, m = len(A), len(e)
    rows = np.repeat(np.arange(m), 2)
    D = sp.csr_matrix((np.tile([-1.0, 1.0], m), (rows, e.ravel())), shape=(m, n))
    w = np.asarray(tri_edge_len, np.float64) / np.asarray(vor_edge_len, np.float64)
    L = (D.T @ D).toarray()
    J = np.full((n, n), 1.0 / n)
    Lp = np.linalg.solve(L + J, np.eye(n)) - J
    Lw = (D.T @ sp.diags(w) @ D).toarray()
    lap_inv = -(Lp @ Lw @ Lp) * A[None, :]
    lap = -(sp.diags(1.0 / A) @ (D.T @ sp.diags(1.0 / w) @ D)).toarray()
    return lap_inv, lap


class DenseOperator:
    def __init__(self, A, forward=None):
        A = np.ascontiguousarray(np.asarray(A, np.float64))
        if A.ndim != 2 or A.shape[0] != A.shape[1]:
            raise ValueError('A must be square')
        self.lib = _lib.load()
        self.n = A.shape[0]
        h = ct.c_void_p()
        _lib.check(self.lib.bx_dense_op_create(_lib.dptr(A), self.n, ct.byref(h)), 'bx_dense_op_create')
        self.h = h
        if forward is not None:
            self.set_forward(forward)

    def set_forward(self, L):
        """L: the operator A inverts, as a scipy.sparse matrix or dense array."""
        try:
            import scipy.sparse as sp
            L = sp.csr_matrix(L)
        except ImportError:  # pragma: no cover - scipy is present where tests run
            raise
        if L.shape != (self.n, self.n):
            raise ValueError('forward operator shape mismatch')
        ptr = np.ascontiguousarray(L.indptr, np.int32)
        col = np.ascontiguousarray(L.indices, np.int32)
        val = np.ascontiguousarray(L.data, np.float64)
        _lib.check(self.lib.bx_dense_op_set_forward(self.h, _lib.iptr(ptr), _lib.iptr(col), _lib.dptr(val)),
                   'bx_dense_op_set_forward')

    def apply(self, X, refine=False, col_scale=None, stream=None):
        import torch
        as_numpy = not isinstance(X, torch.Tensor)
        Xt = torch.as_tensor(np.asarray(X, np.float64) if as_numpy else X, dtype=torch.float64,
                             device='cuda').contiguous()
        squeeze = Xt.ndim == 1
        if squeeze:
            Xt = Xt[:, None].contiguous()
        if Xt.shape[0] != self.n:
            raise ValueError('X must have n rows')
        nrhs = Xt.shape[1]
        Y = torch.empty_like(Xt)
        sc = None
        if col_scale is not None:
            sc = torch.as_tensor(np.asarray(col_scale, np.float64), device='cuda').contiguous()
            if sc.numel() != nrhs:
                raise ValueError('col_scale needs one value per column')
        st = torch.cuda.current_stream().cuda_stream if stream is None else int(stream)
        _lib.check(self.lib.bx_dense_op_apply(self.h, ct.c_void_p(Xt.data_ptr()), ct.c_void_p(Y.data_ptr()),
                                              int(nrhs), None if sc is None else ct.c_void_p(sc.data_ptr()),
                                              int(bool(refine)), ct.c_void_p(st)), 'bx_dense_op_apply')
        self.check()
        if squeeze:
            Y = Y[:, 0]
        return Y.cpu().numpy() if as_numpy else Y

    def check(self):
        t = ct.c_int()
        _lib.check(self.lib.bx_dense_op_status(self.h, ct.byref(t)), 'bx_dense_op_status')
        if t.value:
            raise RuntimeError('tcgen05 pipeline wait timed out')

    def time(self, nrhs, n_iter=10):
        """Mean ms of one GEMM launch for nrhs right-hand sides."""
        import torch
        X = torch.randn(self.n, nrhs, dtype=torch.float64, device='cuda')
        Y = torch.empty_like(X)
        ms = ct.c_double()
        _lib.check(self.lib.bx_dense_op_time(self.h, ct.c_void_p(X.data_ptr()), ct.c_void_p(Y.data_ptr()),
                                             int(nrhs), int(n_iter), ct.byref(ms)), 'bx_dense_op_time')
        self.check()
        return ms.value

    def close(self):
        if getattr(self, 'h', None) is not None and self.h.value:
            self.lib.bx_dense_op_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
