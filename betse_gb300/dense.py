"""Dense inverse-Laplacian products with batched right-hand sides (tcgen05).

``DenseOperator(A)`` keeps ``A`` (``cells.lapGJinv`` or ``cells.lapENVinv``,
FP64 ``[n, n]``) on the GPU as BF16 hi/lo tiles; ``apply(X)`` returns
``A @ X`` for a block of right-hand sides ``X [n, nrhs]`` -- what BETSE
computes one column at a time with ``np.dot(cells.lapGJinv, rhs)``
(``betse/science/physics/pressures.py:59``) or ``np.dot(cells.lapENVinv, rhs)``
(``physics/ion_current.py:90,170``).  With the forward operator ``L`` that
``A`` inverts (``set_forward``), ``apply(X, refine=True)`` adds one FP64
refinement step ``Y += A (X - L Y)``.

``LapGJ`` applies ``cells.lapGJinv`` at any cluster size without forming it:
``-L+ Lw L+ A X`` with ``L+`` by multigrid-preconditioned conjugate gradients
on the GPU (``bx_graph_*``, ``csrc/bx_graph.cu``), and builds the dense
operator for the tensor cores column block by column block from it.

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


def _incidence(tri_edges, n):
    import scipy.sparse as sp
    e = np.asarray(tri_edges, np.int64)
    m = len(e)
    rows = np.repeat(np.arange(m), 2)
    return sp.csr_matrix((np.tile([-1.0, 1.0], m), (rows, e.ravel())), shape=(m, n))


def graph_levels(L, coarse_max=64):
    """The multigrid hierarchy of a graph Laplacian ``L`` (scipy sparse): the
    Galerkin operators ``P^T A P`` of aggregates of 4 consecutive nodes
    (node ``i`` -> ``i // 4``), level by level down to ``coarse_max`` nodes or
    fewer, and the pseudo-inverse of the coarsest.  Consecutive nodes should
    be neighbours (cells along a Z curve)."""
    import scipy.sparse as sp
    levels = [sp.csr_matrix(L)]
    while levels[-1].shape[0] > coarse_max:
        A = levels[-1]
        n = A.shape[0]
        P = sp.csr_matrix((np.ones(n), (np.arange(n), np.arange(n) // 4)), shape=(n, (n + 3) // 4))
        levels.append(sp.csr_matrix(P.T @ A @ P))
    for A in levels:
        A.sum_duplicates()
        A.sort_indices()
    return levels, np.linalg.pinv(levels[-1].toarray())


def lap_gj_inputs(geom, cell_centres, cell_height=1e-5, scale_cell=0.99):
    """``graphLaplacian``'s inputs for a generated cluster: one triangulation
    edge per pair of cells sharing a membrane (lower cell first), its length
    the distance between the cell centres, the dual (Voronoi) edge the shared
    membrane's unscaled length, and the cell areas unscaled from the volumes
    (membranes are scaled by ``scale_cell`` about the centre)."""
    m2c = np.asarray(geom.mem_to_cells, np.int64)
    nn = np.asarray(geom.nn_i, np.int64)
    c, d = m2c, m2c[nn]
    sel = c < d
    edges = np.column_stack((c[sel], d[sel]))
    cc = np.asarray(cell_centres, np.float64)
    tri_len = np.hypot(*(cc[edges[:, 0]] - cc[edges[:, 1]]).T)
    vor_len = np.asarray(geom.mem_sa)[sel] / (cell_height * scale_cell)
    vor_sa = np.asarray(geom.cell_vol) / (cell_height * scale_cell ** 2)
    return edges, tri_len, vor_len, vor_sa


class DenseOperator:
    @classmethod
    def _wrap(cls, handle, n):
        op = cls.__new__(cls)
        op.lib = _lib.load()
        op.n = int(n)
        op.h = handle
        return op

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


class LapGJ:
    """``cells.lapGJinv`` (``Cells.graphLaplacian``, ``cells.py:1845-1894``)
    on the GPU at any size, from the DEC mesh's ``tri_edges``,
    ``tri_edge_len``, ``vor_edge_len`` and ``vor_sa``, as
    ``lap_gj_operators`` takes them.

    ``apply(X)`` = ``lapGJinv @ X`` = ``-L+ Lw L+ (vor_sa * X)`` in FP64 (two
    multigrid-preconditioned CG solves per block of right-hand sides, each
    column to ``tol`` relative residual); ``solve(B)`` = ``L+ B``;
    ``dense()`` the operator as BF16x3 tensor-core tiles (``DenseOperator``),
    built from ``apply`` on identity columns.  The hierarchy groups 4
    consecutive cells, so cells ordered along a Z curve (the generator's
    order) converge fastest."""

    def __init__(self, tri_edges, tri_edge_len, vor_edge_len, vor_sa, max_rhs=64, coarse_max=64):
        import scipy.sparse as sp
        vor_sa = np.ascontiguousarray(vor_sa, np.float64)
        self.n = n = len(vor_sa)
        D = _incidence(tri_edges, n)
        w = np.asarray(tri_edge_len, np.float64) / np.asarray(vor_edge_len, np.float64)
        L = D.T @ D
        Lw = sp.csr_matrix(D.T @ sp.diags(w) @ D)
        Lw.sum_duplicates()
        Lw.sort_indices()
        levels, pinv = graph_levels(L, coarse_max)
        self.n_levels = len(levels)
        self.level_sizes = [A.shape[0] for A in levels]
        keep = []

        def lvl(A):
            ptr = np.ascontiguousarray(A.indptr, np.int32)
            col = np.ascontiguousarray(A.indices, np.int32)
            val = np.ascontiguousarray(A.data, np.float64)
            keep.extend([ptr, col, val])
            return _lib.BxGraphLevel(n=A.shape[0], nnz=len(val), row_ptr=_lib.iptr(ptr), col=_lib.iptr(col),
                                     val=_lib.dptr(val))

        arr = (_lib.BxGraphLevel * len(levels))(*[lvl(A) for A in levels])
        wl = lvl(Lw)
        pinv = np.ascontiguousarray(pinv, np.float64)
        self.lib = _lib.load()
        self.max_rhs = int(max_rhs)
        h = ct.c_void_p()
        _lib.check(self.lib.bx_graph_create(len(levels), arr, _lib.dptr(pinv), ct.byref(wl), _lib.dptr(vor_sa),
                                            self.max_rhs, ct.byref(h)), 'bx_graph_create')
        self.h = h
        self.last_iters = 0
        self.last_rel_res = 0.0

    def _run(self, fn, X, tol, max_iter, stream):
        import torch
        as_numpy = not isinstance(X, torch.Tensor)
        Xt = torch.as_tensor(np.asarray(X, np.float64) if as_numpy else X, dtype=torch.float64,
                             device='cuda')
        squeeze = Xt.ndim == 1
        if squeeze:
            Xt = Xt[:, None]
        if Xt.shape[0] != self.n:
            raise ValueError('X must have n rows')
        st = torch.cuda.current_stream().cuda_stream if stream is None else int(stream)
        outs, worst_it, worst_res = [], 0, 0.0
        for j0 in range(0, Xt.shape[1], self.max_rhs):
            xb = Xt[:, j0:j0 + self.max_rhs].contiguous()
            yb = torch.empty_like(xb)
            it, res = ct.c_int(), ct.c_double()
            _lib.check(fn(self.h, ct.c_void_p(xb.data_ptr()), ct.c_void_p(yb.data_ptr()), int(xb.shape[1]),
                          float(tol), int(max_iter), ct.byref(it), ct.byref(res), ct.c_void_p(st)), fn.__name__)
            worst_it, worst_res = max(worst_it, it.value), max(worst_res, res.value)
            outs.append(yb)
        self.last_iters, self.last_rel_res = worst_it, worst_res
        if worst_res > tol:
            raise RuntimeError(f'graph Laplacian solve did not reach {tol:g} in {max_iter} iterations '
                               f'(relative residual {worst_res:.2e})')
        Y = torch.cat(outs, dim=1)
        if squeeze:
            Y = Y[:, 0]
        return Y.cpu().numpy() if as_numpy else Y

    def solve(self, B, tol=1e-12, max_iter=1000, stream=None):
        return self._run(self.lib.bx_graph_solve, B, tol, max_iter, stream)

    def apply(self, X, tol=1e-12, max_iter=1000, stream=None):
        return self._run(self.lib.bx_lap_gj_apply, X, tol, max_iter, stream)

    def dense(self, tol=1e-10, max_iter=1000, stream=None):
        import torch
        st = torch.cuda.current_stream().cuda_stream if stream is None else int(stream)
        h = ct.c_void_p()
        it, res = ct.c_int(), ct.c_double()
        _lib.check(self.lib.bx_lap_gj_dense(self.h, float(tol), int(max_iter), ct.byref(it), ct.byref(res),
                                            ct.c_void_p(st), ct.byref(h)), 'bx_lap_gj_dense')
        self.last_iters, self.last_rel_res = it.value, res.value
        if res.value > tol:
            self.lib.bx_dense_op_destroy(h)
            raise RuntimeError(f'lapGJinv build did not reach {tol:g} (relative residual {res.value:.2e})')
        return DenseOperator._wrap(h, self.n)

    def close(self):
        if getattr(self, 'h', None) is not None and self.h.value:
            self.lib.bx_graph_destroy(self.h)
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
