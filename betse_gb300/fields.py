"""The environment-grid Laplacian and its inverse (``cells.lapENVinv``).

``FiniteDiffSolver.makeLaplacian`` (``betse/science/math/finitediff.py:252-431``)
builds, on the row-major ``(ny, nx)`` environment grid, the 5-point Laplacian
divided by ``delta**2`` with identity rows (also divided by ``delta**2``) on
the four edges, then ``pinv``s it densely (``cells.py:503-504``).  The matrix
is non-singular, so its inverse is the same operator; it equals
``delta**2 * K(ny, nx)`` with ``K`` the inverse at unit spacing, which is
what lets clusters of one grid shape share it (``bx_batch_set_lap_env_inv``).
The inverse is built on the GPU from the sine-transform eigenvectors of the
interior block (``csrc/bx_lapinv.cuh``), not by dense inversion.
"""
from __future__ import annotations

import numpy as np


def make_laplacian(ny, nx, delta=1.0):
    """The Laplacian as a ``scipy.sparse.csr_matrix`` of shape ``(ny*nx, ny*nx)``."""
    import scipy.sparse as sp
    G = ny * nx
    k = np.arange(G)
    i, j = k // nx, k % nx
    edge = (i == 0) | (j == 0) | (i == ny - 1) | (j == nx - 1)
    inner = k[~edge]
    rows = np.concatenate([k[edge], np.repeat(inner, 5)])
    cols = np.concatenate([k[edge], np.stack([inner - nx, inner - 1, inner, inner + 1, inner + nx], 1).ravel()])
    vals = np.concatenate([np.ones(edge.sum()), np.tile([1.0, 1.0, -4.0, 1.0, 1.0], len(inner))])
    return sp.csr_matrix((vals / delta ** 2, (rows, cols)), shape=(G, G))


def lap_env_inverse(ny, nx, delta=1.0, device=None):
    """``cells.lapENVinv`` for a grid of this shape and spacing, built on the
    GPU (``bx_lap_env_inv_build``: the eigenvector construction, no dense
    inversion).  Returns a CUDA float64 tensor ``[G, G]`` when ``device`` is a
    CUDA device, else a NumPy array copied back to the host."""
    import ctypes as ct
    import torch
    from . import _lib
    G = ny * nx
    dev = torch.device(device) if device is not None else torch.device('cuda', torch.cuda.current_device())
    A = torch.empty((G, G), dtype=torch.float64, device=dev)
    _lib.check(_lib.load().bx_lap_env_inv_build(int(ny), int(nx), float(delta), ct.c_void_p(A.data_ptr()), G,
                                                ct.c_void_p(torch.cuda.current_stream(dev).cuda_stream)),
               'bx_lap_env_inv_build')
    return A if device is not None else A.cpu().numpy()
