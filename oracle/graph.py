"""BETSE's cell-network Poisson operators, restated -- TEST INFRASTRUCTURE
ONLY (the checker of ``betse_gb300.dense.lap_gj_operators``).

``Cells.graphLaplacian`` (``betse/science/cells.py:1845-1894``) builds, from the
DEC triangulation of the cluster (``cells.mesh``): the incidence matrix
``delta_tri_0`` (one row per triangulation edge, -1 at its first vertex and
+1 at its second), its pseudo-inverse ``delta_tri_0_inv``
(``mesh.create_core_operators``), the edge lengths of the triangulation and
of the dual Voronoi edges, and the Voronoi areas, then

    lapGJinv = pinv(D) diag(tri_len / vor_len) (-pinv(D)^T) diag(vor_sa)
    lapGJ    = diag(1 / vor_sa) (-D^T) diag(vor_len / tri_len) D

This restatement takes the same inputs and evaluates the same products with
``np.linalg.pinv``, as BETSE does (dense; small clusters only).
"""
from __future__ import annotations

import numpy as np


def incidence(tri_edges, n_verts):
    """delta_tri_0 as a dense [edges, vertices] array."""
    e = np.asarray(tri_edges, np.int64)
    D = np.zeros((len(e), n_verts))
    D[np.arange(len(e)), e[:, 0]] = -1.0
    D[np.arange(len(e)), e[:, 1]] = 1.0
    return D


def graph_laplacian(tri_edges, tri_edge_len, vor_edge_len, vor_sa):
    """(lapGJinv, lapGJ) as Cells.graphLaplacian computes them."""
    vor_sa = np.asarray(vor_sa, np.float64)
    D = incidence(tri_edges, len(vor_sa))
    Dinv = np.linalg.pinv(D)
    L1 = np.dot(np.diag(np.asarray(vor_edge_len) / np.asarray(tri_edge_len)), D)
    L2 = np.dot(np.diag(1 / vor_sa), -D.T)
    L1_inv = np.dot(Dinv, np.diag(np.asarray(tri_edge_len) / np.asarray(vor_edge_len)))
    L2_inv = np.dot(-Dinv.T, np.diag(vor_sa))
    return np.dot(L1_inv, L2_inv), np.dot(L2, L1)
