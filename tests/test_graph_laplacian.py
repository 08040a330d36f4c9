"""Cells.graphLaplacian (cells.py:1845-1894) restated twice and pinned to
BETSE's own operators on a seeded cluster (tests/golden/lapgj_r80_s1.npz,
written by make_golden.py from BETSE's Cells and DEC mesh):

* the oracle's literal restatement (dense pinv, as BETSE) within 1e-12;
* the product's construction (sparse Laplacians, one dense solve) within
  1e-12, and the pressures.py:59 product it feeds within 1e-12.
"""
import os

import numpy as np

import golden_io as gi
from oracle import graph


def _fixture():
    return dict(np.load(os.path.join(gi.GOLDEN, 'lapgj_r80_s1.npz')))


def _args(d):
    return d['mesh_tri_edges'], d['mesh_tri_edge_len'], d['mesh_vor_edge_len'], d['mesh_vor_sa']


def test_oracle_restatement_matches_betse():
    d = _fixture()
    inv, lap = graph.graph_laplacian(*_args(d))
    assert gi.rel_err(inv, d['lapGJinv']) < 1e-12
    assert gi.rel_err(lap, d['lapGJ']) < 1e-12


def test_product_construction_matches_betse():
    from betse_gb300.dense import lap_gj_operators
    d = _fixture()
    inv, lap = lap_gj_operators(*_args(d))
    assert gi.rel_err(inv, d['lapGJinv']) < 1e-12
    assert gi.rel_err(lap, d['lapGJ']) < 1e-12
    PP = inv @ (-d['press_div_u_osmo'] * d['press_rho'] * d['press_dt'])
    assert gi.rel_err(PP, d['press_PP']) < 1e-12
    # lapGJ does not invert lapGJinv (a property of BETSE's construction)
    assert np.max(np.abs(lap @ inv - np.eye(len(inv)))) > 0.1
