"""Synthetic clusters in the golden-fixture format, for edge cases the
BETSE-generated fixtures do not reach.

``ragged_fixture`` keeps the physical parameters and initial concentrations of
a golden fixture but replaces its geometry with one built here. Cells have
1 to 20 membranes (Voronoi clusters stop near 8), and partners are drawn at
random between different cells. Unpaired membranes are boundary membranes
that name themselves as partner, as ``Cells.nn_i`` does. The dict has the
fixture's keys (``geom_*``, ``par_*``, ``init_*``), so ``golden_io``'s
loaders and tolerance floors apply unchanged. It holds no BETSE outputs: the
oracle is the reference for it.
"""
from __future__ import annotations

import numpy as np

import golden_io as gi


def ragged_fixture(seed=3, n_cells=48, template='noecm_r50_s7'):
    t = gi.load(template)
    d = {k: v for k, v in t.items() if not k.startswith(('geom_', 'init_')) and not (k[:1] == 's' and k[1:2].isdigit())}
    rng = np.random.default_rng(seed)
    counts = rng.integers(1, 8, size=n_cells)
    counts[rng.choice(n_cells, size=6, replace=False)] = [9, 12, 13, 16, 17, 20]   # past the 8 straight-line terms
    C = n_cells
    M = int(counts.sum())
    m2c = np.repeat(np.arange(C), counts).astype(np.int64)
    # partners: shuffled membranes paired greedily across cells; 10 % stay boundary
    nn = np.arange(M, dtype=np.int64)
    order = rng.permutation(M)
    free = [int(m) for m in order if rng.random() > 0.1]
    while len(free) > 1:
        a = free.pop()
        for j in range(len(free) - 1, -1, -1):
            if m2c[free[j]] != m2c[a]:
                b = free.pop(j)
                nn[a], nn[b] = b, a
                break
    boundary = np.nonzero(nn == np.arange(M))[0]
    w = rng.uniform(0.5, 1.0, size=M)
    w = np.minimum(w, w[nn])                      # one weight per pair
    ang = rng.uniform(0, 2 * np.pi, size=M)
    mv = np.zeros((M, 4))
    mv[:, 2], mv[:, 3] = np.cos(ang), np.sin(ang)
    # physically consistent sizes: volume in proportion to membrane area, and
    # diviterm = volume / area (the capacitor of update_V)
    mem_sa = rng.uniform(3e-11, 1.4e-10, size=M)
    cell_sa = np.bincount(m2c, weights=mem_sa, minlength=C)
    cell_vol = cell_sa * rng.uniform(6e-7, 1.2e-6, size=C)
    diviterm = cell_vol / cell_sa
    G = int(np.prod(t['geom_grid_shape']))
    swm = rng.uniform(0.3, 0.7, size=M)
    d.update(geom_mem_to_cells=m2c, geom_nn_i=nn, geom_bflags_mems=boundary.astype(np.int64),
             geom_num_mems=counts.astype(np.int64), geom_mem_sa=mem_sa, geom_cell_vol=cell_vol,
             geom_cell_sa=cell_sa, geom_diviterm=diviterm, geom_mem_vects_flat=mv,
             geom_R_rads=np.full(M, 5e-6), geom_map_mem2ecm=rng.integers(0, G, size=M).astype(np.int64),
             geom_grid_shape=np.asarray(t['geom_grid_shape']), geom_delta=np.float64(t['geom_delta']),
             geom_gj_len=np.float64(t['geom_gj_len']), geom_gj_default_weights=w,
             geom_D_env_weight=np.ones(G), par_smooth_weight_mem=swm, par_smooth_weight_o=1.0 - swm)
    I = len(d['par_zs'])
    Dm = 10.0 ** rng.uniform(-19, -17, size=(I, M))
    names = [str(x) for x in d['par_ion_names']]
    if 'P' in names:
        Dm[names.index('P')] = 0.0                   # proteins do not cross (sim_config.yaml)
    d['par_Dm_cells'] = Dm
    c0 = np.asarray(t['init_cc_cells'])[:, :1]
    cc = np.repeat(c0, C, axis=1)
    rho = (np.asarray(d['par_zs']) * float(d['par_F'])) @ cc
    d.update(init_cc_cells=cc, init_cc_at_mem=cc[:, m2c].copy(),
             init_cc_env=np.repeat(np.asarray(t['init_cc_env'])[:, :1], M, axis=1),
             init_vm=((1.0 / float(d['par_cm'])) * (rho * diviterm))[m2c])
    d['meta_checkpoints'] = np.asarray([1, 30], np.int64)
    return d
