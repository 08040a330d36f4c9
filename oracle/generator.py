"""Synthetic cell clusters with BETSE's conventions in NumPy/SciPy -- TEST
INFRASTRUCTURE ONLY (the checker of the GPU generator,
``betse_gb300.generator.make_cluster`` / ``bx_generate_cluster``).

BETSE seeds a cluster with ``Cells.make_world`` (``betse/science/cells.py:414``):
a jittered hexagonal lattice (``_make_cell_lattice``, cells.py:742-801), a DEC
mesh whose Voronoi vertices are triangle centroids (``DECMesh(use_centroids=
True)``, math/mesh.py:86) clipped to the tissue shape, then per-cell membranes
(``cellVerts``, cells.py:978-1175), volumes (``cell_vols``, :1358-1390), gap
junction pairs (``mem_processing``/``near_neigh``, :1392-1573) and the
environment grid maps (``makeECM``/``environment``, :1576-1843).

This restatement builds the same data with SciPy's Delaunay triangulation:

* the lattice recipe is BETSE's (linspace rows, legacy ``np.random`` jitter
  ``disorder * d_cell * (rand - 0.5)``);
* cells are the Delaunay duals with centroid vertices of every seed whose
  distance to the lattice centre is below ``radius`` and whose triangle fan is
  closed (triangle centroids add their vertices in ascending index order);
  membranes are the polygon edges scaled in by ``scale_cell`` about the
  centroid, listed counter-clockwise per cell exactly as ``cellVerts`` does;
* gap-junction partners come from the shared Delaunay edge (BETSE finds the
  same pairs by a radius search on membrane midpoints); a membrane with no
  partner in the cluster is a boundary membrane, paired with itself;
* cells are ordered along a Z-order curve so that gap-junction partners sit
  close in memory.

``tests/test_generator_betse.py`` pins it to BETSE's own ``Cells``;
``tests/test_gpu_generator.py`` checks the GPU generator against it.
"""
from __future__ import annotations

import numpy as np

from betse_gb300.cluster import ClusterGeometry
from betse_gb300.generator import GeneratedCluster


def hex_lattice(wsx, wsy, d_cell, disorder, rs):
    """BETSE's hexagonal seed lattice (cells.py:742-801) with jitter from ``rs``."""
    r = d_cell / 2
    a_hex = np.sqrt(3) * r
    b_hex = 3 * r
    bx = np.linspace(0, wsy, int(wsy / b_hex))
    by = np.linspace(a_hex / 2, wsx - a_hex / 2, int((wsx - a_hex) / a_hex))
    rx = np.linspace(b_hex / 2, wsy - b_hex / 2, int((wsy - b_hex) / b_hex))
    ry = np.linspace(0, wsx, int(wsx / a_hex))
    xb, yb = np.meshgrid(bx, by)
    xr, yr = np.meshgrid(rx, ry)
    x = np.hstack((xb.ravel(), xr.ravel()))
    y = np.hstack((yb.ravel(), yr.ravel()))
    x = x + disorder * d_cell * (rs.rand(len(x)) - 0.5)
    y = y + disorder * d_cell * (rs.rand(len(y)) - 0.5)
    return np.column_stack((x, y))


def _zorder(xy, bits=16):
    lo = xy.min(axis=0)
    span = np.maximum(xy.max(axis=0) - lo, 1e-30)
    q = ((xy - lo) / span * (2 ** bits - 1)).astype(np.uint64)
    key = np.zeros(len(xy), np.uint64)
    for b in range(bits):
        key |= ((q[:, 0] >> np.uint64(b)) & np.uint64(1)) << np.uint64(2 * b)
        key |= ((q[:, 1] >> np.uint64(b)) & np.uint64(1)) << np.uint64(2 * b + 1)
    return key


def poly_centroid(P):
    """Area centroid of a polygon (vertices in order), as DECMesh.poly_centroid."""
    Q = np.roll(P, -1, axis=0)
    a = P[:, 0] * Q[:, 1] - Q[:, 0] * P[:, 1]
    A = a.sum() / 2
    return np.array([((P[:, 0] + Q[:, 0]) * a).sum(), ((P[:, 1] + Q[:, 1]) * a).sum()]) / (6 * A)


def _centroid_voronoi(pts):
    """Delaunay triangulation of ``pts`` and, per point, its triangles in
    counter-clockwise order; the Voronoi vertices are triangle centroids
    (DECMesh(use_centroids=True)).  Returns (simplices, triangle centroids,
    fan triangle ids, fan pointer, hull mask)."""
    from scipy.spatial import Delaunay
    tri = Delaunay(pts)
    simp = tri.simplices
    simp = np.sort(simp, axis=1)
    tcent = pts[simp].mean(axis=1)
    n = len(pts)
    owner = simp.ravel()
    tid = np.repeat(np.arange(len(simp)), 3)
    ang = np.arctan2(tcent[tid, 1] - pts[owner, 1], tcent[tid, 0] - pts[owner, 0])
    order = np.lexsort((ang, owner))
    owner, tid = owner[order], tid[order]
    fan_ptr = np.concatenate([[0], np.cumsum(np.bincount(owner, minlength=n))])
    hull = np.zeros(n, bool)
    hull[np.unique(tri.convex_hull.ravel())] = True
    return simp, tcent, tid, fan_ptr, hull


def make_cluster(radius, seed, d_cell=10e-6, disorder=0.4, cell_height=1e-5,
                 cell_space=26e-9, scale_cell=0.99, grid_size=20, smooth_cells=2.0):
    """A jittered-hex Voronoi cluster clipped to a disc of ``radius`` (m).

    BETSE's seeding (Cells.make_world -> DECMesh.clip_and_refine,
    math/mesh.py:189, 2290-2372) in two passes: the centroid-Voronoi cells of
    the lattice (plus its four bounding-box corners, Cells.clust_xy), of
    which those whose area centroid lies in the disc are kept; then the
    mesh is rebuilt with those area centroids as its points, and the cells
    are the centroid-Voronoi cells of the rebuilt mesh, centred at their area
    centroids (cells.cell_centres).  BETSE cuts the boundary cells of the
    first pass with the disc before taking their centroids and closes the
    outer cells of the second along the cut; here the first-pass cells are
    whole and the outer ring of the second pass (open Voronoi fans) is left
    out, so the interior is BETSE's and the boundary ring differs."""
    cell_radius = d_cell / 2
    world = 2 * radius + 20e-6
    # the world of BETSE's configuration: world_len plus the disorder margin
    wsx = wsy = world + 5 * disorder * d_cell
    rs = np.random.RandomState(seed)
    lat = hex_lattice(wsx, wsy, d_cell, disorder, rs)
    centre = lat.mean(axis=0)
    lo, hi = lat.min(axis=0), lat.max(axis=0)
    xmin, ymin = lo - cell_radius
    xmax, ymax = hi + cell_radius
    # first pass: the lattice and its bounding-box corners
    corners = np.array([[lo[0], lo[1]], [hi[0], lo[1]], [hi[0], hi[1]], [lo[0], hi[1]]])
    allp = np.vstack([lat, corners])
    simp0, tcent0, tid0, fan0, hull0 = _centroid_voronoi(allp)
    first = [s for s in range(len(lat)) if not hull0[s] and fan0[s + 1] - fan0[s] >= 3]
    c0 = np.array([poly_centroid(tcent0[tid0[fan0[s]:fan0[s + 1]]]) for s in first])
    pts = c0[np.hypot(c0[:, 0] - centre[0], c0[:, 1] - centre[1]) < radius]

    # second pass: the cells of the rebuilt mesh
    simp, tcent, tid, fan_ptr, hull = _centroid_voronoi(pts)
    n = len(pts)
    keep = (~hull) & (np.diff(fan_ptr) >= 3)
    seeds = np.nonzero(keep)[0]
    # polygon of each kept seed, then cell order along a Z curve of the centroid
    polys = [tcent[tid[fan_ptr[s]:fan_ptr[s + 1]]] for s in seeds]
    cents = np.array([poly_centroid(p) for p in polys])
    zo = np.argsort(_zorder(cents), kind='stable')
    seeds = seeds[zo]
    polys = [polys[i] for i in zo]
    C = len(seeds)
    seed_to_cell = -np.ones(n, np.int64)
    seed_to_cell[seeds] = np.arange(C)

    counts = np.array([len(p) for p in polys])
    M = int(counts.sum())
    ptr = np.concatenate([[0], np.cumsum(counts)])
    m2c = np.repeat(np.arange(C), counts)
    # vertices scaled toward the cell centre, the area centroid (cellVerts: p.scale_cell)
    poly_c = cents[zo]
    V = np.concatenate(polys)
    V = scale_cell * (V - poly_c[m2c]) + poly_c[m2c]
    # membrane k of a cell joins vertex k-1 and vertex k (cellVerts' loop)
    prev = np.arange(M) - 1
    prev[ptr[:-1]] = ptr[1:] - 1
    p1, p2 = V[prev], V[np.arange(M)]
    mids = (p1 + p2) / 2
    tang = p2 - p1
    length = np.hypot(tang[:, 0], tang[:, 1])
    tang = tang / length[:, None]
    nx, ny = tang[:, 1], -tang[:, 0]
    mem_sa = length * cell_height
    # cell centre: BETSE's cell_centres are polygon centroids of the unscaled cells
    rad = mids - poly_c[m2c]
    R_rads = np.hypot(rad[:, 0], rad[:, 1])
    mem_vol = 0.5 * R_rads * mem_sa
    cell_vol = np.bincount(m2c, weights=mem_vol, minlength=C)
    cell_sa = np.bincount(m2c, weights=mem_sa, minlength=C)
    diviterm = cell_vol / cell_sa

    # gap junction partners: the edge between triangles (t_prev, t) around seed s is
    # the Voronoi edge dual to the Delaunay edge (s, other); pair by that edge.
    t_prev = tid[np.concatenate([fan_ptr[s] + (np.arange(c) - 1) % c for s, c in
                                 zip(seeds, counts)])] if C else np.zeros(0, np.int64)
    t_cur = tid[np.concatenate([fan_ptr[s] + np.arange(c) for s, c in zip(seeds, counts)])]
    own_seed = seeds[m2c]
    a, b = simp[t_prev], simp[t_cur]
    # the shared vertex of the two triangles that is not the owner seed
    other = np.full(M, -1, np.int64)
    for ka in range(3):
        for kb in range(3):
            same = (a[:, ka] == b[:, kb]) & (a[:, ka] != own_seed)
            other = np.where(same & (other < 0), a[:, ka], other)
    key_lo = np.minimum(own_seed, other)
    key_hi = np.maximum(own_seed, other)
    nn = np.arange(M)
    valid = (other >= 0) & (seed_to_cell[np.maximum(other, 0)] >= 0)
    idx = np.nonzero(valid)[0]
    keys = key_lo[idx] * (n + 1) + key_hi[idx]
    o = np.argsort(keys, kind='stable')
    ks, ix = keys[o], idx[o]
    pair = np.nonzero(ks[1:] == ks[:-1])[0]
    nn[ix[pair]] = ix[pair + 1]
    nn[ix[pair + 1]] = ix[pair]
    bflags = np.nonzero(nn == np.arange(M))[0]

    # environment grid (makeECM / FiniteDiffSolver.cell_grid, environment)
    delta = (xmax - xmin) / grid_size
    gnx = int((xmax - xmin) / delta)
    gny = int((ymax - ymin) / delta)
    xv = np.linspace(xmin, xmax, gnx + 1)
    yv = np.linspace(ymin, ymax, gny + 1)
    cx = (xv[:-1] + xv[1:]) / 2
    cy = (yv[:-1] + yv[1:]) / 2
    jx = np.clip(np.searchsorted(cx, mids[:, 0]), 1, gnx - 1)
    jx = np.where(np.abs(cx[jx - 1] - mids[:, 0]) <= np.abs(cx[jx] - mids[:, 0]), jx - 1, jx)
    iy = np.clip(np.searchsorted(cy, mids[:, 1]), 1, gny - 1)
    iy = np.where(np.abs(cy[iy - 1] - mids[:, 1]) <= np.abs(cy[iy] - mids[:, 1]), iy - 1, iy)
    map_env = iy * gnx + jx
    msa_env = np.bincount(map_env, weights=mem_sa, minlength=gnx * gny)

    # cell adjacency (near_neigh's cell_nn) for the warm-start network
    part = nn != np.arange(M)
    src, dst = m2c[part], m2c[nn[part]]
    oo = np.lexsort((dst, src))
    src, dst = src[oo], dst[oo]
    cnn_ptr = np.concatenate([[0], np.cumsum(np.bincount(src, minlength=C))])

    geom = ClusterGeometry.from_arrays(
        mem_to_cells=m2c, nn_i=nn, bflags_mems=bflags, map_mem2ecm=map_env,
        mem_sa=mem_sa, mem_nx=nx, mem_ny=ny, gj_weight=np.ones(M), cell_vol=cell_vol,
        cell_sa=cell_sa, diviterm=diviterm, grid_shape=(gny, gnx), delta=delta,
        gj_len=cell_space, smooth_cells=smooth_cells, mem_sa_per_env=msa_env,
        D_env_weight=np.ones(gnx * gny), cell_nn_ptr=cnn_ptr, cell_nn=dst, R_rads=R_rads)
    return GeneratedCluster(geom=geom, cell_centres=poly_c, mem_mids=mids,
                            xmin=xmin, xmax=xmax, ymin=ymin, ymax=ymax, world=wsx)
