"""Synthetic cell clusters with BETSE's conventions, generated on the GPU.

BETSE seeds a cluster with ``Cells.make_world`` (``betse/science/cells.py:414``):
a jittered hexagonal lattice (``_make_cell_lattice``, cells.py:742-801), a DEC
mesh whose Voronoi vertices are triangle centroids (``DECMesh(use_centroids=
True)``, math/mesh.py:86) clipped to the tissue shape in two passes
(``clip_and_refine``, math/mesh.py:189, 2290-2372), then per-cell membranes
(``cellVerts``, cells.py:978-1175), volumes (``cell_vols``, :1358-1390), gap
junction pairs (``mem_processing``/``near_neigh``, :1392-1573) and the
environment grid maps (``makeECM``/``environment``, :1576-1843). Its O(N^2)
Python loops and dense ``pinv`` limit it to a few thousand cells.

``make_cluster`` runs the same construction as CUDA kernels
(``bx_generate_cluster``, ``csrc/bx_generator.cu``): BETSE's seed lattice bit
for bit (numpy's linspace rows and legacy ``RandomState`` jitter), per-point
Voronoi cells clipped against the neighbouring buckets' bisectors (Delaunay
stars without a global triangulation), two-pass seeding, Z-ordered cells,
membranes, gap-junction pairs across shared Delaunay edges, the environment
grid map and the cell adjacency.  Clip-edge refinement of the reference mesh
is not reproduced: boundary cells are whole Voronoi cells and the open outer
ring of the second pass is left out.

``workload`` adds the step parameters, diffusivities and initial state of
the seeded synthetic workloads; ``sweep_workload`` a batch of them.
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass

import numpy as np

from . import _lib
from .cluster import ClusterGeometry, StepParams

ION_NAMES = ['Na', 'K', 'Cl', 'Ca', 'P', 'M']
# workload ion set: Na/K/Cl/Ca/P inside and outside (mM); M balances charge
CELL_CONC = {'Na': 8.0, 'K': 125.0, 'Cl': 10.0, 'Ca': 1e-4, 'P': 100.0}
ENV_CONC = {'Na': 145.0, 'K': 5.0, 'Cl': 105.0, 'Ca': 1.0, 'P': 10.0}
Z = {'Na': 1, 'K': 1, 'Cl': -1, 'Ca': 2, 'P': -1, 'M': -1}
D_FREE = {'Na': 1.33e-9, 'K': 1.96e-9, 'Cl': 2.03e-9, 'Ca': 1.0e-10, 'P': 0.0, 'M': 1.0e-9}


@dataclass
class GeneratedCluster:
    geom: ClusterGeometry
    cell_centres: np.ndarray
    mem_mids: np.ndarray
    xmin: float
    xmax: float
    ymin: float
    ymax: float
    world: float       # side of the square world (p.wsx after the disorder margin)

def world_size(radius, d_cell=10e-6, disorder=0.4):
    """(world, wsx): the side of BETSE's square world for a disc of
    ``radius`` (world_len = 2 R + 20 um) and the lattice's side with the
    disorder margin."""
    world = 2 * radius + 20e-6
    return world, world + 5 * disorder * d_cell


def lattice_rows(wsx, wsy, d_cell):
    """The four linspace rows of ``_make_cell_lattice`` (cells.py:742-801):
    ((start, stop, count) of bx, by, rx, ry)."""
    r = d_cell / 2
    a_hex = np.sqrt(3) * r
    b_hex = 3 * r
    return ((0.0, wsy, int(wsy / b_hex)),
            (a_hex / 2, wsx - a_hex / 2, int((wsx - a_hex) / a_hex)),
            (b_hex / 2, wsy - b_hex / 2, int((wsy - b_hex) / b_hex)),
            (0.0, wsx, int(wsx / a_hex)))


def gen_spec(radius, seed, d_cell=10e-6, disorder=0.4, cell_height=1e-5, scale_cell=0.99, grid_size=20):
    wsx = world_size(radius, d_cell, disorder)[1]
    (bx0, bx1, nbx), (by0, by1, nby), (rx0, rx1, nrx), (ry0, ry1, nry) = lattice_rows(wsx, wsx, d_cell)
    return _lib.BxGenSpec(seed=int(seed), grid_size=int(grid_size), nbx=nbx, nby=nby, nrx=nrx, nry=nry,
                          bx0=bx0, bx1=bx1, by0=by0, by1=by1, rx0=rx0, rx1=rx1, ry0=ry0, ry1=ry1,
                          jitter=disorder * d_cell, radius=radius, d_cell=d_cell, cell_radius=d_cell / 2,
                          scale_cell=scale_cell, cell_height=cell_height)


class _Generated:
    """A ``bx_generate_cluster`` result on the device."""

    def __init__(self, spec, stream=None):
        self.lib = _lib.load()
        h = ct.c_void_p()
        _lib.check(self.lib.bx_generate_cluster(ct.byref(spec), stream, ct.byref(h)), 'bx_generate_cluster')
        self.h = h
        sizes = np.zeros(6, np.int32)
        box = np.zeros(5, np.float64)
        _lib.check(self.lib.bx_generated_info(self.h, _lib.iptr(sizes), _lib.dptr(box)), 'bx_generated_info')
        self.C, self.M, self.gny, self.gnx, self.E, self.L = (int(v) for v in sizes)
        self.box = box

    def download(self, lattice=False):
        n = {'C': self.C, 'M': self.M, 'G': self.gny * self.gnx, 'E': self.E, 'L': self.L}
        shapes = {'cell_mem_ptr': n['C'] + 1, 'cell_nn_ptr': n['C'] + 1, 'cell_nn': n['E'],
                  'mem_sa_per_env': n['G'], 'lattice_x': n['L'], 'lattice_y': n['L']}
        cells = {'cell_vol', 'cell_sa', 'diviterm', 'cell_centre_x', 'cell_centre_y'}
        out, ptrs = {}, {}
        for name, t in _lib.GEN_ARRAYS:
            if name.startswith('lattice') and not lattice:
                continue
            size = shapes.get(name, n['C'] if name in cells else n['M'])
            a = np.zeros(size, np.int32 if t == 'i' else np.float64)
            out[name] = a
            ptrs[name] = _lib.iptr(a) if t == 'i' else _lib.dptr(a)
        arr = _lib.BxGenArrays(**ptrs)
        _lib.check(self.lib.bx_generated_download(self.h, ct.byref(arr)), 'bx_generated_download')
        return out

    def close(self):
        if getattr(self, 'h', None) is not None and self.h.value:
            self.lib.bx_generated_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def seed_lattice(radius, seed, d_cell=10e-6, disorder=0.4):
    """BETSE's jittered seed lattice for a disc of ``radius``, made on the GPU
    (the ``lattice_x``/``lattice_y`` of ``bx_generate_cluster``)."""
    g = _Generated(gen_spec(radius, seed, d_cell, disorder))
    try:
        d = g.download(lattice=True)
    finally:
        g.close()
    return np.column_stack((d['lattice_x'], d['lattice_y']))


def make_cluster(radius, seed, d_cell=10e-6, disorder=0.4, cell_height=1e-5,
                 cell_space=26e-9, scale_cell=0.99, grid_size=20, smooth_cells=2.0, stream=None):
    """A jittered-hex Voronoi cluster clipped to a disc of ``radius`` (m),
    generated on the current CUDA device.

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
    world = world_size(radius, d_cell, disorder)[1]
    g = _Generated(gen_spec(radius, seed, d_cell, disorder, cell_height, scale_cell, grid_size), stream)
    try:
        d = g.download()
    finally:
        g.close()
    xmin, xmax, ymin, ymax, delta = (float(v) for v in g.box)
    ptr = d['cell_mem_ptr']
    C, M = g.C, g.M
    m2c = np.repeat(np.arange(C), np.diff(ptr))
    nn = d['nn_i'].astype(np.int64)
    geom = ClusterGeometry.from_arrays(
        mem_to_cells=m2c, nn_i=nn, bflags_mems=np.nonzero(nn == np.arange(M))[0],
        map_mem2ecm=d['map_mem2ecm'], mem_sa=d['mem_sa'], mem_nx=d['mem_nx'], mem_ny=d['mem_ny'],
        gj_weight=np.ones(M), cell_vol=d['cell_vol'], cell_sa=d['cell_sa'], diviterm=d['diviterm'],
        grid_shape=(g.gny, g.gnx), delta=delta, gj_len=cell_space, smooth_cells=smooth_cells,
        mem_sa_per_env=d['mem_sa_per_env'], D_env_weight=np.ones(g.gny * g.gnx),
        cell_nn_ptr=d['cell_nn_ptr'], cell_nn=d['cell_nn'], R_rads=d['R_rads'])
    return GeneratedCluster(geom=geom, cell_centres=np.column_stack((d['cell_centre_x'], d['cell_centre_y'])),
                            mem_mids=np.column_stack((d['mem_mid_x'], d['mem_mid_y'])),
                            xmin=xmin, xmax=xmax, ymin=ymin, ymax=ymax, world=world)


def charge_balanced(conc):
    c = dict(conc)
    q = sum(c[k] * Z[k] for k in c)
    assert q >= 0, 'the balancing ion M must be an anion'
    c['M'] = q
    return c


def workload(radius, seed, is_ecm=False, dt=1e-2, dm_range=(1e-19, 1e-17),
             grid_size=20, cell_space=26e-9, alpha_NaK=5e-8, gj_range=(0.5, 1.0),
             na_k_dm_mult=1.0, pump_mult=1.0, cluster=None):
    """Cluster + parameters + initial state of the seeded synthetic workload.

    Returns (geom, params, Dm, state dict, D_env). Diffusivities are
    log-uniform in ``dm_range`` per membrane and ion (Dm_P = 0), gap-junction
    weights uniform in ``gj_range`` per membrane pair; draws come from
    ``np.random.default_rng(seed + 1)``, the lattice from ``RandomState(seed)``.
    ``cluster`` (a ``GeneratedCluster`` of the same radius and seed) skips
    the generation.
    """
    gc = cluster if cluster is not None else make_cluster(radius, seed, grid_size=grid_size,
                                                          cell_space=cell_space)
    g = gc.geom
    g.extra['cell_centres'] = gc.cell_centres
    M, C, G = g.n_mems, g.n_cells, g.n_grid
    rng = np.random.default_rng(seed + 1)
    Dm = np.exp(rng.uniform(np.log(dm_range[0]), np.log(dm_range[1]), size=(6, M)))
    Dm[ION_NAMES.index('P')] = 0.0
    Dm[ION_NAMES.index('Na')] *= na_k_dm_mult
    Dm[ION_NAMES.index('K')] *= na_k_dm_mult
    w = rng.uniform(gj_range[0], gj_range[1], size=M)
    w = w[np.minimum(np.arange(M), g.nn_i)]
    g.gj_weight = np.ascontiguousarray(w)
    cell = charge_balanced(CELL_CONC)
    env = charge_balanced(ENV_CONC)
    zs = np.array([Z[k] for k in ION_NAMES], np.float64)
    D_free = np.array([D_FREE[k] for k in ION_NAMES])
    cc_cells = np.array([[cell[k]] * C for k in ION_NAMES], np.float64)
    env_v = np.array([env[k] for k in ION_NAMES], np.float64)
    T = 310.15
    F, R, q, kb, eo, er, NAv = 96485.0, 8.314, 1.602e-19, 1.3806e-23, 8.854e-12, 80.0, 6.022e23
    cell_height = 1e-5
    vol_env = gc.world * gc.world * cell_height      # parameters.py:540, multiplier 1
    ko_env = float(np.sqrt(np.dot((NAv * q ** 2 * zs ** 2) / (er * eo * kb * T), env_v)))
    sigma = float((((zs ** 2) * q * F * cell_conc_vec(cell) * D_free) / (kb * T)).sum())
    p = StepParams(zs=zs, D_free=D_free, D_gj=D_free.copy(), iNa=0, iK=1, is_ecm=is_ecm,
                   T=T, dt=dt, cm=0.022, alpha_NaK=alpha_NaK * pump_mult, vol_env=vol_env,
                   cell_height=cell_height, ko_env=ko_env, sigma=sigma,
                   c_env_bound=env_v.copy(), ion_names=list(ION_NAMES))
    if is_ecm:
        cc_env = np.repeat(env_v[:, None], G, axis=1)
    else:
        cc_env = env_v.copy()
    cc_at_mem = cc_cells[:, g.mem_to_cells].copy()
    rho = np.dot(zs * F, cc_cells)
    vm = (1 / p.cm) * (rho * g.diviterm)[g.mem_to_cells]
    state = dict(vm=vm, cc_cells=cc_cells, cc_at_mem=cc_at_mem, cc_env=cc_env)
    if is_ecm:
        # uniform, charge-balanced environment: zero initial field
        state.update(E_env_x=np.zeros(g.grid_shape), E_env_y=np.zeros(g.grid_shape))
    D_env = np.repeat(D_free[:, None], G, axis=1) if is_ecm else None
    return g, p, Dm, state, D_env


def cell_conc_vec(cell):
    return np.array([cell[k] for k in ION_NAMES], np.float64)


def sweep_workload(n_clusters=512, seed=7, cells_range=(200, 5000), mult_range=(0.1, 10.0),
                   dt=5e-3, dm_range=(1e-19, 1e-17), pump_range=None):
    """A parameter sweep: ``n_clusters`` independent clusters with cell counts
    log-uniform in ``cells_range`` and per-cluster Na/K diffusivity and pump
    multipliers log-uniform in ``mult_range`` (the pump's in ``pump_range`` when
    given), each generated on the GPU in turn. Returns lists (geoms, params,
    Dms, states)."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log(cells_range[0]), np.log(cells_range[1])
    counts = np.exp(rng.uniform(lo, hi, n_clusters))
    ml, mh = np.log(mult_range[0]), np.log(mult_range[1])
    pr = mult_range if pump_range is None else pump_range
    dmm = np.exp(rng.uniform(ml, mh, n_clusters))
    pmm = np.exp(rng.uniform(np.log(pr[0]), np.log(pr[1]), n_clusters))
    out = ([], [], [], [])
    for k in range(n_clusters):
        R = np.sqrt(float(counts[k]) / 0.0456) * 1e-6   # cells ~ 0.0456 (R / 1 um)^2 for this lattice
        g, p, Dm, st, _ = workload(R, seed * 1000 + k, dt=dt, dm_range=dm_range,
                                   na_k_dm_mult=float(dmm[k]), pump_mult=float(pmm[k]))
        for lst, v in zip(out, (g, p, Dm, st)):
            lst.append(v)
    return out
