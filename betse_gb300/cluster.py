"""Host-side records of a cell cluster: geometry/index maps and step parameters.

``ClusterGeometry.from_cells`` reads a BETSE ``Cells`` object (or anything
with the same attribute names) and builds the CSR form the GPU step uses. The
CSR is checked to reproduce ``Cells``' own ``mem_to_cells`` bit-exactly
(``betse/science/cells.py:1126``): membranes of a cell are contiguous and in
cell order, exactly as ``Cells.cellVerts`` flattens them.
"""
from __future__ import annotations

from dataclasses import dataclass, field, fields

import numpy as np

from . import _lib


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _i32(a):
    a = np.asarray(a)
    if a.size and (a.min() < np.iinfo(np.int32).min or a.max() > np.iinfo(np.int32).max):
        raise ValueError('index does not fit int32')
    return np.ascontiguousarray(a, dtype=np.int32)


@dataclass
class ClusterGeometry:
    cell_mem_ptr: np.ndarray          # int32 [C+1]
    mem_to_cells: np.ndarray          # int32 [M]
    nn_i: np.ndarray                  # int32 [M]
    bflag: np.ndarray                 # uint8 [M]
    map_mem2ecm: np.ndarray           # int32 [M]
    mem_sa: np.ndarray                # f64 [M]
    mem_nx: np.ndarray
    mem_ny: np.ndarray
    gj_weight: np.ndarray
    smooth_weight_mem: np.ndarray
    smooth_weight_o: np.ndarray
    cell_vol: np.ndarray              # f64 [C]
    cell_sa: np.ndarray
    diviterm: np.ndarray
    num_mems: np.ndarray              # int [C]
    grid_shape: tuple
    delta: float
    gj_len: float
    mem_sa_per_env: np.ndarray | None = None   # f64 [G] (ECM)
    D_env_weight: np.ndarray | None = None     # f64 [G]
    cell_nn_ptr: np.ndarray | None = None      # cell adjacency CSR (warm start)
    cell_nn: np.ndarray | None = None
    R_rads: np.ndarray | None = None           # f64 [M] membrane distance from the cell centre
    extra: dict = field(default_factory=dict)

    @property
    def n_cells(self) -> int:
        return len(self.cell_vol)

    @property
    def n_mems(self) -> int:
        return len(self.mem_sa)

    @property
    def n_grid(self) -> int:
        return int(self.grid_shape[0] * self.grid_shape[1])

    # ------------------------------------------------------------------
    @classmethod
    def from_arrays(cls, *, mem_to_cells, nn_i, bflags_mems, map_mem2ecm, mem_sa,
                    mem_nx, mem_ny, gj_weight, cell_vol, cell_sa, diviterm, grid_shape,
                    delta, gj_len, smooth_cells=2.0, smooth_weight_mem=None,
                    smooth_weight_o=None, mem_sa_per_env=None, D_env_weight=None,
                    cell_nn_ptr=None, cell_nn=None, R_rads=None):
        m2c = np.asarray(mem_to_cells)
        C = len(cell_vol)
        M = len(m2c)
        if M == 0 or C == 0:
            raise ValueError('empty cluster')
        if np.any(np.diff(m2c) < 0) or m2c[0] != 0 or m2c[-1] != C - 1:
            raise ValueError('mem_to_cells must list each cell\'s membranes contiguously, '
                             'in cell order (Cells.cellVerts flattening)')
        counts = np.bincount(m2c, minlength=C)
        if np.any(counts == 0):
            raise ValueError('every cell needs at least one membrane')
        ptr = np.concatenate([[0], np.cumsum(counts)])
        # bit-exact check: the CSR reproduces Cells.mem_to_cells
        rebuilt = np.repeat(np.arange(C), counts)
        if not np.array_equal(rebuilt, m2c):
            raise ValueError('CSR rebuild differs from mem_to_cells')
        bflag = np.zeros(M, np.uint8)
        bflag[np.asarray(bflags_mems, dtype=np.int64)] = 1
        num_mems = counts.astype(np.int64)
        if smooth_weight_mem is None:
            nm = num_mems[m2c].astype(np.float64)
            smooth_weight_mem = (smooth_cells * nm - 1) / (smooth_cells * nm)   # sim.py:783-786
            smooth_weight_o = 1 / (smooth_cells * nm)
        return cls(cell_mem_ptr=_i32(ptr), mem_to_cells=_i32(m2c), nn_i=_i32(nn_i),
                   bflag=bflag, map_mem2ecm=_i32(map_mem2ecm), mem_sa=_f64(mem_sa),
                   mem_nx=_f64(mem_nx), mem_ny=_f64(mem_ny), gj_weight=_f64(gj_weight),
                   smooth_weight_mem=_f64(smooth_weight_mem),
                   smooth_weight_o=_f64(smooth_weight_o), cell_vol=_f64(cell_vol),
                   cell_sa=_f64(cell_sa), diviterm=_f64(diviterm), num_mems=num_mems,
                   grid_shape=tuple(int(x) for x in grid_shape), delta=float(delta),
                   gj_len=float(gj_len),
                   mem_sa_per_env=None if mem_sa_per_env is None else _f64(mem_sa_per_env),
                   D_env_weight=None if D_env_weight is None else _f64(np.ravel(D_env_weight)),
                   cell_nn_ptr=None if cell_nn_ptr is None else _i32(cell_nn_ptr),
                   cell_nn=None if cell_nn is None else _i32(cell_nn),
                   R_rads=None if R_rads is None else _f64(R_rads))

    @classmethod
    def from_cells(cls, cells, sim=None, p=None):
        """Build from a BETSE ``Cells`` (and optionally its ``Simulator``)."""
        mv = np.asarray(cells.mem_vects_flat)
        shape = getattr(cells, 'grid_shape', None)
        if shape is None:
            shape = cells.X.shape
        smooth = getattr(p, 'smooth_cells', 2.0) if p is not None else 2.0
        swm = getattr(sim, 'smooth_weight_mem', None) if sim is not None else None
        swo = getattr(sim, 'smooth_weight_o', None) if sim is not None else None
        dw = getattr(sim, 'D_env_weight', None) if sim is not None else None
        cnn = getattr(cells, 'cell_nn', None)
        cnn_ptr = cnn_flat = None
        if cnn is not None:
            cnn_ptr = np.cumsum([0] + [len(v) for v in cnn])
            cnn_flat = np.concatenate([np.asarray(v, np.int64) for v in cnn]) if cnn_ptr[-1] else np.zeros(0, np.int64)
        return cls.from_arrays(
            mem_to_cells=cells.mem_to_cells, nn_i=cells.nn_i,
            bflags_mems=cells.bflags_mems, map_mem2ecm=cells.map_mem2ecm,
            mem_sa=cells.mem_sa, mem_nx=mv[:, 2], mem_ny=mv[:, 3],
            gj_weight=cells.gj_default_weights, cell_vol=cells.cell_vol,
            cell_sa=cells.cell_sa, diviterm=cells.diviterm, grid_shape=shape,
            delta=cells.delta, gj_len=cells.gj_len, smooth_cells=smooth,
            smooth_weight_mem=swm, smooth_weight_o=swo,
            mem_sa_per_env=getattr(cells, 'memSa_per_envSquare', None),
            D_env_weight=dw, cell_nn_ptr=cnn_ptr, cell_nn=cnn_flat,
            R_rads=getattr(cells, 'R_rads', None))

    def to_c(self):
        """A ``bx_geom`` whose pointers stay valid while ``self`` lives."""
        g = _lib.BxGeom()
        g.n_cells, g.n_mems = self.n_cells, self.n_mems
        g.grid_ny, g.grid_nx = self.grid_shape
        g.cell_mem_ptr = _lib.iptr(self.cell_mem_ptr)
        g.nn_i = _lib.iptr(self.nn_i)
        g.bflag = _lib.u8ptr(self.bflag)
        g.map_mem2ecm = _lib.iptr(self.map_mem2ecm)
        for n in ('mem_sa', 'mem_nx', 'mem_ny', 'gj_weight', 'smooth_weight_mem',
                  'smooth_weight_o', 'cell_vol', 'cell_sa', 'diviterm'):
            setattr(g, n, _lib.dptr(getattr(self, n)))
        g.mem_sa_per_env = _lib.dptr(self.mem_sa_per_env) if self.mem_sa_per_env is not None else None
        g.gj_len, g.delta = self.gj_len, self.delta
        g.R_rads = _lib.dptr(self.R_rads) if self.R_rads is not None else None
        return g


_SCALARS = ('F', 'R', 'T', 'dt', 'cm', 'tm', 'gj_surface', 'gj_block', 'nakatp_block',
            'alpha_NaK', 'KmNK_Na', 'KmNK_K', 'KmNK_ATP', 'cATP', 'cADP', 'cPi',
            'deltaGATP', 'vol_env', 'cell_height', 'q', 'kb', 'eo', 'er', 'sharpness',
            'cell_radius', 'true_cell_size', 'ko_env', 'sigma', 'mu')


@dataclass
class StepParams:
    """Scalars and per-ion constants of the step (BETSE ``Parameters`` plus the
    ``Simulator`` fields ``zs, D_free, D_gj, T, ko_env, sigma``)."""
    zs: np.ndarray
    D_free: np.ndarray
    D_gj: np.ndarray
    iNa: int
    iK: int
    is_ecm: bool
    F: float = 96485.0
    R: float = 8.314
    T: float = 310.0
    dt: float = 1e-2
    cm: float = 0.022
    tm: float = 7.5e-9
    gj_surface: float = 5e-8
    gj_block: float = 1.0
    nakatp_block: float = 1.0
    alpha_NaK: float = 5e-8
    KmNK_Na: float = 12.0
    KmNK_K: float = 0.2
    KmNK_ATP: float = 0.5
    cATP: float = 1.5
    cADP: float = 0.1
    cPi: float = 0.1
    deltaGATP: float = -37000.0
    vol_env: float = 1.0
    cell_height: float = 1e-5
    q: float = 1.602e-19
    kb: float = 1.3806e-23
    eo: float = 8.854e-12
    er: float = 80.0
    sharpness: float = 1.0
    cell_radius: float = 5e-6
    true_cell_size: float = 1e-5
    ko_env: float = 0.0
    sigma: float = 0.0
    mu: float = 1.275e-6
    c_env_bound: np.ndarray | None = None
    ion_names: list | None = None
    v_sensitive_gj: bool = False     # voltage-gated gap junctions (gjopen is then state)
    gj_vthresh: float = 15.0         # mV
    gj_min: float = 0.10
    iCa: int = -1                    # Ca2+ row; the Ca-ATPase runs when iCa >= 0 and alpha_Ca > 0
    alpha_Ca: float = 0.0
    KmCa_Ca: float = 1.0e-3
    KmCa_ATP: float = 0.5
    cell_polarizability: float = 0.0  # != 0: update_V's implicit per-membrane Vmem (plain form)

    @property
    def n_ions(self) -> int:
        return len(self.zs)

    @classmethod
    def from_betse(cls, p, sim):
        """From a BETSE ``Parameters`` ``p`` and an initialised ``Simulator``."""
        kw = {}
        for n in _SCALARS:
            if n in ('gj_block', 'nakatp_block', 'ko_env', 'sigma', 'T'):
                continue
            if hasattr(p, n):
                kw[n] = float(getattr(p, n))
        gjb = getattr(sim, 'gj_block', 1)
        nkb = getattr(sim, 'NaKATP_block', 1)
        if np.ndim(gjb) or np.ndim(nkb):
            if not (np.all(np.asarray(gjb) == 1) and np.all(np.asarray(nkb) == 1)):
                raise NotImplementedError('per-membrane gj/NaKATP blocking vectors')
        D_gj = np.asarray(sim.D_gj, np.float64)
        if D_gj.ndim == 2:
            if not np.all(D_gj == D_gj[:, :1]):
                raise NotImplementedError('per-membrane D_gj')
            D_gj = D_gj[:, 0]
        if bool(getattr(p, 'v_sensitive_gj', False)):
            kw.update(v_sensitive_gj=True, gj_vthresh=float(p.gj_vthresh), gj_min=float(p.gj_min))
        if float(getattr(p, 'cell_polarizability', 0.0)) != 0.0:
            kw.update(cell_polarizability=float(p.cell_polarizability))
        ions = getattr(p, 'ions_dict', {}) or {}
        if ions.get('Ca', 0) == 1 and hasattr(sim, 'iCa'):
            # ca_handler runs for the Ca ion (sim.py:1282-1283)
            kw.update(iCa=int(sim.iCa), alpha_Ca=float(getattr(p, 'alpha_Ca', 0.0)),
                      KmCa_Ca=float(getattr(p, 'KmCa_Ca', 1.0e-3)),
                      KmCa_ATP=float(getattr(p, 'KmCa_ATP', 0.5)))
        return cls(zs=np.asarray(sim.zs, np.float64), D_free=np.asarray(sim.D_free, np.float64),
                   D_gj=D_gj, iNa=int(sim.iNa), iK=int(sim.iK), is_ecm=bool(p.is_ecm),
                   T=float(sim.T), gj_block=float(np.ravel(gjb)[0]),
                   nakatp_block=float(np.ravel(nkb)[0]),
                   ko_env=float(getattr(sim, 'ko_env', 0.0)),
                   sigma=float(getattr(sim, 'sigma', 0.0)),
                   c_env_bound=np.asarray(getattr(sim, 'c_env_bound', np.zeros(len(sim.zs))), np.float64),
                   **kw)

    def to_c(self):
        c = _lib.BxParams()
        I = self.n_ions
        if I > _lib.MAX_IONS:
            raise ValueError('at most 8 ions')
        c.n_ions, c.iNa, c.iK, c.is_ecm = I, int(self.iNa), int(self.iK), int(bool(self.is_ecm))
        for n in _SCALARS:
            setattr(c, n, float(getattr(self, n)))
        cb = np.zeros(I) if self.c_env_bound is None else np.asarray(self.c_env_bound, np.float64)
        for i in range(I):
            c.zs[i] = float(self.zs[i])
            c.D_free[i] = float(self.D_free[i])
            c.D_gj[i] = float(self.D_gj[i])
            c.c_env_bound[i] = float(cb[i])
        c.v_sensitive_gj = int(bool(self.v_sensitive_gj))
        c.gj_vthresh, c.gj_min = float(self.gj_vthresh), float(self.gj_min)
        if not -1 <= int(self.iCa) < I:
            raise ValueError('iCa must be -1 or an ion row')
        c.iCa = int(self.iCa)
        c.alpha_Ca, c.KmCa_Ca, c.KmCa_ATP = float(self.alpha_Ca), float(self.KmCa_Ca), float(self.KmCa_ATP)
        c.cell_polarizability = float(self.cell_polarizability)
        return c

    def replace(self, **kw):
        d = {f.name: getattr(self, f.name) for f in fields(self)}
        d.update(kw)
        return StepParams(**d)
