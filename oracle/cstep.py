"""ctypes wrapper of the C restatement ``oracle/c/bx_oracle.c`` -- TEST
INFRASTRUCTURE AND CPU BASELINE ONLY.

``build()`` compiles it with gcc and OpenMP into ``oracle/_build/``;
``Stepper`` advances a cluster, with or without extracellular spaces, given in
the records ``oracle.step`` reads (``oracle.adapt.from_workload`` or the
golden fixtures), on every host thread OpenMP offers unless told otherwise.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, 'c', 'bx_oracle.c')
OUT_DIR = os.path.join(HERE, '_build')
LIB = os.path.join(OUT_DIR, 'libbx_oracle.so')
MAX_IONS = 8

# IEEE arithmetic without contraction into FMA, so x86 and Arm builds agree;
# no -march=native (the library is rebuilt on each machine)
CFLAGS = ['-O2', '-fopenmp', '-ffp-contract=off', '-fno-fast-math', '-fPIC', '-shared', '-std=c11']


def build(force=False):
    """Compile the C restatement if it is missing or older than its source."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + '.tmp'
    subprocess.run(['gcc', *CFLAGS, '-o', tmp, SRC, '-lm'], check=True)
    os.replace(tmp, LIB)
    return LIB


class _Cluster(ct.Structure):
    _fields_ = [('C', ct.c_int32), ('M', ct.c_int32), ('I', ct.c_int32), ('iNa', ct.c_int32),
                ('iK', ct.c_int32), ('pad0', ct.c_int32),
                ('cell_ptr', ct.c_void_p), ('m2c', ct.c_void_p), ('nn', ct.c_void_p),
                ('bflag', ct.c_void_p), ('mem_sa', ct.c_void_p), ('gj_w', ct.c_void_p),
                ('cell_vol', ct.c_void_p), ('diviterm', ct.c_void_p), ('Dm', ct.c_void_p),
                ('zs', ct.c_double * MAX_IONS), ('D_gj', ct.c_double * MAX_IONS)] + \
        [(n, ct.c_double) for n in ('F', 'R', 'T', 'dt', 'cm', 'tm', 'gj_surface', 'gj_block', 'gj_len',
                                    'nakatp_block', 'alpha_NaK', 'KmNK_Na', 'KmNK_K', 'KmNK_ATP', 'cATP',
                                    'cADP', 'cPi', 'deltaGATP', 'vol_env')] + \
        [('vgj', ct.c_int32), ('iCa', ct.c_int32)] + \
        [(n, ct.c_double) for n in ('gj_vthresh', 'gj_min', 'alpha_Ca', 'KmCa_Ca', 'KmCa_ATP')] + \
        [('is_ecm', ct.c_int32), ('ny', ct.c_int32), ('nx', ct.c_int32), ('pad1', ct.c_int32),
         ('map_env', ct.c_void_p), ('D_env', ct.c_void_p), ('msa_env', ct.c_void_p),
         ('c_bound', ct.c_double * MAX_IONS)] + \
        [(n, ct.c_double) for n in ('delta', 'cell_height', 'q', 'kb', 'eo', 'er', 'ko_env', 'cell_radius',
                                    'true_cell_size', 'sharpness')] + \
        [('polar', ct.c_int32), ('pad2', ct.c_int32), ('R_rads', ct.c_void_p), ('sw_mem', ct.c_void_p),
         ('sw_o', ct.c_void_p), ('cell_sa', ct.c_void_p), ('D_free', ct.c_double * MAX_IONS),
         ('phib', ct.c_void_p)]


_lib = None


def load():
    global _lib
    if _lib is None:
        try:
            lib = ct.CDLL(build())
        except OSError:         # a library built for another machine: rebuild here
            lib = ct.CDLL(build(force=True))
        lib.bxo_step.restype = ct.c_int
        lib.bxo_step.argtypes = [ct.POINTER(_Cluster)] + [ct.c_void_p] * 7 + [ct.c_int, ct.c_int]
        lib.bxo_max_threads.restype = ct.c_int
        _lib = lib
    return _lib


def max_threads():
    return int(load().bxo_max_threads())


def _ptr(a):
    return ct.c_void_p(a.ctypes.data)


class Stepper:
    """A cluster on the C restatement.  ``g``/``p``/``s`` are the records
    ``oracle.step`` reads (BETSE attribute names); the state is copied in and
    ``state()`` returns it in the same shapes."""

    def __init__(self, g, p, s, threads=0):
        self.lib = load()
        self.threads = int(threads)
        m2c = np.ascontiguousarray(g.mem_to_cells, np.int64)
        M = len(m2c)
        C = len(g.cell_vol)
        ptr = np.asarray(getattr(g, 'cell_mem_ptr', None) if getattr(g, 'cell_mem_ptr', None) is not None
                         else np.concatenate([[0], np.cumsum(np.bincount(m2c, minlength=C))]), np.int64)
        bflag = np.zeros(M, np.uint8)
        bf = np.asarray(g.bflag)
        if bf.dtype == bool and bf.shape == (M,):
            bflag[:] = bf
        else:
            bflag[np.asarray(bf, np.int64)] = 1
        Dm = np.ascontiguousarray(p.Dm, np.float64)
        I = Dm.shape[0]
        self._keep = dict(ptr=np.ascontiguousarray(ptr), m2c=m2c, nn=np.ascontiguousarray(g.nn_i, np.int64),
                          bflag=bflag, sa=np.ascontiguousarray(g.mem_sa, np.float64),
                          gjw=np.ascontiguousarray(getattr(g, 'gj_weight', None) if getattr(g, 'gj_weight', None)
                                                   is not None else g.gj_default_weights, np.float64),
                          vol=np.ascontiguousarray(g.cell_vol, np.float64),
                          div=np.ascontiguousarray(g.diviterm, np.float64), Dm=Dm)
        k = _Cluster()
        k.C, k.M, k.I, k.iNa, k.iK = C, M, I, int(p.iNa), int(p.iK)
        kp = self._keep
        k.cell_ptr, k.m2c, k.nn, k.bflag = _ptr(kp['ptr']), _ptr(kp['m2c']), _ptr(kp['nn']), _ptr(kp['bflag'])
        k.mem_sa, k.gj_w, k.cell_vol, k.diviterm = _ptr(kp['sa']), _ptr(kp['gjw']), _ptr(kp['vol']), _ptr(kp['div'])
        k.Dm = _ptr(kp['Dm'])
        for i in range(I):
            k.zs[i] = float(p.zs[i])
            k.D_gj[i] = float(np.ravel(p.D_gj)[i])
        for n in ('F', 'R', 'T', 'dt', 'cm', 'tm', 'gj_surface', 'alpha_NaK', 'KmNK_Na', 'KmNK_K', 'KmNK_ATP',
                  'cATP', 'cADP', 'cPi', 'deltaGATP', 'vol_env'):
            setattr(k, n, float(getattr(p, n)))
        k.gj_block = float(getattr(p, 'gj_block', 1.0))
        k.nakatp_block = float(getattr(p, 'nakatp_block', 1.0))
        k.gj_len = float(g.gj_len)
        k.vgj = int(bool(getattr(p, 'v_sensitive_gj', False)))
        k.iCa = int(getattr(p, 'iCa', -1))
        k.alpha_Ca = float(getattr(p, 'alpha_Ca', 0.0))
        k.KmCa_Ca = float(getattr(p, 'KmCa_Ca', 1e-3))
        k.KmCa_ATP = float(getattr(p, 'KmCa_ATP', 0.5))
        k.gj_vthresh = float(getattr(p, 'gj_vthresh', 15.0))
        k.gj_min = float(getattr(p, 'gj_min', 0.10))
        if float(getattr(p, 'cell_polarizability', 0.0)) != 0.0:
            kp.update(R_rads=np.ascontiguousarray(g.R_rads, np.float64),
                      sw_mem=np.ascontiguousarray(g.smooth_weight_mem, np.float64),
                      sw_o=np.ascontiguousarray(g.smooth_weight_o, np.float64),
                      cell_sa=np.ascontiguousarray(g.cell_sa, np.float64))
            k.polar = 1
            k.R_rads, k.sw_mem, k.sw_o, k.cell_sa = (_ptr(kp['R_rads']), _ptr(kp['sw_mem']), _ptr(kp['sw_o']),
                                                     _ptr(kp['cell_sa']))
            for i in range(I):
                k.D_free[i] = float(np.ravel(p.D_free)[i])
        self.ecm = bool(getattr(p, 'is_ecm', False))
        phib = getattr(s, 'Phi_b', None)
        if phib is not None and np.any(np.asarray(phib) != 0):
            kp.update(phib=np.ascontiguousarray(np.ravel(phib), np.float64),
                      map_env=np.ascontiguousarray(g.map_mem2ecm, np.int64))
            k.phib, k.map_env = _ptr(kp['phib']), _ptr(kp['map_env'])
        if self.ecm:
            ny, nx = (int(x) for x in g.grid_shape)
            G = ny * nx
            kp.update(map_env=np.ascontiguousarray(g.map_mem2ecm, np.int64),
                      D_env=np.ascontiguousarray(np.asarray(g.D_env, np.float64).reshape(I, G)),
                      msa_env=np.ascontiguousarray(np.ravel(g.memSa_per_envSquare), np.float64))
            k.is_ecm, k.ny, k.nx = 1, ny, nx
            k.map_env, k.D_env, k.msa_env = _ptr(kp['map_env']), _ptr(kp['D_env']), _ptr(kp['msa_env'])
            for i in range(I):
                k.c_bound[i] = float(np.ravel(p.c_env_bound)[i])
            for n in ('cell_height', 'q', 'kb', 'eo', 'er', 'cell_radius', 'true_cell_size', 'sharpness'):
                setattr(k, n, float(getattr(p, n)))
            k.delta, k.ko_env = float(g.delta), float(g.ko_env)
        self.k = k
        self.C, self.M, self.I = C, M, I
        self.m2c = m2c
        self.vm = np.ascontiguousarray(s.vm, np.float64).copy()
        self.cc = np.ascontiguousarray(s.cc_cells, np.float64).copy()
        cam = np.asarray(s.cc_at_mem, np.float64)
        first = kp['ptr'][:-1]
        self.ccm = np.ascontiguousarray(cam[:, first])
        ce = np.asarray(s.cc_env, np.float64)
        if self.ecm:
            self.cenv = np.ascontiguousarray(ce.reshape(I, -1)).copy()
            self.grid_shape = tuple(int(x) for x in g.grid_shape)
            self.Ex = np.ascontiguousarray(np.ravel(s.E_env_x), np.float64).copy()
            self.Ey = np.ascontiguousarray(np.ravel(s.E_env_y), np.float64).copy()
        else:
            self.cenv = np.ascontiguousarray(ce[:, 0] if ce.ndim == 2 else ce).copy()
            self.Ex = self.Ey = None
        # the open fraction with gating (sim.gjopen; the static weights before the first step)
        go = getattr(s, 'gjopen', None)
        self.gjopen = (np.ascontiguousarray(go if go is not None else kp['gjw'], np.float64).copy()
                       if k.vgj else None)

    def step(self, n=1):
        opt = lambda a: None if a is None else _ptr(a)  # noqa: E731
        rc = self.lib.bxo_step(ct.byref(self.k), _ptr(self.vm), _ptr(self.cc), _ptr(self.ccm), _ptr(self.cenv),
                               opt(self.gjopen), opt(self.Ex), opt(self.Ey), int(n), self.threads)
        if rc == 1:
            raise FloatingPointError('NaN concentration or Vmem (check_v / no_negs)')
        if rc != 0:
            raise RuntimeError(f'bxo_step_noecm failed ({rc})')

    def state(self):
        out = dict(vm=self.vm.copy(), cc_cells=self.cc.copy(), cc_at_mem=self.ccm[:, self.m2c].copy(),
                   cc_env=self.cenv.copy() if self.ecm else np.repeat(self.cenv[:, None], self.M, axis=1))
        if self.ecm:
            out['E_env_x'] = self.Ex.reshape(self.grid_shape).copy()
            out['E_env_y'] = self.Ey.reshape(self.grid_shape).copy()
        if self.gjopen is not None:
            out['gjopen'] = self.gjopen.copy()
        return out
