"""``ClusterEngine``: one cluster stepping on the GPU through libbx.so.

The engine owns a ``bx_handle``; state lives on the device between calls and
crosses to the host only on ``upload``/``download``/``outputs`` -- BETSE's
sampled steps.  NaN detection (``stb.check_v``/``stb.no_negs``,
``betse/science/sim_toolbox.py:332-344,475-503``) is read back by ``status``
and raised as ``BetseSimUnstableException``.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib
from .cluster import ClusterGeometry, StepParams
from .exceptions import BetseSimUnstableException

PRECISIONS = {'fp64': _lib.PLAIN_FP64, 'plain': _lib.PLAIN_FP64,
              'split': _lib.SPLIT_FP32, 'fp32': _lib.SPLIT_FP32}
# kernels (bx_set_launch_config): the split form's, and 'ion' (the plain
# form's one-lane-per-ion kernel)
KERNELS = {'tile': 0, 'persistent': 1, 'factored': 2, 'resident': 3, 'pipelined': 4, 'ion': 5}
KERNEL_NAMES = {v: k for k, v in KERNELS.items()}


def _c(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _need(a, n, what):
    """The C library reads exactly n values: refuse anything of another size."""
    if a.size != n:
        raise ValueError(f'{what}: expected {n} values, got {a.size}')


def _destinations(shapes, out):
    """Destination arrays for a download: the caller's (checked) or new ones."""
    if out is None:
        return {k: np.empty(v) for k, v in shapes.items()}
    res = {}
    for k, shape in shapes.items():
        a = out.get(k)
        if a is None:
            a = np.empty(shape)
        elif a.shape != tuple(shape) or a.dtype != np.float64 or not a.flags['C_CONTIGUOUS']:
            raise ValueError(f'{k}: need a C-contiguous float64 array of shape {tuple(shape)}')
        res[k] = a
    return res


class ClusterEngine:
    def __init__(self, geom: ClusterGeometry, params: StepParams, precision='fp64'):
        self.lib = _lib.load()
        self.geom = geom
        self.params = params
        self.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        self._cg = geom.to_c()
        self._cp = params.to_c()
        h = ct.c_void_p()
        _lib.check(self.lib.bx_cluster_create(ct.byref(self._cg), ct.byref(self._cp),
                                              self.precision, ct.byref(h)), 'bx_cluster_create')
        self.h = h
        self.I = params.n_ions
        self.C, self.M, self.G = geom.n_cells, geom.n_mems, geom.n_grid
        self.ecm = bool(params.is_ecm)
        self.vgj = bool(params.v_sensitive_gj)

    # ------------------------------------------------------------------
    def close(self):
        if getattr(self, 'h', None) is not None and self.h.value:
            self.lib.bx_destroy(self.h)
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

    # ------------------------------------------------------------------
    def set_params(self, params: StepParams):
        self.params = params
        self._cp = params.to_c()
        _lib.check(self.lib.bx_set_params(self.h, ct.byref(self._cp)), 'bx_set_params')

    def set_membrane_diffusivity(self, Dm):
        Dm = _c(Dm)
        if Dm.shape != (self.I, self.M):
            raise ValueError(f'Dm must be ({self.I}, {self.M})')
        _lib.check(self.lib.bx_set_membrane_diffusivity(self.h, _lib.dptr(Dm)),
                   'bx_set_membrane_diffusivity')

    def set_env_diffusivity(self, D_env):
        D = _c(D_env).reshape(self.I, self.G)
        _lib.check(self.lib.bx_set_env_diffusivity(self.h, _lib.dptr(D)), 'bx_set_env_diffusivity')

    def set_boundary_potential(self, Phi_b=None):
        a = None if Phi_b is None else _c(Phi_b).ravel()
        _lib.check(self.lib.bx_set_boundary_potential(self.h, _lib.dptr(a)),
                   'bx_set_boundary_potential')

    def upload(self, vm, cc_cells, cc_at_mem, cc_env, E_env_x=None, E_env_y=None, gjopen=None):
        """Upload one state. ``gjopen`` (voltage-gated gap junctions only) is the
        per-membrane open fraction; None starts from the static gj weights, as
        BETSE's ``sim.gjopen`` does before its first step."""
        vm = _c(vm)
        cc = _c(cc_cells)
        cam = _c(cc_at_mem)
        ce = _c(cc_env)
        if not self.ecm and ce.ndim == 2:
            # BETSE keeps the well-mixed environment as a uniform (I, M) array
            if not np.all(ce == ce[:, :1]):
                raise ValueError('without ECM, cc_env must be uniform over membranes')
            ce = _c(ce[:, 0])
        ex = _c(E_env_x).ravel() if E_env_x is not None else None
        ey = _c(E_env_y).ravel() if E_env_y is not None else None
        go = _c(gjopen).ravel() if (gjopen is not None and self.vgj) else None
        I, C, M, G = self.I, self.C, self.M, self.G
        _need(vm, M, 'vm')
        _need(cc, I * C, 'cc_cells')
        _need(cam, I * M, 'cc_at_mem')
        _need(ce, I * G if self.ecm else I, 'cc_env')
        for a, k in ((ex, 'E_env_x'), (ey, 'E_env_y')):
            if a is not None:
                _need(a, G, k)
        if go is not None:
            _need(go, M, 'gjopen')
        s = _lib.BxState(_lib.dptr(vm), _lib.dptr(cc), _lib.dptr(cam), _lib.dptr(ce),
                         _lib.dptr(ex), _lib.dptr(ey), _lib.dptr(go))
        _lib.check(self.lib.bx_state_upload(self.h, ct.byref(s)), 'bx_state_upload')

    def step(self, n_steps=1, outputs=False, stream=None):
        st = None if stream is None else ct.c_void_p(int(stream))
        _lib.check(self.lib.bx_step(self.h, int(n_steps), int(bool(outputs)), st), 'bx_step')

    def download(self, out=None):
        """The state in BETSE's layouts.  ``out`` (optional) holds destination
        arrays to fill, e.g. page-locked buffers reused across sampled steps;
        each must be C-contiguous float64 of the shape returned here."""
        I, C, M, G = self.I, self.C, self.M, self.G
        shapes = dict(vm=(M,), cc_cells=(I, C), cc_at_mem=(I, M), cc_env=(I, G) if self.ecm else (I,))
        if self.ecm:
            shapes.update(E_env_x=(G,), E_env_y=(G,))
        if self.vgj:
            shapes['gjopen'] = (M,)
        out = _destinations(shapes, out)
        s = _lib.BxState(*[_lib.dptr(out.get(k)) for k in
                           ('vm', 'cc_cells', 'cc_at_mem', 'cc_env', 'E_env_x', 'E_env_y', 'gjopen')])
        _lib.check(self.lib.bx_state_download(self.h, ct.byref(s)), 'bx_state_download')
        return out

    def outputs(self):
        I, C, M, G = self.I, self.C, self.M, self.G
        shapes = dict(fluxes_mem=(I, M), fluxes_gj=(I, M), rate_NaKATP=M, rho_cells=C, Jn=M,
                      I_mem=M, J_cell_x=C, J_cell_y=C, Jc=M, vm_ave=C, dvm=M, E_cell_x=C,
                      E_cell_y=C, Emc=M, E_gj_x=M, E_gj_y=M, gjopen=M, sigma_cell=C)
        if self.ecm:
            shapes.update(fluxes_env_x=(I, G), fluxes_env_y=(I, G), rho_env=G, v_env=G)
        arrs = {k: np.empty(v) for k, v in shapes.items()}
        o = _lib.BxOutputs(*[_lib.dptr(arrs.get(k)) for k in _lib.OUTPUT_FIELDS])
        _lib.check(self.lib.bx_outputs_download(self.h, ct.byref(o)), 'bx_outputs_download')
        return arrs

    def max_abs_dvm(self):
        """Per-cluster max |dVm/dt| of the last step (which ran with outputs=True)."""
        n = getattr(self, 'n_clusters', 1)
        out = np.empty(n)
        _lib.check(self.lib.bx_max_abs_dvm(self.h, _lib.dptr(out)), 'bx_max_abs_dvm')
        return out

    def build_lap_env_inv(self):
        """Build ``cells.lapENVinv`` for this cluster's grid on the GPU (no
        host array; the eigenvector construction of ``bx_build_lap_env_inv``)."""
        _lib.check(self.lib.bx_build_lap_env_inv(self.h), 'bx_build_lap_env_inv')

    def set_lap_env_inv(self, lap_env_inv):
        """Keep ``cells.lapENVinv`` ([grid, grid]) on the GPU for ``env_fields``."""
        A = _c(lap_env_inv)
        if A.shape != (self.G, self.G):
            raise ValueError(f'lapENVinv must be ({self.G}, {self.G})')
        _lib.check(self.lib.bx_set_lap_env_inv(self.h, _lib.dptr(A)), 'bx_set_lap_env_inv')

    def env_fields(self, D_env_weight=None):
        """Environment fields of the last step (which ran with ``outputs=True``):
        v_env, E_env_x/y, J_env_x/y, B_field, each of length grid."""
        G = self.G
        w = None if D_env_weight is None else _c(D_env_weight).ravel()
        if w is not None and w.shape != (G,):
            raise ValueError(f'D_env_weight must have {G} values')
        names = ('v_env', 'E_env_x', 'E_env_y', 'J_env_x', 'J_env_y', 'B_field')
        out = {k: np.empty(G) for k in names}
        _lib.check(self.lib.bx_env_fields(self.h, _lib.dptr(w), *[_lib.dptr(out[k]) for k in names]),
                   'bx_env_fields')
        return out

    def time_env_fields(self, n=5):
        """(ms of the whole field computation, ms of one two-column lapENVinv product)."""
        a, b = ct.c_double(), ct.c_double()
        _lib.check(self.lib.bx_time_env_fields(self.h, int(n), ct.byref(a), ct.byref(b)),
                   'bx_time_env_fields')
        return a.value, b.value

    def status(self):
        st = _lib.BxStepStatus()
        _lib.check(self.lib.bx_status(self.h, ct.byref(st)), 'bx_status')
        return dict(steps_done=st.steps_done, nan_vm=st.nan_vm, nan_conc=st.nan_conc,
                    neg_clamped=st.neg_clamped, unstable=bool(st.unstable))

    def check_stable(self):
        st = self.status()
        if st['unstable']:
            raise BetseSimUnstableException(
                'Your simulation has become unstable. Please try a smaller time step,'
                'reduce gap junction radius, and/or reduce rate coefficients.')
        return st

    def time_cell_kernel(self, n=20) -> float:
        """Mean ms of one fused-cell-kernel launch (CUDA events, handle stream).
        Advances the state; re-upload afterwards."""
        ms = ct.c_double()
        _lib.check(self.lib.bx_time_cell_kernel(self.h, int(n), ct.byref(ms)), 'bx_time_cell_kernel')
        return ms.value

    def set_launch_config(self, tpb, kernel=0, variant=0):
        """Pin the tile size (membrane slots per tile) and, for the split form,
        the kernel: 0/'tile', 1/'persistent' (True), 2/'factored',
        3/'resident', 4/'pipelined' (factored, persistent); ``variant`` picks
        the factored kernel's (2, 3, 4 or 6 junctions per load round, +10
        with prefetched entries: 2, 4, 12, 13, 14, 16; 0 keeps it). The state
        is kept."""
        k = KERNELS[kernel] if isinstance(kernel, str) else int(kernel)
        _lib.check(self.lib.bx_set_launch_config(self.h, int(tpb), k | (int(variant) << 8)),
                   'bx_set_launch_config')

    def launch_config(self):
        """(membrane slots per tile, kernel number) in use."""
        tpb, kind = ct.c_int(), ct.c_int()
        _lib.check(self.lib.bx_get_launch_config(self.h, ct.byref(tpb), ct.byref(kind)), 'bx_get_launch_config')
        return tpb.value, kind.value

    def resident_barrier_check(self, timeout_s=0.05):
        """Run the resident kernel once with a grid barrier that cannot
        complete; True if its bounded wait ran out and was reported (the
        state is unchanged)."""
        t = ct.c_int()
        _lib.check(self.lib.bx_resident_barrier_check(self.h, int(timeout_s * 1e9), ct.byref(t)),
                   'bx_resident_barrier_check')
        return bool(t.value)

    def resident_info(self):
        """Whether the resident kernel fits this cluster: dict(fits, grid,
        threads, smem_bytes, why)."""
        fits, grid, thr, smem = ct.c_int(), ct.c_int(), ct.c_int(), ct.c_int64()
        rc = self.lib.bx_resident_info(self.h, ct.byref(fits), ct.byref(grid), ct.byref(thr), ct.byref(smem))
        why = '' if rc == _lib.BX_OK else (self.lib.bx_last_error() or b'').decode()
        return dict(fits=bool(fits.value), grid=grid.value, threads=thr.value, smem_bytes=smem.value, why=why)

    def autotune(self, n_steps=20):
        """Pick the fastest CTA size for this cluster; the state is unchanged.
        Returns (threads per CTA, ms per step)."""
        tpb = ct.c_int()
        ms = ct.c_double()
        _lib.check(self.lib.bx_autotune(self.h, int(n_steps), ct.byref(tpb), ct.byref(ms)), 'bx_autotune')
        return tpb.value, ms.value

    def autotune_table(self, n_steps=20):
        """Time every candidate launch configuration (as ``autotune``) and keep
        the fastest; returns the rows as dicts (tpb, kernel, unroll, ms_per_step)."""
        n = 32
        tpb, ker, unr = (np.zeros(n, np.int32) for _ in range(3))
        ms = np.zeros(n)
        rows = ct.c_int()
        _lib.check(self.lib.bx_autotune_table(self.h, int(n_steps), n, ct.byref(rows), _lib.iptr(tpb),
                                              _lib.iptr(ker), _lib.iptr(unr), _lib.dptr(ms)), 'bx_autotune_table')
        return [dict(tpb=int(tpb[r]), kernel=KERNEL_NAMES.get(int(ker[r]), str(ker[r])), unroll=int(unr[r]),
                     ms_per_step=float(ms[r])) for r in range(rows.value)]

    def cell_kernel_bytes(self) -> int:
        return int(self.lib.bx_cell_kernel_bytes(self.h))

    def launch_count(self) -> int:
        return int(self.lib.bx_launch_count(self.h))


class BatchEngine(ClusterEngine):
    """Many independent clusters stepped together (a parameter sweep).

    Arrays are the clusters' arrays concatenated in order; ``layout`` gives
    each cluster's cell and membrane offsets. Clusters may differ in geometry,
    ``alpha_NaK``, ``nakatp_block`` and ``vol_env``.
    """

    def __init__(self, geoms, params, precision='split'):
        self.lib = _lib.load()
        self.geoms = list(geoms)
        self.params_list = list(params)
        self.params = self.params_list[0]
        self.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        n = len(self.geoms)
        self._cgs = (_lib.BxGeom * n)(*[g.to_c() for g in self.geoms])
        self._cps = (_lib.BxParams * n)(*[p.to_c() for p in self.params_list])
        h = ct.c_void_p()
        _lib.check(self.lib.bx_batch_create(self._cgs, self._cps, n, self.precision, ct.byref(h)),
                   'bx_batch_create')
        self.h = h
        self.n_clusters = n
        self.I = self.params.n_ions
        self.C = sum(g.n_cells for g in self.geoms)
        self.M = sum(g.n_mems for g in self.geoms)
        self.G = self.geoms[0].n_grid
        self.ecm = False
        self.vgj = bool(self.params.v_sensitive_gj)
        co = np.zeros(n + 1, np.int32)
        mo = np.zeros(n + 1, np.int32)
        _lib.check(self.lib.bx_batch_layout(self.h, _lib.iptr(co), _lib.iptr(mo)), 'bx_batch_layout')
        self.cell_offsets, self.mem_offsets = co, mo

    def set_membrane_diffusivity(self, Dm_list):
        Dm = np.concatenate([_c(d) for d in Dm_list], axis=1) if isinstance(Dm_list, (list, tuple)) else _c(Dm_list)
        super().set_membrane_diffusivity(Dm)

    def upload_states(self, states):
        """Upload a list of per-cluster state dicts (as ``ClusterEngine.upload``)."""
        cat = lambda k, ax: np.concatenate([_c(s[k]) for s in states], axis=ax)  # noqa: E731
        ce = []
        for s in states:
            e = _c(s['cc_env'])
            if e.ndim == 2:
                if not np.all(e == e[:, :1]):
                    raise ValueError('without ECM, cc_env must be uniform over membranes')
                e = e[:, 0]
            ce.append(e)
        vm, cc, cam, cenv = cat('vm', 0), cat('cc_cells', 1), cat('cc_at_mem', 1), _c(np.stack(ce))
        for a, n, k in ((vm, self.M, 'vm'), (cc, self.I * self.C, 'cc_cells'), (cam, self.I * self.M, 'cc_at_mem'),
                        (cenv, self.n_clusters * self.I, 'cc_env')):
            _need(a, n, k)
        go = None
        if self.vgj and all(s.get('gjopen') is not None for s in states):
            go = cat('gjopen', 0)
            _need(go, self.M, 'gjopen')
        st = _lib.BxState(_lib.dptr(vm), _lib.dptr(cc), _lib.dptr(cam), _lib.dptr(cenv), None, None,
                          _lib.dptr(go))
        _lib.check(self.lib.bx_state_upload(self.h, ct.byref(st)), 'bx_state_upload')

    def upload_concat(self, vm, cc_cells, cc_at_mem, cc_env):
        """Upload the concatenated state directly (cc_env is [n_clusters, n_ions]);
        the arrays are passed to the C ABI as they are (e.g. pinned views)."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (vm, cc_cells, cc_at_mem, cc_env)]
        for a, n, k in zip(arrs, (self.M, self.I * self.C, self.I * self.M, self.n_clusters * self.I),
                           ('vm', 'cc_cells', 'cc_at_mem', 'cc_env')):
            _need(a, n, k)
        st = _lib.BxState(*[_lib.dptr(a) for a in arrs], None, None, None)
        _lib.check(self.lib.bx_state_upload(self.h, ct.byref(st)), 'bx_state_upload')

    def download_concat(self, out=None):
        """The concatenated state (``out``: optional destination arrays, as in
        ``ClusterEngine.download``)."""
        I = self.I
        out = _destinations(dict(vm=(self.M,), cc_cells=(I, self.C), cc_at_mem=(I, self.M),
                                 cc_env=(self.n_clusters, I)), out)
        st = _lib.BxState(*[_lib.dptr(out[k]) for k in ('vm', 'cc_cells', 'cc_at_mem', 'cc_env')], None, None, None)
        _lib.check(self.lib.bx_state_download(self.h, ct.byref(st)), 'bx_state_download')
        return out

    def set_lap_env_inv_shape(self, lap_env_inv, grid_shape, delta):
        """lapENVinv of one cluster of the batch with this grid shape and spacing;
        every cluster of that shape uses it (scaled by its own delta^2)."""
        ny, nx = (int(x) for x in grid_shape)
        A = _c(lap_env_inv)
        if A.shape != (ny * nx, ny * nx):
            raise ValueError(f'lapENVinv must be ({ny * nx}, {ny * nx})')
        _lib.check(self.lib.bx_batch_set_lap_env_inv(self.h, ny, nx, float(delta), _lib.dptr(A)),
                   'bx_batch_set_lap_env_inv')

    def env_fields(self, D_env_weights=None):
        """Environment fields of the last step for every cluster (list of dicts),
        the dense products of each grid shape done as one tensor-core GEMM."""
        sizes = [g.n_grid for g in self.geoms]
        offs = np.concatenate([[0], np.cumsum(sizes)])
        w = None
        if D_env_weights is not None:
            w = _c(np.concatenate([np.ravel(x) for x in D_env_weights]))
            if w.shape != (offs[-1],):
                raise ValueError('one D_env_weight per grid cell of every cluster')
        names = ('v_env', 'E_env_x', 'E_env_y', 'J_env_x', 'J_env_y', 'B_field')
        out = {k: np.empty(offs[-1]) for k in names}
        _lib.check(self.lib.bx_batch_env_fields(self.h, _lib.dptr(w), *[_lib.dptr(out[k]) for k in names]),
                   'bx_batch_env_fields')
        return [{k: out[k][offs[c]:offs[c + 1]].copy() for k in names} for c in range(len(sizes))]

    def download_states(self):
        I = self.I
        vm, cc, cam = np.empty(self.M), np.empty((I, self.C)), np.empty((I, self.M))
        cenv = np.empty((self.n_clusters, I))
        go = np.empty(self.M) if self.vgj else None
        st = _lib.BxState(_lib.dptr(vm), _lib.dptr(cc), _lib.dptr(cam), _lib.dptr(cenv), None, None,
                          _lib.dptr(go))
        _lib.check(self.lib.bx_state_download(self.h, ct.byref(st)), 'bx_state_download')
        out = []
        for k in range(self.n_clusters):
            c0, c1 = self.cell_offsets[k], self.cell_offsets[k + 1]
            m0, m1 = self.mem_offsets[k], self.mem_offsets[k + 1]
            out.append(dict(vm=vm[m0:m1].copy(), cc_cells=cc[:, c0:c1].copy(),
                            cc_at_mem=cam[:, m0:m1].copy(), cc_env=cenv[k].copy()))
            if go is not None:
                out[-1]['gjopen'] = go[m0:m1].copy()
        return out
