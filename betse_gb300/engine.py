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


def _c(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


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

    def upload(self, vm, cc_cells, cc_at_mem, cc_env, E_env_x=None, E_env_y=None):
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
        s = _lib.BxState(_lib.dptr(vm), _lib.dptr(cc), _lib.dptr(cam), _lib.dptr(ce),
                         _lib.dptr(ex), _lib.dptr(ey))
        _lib.check(self.lib.bx_state_upload(self.h, ct.byref(s)), 'bx_state_upload')

    def step(self, n_steps=1, outputs=False, stream=None):
        st = None if stream is None else ct.c_void_p(int(stream))
        _lib.check(self.lib.bx_step(self.h, int(n_steps), int(bool(outputs)), st), 'bx_step')

    def download(self):
        I, C, M, G = self.I, self.C, self.M, self.G
        out = dict(vm=np.empty(M), cc_cells=np.empty((I, C)), cc_at_mem=np.empty((I, M)),
                   cc_env=np.empty((I, G) if self.ecm else I))
        if self.ecm:
            out['E_env_x'] = np.empty(G)
            out['E_env_y'] = np.empty(G)
        s = _lib.BxState(*[_lib.dptr(out.get(k)) for k in
                           ('vm', 'cc_cells', 'cc_at_mem', 'cc_env', 'E_env_x', 'E_env_y')])
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

    def cell_kernel_bytes(self) -> int:
        return int(self.lib.bx_cell_kernel_bytes(self.h))

    def launch_count(self) -> int:
        return int(self.lib.bx_launch_count(self.h))
