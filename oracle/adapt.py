"""Oracle inputs from a library workload (TEST INFRASTRUCTURE ONLY).

Turns a ``betse_gb300.cluster.ClusterGeometry`` / ``StepParams`` pair, the
membrane diffusivities and an initial state (as ``betse_gb300.generator``
makes them) into the (geometry, parameters, state) records ``oracle.step``
reads, with BETSE's attribute names.
"""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np

from .step import OracleState, init_fields

_GEOM = ('mem_to_cells', 'nn_i', 'map_mem2ecm', 'mem_sa', 'mem_nx', 'mem_ny', 'cell_vol',
         'cell_sa', 'diviterm', 'num_mems', 'smooth_weight_mem', 'smooth_weight_o', 'delta',
         'gj_len', 'cell_mem_ptr', 'gj_weight')
_PAR = ('F', 'R', 'T', 'dt', 'cm', 'tm', 'gj_surface', 'alpha_NaK', 'KmNK_Na', 'KmNK_K',
        'KmNK_ATP', 'cATP', 'cADP', 'cPi', 'deltaGATP', 'vol_env', 'zs', 'D_free', 'D_gj',
        'iNa', 'iK', 'is_ecm', 'gj_block', 'nakatp_block', 'cell_height', 'q', 'kb', 'eo',
        'er', 'sharpness', 'cell_radius', 'true_cell_size', 'mu')


def from_workload(g, p, Dm, st, D_env=None):
    geo = SimpleNamespace(**{k: getattr(g, k) for k in _GEOM})
    geo.bflag = np.asarray(g.bflag).astype(bool)
    geo.grid_shape = tuple(int(x) for x in g.grid_shape)
    geo.mem_to_cells = np.asarray(g.mem_to_cells, np.int64)
    geo.nn_i = np.asarray(g.nn_i, np.int64)
    geo.map_mem2ecm = np.asarray(g.map_mem2ecm, np.int64)
    geo.sigma = float(p.sigma)
    if getattr(g, 'R_rads', None) is not None:
        geo.R_rads = np.asarray(g.R_rads, np.float64)
    geo.ko_env = float(p.ko_env)
    if g.D_env_weight is not None:
        geo.D_env_weight = np.asarray(g.D_env_weight)
    par = SimpleNamespace(**{k: getattr(p, k) for k in _PAR})
    par.is_ecm = bool(p.is_ecm)
    par.Dm = np.asarray(Dm, np.float64)
    I, M = par.Dm.shape
    G = int(np.prod(geo.grid_shape))
    if par.is_ecm:
        geo.D_env = np.asarray(D_env, np.float64).reshape(I, G)
        geo.memSa_per_envSquare = np.asarray(g.mem_sa_per_env)
        par.c_env_bound = np.asarray(p.c_env_bound, np.float64)
        ce = np.asarray(st['cc_env'], np.float64).reshape(I, G).copy()
    else:
        ce = np.repeat(np.asarray(st['cc_env'], np.float64)[:, None], M, axis=1)
    s = OracleState(vm=np.asarray(st['vm'], np.float64).copy(),
                    cc_cells=np.asarray(st['cc_cells'], np.float64).copy(),
                    cc_at_mem=np.asarray(st['cc_at_mem'], np.float64).copy(),
                    cc_env=ce, Phi_b=np.zeros(G))
    if par.is_ecm:
        if st.get('E_env_x') is not None:
            s.E_env_x = np.asarray(st['E_env_x'], np.float64).reshape(geo.grid_shape).copy()
            s.E_env_y = np.asarray(st['E_env_y'], np.float64).reshape(geo.grid_shape).copy()
        else:
            init_fields(geo, par, s)
    return geo, par, s
