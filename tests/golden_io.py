"""Load the committed golden fixtures into (geometry, params, state) records.

The fixtures were written by ``tests/golden/make_golden.py`` from BETSE's own
``Cells``/``Simulator`` objects; field names follow BETSE's attributes.
"""
from __future__ import annotations

import os
from types import SimpleNamespace

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
CASES = ['noecm_r80_s1', 'noecm_r50_s7', 'ecm_r50_s3', 'ecm_r40_s5_sharp', 'noecm_r50_s9_vgj',
         'noecm_r50_s11_ca', 'ecm_r40_s13_ca', 'noecm_r50_s17_pol', 'noecm_r20_s2']


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + '.npz')))


def polar(d):
    """Cell polarizability on: Vmem is per-membrane state, which only the
    plain FP64 form keeps (the split form refuses the configuration)."""
    return float(d.get('par_cell_polarizability', 0.0)) != 0.0


def geometry(d):
    g = SimpleNamespace()
    for k, v in d.items():
        if k.startswith('geom_'):
            setattr(g, k[5:], v)
    M = len(g.mem_to_cells)
    C = len(g.cell_vol)
    g.n_mems, g.n_cells = M, C
    g.cell_mem_ptr = np.concatenate([[0], np.cumsum(np.bincount(g.mem_to_cells, minlength=C))]).astype(np.int64)
    g.bflag = np.zeros(M, bool)
    g.bflag[g.bflags_mems] = True
    g.mem_nx = np.ascontiguousarray(g.mem_vects_flat[:, 2])
    g.mem_ny = np.ascontiguousarray(g.mem_vects_flat[:, 3])
    g.gj_weight = g.gj_default_weights
    g.grid_shape = tuple(int(x) for x in g.grid_shape)
    g.delta = float(g.delta)
    g.gj_len = float(g.gj_len)
    g.smooth_weight_mem = d['par_smooth_weight_mem']
    g.smooth_weight_o = d['par_smooth_weight_o']
    g.sigma = float(d['par_sigma'])
    g.D_env_weight = g.D_env_weight.ravel()
    if hasattr(g, 'ko_env'):
        g.ko_env = float(g.ko_env)
    return g


def params(d):
    p = SimpleNamespace()
    for k, v in d.items():
        if k.startswith('par_') and np.ndim(v) == 0 and v.dtype.kind == 'f':
            setattr(p, k[4:], float(v))
    p.zs = d['par_zs']
    p.D_free = d['par_D_free']
    p.D_gj = d['par_D_gj']
    p.Dm = d['par_Dm_cells']
    names = [str(x) for x in d['par_ion_names']]
    p.ion_names = names
    p.iNa, p.iK = names.index('Na'), names.index('K')
    p.iCa = names.index('Ca') if 'Ca' in names else -1
    p.alpha_Ca = float(getattr(p, 'alpha_Ca', 0.0))
    p.is_ecm = bool(p.is_ecm)
    p.v_sensitive_gj = bool(getattr(p, 'v_sensitive_gj', 0.0))
    p.nakatp_block = 1.0
    p.gj_block = 1.0
    if 'geom_c_env_bound' in d:
        p.c_env_bound = d['geom_c_env_bound']
    return p


def state(d, prefix='init'):
    from oracle import OracleState
    g = geometry(d)
    G = int(np.prod(g.grid_shape))
    s = OracleState(vm=d[prefix + '_vm'].copy(),
                    cc_cells=d[prefix + '_cc_cells'].copy(),
                    cc_at_mem=d[prefix + '_cc_at_mem'].copy(),
                    cc_env=d[prefix + '_cc_env'].copy(),
                    Phi_b=np.zeros(G))
    if prefix + '_gjopen' in d:
        s.gjopen = d[prefix + '_gjopen'].copy()
    if bool(d['par_is_ecm']):
        s.E_env_x = np.zeros(g.grid_shape)
        s.E_env_y = np.zeros(g.grid_shape)
        from oracle import init_fields
        init_fields(g, params(d), s)
    return s


def rel_err(a, b):
    """max |a-b| / max |b| (0 when both vanish)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.max(np.abs(b)) if b.size else 0.0
    num = np.max(np.abs(a - b)) if b.size else 0.0
    return 0.0 if num == 0.0 else num / (den if den > 0 else 1.0)


def engine_inputs(d):
    """(ClusterGeometry, StepParams, Dm, state kwargs, D_env) for ClusterEngine."""
    from betse_gb300.cluster import ClusterGeometry, StepParams
    g = geometry(d)
    p = params(d)
    cg = ClusterGeometry.from_cells(g, sim=SimpleNamespace(
        smooth_weight_mem=g.smooth_weight_mem, smooth_weight_o=g.smooth_weight_o,
        D_env_weight=g.D_env_weight))
    kw = {k: getattr(p, k) for k in ('F', 'R', 'T', 'dt', 'cm', 'tm', 'gj_surface',
                                     'alpha_NaK', 'KmNK_Na', 'KmNK_K', 'KmNK_ATP', 'cATP',
                                     'cADP', 'cPi', 'deltaGATP', 'vol_env', 'cell_height',
                                     'q', 'kb', 'eo', 'er', 'mu', 'sharpness',
                                     'cell_radius', 'true_cell_size')}
    sp = StepParams(zs=p.zs, D_free=p.D_free, D_gj=p.D_gj, iNa=p.iNa, iK=p.iK,
                    is_ecm=p.is_ecm, ko_env=getattr(g, 'ko_env', 0.0), sigma=g.sigma,
                    c_env_bound=getattr(p, 'c_env_bound', None), ion_names=p.ion_names,
                    v_sensitive_gj=p.v_sensitive_gj, gj_vthresh=getattr(p, 'gj_vthresh', 15.0),
                    gj_min=getattr(p, 'gj_min', 0.10), iCa=p.iCa, alpha_Ca=p.alpha_Ca,
                    KmCa_Ca=getattr(p, 'KmCa_Ca', 1.0e-3), KmCa_ATP=getattr(p, 'KmCa_ATP', 0.5),
                    cell_polarizability=getattr(p, 'cell_polarizability', 0.0), **kw)
    s = state(d)
    st = dict(vm=s.vm, cc_cells=s.cc_cells, cc_at_mem=s.cc_at_mem, cc_env=s.cc_env)
    if p.v_sensitive_gj:
        st['gjopen'] = s.gjopen
    if p.is_ecm:
        st.update(E_env_x=s.E_env_x, E_env_y=s.E_env_y)
    D_env = getattr(g, 'D_env', None)
    return cg, sp, p.Dm, st, D_env


def vm_floor(d, cc_cells, ulps=4.0):
    """FP64 cancellation floor of Vmem (volts).

    Vmem = (sum_i z_i F c_i) * diviterm / cm is a small difference of charges of
    ~1e7 C/m3 (betse/science/sim.py:2027-2029); any two summation orders of that
    sum differ by a few ulp of the largest term, mapped to volts here."""
    zF = np.abs(d['par_zs'] * d['par_F'])
    charge = (zF[:, None] * np.abs(cc_cells)).sum(axis=0)
    div = d['geom_diviterm']
    return ulps * np.finfo(np.float64).eps * np.max(charge * div) / float(d['par_cm'])


def vm_err_ok(d, vm, vm_ref, cc_ref, rel=1e-10):
    err = np.max(np.abs(vm - vm_ref))
    bound = rel * np.max(np.abs(vm_ref)) + vm_floor(d, cc_ref)
    return err <= bound, err, bound


def output_floors(d, cc, o):
    """Absolute FP64 cancellation floors of the step outputs (see vm_floor).

    * rho_cells, vm_ave, dvm: the charge sum (~1e7 C/m3 terms);
    * fluxes: the GHK numerator cB - cA*exp(-alpha) cancels near equilibrium and
      between nearly equal neighbour cells (a few ulp of one term), and alpha =
      z F V/(R T) carries the Vmem floor (for gap junctions twice, through
      vm[nn] - vm[m]); the currents built from the fluxes (Jn, I_mem, J_cell,
      Jc, E_cell, Emc) carry the same floors times |z| F."""
    eps = np.finfo(np.float64).eps
    zF = np.abs(d['par_zs'] * d['par_F'])
    rho_floor = 4 * eps * np.max((zF[:, None] * cc).sum(axis=0))
    vfl = vm_floor(d, cc)
    F_RT = float(d['par_F']) / (float(d['par_R']) * float(d['par_T']))
    cmax = np.max(np.abs(cc), axis=1)
    env = np.asarray(d['init_cc_env'])
    cenv = np.max(np.abs(env), axis=1) if env.ndim == 2 else np.abs(env)
    mem_term = np.max(d['par_Dm_cells'], axis=1) / float(d['par_tm']) * np.maximum(cmax, cenv)
    gj_term = d['par_D_gj'] * float(d['par_gj_surface']) / float(d['geom_gj_len']) * cmax
    f_mem = 8 * eps * mem_term + mem_term * F_RT * 2 * vfl
    f_gj = 8 * eps * gj_term + gj_term * F_RT * 4 * vfl
    j_floor = float(np.sum(zF * (f_mem + f_gj)))
    sig = np.min(np.abs(o['sigma_cell'])) if 'sigma_cell' in o else 1.0
    return {'rho_cells': rho_floor, 'vm_ave': vfl, 'dvm': 2 * vfl / float(d['par_dt']),
            'fluxes_mem': float(np.max(f_mem)), 'fluxes_gj': float(np.max(f_gj)),
            'rate_NaKATP': float(np.max(f_mem)), 'Jn': j_floor,
            'I_mem': j_floor * np.max(d['geom_mem_sa']),
            'J_cell_x': j_floor, 'J_cell_y': j_floor, 'Jc': j_floor,
            'E_cell_x': j_floor / sig, 'E_cell_y': j_floor / sig, 'Emc': j_floor / sig,
            # E_gj = -(vm[nn] - vm[m]) / gj_len: two Vmem floors over 26 nm
            'E_gj_x': 2 * vfl / float(d['geom_gj_len']), 'E_gj_y': 2 * vfl / float(d['geom_gj_len'])}
