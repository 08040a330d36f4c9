"""One explicit-Euler electrodiffusion step of BETSE's full solver, restated.

The operator order is that of ``Simulator._run_sim_core_loop``
(``betse/science/sim.py:1169-1363``). Dense products with ``cells.M_sum_mems``
become CSR segment sums over the contiguous membranes of each cell
(``np.add.reduceat`` on ``cell_mem_ptr``); products with
``cells.M_divmap_mem2ecm`` become a scatter-add with ``np.bincount``.

Inputs are duck-typed: ``g`` carries the cluster geometry and index maps, ``p``
the scalar parameters and per-ion constants, ``s`` the evolving state. The
field names follow BETSE's ``Cells``/``Simulator`` attributes.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import fields as fd

FLOAT_NONCE = 1.0e-25   # sim_toolbox.py:52


# ---------------------------------------------------------------------------
# membrane kernels
# ---------------------------------------------------------------------------
def electroflux(cA, cB, Dc, d, zc, vBA, T, F, R):
    """GHK flux from A (outside) into B (inside) (sim_toolbox.py:18-69).

    ``vBA`` is NOT mutated here; the reference adds ``FLOAT_NONCE`` to the
    caller's array in place (``:54``) and ``step`` reproduces that on ``vm``.
    """
    vBA = vBA + FLOAT_NONCE
    zc = zc + FLOAT_NONCE
    alpha = (zc * vBA * F) / (R * T)
    exp_alpha = np.exp(-alpha)
    deno = -np.expm1(-alpha)
    return -((Dc * alpha) / d) * ((cB - cA * exp_alpha) / deno)


def pump_nakatp(cNai, cNao, cKi, cKo, Vm, T, p, block=1.0):
    """Na/K-ATPase rate (sim_toolbox.py:71-122); returns (f_Na, f_K, rate)."""
    Qnumo = (p.cADP * 1e-3) * (p.cPi * 1e-3) * ((cNao * 1e-3) ** 3) * ((cKi * 1e-3) ** 2)
    Qdenomo = (p.cATP * 1e-3) * ((cNai * 1e-3) ** 3) * ((cKo * 1e-3) ** 2)
    Qdenomo = np.where(Qdenomo == 0.0, 1.0e-15, Qdenomo)
    Q = Qnumo / Qdenomo
    Keq = np.exp(-(p.deltaGATP / (p.R * T) - ((p.F * Vm) / (p.R * T))))
    numo_E = ((cNai / p.KmNK_Na) ** 3) * ((cKo / p.KmNK_K) ** 2) * (p.cATP / p.KmNK_ATP)
    denomo_E = (1 + (cNai / p.KmNK_Na) ** 3) * (1 + (cKo / p.KmNK_K) ** 2) * (1 + (p.cATP / p.KmNK_ATP))
    fwd_co = numo_E / denomo_E
    f_Na = -3 * block * p.alpha_NaK * fwd_co * (1 - (Q / Keq))
    f_K = -(2 / 3) * f_Na
    return f_Na, f_K, -f_Na


def pump_caatp(cCai, cCao, Vm, T, p):
    """Ca-ATPase flux, into the cell positive (sim_toolbox.py:124-180).

    The reference clamps both concentration arrays in place first
    (``no_negs``) and computes, but never uses, a backward coefficient; its
    ``block`` and ``met`` arguments are unused as well."""
    cCai = np.maximum(cCai, 0.0)
    cCao = np.maximum(cCao, 0.0)
    Qnumo = p.cADP * p.cPi * cCao
    Qdenomo = p.cATP * cCai
    Qdenomo = np.where(Qdenomo == 0.0, 1.0e-16, Qdenomo)
    Q = Qnumo / Qdenomo
    Keq = np.exp(-(p.deltaGATP / (p.R * T) - 2 * ((p.F * Vm) / (p.R * T))))
    numo_E = (cCai / p.KmCa_Ca) * (p.cATP / p.KmCa_ATP)
    denomo_E = (1 + (cCai / p.KmCa_Ca)) * (1 + (p.cATP / p.KmCa_ATP))
    frwd = numo_E / denomo_E
    return -p.alpha_Ca * frwd * (1 - (Q / Keq))


def ca_pump_on(p):
    """ca_handler runs its pump when Ca is an ion and alpha_Ca > 0
    (sim.py:1282-1283, 2129)."""
    return getattr(p, 'iCa', -1) >= 0 and float(getattr(p, 'alpha_Ca', 0.0)) > 0.0


def seg_sum(g, x):
    """``cells.M_sum_mems @ x`` (cells.py:1297-1306): sum over each cell's
    contiguous membrane range."""
    ptr = np.asarray(g.cell_mem_ptr)
    out = np.zeros(len(ptr) - 1)
    nz = ptr[1:] > ptr[:-1]
    out[nz] = np.add.reduceat(x, ptr[:-1][nz])
    return out


def env_scatter(g, x):
    """``cells.M_divmap_mem2ecm @ x`` with ``M_divmap[k, m] = mem_sa[m]`` for
    ``k = map_mem2ecm[m]`` (cells.py:1838-1843)."""
    G = int(np.prod(g.grid_shape))
    return np.bincount(g.map_mem2ecm, weights=g.mem_sa * x, minlength=G)


# ---------------------------------------------------------------------------
# state
# ---------------------------------------------------------------------------
@dataclass
class OracleState:
    vm: np.ndarray
    cc_cells: np.ndarray          # (I, C)
    cc_at_mem: np.ndarray         # (I, M)
    cc_env: np.ndarray            # (I, M) without ECM, (I, G) with ECM
    Phi_b: np.ndarray | None = None
    E_env_x: np.ndarray | None = None   # (ny, nx), ECM only
    E_env_y: np.ndarray | None = None
    extra: dict = field(default_factory=dict)
    gjopen: np.ndarray | None = None     # (M,), voltage-gated gap junctions only

    def copy(self):
        c = lambda a: None if a is None else np.array(a, copy=True)  # noqa: E731
        return OracleState(c(self.vm), c(self.cc_cells), c(self.cc_at_mem),
                           c(self.cc_env), c(self.Phi_b), c(self.E_env_x),
                           c(self.E_env_y), dict(self.extra), c(self.gjopen))


# Harris et al. (1983) gating constants of channels/gap_junction.py:26-31
GJ_LAMBDA, GJ_A1, GJ_A2 = 0.0013, 0.077, 0.14


def gap_junction_run(gjopen, vgj, p):
    """One ``Gap_Junction.run`` (channels/gap_junction.py:52-81): implicit
    Euler step of the open fraction in ms units, then the block factor."""
    V1 = 1.0e3 * np.abs(vgj)
    alpha = GJ_LAMBDA * np.exp(-GJ_A1 * (V1 - p.gj_vthresh))
    beta = GJ_LAMBDA * np.exp(GJ_A2 * (V1 - p.gj_vthresh))
    beta = beta / (1 + 50 * beta)
    dt = p.dt * 1e3
    g = (gjopen + dt * (alpha + beta * p.gj_min)) / (1 + alpha * dt + beta * dt)
    return p.gj_block * g


def init_vm(g, p, s):
    """Initial ``update_V`` (sim.py:1041 -> 2007-2029) for a fresh state.  With
    cell polarizability the implicit form runs from vm = 0 (sim.py:550) with no
    fluxes yet, so Jn = 0 (sim.py:2048-2058)."""
    rho = np.dot(p.zs * p.F, s.cc_cells)
    if float(getattr(p, 'cell_polarizability', 0.0)) != 0.0:
        sigma_cell = np.asarray([((z ** 2) * (p.F ** 2) * cc * D * 0.1) / (p.R * p.T)
                                 for z, cc, D in zip(p.zs, s.cc_cells, p.D_free)]).mean(axis=0)
        vm_o = (1 / p.cm) * (rho * g.diviterm)[g.mem_to_cells]
        sig = sigma_cell[g.mem_to_cells]
        return ((0.0 - (p.dt / p.cm) * 0.0 + ((p.dt * sig * vm_o) / (p.cm * g.R_rads)))
                / (1 + ((p.dt * sig) / (p.cm * g.R_rads))))
    Phi_b = s.Phi_b if s.Phi_b is not None else np.zeros(int(np.prod(g.grid_shape)))
    return (1 / p.cm) * (rho * g.diviterm)[g.mem_to_cells] - Phi_b[g.map_mem2ecm]


def init_fields(g, p, s):
    """Environment field that the initial ``update_V`` leaves behind (ECM):
    ``E_env`` feeds the first step's stencil."""
    if bool(p.is_ecm):
        s.E_env_x, s.E_env_y, _, _ = _env_E_field(g, p, s)
    return s


def _env_E_field(g, p, s):
    """ECM branch of ``get_current`` that feeds the state: E_env from the
    environment charge (ion_current.py:79-110)."""
    shape = tuple(g.grid_shape)
    rho_env = np.dot(p.zs * p.F, s.cc_env)
    G = rho_env.shape[0]
    msa = g.memSa_per_envSquare[g.map_mem2ecm].mean()
    rho_env_surf = np.zeros(G)
    rho_env_surf[g.map_mem2ecm] = rho_env[g.map_mem2ecm] * (p.cell_height * g.delta ** 2) / msa
    v_env = rho_env_surf / (g.ko_env * p.eo * p.er)
    screen = (2 / (g.ko_env * g.delta)) * (p.cell_radius / p.true_cell_size)
    v_env = fd.gaussian_filter(v_env.reshape(shape), 1.0, mode='constant').ravel() + s.Phi_b
    gVex, gVey = fd.gradient(screen * v_env.reshape(shape), g.delta)
    return -gVex, -gVey, v_env, rho_env


def step(g, p, s, outputs=False):
    """Advance ``s`` by one time step in place; return step outputs if asked.

    Order (sim.py:1169-1363): pump -> per ion {GHK flux, GJ flux, ECM stencil}
    -> update_all_concs -> update_V -> check_v.
    """
    I, M = s.cc_at_mem.shape
    m2c, nn = g.mem_to_cells, g.nn_i
    is_ecm = bool(p.is_ecm)
    T, F, R = p.T, p.F, p.R
    shape = tuple(g.grid_shape)
    fluxes_mem = np.zeros((I, M))
    fluxes_gj = np.zeros((I, M))
    vm = s.vm.copy()
    env_at_mem = (lambda i: s.cc_env[i][g.map_mem2ecm]) if is_ecm else (lambda i: s.cc_env[i])
    out = {}

    # ---- Na/K-ATPase (sim.py:1196-1234); cluster_open is True in BETSE
    iNa, iK = p.iNa, p.iK
    if p.alpha_NaK > 0.0:
        fNa, fK, rate = pump_nakatp(s.cc_at_mem[iNa], env_at_mem(iNa),
                                    s.cc_at_mem[iK], env_at_mem(iK), vm, T, p,
                                    p.nakatp_block)
        fluxes_mem[iNa] += fNa
        fluxes_mem[iK] += fK
    else:
        rate = np.zeros(M)

    fenv_x = np.zeros((I, int(np.prod(shape)))) if is_ecm else None
    fenv_y = np.zeros_like(fenv_x) if is_ecm else None
    for i in range(I):
        # GHK transmembrane flux (sim.py:1256-1269); vm += nonce in place
        f_ED = electroflux(env_at_mem(i), s.cc_at_mem[i], p.Dm[i], p.tm,
                           p.zs[i], vm, T, F, R)
        vm = vm + FLOAT_NONCE
        fluxes_mem[i] += f_ED
        # gap junctions (sim.py:2162-2206)
        vgj = vm[nn] - vm
        if getattr(p, 'v_sensitive_gj', False):
            # update_gj runs the gating object once per ion (sim.py:2181-2183)
            s.gjopen = gap_junction_run(s.gjopen, vgj, p)
            gjopen = s.gjopen
        else:
            gjopen = p.gj_block * g.gj_weight
        conc_mem = s.cc_at_mem[i]
        fgj = electroflux(conc_mem, conc_mem[nn],
                          p.D_gj[i] * p.gj_surface * gjopen, g.gj_len,
                          p.zs[i], vgj, T, F, R)
        fgj[g.bflag] = 0.0
        fluxes_gj[i] = fluxes_gj[i] + fgj
        # extracellular stencil (sim.py:2209-2254)
        if is_ecm:
            cenv = s.cc_env[i].reshape(shape)
            cenv[:, 0] = p.c_env_bound[i]
            cenv[:, -1] = p.c_env_bound[i]
            cenv[0, :] = p.c_env_bound[i]
            cenv[-1, :] = p.c_env_bound[i]
            gcx, gcy = fd.gradient(cenv, g.delta)
            denv = g.D_env[i].reshape(shape)
            alpha = (denv * p.zs[i] * p.q) / (p.kb * T)
            gvx, gvy = -s.E_env_x, -s.E_env_y
            fx = -denv * gcx - alpha * gvx * cenv
            fy = -denv * gcy - alpha * gvy * cenv
            fenv_x[i] = fx.ravel()
            fenv_y[i] = fy.ravel()
            div_fa = fd.divergence(-fx, -fy, g.delta, g.delta)
            cenv = cenv + div_fa * p.dt
            if p.sharpness < 1.0:
                cenv = fd.integrator(cenv, sharp=p.sharpness)
            s.cc_env[i] = cenv.ravel()
        # update_intra (sim.py:2310): cc_at_mem[i] = cc_cells[i][m2c]
        s.cc_at_mem[i] = s.cc_cells[i][m2c]
        if outputs and i == I - 1:
            out['E_gj_x'] = (-vgj / g.gj_len) * g.mem_nx
            out['E_gj_y'] = (-vgj / g.gj_len) * g.mem_ny
            out['gjopen'] = gjopen * np.ones(M)

    # ---- ca_handler (sim.py:2126-2155): after every ion's update_intra, so the
    # cell side is cc_cells at the start of the step and, with extracellular
    # spaces, the environment side is after this step's Nernst-Planck update;
    # vm carries the I in-place nonces (irrelevant at FP64 resolution)
    if ca_pump_on(p):
        iCa = p.iCa
        f_Ca = pump_caatp(s.cc_at_mem[iCa], env_at_mem(iCa), vm, T, p)
        fluxes_mem[iCa] += f_Ca
        out['rate_CaATP'] = f_Ca

    # ---- update_all_concs (sim.py:2086-2111, sim_toolbox.py:1155-1232)
    for i in range(I):
        flux = fluxes_mem[i]
        delta_cells = seg_sum(g, flux * g.mem_sa) / g.cell_vol
        cX_cell = s.cc_cells[i] + delta_cells * p.dt
        s.cc_at_mem[i] = cX_cell[m2c]
        if is_ecm:
            delta_env = env_scatter(g, -flux) / (p.cell_height * g.delta ** 2)
            s.cc_env[i] = s.cc_env[i] + delta_env * p.dt
        else:
            delta_env = -flux * (g.mem_sa / p.vol_env)
            s.cc_env[i] = (s.cc_env[i] + delta_env * p.dt).mean()
        delta_cgj = seg_sum(g, -fluxes_gj[i] * g.mem_sa) / g.cell_vol
        cX_cell = cX_cell + p.dt * delta_cgj
        if np.isnan(cX_cell).any():
            raise FloatingPointError('NaN concentration (no_negs)')
        cX_cell[cX_cell < 0.0] = 0.0
        s.cc_cells[i] = cX_cell

    # ---- update_V / get_current (sim.py:2007-2083, ion_current.py:13-171)
    vmo = vm
    rho_cells = np.dot(p.zs * F, s.cc_cells)
    if is_ecm:
        s.E_env_x, s.E_env_y, v_env, rho_env = _env_E_field(g, p, s)
    polar = float(getattr(p, 'cell_polarizability', 0.0)) != 0.0
    if polar or outputs:
        # get_current (ion_current.py:19-37): smoothed normal current density
        zF = p.zs * F
        Jn = -np.dot(zF, fluxes_mem) + np.dot(zF, fluxes_gj)
        Jn_ave = seg_sum(g, Jn * g.mem_sa) / g.cell_sa
        Jn = g.smooth_weight_mem * Jn + Jn_ave[m2c] * g.smooth_weight_o
        sigma_cell = np.asarray([((z ** 2) * (F ** 2) * cc * D * 0.1) / (R * T)
                                 for z, cc, D in zip(p.zs, s.cc_cells, p.D_free)]).mean(axis=0)
    if polar:
        # implicit polarizable form (sim.py:2048-2058): vm relaxes towards the
        # cell's charge potential through the cytoplasm, driven by Jn; vm here
        # carries the in-place nonces, as self.vm does in the reference
        vm_o = (1 / p.cm) * (rho_cells * g.diviterm)[m2c]
        sig = sigma_cell[m2c]
        vm_new = ((vm - (p.dt / p.cm) * Jn + ((p.dt * sig * vm_o) / (p.cm * g.R_rads)))
                  / (1 + ((p.dt * sig) / (p.cm * g.R_rads))))
    else:
        vm_new = (1 / p.cm) * (rho_cells * g.diviterm)[m2c] - s.Phi_b[g.map_mem2ecm]
    if np.isnan(vm_new).any():
        raise FloatingPointError('NaN Vmem (check_v)')
    s.vm = vm_new

    if outputs:
        J_cell_x = seg_sum(g, Jn * g.mem_nx * g.mem_sa) / g.cell_sa
        J_cell_y = seg_sum(g, Jn * g.mem_ny * g.mem_sa) / g.cell_sa
        vm_ave = seg_sum(g, s.vm) / g.num_mems
        if polar:
            # cell field from the membrane voltage profile (sim.py:2063-2074)
            Rcells = g.R_rads * (p.true_cell_size / p.cell_radius)
            gE = (s.vm - vm_ave[m2c]) / Rcells
            E_cell_x = seg_sum(g, -gE * g.mem_nx * g.mem_sa) / g.cell_sa
            E_cell_y = seg_sum(g, -gE * g.mem_ny * g.mem_sa) / g.cell_sa
        else:
            E_cell_x = J_cell_x / sigma_cell
            E_cell_y = J_cell_y / sigma_cell
        out.update(
            fluxes_mem=fluxes_mem, fluxes_gj=fluxes_gj, rate_NaKATP=rate,
            rho_cells=rho_cells, Jn=Jn, I_mem=-Jn * g.mem_sa,
            J_cell_x=J_cell_x, J_cell_y=J_cell_y,
            Jc=J_cell_x[m2c] * g.mem_nx + J_cell_y[m2c] * g.mem_ny,
            vm_ave=vm_ave,
            dvm=(s.vm - vmo) / p.dt, sigma_cell=sigma_cell,
            E_cell_x=E_cell_x, E_cell_y=E_cell_y,
            Emc=E_cell_x[m2c] * g.mem_nx + E_cell_y[m2c] * g.mem_ny,
            Phi_b=s.Phi_b.copy())
        if is_ecm:
            out.update(v_env=v_env, E_env_x=s.E_env_x, E_env_y=s.E_env_y,
                       rho_env=rho_env, fluxes_env_x=fenv_x, fluxes_env_y=fenv_y)
            if getattr(g, 'lap_inv', None) is not None:
                Jx = np.dot(F * p.zs, fenv_x).reshape(shape)
                Jy = np.dot(F * p.zs, fenv_y).reshape(shape)
                BB, Jex, Jey, _, Ja, Jb = fd.hh_decomp(Jx, Jy, g.lap_inv, shape, g.delta)
                out.update(J_env_x=Jex, J_env_y=Jey, B_field=BB * p.mu)
        elif getattr(g, 'lap_inv', None) is not None:
            # get_current runs before vm is replaced (sim.py:2013)
            out.update(_noecm_fields(g, p, vmo))
    return out


def _noecm_fields(g, p, vm):
    """Output-only environment fields without ECM (ion_current.py:116-171)."""
    shape = tuple(g.grid_shape)
    G = int(np.prod(shape))
    vce = np.zeros(G)
    # the reference indexes the membrane vector vm/2 with cell indices here
    vce[g.map_mem2ecm] = (vm / 2)[g.mem_to_cells]
    Phi = fd.gaussian_filter(-vce.reshape(shape), 1.0)
    gVex, gVey = fd.gradient(g.delta * Phi, g.delta)
    _, Frx, Fry, _, Fdx, Fdy = fd.hh_decomp(gVex, gVey, g.lap_inv, shape, g.delta)
    gVex, gVey = Frx + Fdx, Fry + Fdy
    E_env_x, E_env_y = -gVex, -gVey
    Dw = np.asarray(g.D_env_weight).reshape(shape)
    Jxo = g.sigma * E_env_x * Dw
    Jyo = g.sigma * E_env_y * Dw
    BB, Jex, Jey, _, Ja, Jb = fd.hh_decomp(Jxo, Jyo, g.lap_inv, shape, g.delta)
    return dict(E_env_x=E_env_x, E_env_y=E_env_y, J_env_x=Jex, J_env_y=Jey,
                B_field=BB * p.mu, v_env=Phi.ravel())


def run(g, p, s, n_steps, outputs_last=False):
    """Run ``n_steps`` steps; return the outputs of the last one if asked."""
    out = {}
    for k in range(n_steps):
        out = step(g, p, s, outputs=outputs_last and k == n_steps - 1)
    return out
