"""The drop-in: BETSE's ``Simulator._run_sim_core_loop`` on the GPU.

``run_sim_core_loop`` has the signature and the observable behaviour of
``Simulator._run_sim_core_loop`` (``betse/science/sim.py:1132-1390``) for the
electrodiffusion step: Na/K-ATPase, transmembrane GHK fluxes, gap junctions
(static, or voltage-gated as ``Gap_Junction.run`` gates them when
``p.v_sensitive_gj``, ``betse/science/channels/gap_junction.py:52-75``), the
Ca-ATPase of ``ca_handler`` (``sim.py:2126-2155``), extracellular spaces when ``p.is_ecm``, ``update_all_concs``, ``update_V`` /
``get_current`` and ``check_v``.  The state stays on the GPU between sampled
time steps; at each sampled step the Simulator's attributes are refreshed from
the device under BETSE's names, then -- as the reference loop does --
``phase.callbacks.progressed_next()``, ``sim.write2storage(t, cells, p)`` and
``anim_cells.plot_frame(time_step=-1)`` run.  After the loop the attributes
hold the last step, so ``run_sim_core``'s pickling and the plotting pipeline
see what the reference would leave.

A general network (``p.molecules_enabled``) or a gene regulatory network
(``p.grn_enabled``) steps with the ions in the plain FP64 form
(``betse_gb300.network``; ``sim.py:1290-1319``): its substances are uploaded
from the ``Molecule`` objects, and at each sampled step their concentrations,
fluxes and the reaction rates are written back before ``write2storage`` (whose
``core.write_data`` reads them).

Features of the reference loop outside the step (endoplasmic reticulum
calcium dynamics, pressures, flow, deformation, polarizability in the split
form, networks in the split form or both networks at once, the network
features ``NetworkSpec.from_betse`` names, scheduled events of the SIM phase,
dynamic protein noise) are refused with ``NotImplementedError`` naming them,
before any work.

``install()`` patches the method on BETSE's ``Simulator`` class.
"""
from __future__ import annotations

import time

import numpy as np

from .cluster import ClusterGeometry, StepParams
from .engine import ClusterEngine
from .network import Network, NetworkSpec


def unsupported_features(sim, phase, assume_no_events=False, precision='fp64'):
    """Reasons the GPU loop cannot stand in for the reference loop here
    (empty when it can).  Each names the option of ``phase.p`` that enables a
    branch of ``sim.py:1169-1363`` this step does not compute (with
    ``precision``, the form that would run)."""
    p = phase.p
    reasons = []
    ions = getattr(p, 'ions_dict', {}) or {}
    if ions.get('Ca', 0) == 1 and bool(getattr(p, 'Ca_dyn', False)):
        reasons.append('endoplasmic reticulum calcium dynamics (Ca_dyn, sim.py:2157-2159)')
    nets = [f for f in ('molecules_enabled', 'grn_enabled') if bool(getattr(p, f, False))]
    if len(nets) == 2:
        reasons.append('a general network and a gene regulatory network at once '
                       '(molecules_enabled and grn_enabled)')
    if nets and precision != 'fp64':
        reasons.append('networks in the split form (the plain form, precision="fp64", steps them)')
    if nets and bool(getattr(p, 'is_ecm', False)):
        reasons.append('networks with extracellular spaces (is_ecm)')
    for flag, holder in (('molecules_enabled', 'molecules'), ('grn_enabled', 'grn')):
        h = getattr(sim, holder, None) if flag in nets else None
        for what in ('transporters', 'channels', 'modulators'):
            if h is not None and getattr(h, what, False):
                reasons.append(f'network {what} ({holder})')
    for flag, what in (('deform_osmo', 'osmotic pressure'),
                       ('fluid_flow', 'fluid flow'),
                       ('deformation', 'deformation')):
        if bool(getattr(p, flag, False)):
            reasons.append(f'{what} ({flag})')
    if float(getattr(p, 'cell_polarizability', 0.0)) != 0.0 and precision != 'fp64':
        reasons.append('cell polarizability in the split form (sim.py:2048-2080 makes Vmem per-membrane '
                       'state; the plain form, precision="fp64", computes it)')
    if not bool(getattr(p, 'cluster_open', True)):
        reasons.append('closed cluster boundary (cluster_open False)')
    kind = getattr(getattr(phase, 'kind', None), 'name', str(getattr(phase, 'kind', '')))
    if kind == 'SIM':
        if not assume_no_events:
            reasons.append('scheduled events of the SIM phase (phase.dyna.fire_events); '
                           'pass assume_no_events=True when the configuration schedules none')
        if getattr(p, 'dynamic_noise', 0) == 1 and ions.get('P', 0) == 1:
            reasons.append('dynamic protein noise (dynamic_noise)')
    return reasons


def _network_core(sim, p):
    """The MasterOfNetworks the loop steps (sim.molecules.core or
    sim.grn.core), or None."""
    if bool(getattr(p, 'molecules_enabled', False)):
        return sim.molecules.core
    if bool(getattr(p, 'grn_enabled', False)):
        return sim.grn.core
    return None


def _network_upload(net, core, M):
    mols = list(core.molecules.values())
    net.upload(np.stack([np.asarray(m.c_cells, np.float64) for m in mols]),
               np.stack([np.asarray(m.cc_at_mem, np.float64) for m in mols]),
               np.stack([np.asarray(m.c_env, np.float64) * np.ones(M) for m in mols]))


def _network_mirror(sim, core, net, M):
    """Write the substances back on BETSE's objects (Molecule.c_cells,
    cc_at_mem, c_env as the uniform length-M vector, f_mem, f_gj;
    MasterOfNetworks.reaction_rates) and let BETSE's own energy_charge
    (networks.py:3996-4013) refresh chi from them."""
    st = net.download()
    fl = net.fluxes()
    for k, m in enumerate(core.molecules.values()):
        m.c_cells = st['c_cells'][k].copy()
        m.cc_at_mem = st['cc_at_mem'][k].copy()
        m.c_env = np.full(M, st['c_env'][k])
        m.f_mem = fl['f_mem'][k].copy()
        m.f_gj = fl['f_gj'][k].copy()
    core.reaction_rates = fl['reaction_rates'] if len(core.reactions) else np.asarray([])
    if hasattr(core, 'energy_charge'):
        core.energy_charge(sim)


def _grid_shape(cells):
    shape = getattr(cells, 'grid_shape', None)
    return tuple(int(x) for x in (shape if shape is not None else cells.X.shape))


def _mirror(sim, cells, eng, fields, D_env_weight):
    """Refresh the Simulator's attributes from the device (BETSE names and shapes)."""
    shape = _grid_shape(cells)
    st = eng.download()
    sim.vm = st['vm']
    sim.cc_cells = st['cc_cells']
    sim.cc_at_mem = st['cc_at_mem']
    if eng.ecm:
        sim.cc_env = st['cc_env']
        sim.E_env_x = st['E_env_x'].reshape(shape)
        sim.E_env_y = st['E_env_y'].reshape(shape)
    else:
        # the well-mixed environment is a uniform (I, n_mems) array in BETSE
        sim.cc_env = np.repeat(st['cc_env'][:, None], eng.M, axis=1)
    for k, v in eng.outputs().items():
        setattr(sim, k, v)
    if fields:
        f = eng.env_fields(D_env_weight)
        sim.v_env = f['v_env']
        sim.B_field = f['B_field']
        sim.J_env_x = f['J_env_x'].reshape(shape)
        sim.J_env_y = f['J_env_y'].reshape(shape)
        if not eng.ecm:
            sim.E_env_x = f['E_env_x'].reshape(shape)
            sim.E_env_y = f['E_env_y'].reshape(shape)
    if getattr(sim, 'E_env_x', None) is not None:
        # environment field at the membranes (ion_current.py:112-113, 150-151)
        mv = np.asarray(cells.mem_vects_flat)
        idx = np.asarray(cells.map_mem2ecm)
        sim.Eme = (np.ravel(sim.E_env_x)[idx] * mv[:, 2] + np.ravel(sim.E_env_y)[idx] * mv[:, 3])


def run_sim_core_loop(sim, phase, time_steps, time_steps_sampled, anim_cells=None, *,
                      precision='fp64', assume_no_events=False, fields=True, launch_config=None):
    """GPU stand-in for ``Simulator._run_sim_core_loop(phase, time_steps,
    time_steps_sampled, anim_cells)``.

    precision: 'fp64' (every term in FP64, BETSE's arithmetic) or 'split'
    (FP32 fluxes, FP64 concentrations and Vmem).  fields: compute v_env,
    E_env, J_env and B_field at sampled steps from ``cells.lapENVinv`` (False,
    or no ``lapENVinv`` on ``cells``, leaves those attributes untouched).
    launch_config: (membrane slots per tile, kernel) to pin, or 'auto' to time
    the candidates once before stepping.
    """
    reasons = unsupported_features(sim, phase, assume_no_events, precision)
    if reasons:
        raise NotImplementedError('the GPU step does not cover: ' + '; '.join(reasons))
    p, cells = phase.p, phase.cells
    time_steps = np.asarray(time_steps)
    n = len(time_steps)
    if n == 0:
        return
    core = _network_core(sim, p)
    spec = NetworkSpec.from_betse(core, cells, p, sim) if core is not None else None
    geom = ClusterGeometry.from_cells(cells, sim=sim, p=p)
    params = StepParams.from_betse(p, sim)
    lap = getattr(cells, 'lapENVinv', None) if fields else None
    D_env_weight = getattr(sim, 'D_env_weight', None)
    with ClusterEngine(geom, params, precision) as eng:
        eng.set_membrane_diffusivity(sim.Dm_cells)
        if eng.ecm:
            D_env = np.asarray(sim.D_env, np.float64)
            tj = getattr(sim, 'TJ_modulator', None)
            if tj is not None:
                D_env = D_env * np.asarray(tj, np.float64)
            eng.set_env_diffusivity(D_env)
        Phi_b = getattr(sim, 'Phi_b', None)
        if Phi_b is not None and np.any(np.asarray(Phi_b) != 0):
            eng.set_boundary_potential(Phi_b)
        # with voltage-gated gap junctions sim.gjopen is state (sim.py:732 sets
        # it to the static weights; Gap_Junction.run updates it every step)
        eng.upload(sim.vm, sim.cc_cells, sim.cc_at_mem, sim.cc_env,
                   getattr(sim, 'E_env_x', None) if eng.ecm else None,
                   getattr(sim, 'E_env_y', None) if eng.ecm else None,
                   getattr(sim, 'gjopen', None) if eng.vgj else None)
        if lap is not None:
            eng.set_lap_env_inv(lap)
        if launch_config == 'auto':
            eng.autotune()
        elif launch_config is not None:
            eng.set_launch_config(*launch_config)
        net = None
        if spec is not None:
            net = Network(eng, spec)
            _network_upload(net, core, eng.M)
        sampled = {k for k, t in enumerate(time_steps) if t in time_steps_sampled}
        # the first step runs alone so the solver-time estimate sees one step
        stops = sorted(sampled | {0, n - 1})
        done = 0
        loop_measure = time.time()
        try:
            for k in stops:
                if net is not None:
                    net.step(k + 1 - done, with_ions=True, outputs=True)
                else:
                    eng.step(k + 1 - done, outputs=True)
                done = k + 1
                eng.check_stable()  # check_v: BetseSimUnstableException on NaN
                if net is not None:
                    net.check_stable()   # negative substance concentrations
                if k in sampled or k == n - 1:
                    _mirror(sim, cells, eng, lap is not None, D_env_weight)
                    if net is not None:
                        _network_mirror(sim, core, net, eng.M)
                if k in sampled:
                    t = time_steps[k]
                    phase.callbacks.progressed_next()
                    sim.write2storage(t, cells, p)
                    if anim_cells is not None:
                        anim_cells.plot_frame(time_step=-1)
                if k == 0 and hasattr(sim, '_log_solver_time_estimate'):
                    sim._log_solver_time_estimate(phase=phase, step_first_time=loop_measure)
        finally:
            if net is not None:
                net.close()


def install(simulator_cls=None, **options):
    """Make ``simulator_cls._run_sim_core_loop`` (default: BETSE's
    ``betse.science.sim.Simulator``) run on the GPU with ``options`` (those of
    ``run_sim_core_loop``).  Returns the original method."""
    if simulator_cls is None:
        from betse.science.sim import Simulator as simulator_cls
    original = simulator_cls._run_sim_core_loop

    def _run_sim_core_loop(self, phase, time_steps, time_steps_sampled, anim_cells):
        return run_sim_core_loop(self, phase, time_steps, time_steps_sampled, anim_cells, **options)

    _run_sim_core_loop.__wrapped__ = original
    simulator_cls._run_sim_core_loop = _run_sim_core_loop
    return original
