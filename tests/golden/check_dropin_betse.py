#!/usr/bin/env python3
"""The drop-in inside BETSE's own ``Simulator``, checked against BETSE's loop.

Test infrastructure, like ``make_golden.py`` beside it: it needs a BETSE
checkout and runs on the host, without a GPU. It builds two identical seeded
BETSE simulations (``Cells``, ``Simulator.init_core``/``init_dynamics``, a
molecule network from ``make_golden.NETWORK`` built by BETSE's own
``MasterOfNetworks``), then:

* runs BETSE's ``Simulator._run_sim_core_loop`` on the first, with sampled
  steps, so BETSE's ``write2storage`` (``sim.py:1789-1884``, including the
  network's ``write_data``) records its time series;
* runs ``betse_gb300.simulator.run_sim_core_loop`` on the second, with the
  same sampled steps. That is the drop-in's host code, unchanged:
  - ``ClusterGeometry.from_cells`` and ``StepParams.from_betse`` on BETSE's
    objects;
  - ``NetworkSpec.from_betse`` on BETSE's ``MasterOfNetworks``;
  - the attribute mirroring and the calls to BETSE's own
    ``write2storage`` and ``energy_charge``.

  Only the device engines are replaced, by stand-ins that step the oracle
  (``oracle.step``, ``oracle.network``), because this host has no GPU;
* compares every time series ``write2storage`` recorded (and the network
  tables ``from_betse`` built against ``from_config`` on the same
  configuration).

    python tests/golden/check_dropin_betse.py --ref <path of a BETSE checkout>

It prints the largest difference per series (relative to the series' largest
value) and exits non-zero if one exceeds 1e-10 (1e-9 for currents and
fields).
"""
from __future__ import annotations

import argparse
import copy
import os
import sys
from types import SimpleNamespace

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)

import make_golden as mg  # noqa: E402


# ---------------------------------------------------------------------------
# device stand-ins (oracle-backed), with the engine API the drop-in calls
# ---------------------------------------------------------------------------
class OracleEngine:
    def __init__(self, geom, params, precision='fp64'):
        self.geom, self.params = geom, params
        self.M, self.C = geom.n_mems, geom.n_cells
        self.ecm = bool(params.is_ecm)
        self.vgj = bool(params.v_sensitive_gj)
        self.lap = None
        self.out = {}

    def __enter__(self):
        return self

    def __exit__(self, *a):
        pass

    def set_membrane_diffusivity(self, Dm):
        self.Dm = np.array(Dm, np.float64)

    def upload(self, vm, cc_cells, cc_at_mem, cc_env, E_env_x=None, E_env_y=None, gjopen=None):
        from oracle.adapt import from_workload
        ce = np.asarray(cc_env, np.float64)
        st = dict(vm=vm, cc_cells=cc_cells, cc_at_mem=cc_at_mem, cc_env=ce[:, 0] if ce.ndim == 2 else ce)
        self.g, self.p, self.s = from_workload(self.geom, self.params, self.Dm, st)
        self.p.v_sensitive_gj = self.vgj
        if self.vgj:
            self.p.gj_vthresh, self.p.gj_min = self.params.gj_vthresh, self.params.gj_min
            self.s.gjopen = np.array(gjopen if gjopen is not None else self.g.gj_weight, np.float64)

    def set_lap_env_inv(self, lap):
        self.g.lap_inv = np.asarray(lap, np.float64)

    def step_one(self, outputs):
        from oracle.step import step
        o = step(self.g, self.p, self.s, outputs=outputs)
        if outputs:
            self.out = o

    def step(self, n, outputs=False):
        for k in range(n):
            self.step_one(outputs and k == n - 1)

    def check_stable(self):
        pass

    def download(self):
        return {'vm': self.s.vm.copy(), 'cc_cells': self.s.cc_cells.copy(), 'cc_at_mem': self.s.cc_at_mem.copy(),
                'cc_env': self.s.cc_env[:, 0].copy()}

    def outputs(self):
        from betse_gb300 import _lib
        o = {k: np.array(self.out[k]) for k in _lib.OUTPUT_FIELDS if k in self.out}
        o['E_gj_x'], o['E_gj_y'] = self.out['E_gj_x'], self.out['E_gj_y']
        o['gjopen'] = self.out['gjopen']
        return o

    def env_fields(self, D_env_weight=None):
        return {k: np.ravel(self.out[k]) for k in ('v_env', 'E_env_x', 'E_env_y', 'J_env_x', 'J_env_y', 'B_field')}


class OracleNetworkEngine:
    """Stand-in for ``betse_gb300.network.Network``: the oracle network on the
    same configuration, stepped after each oracle ion step."""
    config = None

    def __init__(self, eng, spec):
        from oracle.network import Network
        cfg, targets, mods = self.config
        self.eng, self.spec = eng, spec
        eng.g.R_rads = np.asarray(eng.geom.R_rads)
        self.net = Network(cfg['substances'], cfg['reactions'], eng.g, eng.p, cfg['mem_vol'], cfg['time_dilation'],
                           targets, mods)

    def upload(self, c_cells, cc_at_mem, c_env):
        from oracle.network import NetworkState
        ce = np.asarray(c_env)
        self.st = NetworkState(c_cells, cc_at_mem, ce[:, 0] if ce.ndim == 2 else ce)

    def step(self, n, with_ions=True, outputs=False):
        from oracle.network import run_with_ions
        e = self.eng
        for k in range(n):
            out = outputs and k == n - 1
            if out:
                # run_with_ions takes no outputs: step the ions with outputs by hand
                from oracle.step import FLOAT_NONCE
                vm = e.s.vm.copy()
                e.step_one(True)
                for _ in range(e.s.cc_at_mem.shape[0]):
                    vm = vm + FLOAT_NONCE
                vgj = (vm[e.g.nn_i] - vm) + FLOAT_NONCE
                gjo = e.s.gjopen if e.vgj else e.p.gj_block * e.g.gj_weight
                self.rates_before = self._rates()
                self.net.step(self.st, vm, vgj, gjo, e.p.gj_block)
            else:
                run_with_ions(self.net, self.st, e.g, e.p, e.s, 1)

    def _rates(self):
        C = len(self.eng.g.cell_vol)
        cc = {s.name: self.st.c_cells[k] for k, s in enumerate(self.net.subs)}
        env = {s.name: self.st.c_env[k] for k, s in enumerate(self.net.subs)}
        return np.asarray([r.rate(cc, env, C) for r in self.net.reactions])

    def check_stable(self):
        assert self.st.unstable == 0

    def download(self):
        return {'c_cells': self.st.c_cells.copy(), 'cc_at_mem': self.st.cc_at_mem.copy(), 'c_env': self.st.c_env.copy()}

    def fluxes(self):
        return {'f_mem': self.st.f_mem.copy(), 'f_gj': self.st.f_gj.copy(), 'reaction_rates': self.rates_before}

    def close(self):
        pass


# ---------------------------------------------------------------------------
def build(radius, seed, dt, n_steps, network):
    from betse.science.sim import Simulator
    from betse.science.enum.enumphase import SimPhaseKind
    p = mg.make_params(radius, 20, False, dt, n_steps)
    p.GHK_calc = False
    c = mg.build_cells(p, radius, seed)
    dm, w = mg.draw_cluster_parameters(c, seed)
    c.gj_default_weights = w.copy()
    fake = mg._Fake(dm)
    phase = SimpleNamespace(p=p, cells=c, kind=SimPhaseKind.INIT, dyna=fake, callbacks=fake)
    s = Simulator()
    phase.sim = s
    s.init_core(phase)
    s.init_dynamics(phase)
    s.clear_storage(c, p)
    s.update_V(c, p)
    out = {}
    core = mg.attach_network(phase, network, out)
    for mol in core.molecules.values():
        mol.c_mems_time, mol.c_cells_time, mol.c_env_time = [], [], []
    for r in core.reactions.values():
        r.rate_time = []
    core.chi_time = []
    core.report = lambda sim, p: None
    return phase, out


SERIES = ['vm_time', 'cc_time', 'cc_env_time', 'I_cell_x_time', 'I_cell_y_time', 'I_mem_time', 'rho_cells_time',
          'rate_NaKATP_time', 'efield_gj_x_time', 'efield_gj_y_time', 'gjopen_time', 'venv_time', 'I_tot_x_time',
          'I_tot_y_time', 'vm_ave_time', 'dd_time', 'time']


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    den = np.max(np.abs(b)) if b.size else 0.0
    num = np.max(np.abs(a - b)) if b.size else 0.0
    return 0.0 if num == 0.0 else num / (den if den > 0 else 1.0)


def series_rel(va, vb, scale=0.0):
    """max over samples of |a - b|, relative to the largest |b| over all
    samples (or to ``scale`` when larger): a uniform start makes the first
    step's fields pure 1e-25 V nonce, which BETSE's network also adds to vm in
    place, and without extracellular spaces J_env is the divergence-free part
    of a gradient field, zero up to rounding."""
    den = max([np.max(np.abs(np.asarray(y, np.float64))) for y in va if np.size(y)] + [scale])
    num = max((np.max(np.abs(np.asarray(x, np.float64) - np.asarray(y, np.float64)))
               for x, y in zip(vb, va) if np.size(y)), default=0.0)
    return 0.0 if num == 0.0 else num / (den if den > 0 else 1.0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', default=os.environ.get('BETSE_REF'),
                    help='path of a BETSE source checkout (or set BETSE_REF)')
    ap.add_argument('--steps', type=int, default=60)
    a = ap.parse_args()
    if not a.ref:
        ap.error('give --ref <path of a BETSE checkout> or set BETSE_REF')
    mg.install_reference(a.ref)
    from betse_gb300 import simulator
    from betse_gb300.network import NetworkSpec
    radius, seed, dt, n = 50e-6, 21, 1e-2, a.steps
    time_steps = np.arange(n) * dt
    sampled = set(time_steps[[0, 9, 30, n - 1]])
    ph_a, _ = build(radius, seed, dt, n, mg.NETWORK)
    ph_b, out_b = build(radius, seed, dt, n, mg.NETWORK)
    # BETSE's loop
    ph_a.sim._run_sim_core_loop(ph_a, time_steps, sampled, None)
    # the drop-in's host code with oracle-backed engines
    core_b = ph_b.sim.molecules.core
    names = list(core_b.molecules)
    targets = {nm: np.asarray(m.growth_targets_cell) for nm, m in core_b.molecules.items()
               if len(m.growth_targets_cell) != len(ph_b.cells.cell_i)}
    mods = {nm: np.asarray(m.growth_mod_function_cells) * np.ones(len(ph_b.cells.cell_i))
            for nm, m in core_b.molecules.items() if m.simple_growth}
    cfg = dict(copy.deepcopy(mg.NETWORK), mem_vol=np.asarray(ph_b.cells.mem_vol))
    OracleNetworkEngine.config = (cfg, targets, mods)
    spec_betse = NetworkSpec.from_betse(core_b, ph_b.cells, ph_b.p)
    spec_cfg = NetworkSpec.from_config(mg.NETWORK['substances'], mg.NETWORK['reactions'],
                                       mg.NETWORK['time_dilation'], n_cells=len(ph_b.cells.cell_i),
                                       profiles={'spot': out_b['net_spot_cells']},
                                       growth_mod={'A': mods['A']}, ion_names=mg.ION_ORDER,
                                       mem_vol=ph_b.cells.mem_vol, R_rads=ph_b.cells.R_rads)
    bad = []
    same_tables = (spec_betse.terms == spec_cfg.terms and len(spec_betse.subs) == len(spec_cfg.subs) and all(
        all((x[k] is None and y[k] is None) or np.array_equal(x[k], y[k]) for k in x)
        for x, y in zip(spec_betse.subs, spec_cfg.subs)) and all(
        x == y for x, y in zip(spec_betse.reactions, spec_cfg.reactions)))
    print(f'NetworkSpec.from_betse == from_config: {same_tables}')
    if not same_tables:
        bad.append('network tables')
    saved = simulator.ClusterEngine, simulator.Network
    simulator.ClusterEngine, simulator.Network = OracleEngine, OracleNetworkEngine
    try:
        simulator.run_sim_core_loop(ph_b.sim, ph_b, time_steps, sampled, None, precision='fp64')
    finally:
        simulator.ClusterEngine, simulator.Network = saved
    sa, sb = ph_a.sim, ph_b.sim
    # the scale of the environment current: sigma |E_env| ~ sigma |v_env| / delta
    j_scale = float(sa.sigma) * max(np.max(np.abs(v)) for v in sa.venv_time) / float(ph_a.cells.delta)
    for k in SERIES:
        va, vb = getattr(sa, k), getattr(sb, k)
        if len(va) != len(vb):
            bad.append(k)
            print(f'{k}: {len(va)} vs {len(vb)} samples')
            continue
        r = series_rel(va, vb, j_scale if k in ('I_tot_x_time', 'I_tot_y_time') else 0.0)
        tol = 1e-9 if k in ('I_tot_x_time', 'I_tot_y_time', 'venv_time', 'I_cell_x_time', 'I_cell_y_time',
                            'I_mem_time') else 1e-10
        print(f'{k:18s} {len(va)} samples, max rel diff {r:.2e}')
        if r > tol:
            bad.append(k)
    ca, cb = sa.molecules.core, sb.molecules.core
    for nm in names:
        for k in ('c_cells_time', 'c_mems_time', 'c_env_time'):
            va, vb = getattr(ca.molecules[nm], k), getattr(cb.molecules[nm], k)
            r = max((rel(x, y) for x, y in zip(vb, va)), default=0.0)
            print(f'{nm}.{k:14s} {len(va)} samples, max rel diff {r:.2e}')
            if len(va) != len(vb) or r > 1e-10:
                bad.append(f'{nm}.{k}')
    for rn in ca.reactions:
        va, vb = ca.reactions[rn].rate_time, cb.reactions[rn].rate_time
        r = max((rel(x, y) for x, y in zip(vb, va)), default=0.0)
        print(f'reaction {rn}.rate_time {len(va)} samples, max rel diff {r:.2e}')
        if len(va) != len(vb) or r > 1e-10:
            bad.append(f'{rn}.rate_time')
    print('FAILED: ' + ', '.join(bad) if bad else 'all series match')
    return 1 if bad else 0


if __name__ == '__main__':
    sys.exit(main())
