"""CPU restatement of BETSE's molecule-network step -- TEST INFRASTRUCTURE ONLY.

``MasterOfNetworks.run_loop`` (``betse/science/chemistry/networks.py:2805-2983``)
advances the user-defined substances of a general network (``p.molecules_enabled``,
``sim.py:1290-1303``) or a gene regulatory network (``p.grn_enabled``,
``sim.py:1305-1319``; ``gene.py:220-308`` runs it alone, without the ions).
BETSE writes every rate as a Python string at initialisation and ``eval``s it
each step; this module states the same arithmetic as functions:

* influencer factors (``get_influencers``, ``networks.py:5084-5600``):
  multiplicative Hill activators ``(c/K)^n / (1 + (c/K)^n)``, ``!``
  independent activators added to their product, ``&`` direct terms
  (``+c`` for activators, ``-c`` for inhibitors) summed and multiplied in, and
  inhibitors ``1 / (1 + (c/K)^n)``, each reading the cell (``'cell'`` zone) or
  the well-mixed environment (``'env'`` zone);
* growth and decay (``write_growth_and_decay``, ``networks.py:1187-1310``):
  ``mod * r_prod * alpha - r_decay * c/s - decay_max * alpha_decay * c/s``,
  zero outside the growth targets (``run_loop``, ``:2840-2845``);
* cell-zone reactions (``write_reactions``, ``networks.py:1312-1572``):
  ``vmax * alpha * prod (c_r/K_r)^n_r / (1 + (c_r/K_r)^n_r)``, or with a
  standard free energy ``vmax * alpha * (1 - Q / Keq)``, where BETSE's ``Q``
  is ``prod 1e-3 c_p^n_p / prod 1e-3 c_r^n_r`` (its string applies the power
  before the 1e-3 factor);
* the reaction matrix (``create_reaction_matrix``, ``:2686-2725``) applied
  as ``c += (RM @ rates) * dt``;
* ``Molecule.update_intra`` (``networks.py:5714-5807``) and
  ``stb.molecule_mover`` without extracellular spaces
  (``sim_toolbox.py:909-1153``): GHK flux across the membrane, ``update_Co``
  (``:1155-1207``) with the auto-mixed environment, GHK flux through the gap
  junctions, and the negative-concentration checks.

It is the checker, never the product: only ``tests/`` may import it. Parity is
pinned to BETSE's own ``MasterOfNetworks`` run on a seeded cluster
(``tests/golden/net_r50_s21.npz``, made by ``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import numpy as np

from .step import FLOAT_NONCE, electroflux, seg_sum


def _absent(x):
    if x is None or (isinstance(x, str) and x == 'None'):
        return True
    return hasattr(x, '__len__') and not isinstance(x, str) and len(x) == 0


def _zones(zones, names):
    """``default_zones`` (``networks.py:4738-4750``)."""
    if names is None or _absent(names):
        return zones
    if zones is None or _absent(zones):
        return ['cell'] * len(names)
    return list(zones)


class Influence:
    """One factor of ``get_influencers`` for reaction zone ``'cell'``."""

    def __init__(self, a_names, a_km, a_n, a_zone, i_names, i_km, i_n, i_zone):
        self.mult, self.indep, self.direct, self.inhib = [], [], [], []
        a_zone, i_zone = _zones(a_zone, a_names), _zones(i_zone, i_names)
        self.has_a = not _absent(a_names)
        self.has_i = not _absent(i_names)
        if self.has_a:
            for name, km, n, zone in zip(a_names, a_km, a_n, a_zone):
                name = name[:-1] if name.endswith('*') else name  # Vmem-sensitive: membrane zone only
                if name.endswith('!'):
                    self.indep.append((name[:-1], float(km), float(n), zone))
                elif name.endswith('&'):
                    self.direct.append((name[:-1], +1.0, zone))
                else:
                    self.mult.append((name, float(km), float(n), zone))
        if self.has_i:
            seen_direct = False
            for name, km, n, zone in zip(i_names, i_km, i_n, i_zone):
                name = name[:-1] if name.endswith('*') else name
                if name.endswith('!'):
                    name = name[:-1]
                if name.endswith('&'):
                    self.direct.append((name[:-1], -1.0, zone))
                    seen_direct = True
                else:
                    if seen_direct:
                        raise ValueError('a direct (&) inhibitor followed by another inhibitor: '
                                         'BETSE composes no valid expression for it')
                    self.inhib.append((name, float(km), float(n), zone))
        self.act_empty = self.has_a and not self.mult and not self.indep
        self.inh_empty = self.has_i and not self.inhib
        if self.act_empty and self.inh_empty:
            raise ValueError('only direct (&) influencers: BETSE composes no valid expression for it')

    @staticmethod
    def _conc(name, zone, cc, env):
        return cc[name] if zone == 'cell' else env[name]

    def __call__(self, cc, env, n_cells):
        one = np.ones(n_cells)
        if not self.has_a:
            act = one
        elif self.mult:
            act = one
            for k, (name, km, n, zone) in enumerate(self.mult):
                x = (self._conc(name, zone, cc, env) / km) ** n
                t = x / (1 + x)
                act = t if k == 0 else act * t
            for name, km, n, zone in self.indep:
                x = (self._conc(name, zone, cc, env) / km) ** n
                act = act + x / (1 + x)
        elif self.indep:
            act = 1.0
            for name, km, n, zone in self.indep:
                x = (self._conc(name, zone, cc, env) / km) ** n
                act = act + x / (1 + x)
        else:
            act = None
        if not self.has_i:
            inh = one
        elif self.inhib:
            inh = None
            for name, km, n, zone in self.inhib:
                t = 1 / (1 + (self._conc(name, zone, cc, env) / km) ** n)
                inh = t if inh is None else inh * t
        else:
            inh = None
        alpha = act if inh is None else (inh if act is None else act * inh)
        if self.direct:
            dsum = None
            for name, sign, zone in self.direct:
                c = self._conc(name, zone, cc, env)
                dsum = sign * c if dsum is None else dsum + sign * c
            alpha = alpha * dsum
        return alpha * one


class Substance:
    def __init__(self, d, time_dila, n_cells, targets=None, growth_mod=None):
        self.name = str(d['name'])
        self.z = float(d['z'])
        self.Dm = float(d['Dm'])
        self.Do = float(d['Do'])
        self.Dgj = float(d.get('Dgj', 1.0e-16))
        self.c_env0 = float(d['env conc'])
        self.c_cell0 = float(d['cell conc'])
        self.update_intra = bool(d.get('update intracellular', True))
        self.ignore_gj = bool(d['GJ impermeable'])
        self.Mu_mem = float(d.get('Mu_mem', 0.0))
        self.tdf = float(time_dila) if d.get('use time dilation', False) else 1.0
        gad = d.get('growth and decay', None)
        self.growth = isinstance(gad, dict)
        self.mod = np.ones(n_cells) if growth_mod is None else np.asarray(growth_mod, np.float64)
        self.targets = np.ones(n_cells, bool)
        if targets is not None:
            self.targets = np.zeros(n_cells, bool)
            self.targets[np.asarray(targets, np.int64)] = True
        if self.growth:
            self.r_prod = float(gad['production rate'])
            self.r_decay = float(gad['decay rate'])
            self.gsf = float(gad.get('scale factor', 1.0))
            self.decay_max = float(gad.get('decay max', 0.0))
            self.alpha = Influence(gad.get('activators'), gad.get('Km activators'), gad.get('n activators'),
                                   gad.get('zone activators'), gad.get('inhibitors'), gad.get('Km inhibitors'),
                                   gad.get('n inhibitors'), gad.get('zone inhibitors'))
            self.alpha_dec = Influence(gad.get('decay activators'), gad.get('Km decay activators'),
                                       gad.get('n decay activators'), gad.get('zone decay activators'),
                                       gad.get('decay inhibitors'), gad.get('Km decay inhibitors'),
                                       gad.get('n decay inhibitors'), gad.get('zone decay inhibitors'))

    def gad_rate(self, cc, env, n_cells):
        if not self.growth:
            return np.zeros(n_cells)
        c = cc[self.name] / self.gsf
        r = (self.mod * (self.r_prod * self.tdf) * self.alpha(cc, env, n_cells)
             - (self.r_decay * self.tdf) * c
             - (self.decay_max * self.tdf) * self.alpha_dec(cc, env, n_cells) * c)
        out = np.zeros(n_cells)
        out[self.targets] = r[self.targets]
        return out


class Reaction:
    def __init__(self, d, R, T):
        self.reactants = [str(x) for x in d['reactants']]
        self.r_coeff = [float(x) for x in d['reactant multipliers']]
        self.r_km = [float(x) for x in d['Km reactants']]
        self.products = [str(x) for x in d['products']]
        self.p_coeff = [float(x) for x in d['product multipliers']]
        self.vmax = float(d['max rate'])
        dg = d['standard free energy']
        self.keq = None if _absent(dg) else np.exp(-float(dg) / (R * T))
        self.alpha = Influence(d.get('reaction activators'), d.get('activator Km'), d.get('activator n'),
                               d.get('activator zone'), d.get('reaction inhibitors'), d.get('inhibitor Km'),
                               d.get('inhibitor n'), d.get('inhibitor zone'))

    def rate(self, cc, env, n_cells):
        a = self.alpha(cc, env, n_cells)
        if self.keq is None:
            fwd = None
            for name, n, km in zip(self.reactants, self.r_coeff, self.r_km):
                x = (cc[name] / km) ** n
                t = x / (1 + x)
                fwd = t if fwd is None else fwd * t
            return self.vmax * a * fwd
        # BETSE's string is '(1.0e-3*c**n)': the power binds first
        # (write_reactions, networks.py:1364-1396)
        num = None
        for name, n in zip(self.products, self.p_coeff):
            t = 1.0e-3 * cc[name] ** n
            num = t if num is None else num * t
        den = None
        for name, n in zip(self.reactants, self.r_coeff):
            t = 1.0e-3 * cc[name] ** n
            den = t if den is None else den * t
        return self.vmax * a * (1.0 - (num / den) / self.keq)


class NetworkState:
    def __init__(self, c_cells, cc_at_mem, c_env):
        self.c_cells = np.array(c_cells, np.float64)       # [S][C]
        self.cc_at_mem = np.array(cc_at_mem, np.float64)   # [S][M]
        self.c_env = np.array(c_env, np.float64)           # [S] (well-mixed environment)
        self.f_mem = np.zeros_like(self.cc_at_mem)
        self.f_gj = np.zeros_like(self.cc_at_mem)
        self.unstable = 0


class Network:
    """The substances and cell-zone reactions of one network on one cluster
    without extracellular spaces."""

    def __init__(self, substances, reactions, geom, p, mem_vol, time_dila=1.0, targets=None, growth_mod=None):
        C = len(geom.cell_vol)
        targets = targets or {}
        growth_mod = growth_mod or {}
        self.subs = [Substance(d, time_dila, C, targets.get(str(d['name'])), growth_mod.get(str(d['name'])))
                     for d in substances]
        self.names = [s.name for s in self.subs]
        self.reactions = [Reaction(d, p.R, p.T) for d in (reactions or [])]
        S, R = len(self.subs), len(self.reactions)
        # create_reaction_matrix (networks.py:2686-2725), substance rows only
        self.rm = np.zeros((S, S + R))
        for i in range(S):
            self.rm[i, i] += 1
        for j, r in enumerate(self.reactions):
            for name, c in zip(r.reactants, r.r_coeff):
                self.rm[self.names.index(name), S + j] += -c
            for name, c in zip(r.products, r.p_coeff):
                self.rm[self.names.index(name), S + j] += c
        self.g, self.p = geom, p
        self.mem_vol = np.asarray(mem_vol, np.float64)
        self.gamma = geom.mem_sa / ((3 / 4) * self.mem_vol)

    def initial_state(self):
        g = self.g
        C, M = len(g.cell_vol), len(g.mem_to_cells)
        cc = np.stack([np.full(C, s.c_cell0) for s in self.subs])
        return NetworkState(cc, cc[:, g.mem_to_cells], np.array([s.c_env0 for s in self.subs]))

    def step(self, st, vm, vgj, gjopen, gj_block=1.0):
        """One ``run_loop`` on ``st`` in place. ``vm``: Vmem BETSE's network
        reads (the start of the step); ``vgj``: ``sim.vgj`` as the ion loop
        leaves it; ``gjopen``: ``sim.gjopen`` after the ion loop."""
        g, p = self.g, self.p
        C = len(g.cell_vol)
        m2c, nn = g.mem_to_cells, g.nn_i
        dt, T = p.dt, p.T
        vm = np.array(vm, np.float64)
        vgj = np.array(vgj, np.float64)
        # update_intra of every substance (networks.py:5714-5807; En = 0 for
        # neutral substances without Mu_mem)
        for k, s in enumerate(self.subs):
            cav = st.c_cells[k][m2c]
            if not s.update_intra:
                st.cc_at_mem[k] = cav * 1
            else:
                if s.z != 0.0 or s.Mu_mem != 0.0:
                    raise NotImplementedError('intracellular transport of a charged substance reads E_cell')
                a_tot = 0.0
                dts = dt * s.tdf
                gm = self.gamma
                st.cc_at_mem[k] = (((gm * s.Do * dts * cav) / g.R_rads) + ((gm * a_tot * cav * dts) / 2)
                                   + st.cc_at_mem[k]) / (1 + ((gm * s.Do * dts) / g.R_rads)
                                                         - ((gm * a_tot * dts) / 2))
            if np.any(st.cc_at_mem[k] < 0):
                st.unstable += 1
        cc = {s.name: st.c_cells[k] for k, s in enumerate(self.subs)}
        env = {s.name: st.c_env[k] for k, s in enumerate(self.subs)}
        rates = [s.gad_rate(cc, env, C) for s in self.subs]
        rates += [r.rate(cc, env, C) for r in self.reactions]
        delta = self.rm @ np.asarray(rates)
        for k, s in enumerate(self.subs):
            c = st.c_cells[k] + delta[k] * dt
            cm = st.cc_at_mem[k]
            # molecule_mover without extracellular spaces (sim_toolbox.py:909-1153)
            if s.Dm != 0.0:
                f = electroflux(st.c_env[k], cm, s.Dm, p.tm, s.z, vm, T, p.F, p.R)
                vm = vm + FLOAT_NONCE
            else:
                f = np.zeros(len(cm))
            dcell = seg_sum(g, f * g.mem_sa) / g.cell_vol
            if not s.update_intra:
                c = c + dcell * dt
                cm = c[m2c]
            else:
                cm = cm + f * self.gamma * dt
                c = c + dcell * dt
            env_o = st.c_env[k] + (-f * (g.mem_sa / p.vol_env)) * dt
            e = env_o.mean()
            if not s.ignore_gj:
                fgj = electroflux(cm, cm[nn], s.Dgj * gj_block * gjopen, g.gj_len, s.z, vgj, T, p.F, p.R)
                vgj = vgj + FLOAT_NONCE
                fgj[g.bflag] = 0.0
                dcc = seg_sum(g, -fgj * g.mem_sa) / g.cell_vol
                c = c + dt * dcc * s.tdf
                if not s.update_intra:
                    cm = c[m2c]
                else:
                    cm = cm + (-fgj) * self.gamma * s.tdf * dt
            else:
                fgj = np.zeros(len(cm))
            if np.any(c < 0) or np.any(cm < 0) or e < 0:
                st.unstable += 1
            st.c_cells[k], st.cc_at_mem[k], st.c_env[k] = c, cm, e
            st.f_mem[k], st.f_gj[k] = f, fgj


def run_with_ions(net, st, g, p, s, n_steps):
    """Step the ions (``oracle.step``) and the network together in BETSE's
    order: the network of step t reads Vmem from the start of the step and the
    gap-junction state and ``sim.vgj`` the ion loop of step t leaves."""
    from .step import step as ion_step
    I = s.cc_at_mem.shape[0]
    for _ in range(n_steps):
        vm = s.vm.copy()
        ion_step(g, p, s)
        for _i in range(I):           # the ion loop's in-place nonce on vm (sim_toolbox.py:54)
            vm = vm + FLOAT_NONCE
        vgj = (vm[g.nn_i] - vm) + FLOAT_NONCE
        gjopen = s.gjopen if getattr(p, 'v_sensitive_gj', False) else p.gj_block * g.gj_weight
        net.step(st, vm, vgj, gjopen, p.gj_block)
