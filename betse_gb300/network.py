"""Molecule and gene regulatory networks on the GPU (``bx_network_*``).

``MasterOfNetworks`` (``betse/science/chemistry/networks.py``) reads the
'biomolecules' and 'reactions' of a general network (``p.network_config``,
stepped in ``sim.py:1290-1303``) or of a gene regulatory network
(``gene.py``, stepped in ``sim.py:1305-1319`` or alone by
``MasterOfGenes.run_core_sim``, ``gene.py:220-308``), writes every rate as a
Python string and ``eval``s it each step (``run_loop``, ``networks.py:
2805-2983``). Here the same network is a set of tables -- substances,
influencer terms, reactions -- that ``csrc/bx_network.cuh`` evaluates per cell.

``NetworkSpec.from_config`` reads the configuration dicts (the YAML entries,
``'None'`` strings included); ``NetworkSpec.from_betse`` reads an initialised
``MasterOfNetworks``. Both refuse, naming the BETSE option, what the kernels do
not compute: transporters, channels, modulators, environment- and
mitochondria-zone reactions, active pumping, ion-channel gating, concentration
clamps and boundary changes, transmembrane substances, 'Mu_mem',
'substances affect Vmem', extracellular spaces, influencers or reactants that
are ions, and intracellular transport of charged substances.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib
from .exceptions import BetseSimUnstableException


def _absent(x):
    if x is None or (isinstance(x, str) and x == 'None'):
        return True
    return hasattr(x, '__len__') and not isinstance(x, str) and len(x) == 0


def _default_zones(zones, names):
    """``default_zones`` (networks.py:4738-4750): 'cell' for every name when
    no zones are given."""
    if _absent(names):
        return []
    if _absent(zones):
        return ['cell'] * len(names)
    return list(zones)


class NetworkSpec:
    """The tables of one network (``bx_net_spec``)."""

    def __init__(self, names):
        self.names = list(names)
        self.subs = []       # dicts of bx_net_substance fields (+ 'growth_mod', 'growth_target' arrays)
        self.reactions = []  # dicts of bx_net_reaction fields
        self.terms = []      # (kind, substance, env_zone, Km, n)
        self.mem_vol = None
        self.R_rads = None
        self.c_cell0 = []
        self.c_env0 = []

    # ------------------------------------------------------------------
    def _index(self, name, ions, what):
        if name in ions:
            raise NotImplementedError(f'{what} {name!r} is an ion: network terms that read or change the '
                                      'ion concentrations are not built')
        if name not in self.names:
            raise ValueError(f'{what} {name!r} is not a substance of the network')
        return self.names.index(name)

    def _factor(self, a_names, a_km, a_n, a_zone, i_names, i_km, i_n, i_zone, ions):
        """Append the terms of one ``get_influencers`` factor (reaction zone
        'cell', networks.py:5084-5600) in the order BETSE composes its string:
        multiplicative activators, '!' independent activators, inhibitors,
        then the '&' direct terms. Returns (first term, count)."""
        a_zone, i_zone = _default_zones(a_zone, a_names), _default_zones(i_zone, i_names)
        mult, indep, inh, direct = [], [], [], []
        if not _absent(a_names):
            for name, km, n, zone in zip(a_names, a_km, a_n, a_zone):
                if name.endswith('*'):        # Vmem-sensitive Km: membrane-bound targets only
                    name = name[:-1]
                if name.endswith('!'):
                    indep.append((_lib.TERM_ACT_INDEP, name[:-1], zone, km, n))
                elif name.endswith('&'):
                    direct.append((_lib.TERM_DIRECT_POS, name[:-1], zone, 1.0, 1.0))
                else:
                    mult.append((_lib.TERM_ACT, name, zone, km, n))
        if not _absent(i_names):
            seen_direct = False
            for name, km, n, zone in zip(i_names, i_km, i_n, i_zone):
                if name.endswith('*'):
                    name = name[:-1]
                if name.endswith('!'):
                    name = name[:-1]
                if name.endswith('&'):
                    direct.append((_lib.TERM_DIRECT_NEG, name[:-1], zone, 1.0, 1.0))
                    seen_direct = True
                elif seen_direct:
                    raise ValueError('a direct (&) inhibitor followed by another inhibitor: BETSE composes '
                                     'no valid rate expression for it')
                else:
                    inh.append((_lib.TERM_INH, name, zone, km, n))
        if not _absent(a_names) and not mult and not indep and not _absent(i_names) and not inh:
            raise ValueError('only direct (&) influencers: BETSE composes no valid rate expression for it')
        t0 = len(self.terms)
        for kind, name, zone, km, n in mult + indep + inh + direct:
            if zone not in ('cell', 'env'):
                raise NotImplementedError(f'influencer zone {zone!r}: only cell and env are built')
            self.terms.append((kind, self._index(name, ions, 'influencer'), 1 if zone == 'env' else 0,
                               float(km), float(n)))
        return t0, len(self.terms) - t0

    # ------------------------------------------------------------------
    @classmethod
    def from_config(cls, substances, reactions=None, time_dilation=1.0, n_cells=None, profiles=None,
                    growth_mod=None, ion_names=(), mem_vol=None, R_rads=None, mit_enabled=False,
                    transporters=None, channels=None, modulators=None, substances_affect_charge=False,
                    is_ecm=False):
        """The network of BETSE's configuration dicts ('biomolecules',
        'reactions'; read_substances/tissue_init/read_reactions,
        networks.py:120-657, 814-922). ``profiles`` maps a tissue-profile name
        to its cell indices ('apply to'); ``growth_mod`` maps a substance name
        to its ``growth_mod_function_cells`` values (a 'modulator function')."""
        for what, v in (('transporters', transporters), ('channels', channels), ('modulators', modulators)):
            if not _absent(v):
                raise NotImplementedError(f"network {what} are not built")
        if mit_enabled:
            raise NotImplementedError('mitochondria (enable mitochondria) are not built')
        if substances_affect_charge:
            raise NotImplementedError("'substances affect Vmem' is not built")
        if is_ecm:
            raise NotImplementedError('networks with extracellular spaces are not built')
        ions = set(ion_names)
        names = [str(d['name']) for d in substances]
        spec = cls(names)
        profiles = profiles or {}
        growth_mod = growth_mod or {}
        any_ui = False
        for d in substances:
            name = str(d['name'])
            for key in ('active pumping', 'ion channel gating', 'clamp cell conc', 'change at bounds'):
                if d.get(key) is not None and not _absent(d.get(key)):
                    raise NotImplementedError(f"substance {name!r}: '{key}' is not built")
            if d.get('transmem', False):
                raise NotImplementedError(f"substance {name!r}: 'transmem' is not built")
            if float(d.get('Mu_mem', 0.0)) != 0.0 or float(d.get('u_mtube', 0.0)) != 0.0:
                raise NotImplementedError(f"substance {name!r}: 'Mu_mem' / 'u_mtube' transport is not built")
            init_asym = d.get('initial asymmetry', None)
            if not _absent(init_asym):
                raise NotImplementedError(f"substance {name!r}: 'initial asymmetry' is read from BETSE's "
                                          "objects (NetworkSpec.from_betse)")
            ui = bool(d.get('update intracellular', True))
            z = float(d['z'])
            if ui and z != 0.0:
                raise NotImplementedError(f"substance {name!r}: 'update intracellular' of a charged substance "
                                          'reads the intracellular field E_cell; not built')
            any_ui |= ui
            tdf = float(time_dilation) if d.get('use time dilation', False) else 1.0
            rec = dict(z=z, Dm=float(d['Dm']), Do=float(d['Do']), Dgj=float(d.get('Dgj', 1.0e-16)),
                       time_factor=tdf, update_intra=int(ui), gj_impermeable=int(bool(d['GJ impermeable'])),
                       growth=0, r_production=0.0, r_decay=0.0, decay_max=0.0, gad_scale_factor=1.0,
                       growth_term0=0, growth_nterm=0, decay_term0=0, decay_nterm=0,
                       growth_mod=None, growth_target=None)
            gad = d.get('growth and decay', None)
            if isinstance(gad, dict):
                rec.update(growth=1, r_production=float(gad['production rate']), r_decay=float(gad['decay rate']),
                           decay_max=float(gad.get('decay max', 0.0)),
                           gad_scale_factor=float(gad.get('scale factor', 1.0)))
                apply_to = gad.get('apply to', 'all')
                if apply_to == 'express':
                    raise NotImplementedError(f"substance {name!r}: 'apply to: express' is not built")
                if not (_absent(apply_to) or apply_to == 'all'):
                    if n_cells is None:
                        raise ValueError('n_cells is needed for growth restricted to tissue profiles')
                    mask = np.zeros(int(n_cells), np.uint8)
                    for prof in apply_to:
                        if prof not in profiles:
                            raise ValueError(f"substance {name!r}: no cell indices for profile {prof!r}")
                        mask[np.asarray(profiles[prof], np.int64)] = 1
                    rec['growth_target'] = mask
                mf = gad.get('modulator function', None)
                if not _absent(mf):
                    if name not in growth_mod:
                        raise ValueError(f"substance {name!r}: modulator function {mf!r} needs its "
                                         'growth_mod values')
                    rec['growth_mod'] = np.ascontiguousarray(growth_mod[name], np.float64)
                rec['growth_term0'], rec['growth_nterm'] = spec._factor(
                    gad.get('activators'), gad.get('Km activators'), gad.get('n activators'),
                    gad.get('zone activators'), gad.get('inhibitors'), gad.get('Km inhibitors'),
                    gad.get('n inhibitors'), gad.get('zone inhibitors'), ions)
                rec['decay_term0'], rec['decay_nterm'] = spec._factor(
                    gad.get('decay activators'), gad.get('Km decay activators'), gad.get('n decay activators'),
                    gad.get('zone decay activators'), gad.get('decay inhibitors'),
                    gad.get('Km decay inhibitors'), gad.get('n decay inhibitors'),
                    gad.get('zone decay inhibitors'), ions)
            spec.subs.append(rec)
            spec.c_cell0.append(float(d['cell conc']))
            spec.c_env0.append(float(d['env conc']))
        for d in (reactions or []):
            spec._add_reaction(d.get('reaction zone', 'cell'), d['reactants'], d['reactant multipliers'],
                               d['Km reactants'], d['products'], d['product multipliers'], d['max rate'],
                               d['standard free energy'], d.get('reaction activators'), d.get('activator Km'),
                               d.get('activator n'), d.get('activator zone'), d.get('reaction inhibitors'),
                               d.get('inhibitor Km'), d.get('inhibitor n'), d.get('inhibitor zone'), ions)
        if any_ui:
            if mem_vol is None or R_rads is None:
                raise ValueError("'update intracellular' needs cells.mem_vol and cells.R_rads")
        spec.mem_vol = None if mem_vol is None else np.ascontiguousarray(mem_vol, np.float64)
        spec.R_rads = None if R_rads is None else np.ascontiguousarray(R_rads, np.float64)
        return spec

    def _add_reaction(self, zone, reactants, r_coeff, r_km, products, p_coeff, vmax, dG, a_names, a_km, a_n,
                      a_zone, i_names, i_km, i_n, i_zone, ions, keq_RT=None):
        if zone != 'cell':
            raise NotImplementedError(f"reaction zone {zone!r}: only cell-zone reactions are built")
        reactants = [str(x) for x in reactants]
        products = [] if _absent(products) else [str(x) for x in products]
        if not 1 <= len(reactants) <= _lib.NET_MAX_STOICH or len(products) > _lib.NET_MAX_STOICH:
            raise ValueError(f'reactions take 1..{_lib.NET_MAX_STOICH} reactants and products')
        rec = dict(reactant=[self._index(n, ions, 'reactant') for n in reactants],
                   product=[self._index(n, ions, 'product') for n in products],
                   reactant_coeff=[float(x) for x in r_coeff], reactant_Km=[float(x) for x in r_km],
                   product_coeff=[] if _absent(p_coeff) else [float(x) for x in p_coeff], vmax=float(vmax),
                   delta_Go=None if _absent(dG) else float(dG))
        rec['term0'], rec['nterm'] = self._factor(a_names, a_km, a_n, a_zone, i_names, i_km, i_n, i_zone, ions)
        self.reactions.append(rec)

    # ------------------------------------------------------------------
    @classmethod
    def from_betse(cls, core, cells, p, sim=None):
        """The network of an initialised ``MasterOfNetworks`` (after
        ``tissue_init`` and ``read_reactions``): the values BETSE's own
        strings read, taken from its objects."""
        if getattr(core, 'mit_enabled', False):
            raise NotImplementedError('mitochondria (enable mitochondria) are not built')
        for what in ('transporters', 'channels', 'modulators', 'reactions_env'):
            if len(getattr(core, what, {}) or {}):
                raise NotImplementedError(f'network {what} are not built')
        if getattr(p, 'substances_affect_charge', False):
            raise NotImplementedError("'substances affect Vmem' is not built")
        if getattr(p, 'is_ecm', False):
            raise NotImplementedError('networks with extracellular spaces are not built')
        ions = set(k for k, v in p.ions_dict.items() if v == 1)
        names = list(core.molecules)
        spec = cls(names)
        n_cells = len(cells.cell_i)
        any_ui = False
        for name, mol in core.molecules.items():
            for attr, what in (('active_pumping', 'active pumping'), ('ion_channel_gating', 'ion channel gating'),
                               ('cell_clamp', 'clamp cell conc'), ('change_bounds', 'change at bounds'),
                               ('transmem', 'transmem')):
                if getattr(mol, attr, False):
                    raise NotImplementedError(f"substance {name!r}: '{what}' is not built")
            if float(getattr(mol, 'Mu_mem', 0.0)) != 0.0 or float(getattr(mol, 'u_mt', 0.0)) != 0.0:
                raise NotImplementedError(f"substance {name!r}: 'Mu_mem' / 'u_mtube' transport is not built")
            ui = bool(mol.update_intra_conc)
            if ui and float(mol.z) != 0.0:
                raise NotImplementedError(f"substance {name!r}: 'update intracellular' of a charged substance "
                                          'reads the intracellular field E_cell; not built')
            any_ui |= ui
            rec = dict(z=float(mol.z), Dm=float(mol.Dm), Do=float(mol.Do), Dgj=float(mol.Dgj),
                       time_factor=float(mol.modify_time_factor), update_intra=int(ui),
                       gj_impermeable=int(bool(mol.ignoreGJ)), growth=0, r_production=0.0, r_decay=0.0,
                       decay_max=0.0, gad_scale_factor=1.0, growth_term0=0, growth_nterm=0, decay_term0=0,
                       decay_nterm=0, growth_mod=None, growth_target=None)
            if mol.simple_growth:
                if mol.growth_profiles_list == 'express':
                    raise NotImplementedError(f"substance {name!r}: 'apply to: express' is not built")
                rec.update(growth=1, r_production=float(mol.r_production), r_decay=float(mol.r_decay),
                           decay_max=float(mol.decay_max), gad_scale_factor=float(mol.gad_scale_factor))
                targets = np.asarray(mol.growth_targets_cell, np.int64)
                if len(targets) != n_cells or not np.array_equal(np.sort(targets), np.arange(n_cells)):
                    mask = np.zeros(n_cells, np.uint8)
                    mask[targets] = 1
                    rec['growth_target'] = mask
                gm = np.asarray(mol.growth_mod_function_cells, np.float64) * np.ones(n_cells)
                if not np.all(gm == 1.0):
                    rec['growth_mod'] = np.ascontiguousarray(gm)
                rec['growth_term0'], rec['growth_nterm'] = spec._factor(
                    mol.growth_activators_list, mol.growth_activators_Km, mol.growth_activators_n,
                    mol.growth_activators_zone, mol.growth_inhibitors_list, mol.growth_inhibitors_Km,
                    mol.growth_inhibitors_n, mol.growth_inhibitors_zone, ions)
                rec['decay_term0'], rec['decay_nterm'] = spec._factor(
                    mol.decay_activators_list, mol.decay_activators_Km, mol.decay_activators_n,
                    mol.decay_activators_zone, mol.decay_inhibitors_list, mol.decay_inhibitors_Km,
                    mol.decay_inhibitors_n, mol.decay_inhibitors_zone, ions)
            spec.subs.append(rec)
        for rname, r in core.reactions.items():
            spec._add_reaction(r.reaction_zone, r.reactants_list, r.reactants_coeff, r.Km_reactants_list,
                               r.products_list, r.products_coeff, r.vmax, r.delta_Go,
                               r.reaction_activators_list, r.reaction_activators_Km, r.reaction_activators_n,
                               r.reaction_activators_zone, r.reaction_inhibitors_list, r.reaction_inhibitors_Km,
                               r.reaction_inhibitors_n, r.reaction_inhibitors_zone, ions)
        if any_ui:
            spec.mem_vol = np.ascontiguousarray(cells.mem_vol, np.float64)
            spec.R_rads = np.ascontiguousarray(cells.R_rads, np.float64)
        return spec

    # ------------------------------------------------------------------
    def to_c(self, R, T):
        """``bx_net_spec`` and the arrays it points to (kept on the object)."""
        S, NR, NT = len(self.subs), len(self.reactions), len(self.terms)
        if not 1 <= S <= _lib.NET_MAX_SUBSTANCES:
            raise ValueError(f'a network holds 1..{_lib.NET_MAX_SUBSTANCES} substances')
        if NR > _lib.NET_MAX_REACTIONS or NT > _lib.NET_MAX_TERMS:
            raise ValueError('too many reactions or influencer terms')
        subs = (_lib.BxNetSubstance * S)()
        keep = []
        for k, r in enumerate(self.subs):
            s = subs[k]
            for f in ('z', 'Dm', 'Do', 'Dgj', 'time_factor', 'r_production', 'r_decay', 'decay_max',
                      'gad_scale_factor', 'growth', 'update_intra', 'gj_impermeable', 'growth_term0',
                      'growth_nterm', 'decay_term0', 'decay_nterm'):
                setattr(s, f, r[f])
            if r['growth_mod'] is not None:
                keep.append(r['growth_mod'])
                s.growth_mod = _lib.dptr(r['growth_mod'])
            if r['growth_target'] is not None:
                keep.append(r['growth_target'])
                s.growth_target = _lib.u8ptr(r['growth_target'])
        reacts = (_lib.BxNetReaction * max(NR, 1))()
        for j, r in enumerate(self.reactions):
            x = reacts[j]
            x.n_reactants, x.n_products = len(r['reactant']), len(r['product'])
            for q, v in enumerate(r['reactant']):
                x.reactant[q] = v
                x.reactant_coeff[q] = r['reactant_coeff'][q]
                x.reactant_Km[q] = r['reactant_Km'][q]
            for q, v in enumerate(r['product']):
                x.product[q] = v
                x.product_coeff[q] = r['product_coeff'][q]
            x.vmax = r['vmax']
            # exp(-delta_Go / (R T)) of write_reactions (networks.py:1462-1470)
            x.keq = 0.0 if r['delta_Go'] is None else float(np.exp(-r['delta_Go'] / (R * T)))
            x.term0, x.nterm = r['term0'], r['nterm']
        terms = (_lib.BxNetTerm * max(NT, 1))()
        for q, (kind, sub, env, km, n) in enumerate(self.terms):
            terms[q].kind, terms[q].substance, terms[q].env_zone = kind, sub, env
            terms[q].Km, terms[q].n = km, n
        spec = _lib.BxNetSpec()
        spec.n_substances, spec.n_reactions, spec.n_terms = S, NR, NT
        spec.substances = ct.cast(subs, ct.POINTER(_lib.BxNetSubstance))
        spec.reactions = ct.cast(reacts, ct.POINTER(_lib.BxNetReaction))
        spec.terms = ct.cast(terms, ct.POINTER(_lib.BxNetTerm))
        if self.mem_vol is not None:
            spec.mem_vol = _lib.dptr(self.mem_vol)
        if self.R_rads is not None:
            spec.R_rads = _lib.dptr(self.R_rads)
        self._c = (spec, subs, reacts, terms, keep)
        return spec


class Network:
    """A network stepping on a plain FP64 ``ClusterEngine``'s cluster."""

    def __init__(self, engine, spec: NetworkSpec):
        self.lib = _lib.load()
        self.engine = engine
        self.spec = spec
        self.names = list(spec.names)
        self.S, self.C, self.M = len(spec.names), engine.C, engine.M
        c = spec.to_c(engine.params.R, engine.params.T)
        h = ct.c_void_p()
        _lib.check(self.lib.bx_network_create(engine.h, ct.byref(c), ct.byref(h)), 'bx_network_create')
        self.h = h

    def close(self):
        if getattr(self, 'h', None) is not None and self.h.value:
            self.lib.bx_network_destroy(self.h)
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

    def upload(self, c_cells, cc_at_mem, c_env):
        """``Molecule.c_cells`` [S][C], ``cc_at_mem`` [S][M] and ``c_env``: one
        well-mixed value per substance (BETSE's uniform length-M vector is
        accepted)."""
        cc = np.ascontiguousarray(c_cells, np.float64).reshape(self.S, self.C)
        cm = np.ascontiguousarray(cc_at_mem, np.float64).reshape(self.S, self.M)
        ce = np.asarray(c_env, np.float64)
        if ce.ndim == 2:
            if not np.all(ce == ce[:, :1]):
                raise ValueError('without ECM, c_env must be uniform over membranes')
            ce = ce[:, 0]
        ce = np.ascontiguousarray(ce).reshape(self.S)
        _lib.check(self.lib.bx_network_upload(self.h, cc.ctypes.data, cm.ctypes.data, ce.ctypes.data),
                   'bx_network_upload')

    def upload_initial(self):
        """The initial concentrations of the configuration ('cell conc',
        'env conc'; read_substances, networks.py:221-262)."""
        cc = np.repeat(np.asarray(self.spec.c_cell0)[:, None], self.C, 1)
        m2c = np.repeat(np.arange(self.C), np.diff(self.engine.geom.cell_mem_ptr))
        self.upload(cc, cc[:, m2c], np.asarray(self.spec.c_env0))

    def download(self):
        cc = np.empty((self.S, self.C))
        cm = np.empty((self.S, self.M))
        ce = np.empty(self.S)
        _lib.check(self.lib.bx_network_download(self.h, cc.ctypes.data, cm.ctypes.data, ce.ctypes.data),
                   'bx_network_download')
        return {'c_cells': cc, 'cc_at_mem': cm, 'c_env': ce}

    def step(self, n_steps, with_ions=True, outputs=False):
        _lib.check(self.lib.bx_network_step(self.h, int(n_steps), int(bool(with_ions)), int(bool(outputs))),
                   'bx_network_step')

    def fluxes(self):
        """The last output step's ``f_mem``, ``f_gj`` [S][M] and the cell-zone
        ``reaction_rates`` [R][C]."""
        fm = np.empty((self.S, self.M))
        fg = np.empty((self.S, self.M))
        rr = np.empty((len(self.spec.reactions), self.C))
        _lib.check(self.lib.bx_network_fluxes(self.h, fm.ctypes.data, fg.ctypes.data,
                                              rr.ctypes.data if rr.size else None), 'bx_network_fluxes')
        return {'f_mem': fm, 'f_gj': fg, 'reaction_rates': rr}

    def time_step(self, n_steps, with_ions=True):
        """ms per time step of ``n_steps`` steps, timed with CUDA events on the
        cluster's stream (the state advances)."""
        v = ct.c_double()
        _lib.check(self.lib.bx_network_time_step(self.h, int(n_steps), int(bool(with_ions)), ct.byref(v)),
                   'bx_network_time_step')
        return float(v.value)

    def algorithmic_bytes(self):
        """Bytes one network step (both kernels) moves, each array once at
        its stored width: per cell the concentrations in and out of both
        kernels (16 S each), the CSR pointer and volume; per membrane Vmem,
        mem_sa, the partner maps, boundary flag and gap-junction weight; per
        membrane and substance the cc_at_mem write, and for 'update
        intracellular' substances the membrane values in, mid out and in, and
        gamma / R_rads; growth modulation and target rows per cell."""
        S, C, M = self.S, self.C, self.M
        n_ui = sum(r['update_intra'] for r in self.spec.subs)
        rows = sum(r['growth_mod'] is not None for r in self.spec.subs) * 8 + \
            sum(r['growth_target'] is not None for r in self.spec.subs)
        cell = C * (2 * 16 * S + 2 * 12) + C * rows
        mem = M * (8 + 8 + 4 + 4 + 1 + 8) + M * 8 * S + n_ui * M * (8 + 8 + 8 + 8 + 8)
        return int(cell + mem)

    def negative_count(self):
        v = ct.c_int64()
        _lib.check(self.lib.bx_network_status(self.h, ct.byref(v)), 'bx_network_status')
        return int(v.value)

    def check_stable(self):
        """BETSE raises on a negative substance concentration
        (sim_toolbox.py:1132-1151, networks.py:5802-5807)."""
        n = self.negative_count()
        if n:
            raise BetseSimUnstableException(
                f'Network concentration below zero ({n} values)! Your simulation has become unstable.')
