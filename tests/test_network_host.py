"""Host side of the network path (``betse_gb300/network.py``), no GPU: the
tables built from BETSE's configuration dicts reproduce the oracle's rates
when evaluated the way ``csrc/bx_network.cuh`` evaluates them, and options the
kernels do not compute are refused by name."""
import copy

import numpy as np
import pytest

import golden_io as gi
from betse_gb300 import _lib
from betse_gb300.network import NetworkSpec
from oracle.network import Network as OracleNetwork
from test_oracle_network import network_inputs


def _factor(spec, t0, nt, cs, env):
    """The kernel's single pass over one factor's terms (bx_network.cuh)."""
    act, inh, dsum = 1.0, 1.0, 0.0
    any_mult = any_inh = any_direct = False
    for kind, sub, ez, km, n in spec.terms[t0:t0 + nt]:
        c = env[sub] if ez else cs[sub]
        if kind == _lib.TERM_ACT:
            x = (c / km) ** n
            act = act * (x / (1 + x)) if any_mult else x / (1 + x)
            any_mult = True
        elif kind == _lib.TERM_ACT_INDEP:
            x = (c / km) ** n
            act = act + x / (1 + x)
        elif kind == _lib.TERM_INH:
            h = 1 / (1 + (c / km) ** n)
            inh = inh * h if any_inh else h
            any_inh = True
        else:
            s = c if kind == _lib.TERM_DIRECT_POS else -c
            dsum = dsum + s if any_direct else s
            any_direct = True
    a = act * inh
    return a * dsum if any_direct else a


def _rates(spec, cs, env, cell):
    out = []
    for r in spec.subs:
        if not r['growth'] or (r['growth_target'] is not None and not r['growth_target'][cell]):
            out.append(0.0)
            continue
        k = len(out)
        mod = 1.0 if r['growth_mod'] is None else r['growth_mod'][cell]
        cc = cs[k] / r['gad_scale_factor']
        out.append(mod * (r['r_production'] * r['time_factor']) * _factor(spec, r['growth_term0'], r['growth_nterm'], cs, env)
                   - (r['r_decay'] * r['time_factor']) * cc
                   - (r['decay_max'] * r['time_factor']) * _factor(spec, r['decay_term0'], r['decay_nterm'], cs, env) * cc)
    return out


def _spec(d):
    cfg, names, targets, mods = network_inputs(d)
    g = gi.geometry(d)
    spec = NetworkSpec.from_config(cfg['substances'], cfg['reactions'], cfg['time_dilation'],
                                   n_cells=len(g.cell_vol), profiles={'spot': targets['B']},
                                   growth_mod={'A': mods['A']}, ion_names=[str(x) for x in d['par_ion_names']],
                                   mem_vol=d['net_mem_vol'], R_rads=g.R_rads)
    return cfg, names, targets, mods, g, spec


def test_tables_reproduce_oracle_growth_rates():
    d = gi.load('net_r50_s21')
    cfg, names, targets, mods, g, spec = _spec(d)
    p = gi.params(d)
    onet = OracleNetwork(cfg['substances'], cfg['reactions'], g, p, d['net_mem_vol'], cfg['time_dilation'],
                         targets, mods)
    rng = np.random.default_rng(3)
    C = len(g.cell_vol)
    cc = rng.uniform(0.01, 1.0, size=(4, C))
    env = np.array([0.0, 0.0, 0.45, 0.9])
    want = np.asarray([s.gad_rate(dict(zip(names, cc)), dict(zip(names, env)), C) for s in onet.subs])
    got = np.asarray([_rates(spec, cc[:, c], env, c) for c in range(C)]).T
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-18)
    # reactions: irreversible and with a standard free energy
    for j, r in enumerate(onet.reactions):
        rec = spec.reactions[j]
        keq = np.exp(-rec['delta_Go'] / (p.R * p.T)) if rec['delta_Go'] is not None else None
        assert (keq is None) == (r.keq is None)
        assert rec['reactant'] == [names.index(x) for x in r.reactants]


def test_term_order_and_refusals():
    d = gi.load('net_r50_s21')
    cfg, names, targets, mods, g, spec = _spec(d)
    # B's growth: multiplicative 'A', then independent 'C!'
    rec = spec.subs[names.index('B')]
    kinds = [t[0] for t in spec.terms[rec['growth_term0']:rec['growth_term0'] + rec['growth_nterm']]]
    assert kinds == [_lib.TERM_ACT, _lib.TERM_ACT_INDEP]
    rec = spec.subs[names.index('C')]
    kinds = [t[0] for t in spec.terms[rec['growth_term0']:rec['growth_term0'] + rec['growth_nterm']]]
    assert kinds == [_lib.TERM_ACT, _lib.TERM_DIRECT_POS]
    rec = spec.subs[names.index('D')]
    (t,) = spec.terms[rec['growth_term0']:rec['growth_term0'] + rec['growth_nterm']]
    assert t[0] == _lib.TERM_INH and t[2] == 1          # env-zone inhibitor
    c = spec.to_c(8.314, 310.15)
    assert c.n_substances == 4 and c.n_reactions == 2 and c.n_terms == len(spec.terms)
    ions = [str(x) for x in d['par_ion_names']]
    kw = dict(n_cells=len(g.cell_vol), profiles={'spot': targets['B']}, growth_mod={'A': mods['A']},
              ion_names=ions, mem_vol=d['net_mem_vol'], R_rads=g.R_rads)
    for key, val in (('active pumping', {'turn on': True}), ('ion channel gating', {'x': 1}),
                     ('transmem', True)):
        subs = copy.deepcopy(cfg['substances'])
        subs[0][key] = val
        with pytest.raises(NotImplementedError, match=key):
            NetworkSpec.from_config(subs, cfg['reactions'], **kw)
    subs = copy.deepcopy(cfg['substances'])
    subs[0]['growth and decay']['activators'] = ['Na']
    subs[0]['growth and decay']['Km activators'] = [1.0]
    subs[0]['growth and decay']['n activators'] = [1.0]
    with pytest.raises(NotImplementedError, match='ion'):
        NetworkSpec.from_config(subs, cfg['reactions'], **kw)
    subs = copy.deepcopy(cfg['substances'])
    subs[2]['update intracellular'] = True
    with pytest.raises(NotImplementedError, match='E_cell'):
        NetworkSpec.from_config(subs, cfg['reactions'], **kw)
    reacts = copy.deepcopy(cfg['reactions'])
    reacts[0]['reaction zone'] = 'env'
    with pytest.raises(NotImplementedError, match='zone'):
        NetworkSpec.from_config(cfg['substances'], reacts, **kw)
    with pytest.raises(NotImplementedError, match='transporters'):
        NetworkSpec.from_config(cfg['substances'], cfg['reactions'], transporters=[{'name': 't'}], **kw)
