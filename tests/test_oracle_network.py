"""The molecule-network oracle (``oracle/network.py``) against BETSE's own
``MasterOfNetworks`` stepped with the ions (``tests/golden/net_r50_s21.npz``):
substance concentrations in cells, at membranes and in the environment, and
the membrane and gap-junction fluxes, at every checkpoint up to 300 steps."""
import json

import numpy as np
import pytest

import golden_io as gi
from oracle.network import Influence, Network, NetworkState, run_with_ions


def network_inputs(d):
    """The network description a drop-in reads from BETSE's objects: the
    configuration dicts, the growth targets and modulator values per substance."""
    cfg = json.loads(str(d['net_config']))
    names = [str(x) for x in d['net_names']]
    targets = {'B': d['net_spot_cells']}
    mods = {n: d['net_growth_mod'][k] for k, n in enumerate(names)}
    return cfg, names, targets, mods


def test_network_oracle_matches_betse():
    d = gi.load('net_r50_s21')
    g, p, s = gi.geometry(d), gi.params(d), gi.state(d)
    cfg, names, targets, mods = network_inputs(d)
    net = Network(cfg['substances'], cfg['reactions'], g, p, d['net_mem_vol'], cfg['time_dilation'],
                  targets, mods)
    assert np.array_equal(net.rm, d['net_reaction_matrix'][-len(names):])
    st = NetworkState(d['init_net_c_cells'], d['init_net_cc_at_mem'], d['init_net_c_env'][:, 0])
    done = 0
    for cp in d['meta_checkpoints']:
        run_with_ions(net, st, g, p, s, int(cp - done))
        done = int(cp)
        assert st.unstable == 0
        for k in ('c_cells', 'cc_at_mem', 'f_mem', 'f_gj'):
            ref = d[f's{cp}_net_{k}']
            got = getattr(st, k)
            assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref)), (cp, k)
        np.testing.assert_allclose(st.c_env, d[f's{cp}_net_c_env'][:, 0], rtol=1e-12, atol=0)
        np.testing.assert_allclose(s.vm, d[f's{cp}_vm'], rtol=1e-10, atol=0)


def test_influencer_composition():
    """get_influencers' composition rules on a single cell: product of
    multiplicative activators plus independent ones, inhibitors, direct terms."""
    cc = {'A': np.array([0.2]), 'B': np.array([0.5]), 'C': np.array([1.5])}
    env = {'A': 0.0, 'B': 2.0, 'C': 0.1}
    h = lambda c, k, n: (c / k) ** n / (1 + (c / k) ** n)  # noqa: E731
    f = Influence(['A', 'B!'], [0.1, 0.4], [2, 1], None, ['C'], [1.0], [3], ['env'], )
    assert np.allclose(f(cc, env, 1), (h(0.2, 0.1, 2) + h(0.5, 0.4, 1)) / (1 + (0.1 / 1.0) ** 3))
    f = Influence(['B!'], [0.4], [1], None, 'None', None, None, None)
    assert np.allclose(f(cc, env, 1), 1 + h(0.5, 0.4, 1))
    f = Influence(['A', 'C&'], [0.1, 1.0], [1, 1], None, ['B&'], [1.0], [1], None)
    assert np.allclose(f(cc, env, 1), h(0.2, 0.1, 1) * (1.5 - 0.5))
    with pytest.raises(ValueError):
        Influence('None', None, None, None, ['A&', 'B'], [1, 1], [1, 1], None)
