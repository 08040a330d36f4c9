"""GPU parity of the molecule / gene-regulatory-network step
(``bx_network_*``, ``csrc/bx_network.cuh``):

* stepped with the ions against BETSE's own ``MasterOfNetworks`` run
  (``tests/golden/net_r50_s21.npz``, 300 steps; the coupled CUDA-graph path
  runs from step 2 on): substance concentrations in cells, at membranes and in
  the environment within 1e-10 relative, fluxes at the checkpoints;
* the network alone (``MasterOfGenes.run_core_sim``, gene.py:220-308) against
  the oracle on a frozen Vmem;
* a generated 3800-cell cluster against the oracle over 100 steps;
* a negative concentration is reported (BETSE raises
  ``BetseSimUnstableException``), computed on the host side of the check.
"""
import copy

import numpy as np
import pytest

import golden_io as gi
from oracle.network import Network as OracleNetwork, NetworkState, run_with_ions
from test_oracle_network import network_inputs

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def _rel(a, b):
    den = np.max(np.abs(b))
    return np.max(np.abs(a - b)) / (den if den > 0 else 1.0)


def _setup(d, substances=None):
    from betse_gb300.engine import ClusterEngine
    from betse_gb300.network import Network, NetworkSpec
    cfg, names, targets, mods = network_inputs(d)
    cg, sp, Dm, st, _ = gi.engine_inputs(d)
    g = gi.geometry(d)
    eng = ClusterEngine(cg, sp, 'fp64')
    eng.set_membrane_diffusivity(Dm)
    eng.upload(**st)
    spec = NetworkSpec.from_config(substances or cfg['substances'], cfg['reactions'], cfg['time_dilation'],
                                   n_cells=len(g.cell_vol), profiles={'spot': targets['B']},
                                   growth_mod={'A': mods['A']}, ion_names=[str(x) for x in d['par_ion_names']],
                                   mem_vol=d['net_mem_vol'], R_rads=g.R_rads)
    net = Network(eng, spec)
    net.upload(d['init_net_c_cells'], d['init_net_cc_at_mem'], d['init_net_c_env'])
    return eng, net


def test_network_with_ions_matches_betse():
    d = gi.load('net_r50_s21')
    eng, net = _setup(d)
    with eng, net:
        done = 0
        for cp in d['meta_checkpoints']:
            net.step(int(cp - done), with_ions=True, outputs=True)
            done = int(cp)
            net.check_stable()
            eng.check_stable()
            got = net.download()
            for k in ('c_cells', 'cc_at_mem'):
                assert _rel(got[k], d[f's{cp}_net_{k}']) < RTOL, (cp, k, _rel(got[k], d[f's{cp}_net_{k}']))
            np.testing.assert_allclose(got['c_env'], d[f's{cp}_net_c_env'][:, 0], rtol=RTOL, atol=0)
            fl = net.fluxes()
            for k in ('f_mem', 'f_gj'):
                ref = d[f's{cp}_net_{k}']
                for s in range(ref.shape[0]):
                    assert np.max(np.abs(fl[k][s] - ref[s])) <= 1e-9 * max(np.max(np.abs(ref[s])), 1e-300), (cp, k, s)
            assert _rel(eng.download()['vm'], d[f's{cp}_vm']) < 1e-9


def test_network_alone_matches_oracle():
    """The network without the ion step (gene.py:220-308): Vmem and the gap
    junctions stay as uploaded."""
    d = gi.load('net_r50_s21')
    g, p, s = gi.geometry(d), gi.params(d), gi.state(d)
    cfg, names, targets, mods = network_inputs(d)
    onet = OracleNetwork(cfg['substances'], cfg['reactions'], g, p, d['net_mem_vol'], cfg['time_dilation'],
                         targets, mods)
    st = NetworkState(d['init_net_c_cells'], d['init_net_cc_at_mem'], d['init_net_c_env'][:, 0])
    vm = s.vm
    n = 70
    for _ in range(n):
        onet.step(st, vm, vm[g.nn_i] - vm, p.gj_block * g.gj_weight, p.gj_block)
    eng, net = _setup(d)
    with eng, net:
        net.step(n, with_ions=False)
        net.check_stable()
        got = net.download()
        assert np.array_equal(eng.download()['vm'], d['init_vm'])
    for k in ('c_cells', 'cc_at_mem'):
        assert _rel(got[k], getattr(st, k)) < RTOL, k
    np.testing.assert_allclose(got['c_env'], st.c_env, rtol=RTOL, atol=0)


def test_network_generated_cluster_matches_oracle():
    """A 3800-cell generated cluster (BETSE's seeding recipe) with the same
    network: 100 coupled steps against the oracle run with the ion oracle."""
    from betse_gb300 import generator as gen
    from betse_gb300.engine import ClusterEngine
    from betse_gb300.network import Network, NetworkSpec
    from oracle.adapt import from_workload
    d = gi.load('net_r50_s21')
    cfg, names, targets, mods = network_inputs(d)
    geom, params, Dm, st0, _ = gen.workload(290e-6, 5, is_ecm=False, dt=1e-2, dm_range=(1e-19, 1e-17))
    C, M = geom.n_cells, geom.n_mems
    rng = np.random.default_rng(7)
    spot = np.sort(rng.choice(C, size=C // 3, replace=False))
    gmod = rng.uniform(0.2, 1.2, size=C)
    R_rads = np.asarray(geom.R_rads)
    mem_vol = 0.5 * R_rads * geom.mem_sa          # cells.py:1382
    spec = NetworkSpec.from_config(cfg['substances'], cfg['reactions'], cfg['time_dilation'], n_cells=C,
                                   profiles={'spot': spot}, growth_mod={'A': gmod}, ion_names=params.ion_names,
                                   mem_vol=mem_vol, R_rads=R_rads)
    og, op, os_ = from_workload(geom, params, Dm, st0)
    onet = OracleNetwork(cfg['substances'], cfg['reactions'], og, op, mem_vol, cfg['time_dilation'],
                         {'B': spot}, {'A': gmod})
    og.R_rads = R_rads
    ost = onet.initial_state()
    n = 100
    run_with_ions(onet, ost, og, op, os_, n)
    assert ost.unstable == 0
    with ClusterEngine(geom, params, 'fp64') as eng:
        eng.set_membrane_diffusivity(Dm)
        eng.upload(**st0)
        with Network(eng, spec) as net:
            net.upload_initial()
            net.step(n, with_ions=True)
            net.check_stable()
            got = net.download()
    for k in ('c_cells', 'cc_at_mem'):
        assert _rel(got[k], getattr(ost, k)) < RTOL, k
    np.testing.assert_allclose(got['c_env'], ost.c_env, rtol=RTOL, atol=0)


def test_network_negative_concentration_is_reported():
    from betse_gb300.exceptions import BetseSimUnstableException
    d = gi.load('net_r50_s21')
    cfg, names, targets, mods = network_inputs(d)
    subs = copy.deepcopy(cfg['substances'])
    subs[3]['growth and decay']['decay rate'] = 500.0     # c - 500 c dt < 0 within a step
    eng, net = _setup(d, subs)
    with eng, net:
        net.step(3, with_ions=True)
        assert net.negative_count() > 0
        with pytest.raises(BetseSimUnstableException):
            net.check_stable()
