"""Host logic of the ``_run_sim_core_loop`` drop-in (no GPU needed)."""
from types import SimpleNamespace

import numpy as np
import pytest

from betse_gb300 import simulator


def _phase(kind='INIT', **popts):
    p = SimpleNamespace(ions_dict={'Na': 1, 'K': 1, 'Cl': 1, 'Ca': 1, 'P': 1}, alpha_Ca=0.0,
                        cluster_open=True, cell_polarizability=0.0, dynamic_noise=0, **popts)
    return SimpleNamespace(p=p, kind=SimpleNamespace(name=kind))


def test_default_electrodiffusion_config_is_supported():
    assert simulator.unsupported_features(None, _phase()) == []
    # BETSE's default configuration gates its gap junctions by voltage
    assert simulator.unsupported_features(None, _phase(v_sensitive_gj=True)) == []
    # the mammal/amphibian profiles run ca_handler's Ca-ATPase with alpha_Ca > 0
    ph = _phase()
    ph.p.alpha_Ca = 5e-8
    assert simulator.unsupported_features(None, ph) == []


@pytest.mark.parametrize('opt,frag', [
    (dict(Ca_dyn=True), 'endoplasmic reticulum'),
    (dict(molecules_enabled=True, grn_enabled=True), 'gene regulatory'),
    (dict(deform_osmo=True), 'osmotic'),
    (dict(fluid_flow=True), 'fluid flow'),
    (dict(deformation=True), 'deformation'),
    (dict(cluster_open=False), 'closed cluster'),
])
def test_unsupported_options_are_named(opt, frag):
    ph = _phase()
    for k, v in opt.items():
        setattr(ph.p, k, v)
    reasons = simulator.unsupported_features(None, ph)
    assert len(reasons) == 1 and frag in reasons[0]


def test_networks_need_the_plain_form_without_ecm():
    """A general or gene regulatory network steps with the plain FP64 form;
    the split form, extracellular spaces and network transporters are named."""
    sim = SimpleNamespace(molecules=SimpleNamespace(transporters=False, channels=False, modulators=False),
                          grn=SimpleNamespace(transporters=True, channels=False, modulators=False))
    for flag in ('molecules_enabled', 'grn_enabled'):
        ph = _phase(**{flag: True})
        r = simulator.unsupported_features(sim, ph, precision='fp64')
        assert r == [] if flag == 'molecules_enabled' else ('network transporters (grn)' in r[0] and len(r) == 1)
        r = simulator.unsupported_features(sim, ph, precision='split')
        assert any('split form' in x for x in r)
        ph.p.is_ecm = True
        assert any('extracellular' in x for x in simulator.unsupported_features(sim, ph, precision='fp64'))


def test_polarizability_needs_the_plain_form():
    ph = _phase()
    ph.p.cell_polarizability = 1e-4
    assert simulator.unsupported_features(None, ph, precision='fp64') == []
    reasons = simulator.unsupported_features(None, ph, precision='split')
    assert len(reasons) == 1 and 'polarizability' in reasons[0]


def test_sim_phase_needs_event_free_configuration():
    ph = _phase('SIM')
    assert 'scheduled events' in simulator.unsupported_features(None, ph)[0]
    assert simulator.unsupported_features(None, ph, assume_no_events=True) == []
    ph.p.dynamic_noise = 1
    assert 'dynamic protein noise' in simulator.unsupported_features(None, ph, True)[0]


def test_refusal_happens_before_any_device_work():
    ph = _phase(fluid_flow=True)
    with pytest.raises(NotImplementedError, match='fluid flow'):
        simulator.run_sim_core_loop(None, ph, np.arange(3) * 0.1, set())


def test_install_patches_and_returns_original():
    class Simulator:
        def _run_sim_core_loop(self, phase, time_steps, time_steps_sampled, anim_cells):
            return 'cpu'

    orig = simulator.install(Simulator, precision='split')
    assert orig(Simulator(), None, None, None, None) == 'cpu'
    assert Simulator._run_sim_core_loop.__wrapped__ is orig
    ph = _phase(grn_enabled=True)
    with pytest.raises(NotImplementedError, match='networks in the split form'):
        Simulator()._run_sim_core_loop(ph, np.arange(2), set(), None)


def test_product_laplacian_matches_oracle():
    """The forward operator (its GPU inverse is checked in test_gpu_lapinv.py)."""
    import oracle
    from betse_gb300.fields import make_laplacian
    L = make_laplacian(9, 11, 2.5e-6).toarray()
    assert np.array_equal(L, oracle.fields.make_laplacian(9, 11, 2.5e-6))


def _betse_objects(**popts):
    """A BETSE Parameters / Simulator pair with the fields StepParams reads."""
    p = SimpleNamespace(F=96485.0, R=8.314, dt=1e-2, cm=0.022, tm=7.5e-9, gj_surface=5e-8, alpha_NaK=5e-8,
                        KmNK_Na=12.0, KmNK_K=0.2, KmNK_ATP=0.5, cATP=1.5, cADP=0.1, cPi=0.1,
                        deltaGATP=-37000.0, vol_env=1e-12, is_ecm=False,
                        ions_dict={'Na': 1, 'K': 1, 'Cl': 1, 'Ca': 1, 'P': 1, 'M': 1}, alpha_Ca=0.0,
                        KmCa_Ca=1e-3, KmCa_ATP=0.5, v_sensitive_gj=False, gj_vthresh=15.0, gj_min=0.1,
                        cell_polarizability=0.0)
    for k, v in popts.items():
        setattr(p, k, v)
    sim = SimpleNamespace(zs=np.array([1, 1, -1, 2, -1, -1.0]), D_free=np.ones(6) * 1e-9,
                          D_gj=np.ones(6) * 1e-18, iNa=0, iK=1, iCa=3, T=310.15, gj_block=1, NaKATP_block=1)
    return p, sim


def test_step_params_follow_betse_options():
    from betse_gb300.cluster import StepParams
    p, sim = _betse_objects()
    sp = StepParams.from_betse(p, sim)
    assert (sp.iCa, sp.alpha_Ca, sp.v_sensitive_gj, sp.cell_polarizability) == (3, 0.0, False, 0.0)
    c = sp.to_c()
    assert c.iCa == 3 and c.alpha_Ca == 0.0          # the pump stays off with alpha_Ca == 0
    p, sim = _betse_objects(alpha_Ca=5e-8, v_sensitive_gj=True, gj_vthresh=12.0, cell_polarizability=1e-4)
    sp = StepParams.from_betse(p, sim)
    assert sp.iCa == 3 and sp.alpha_Ca == 5e-8
    assert sp.v_sensitive_gj and sp.gj_vthresh == 12.0
    assert sp.cell_polarizability == 1e-4
    c = sp.to_c()
    assert (c.v_sensitive_gj, c.gj_vthresh, c.cell_polarizability, c.alpha_Ca) == (1, 12.0, 1e-4, 5e-8)
    # a profile without Ca leaves ca_handler's pump out whatever alpha_Ca says
    p, sim = _betse_objects(alpha_Ca=5e-8)
    p.ions_dict = dict(p.ions_dict, Ca=0)
    assert StepParams.from_betse(p, sim).iCa == -1


def test_step_params_reject_a_ca_row_out_of_range():
    from betse_gb300.cluster import StepParams
    p, sim = _betse_objects(alpha_Ca=5e-8)
    sp = StepParams.from_betse(p, sim).replace(iCa=9)
    with pytest.raises(ValueError, match='iCa'):
        sp.to_c()


class _FakeEngine:
    """Stands in for ClusterEngine: arrays of the shapes the device returns."""

    def __init__(self, I, C, M, shape, ecm):
        self.I, self.C, self.M, self.ecm = I, C, M, ecm
        self.G = int(np.prod(shape))
        self.shape = shape

    def download(self):
        st = dict(vm=np.zeros(self.M), cc_cells=np.ones((self.I, self.C)), cc_at_mem=np.ones((self.I, self.M)),
                  cc_env=np.ones((self.I, self.G)) if self.ecm else np.ones(self.I))
        if self.ecm:
            st.update(E_env_x=np.zeros(self.G), E_env_y=np.zeros(self.G))
        return st

    def outputs(self):
        I, C, M = self.I, self.C, self.M
        o = dict(fluxes_mem=np.zeros((I, M)), fluxes_gj=np.zeros((I, M)), rate_NaKATP=np.zeros(M),
                 rho_cells=np.zeros(C), Jn=np.zeros(M), I_mem=np.zeros(M), J_cell_x=np.zeros(C),
                 J_cell_y=np.zeros(C), Jc=np.zeros(M), vm_ave=np.zeros(C), dvm=np.zeros(M),
                 E_cell_x=np.zeros(C), E_cell_y=np.zeros(C), Emc=np.zeros(M), E_gj_x=np.zeros(M),
                 E_gj_y=np.zeros(M), gjopen=np.ones(M), sigma_cell=np.ones(C))
        if self.ecm:
            o['rho_env'] = np.zeros(self.G)
        return o

    def env_fields(self, D_env_weight=None):
        return {k: np.zeros(self.G) for k in ('v_env', 'E_env_x', 'E_env_y', 'J_env_x', 'J_env_y', 'B_field')}


@pytest.mark.parametrize('ecm', [False, True])
def test_mirror_leaves_what_write2storage_reads(ecm):
    """After a sampled step the Simulator holds, under BETSE's names and shapes,
    every step quantity Simulator.write2storage stores (sim.py:1789-1884)."""
    I, C, M, shape = 6, 10, 46, (4, 5)
    cells = SimpleNamespace(grid_shape=shape, mem_vects_flat=np.zeros((M, 4)),
                            map_mem2ecm=np.zeros(M, np.int64))
    sim = SimpleNamespace()
    simulator._mirror(sim, cells, _FakeEngine(I, C, M, shape, ecm), True, None)
    G = int(np.prod(shape))
    want = dict(vm=(M,), cc_cells=(I, C), cc_env=(I, G) if ecm else (I, M), E_gj_x=(M,), E_gj_y=(M,),
                I_mem=(M,), J_cell_x=(C,), J_cell_y=(C,), J_env_x=shape, J_env_y=shape, gjopen=(M,),
                rate_NaKATP=(M,), rho_cells=(C,), v_env=(G,), vm_ave=(C,), E_env_x=shape, E_env_y=shape,
                B_field=(G,), cc_at_mem=(I, M), Eme=(M,))
    for k, shp in want.items():
        assert hasattr(sim, k), k
        assert np.shape(getattr(sim, k)) == shp, (k, np.shape(getattr(sim, k)), shp)
