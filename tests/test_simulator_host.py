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
    (dict(molecules_enabled=True), 'molecules'),
    (dict(grn_enabled=True), 'gene regulatory'),
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
    with pytest.raises(NotImplementedError, match='gene regulatory'):
        Simulator()._run_sim_core_loop(ph, np.arange(2), set(), None)


def test_product_laplacian_matches_oracle():
    import oracle
    from betse_gb300.fields import lap_env_inverse, make_laplacian
    L = make_laplacian(9, 11, 2.5e-6).toarray()
    assert np.array_equal(L, oracle.fields.make_laplacian(9, 11, 2.5e-6))
    A = lap_env_inverse(9, 11, 2.5e-6)
    assert np.allclose(A @ L, np.eye(99), atol=1e-10)
