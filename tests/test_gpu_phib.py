"""Applied boundary potential (sim.Phi_b, the lapENVinv solution of an
applied-voltage event, ion_current.py:164-171) against the oracle.

A smooth Phi_b of a few mV on the environment grid makes Vmem differ between
the membranes of one cell (vm = (rho diviterm)[mem_to_cells]/cm -
Phi_b[map_mem2ecm], sim.py:2027-2029).  Tolerances as in test_gpu_parity.py.
"""
import numpy as np
import pytest

import golden_io as gi
import oracle

pytestmark = pytest.mark.gpu


def _phib(shape):
    ny, nx = shape
    yy, xx = np.mgrid[0:ny, 0:nx]
    return (3e-3 * np.sin(np.pi * xx / (nx - 1)) * np.cos(np.pi * yy / (ny - 1)) + 1e-3 * yy / ny).ravel()


@pytest.mark.parametrize('precision', ['fp64', 'split'])
@pytest.mark.parametrize('name', ['noecm_r50_s7', 'ecm_r50_s3'])
def test_boundary_potential_matches_oracle(name, precision):
    from betse_gb300.engine import ClusterEngine
    d = gi.load(name)
    g, p, s = gi.geometry(d), gi.params(d), gi.state(d)
    s.Phi_b = _phib(g.grid_shape)
    s.vm = oracle.init_vm(g, p, s)
    if p.is_ecm:
        oracle.init_fields(g, p, s)
    cg, sp, Dm, st, D_env = gi.engine_inputs(d)
    st = dict(st, vm=s.vm.copy())
    if p.is_ecm:
        st.update(E_env_x=s.E_env_x.copy(), E_env_y=s.E_env_y.copy())
    n = 10
    with ClusterEngine(cg, sp, precision) as e:
        e.set_membrane_diffusivity(Dm)
        if p.is_ecm:
            e.set_env_diffusivity(D_env)
        e.set_boundary_potential(s.Phi_b)
        e.upload(**st)
        e.step(n)
        e.check_stable()
        out = e.download()
    for _ in range(n):
        oracle.step(g, p, s)
    if precision == 'fp64':
        ok, err, bound = gi.vm_err_ok(d, out['vm'], s.vm, s.cc_cells)
        assert ok, (err, bound)
        assert gi.rel_err(out['cc_cells'], s.cc_cells) < 1e-10
    else:
        assert np.max(np.abs(out['vm'] - s.vm)) < 1e-6
        assert gi.rel_err(out['cc_cells'], s.cc_cells) < 1e-6
    # Vmem really differs within cells
    ptr = np.asarray(cg.cell_mem_ptr)
    spread = max(np.ptp(out['vm'][ptr[c]:ptr[c + 1]]) for c in range(len(ptr) - 1))
    assert spread > 1e-4
