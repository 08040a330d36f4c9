"""A cluster stepped through the PyTorch operators (torch.ops.bx.*, state in
CUDA tensors) gives the state and outputs of the ctypes engine on the same
handle calls, bit for bit (the operators are a thin layer over the C ABI)."""
import numpy as np
import pytest

import golden_io as gi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('precision', ['fp64', 'split'])
def test_torch_ops_step_equals_engine(precision):
    import torch
    import betse_gb300.torch_ops as tops
    from betse_gb300.engine import ClusterEngine
    d = gi.load('noecm_r80_s1')
    cg, sp, Dm, st, _ = gi.engine_inputs(d)
    dev = torch.device('cuda', 0)
    torch.cuda.set_device(0)
    h = tops.create(cg, sp, precision)
    try:
        torch.ops.bx.set_membrane_diffusivity(h, torch.as_tensor(Dm, device=dev))
        cuda = {k: torch.as_tensor(np.ascontiguousarray(v), device=dev) for k, v in st.items()}
        env = cuda['cc_env'][:, 0].contiguous()
        torch.ops.bx.state_upload(h, cuda['vm'], cuda['cc_cells'], cuda['cc_at_mem'], env)
        torch.ops.bx.step(h, 70, False)
        torch.ops.bx.step(h, 5, True)
        vm, cc, cam, cenv = torch.ops.bx.state_download(h)
        assert vm.is_cuda and cc.shape == (sp.n_ions, cg.n_cells)
        outs = torch.ops.bx.outputs(h)
        status = tops.check_stable(h)
        assert int(status[0]) == 75
    finally:
        tops.release(h)
    with ClusterEngine(cg, sp, precision) as e:
        e.set_membrane_diffusivity(Dm)
        e.upload(**st)
        e.step(70)
        e.step(5, outputs=True)
        ref = e.download()
        ref_out = e.outputs()
    assert np.array_equal(vm.cpu().numpy(), ref['vm'])
    assert np.array_equal(cc.cpu().numpy(), ref['cc_cells'])
    assert np.array_equal(cam.cpu().numpy(), ref['cc_at_mem'])
    assert np.array_equal(cenv.cpu().numpy(), ref['cc_env'])
    from betse_gb300 import _lib
    for name, t in zip(_lib.OUTPUT_FIELDS, outs):
        if name in ref_out and t.numel():
            assert np.array_equal(t.cpu().numpy().reshape(ref_out[name].shape), ref_out[name]), name


def test_torch_ops_report_nan_as_unstable():
    import torch
    import betse_gb300.torch_ops as tops
    from betse_gb300.exceptions import BetseSimUnstableException
    d = gi.load('noecm_r20_s2')
    cg, sp, Dm, st, _ = gi.engine_inputs(d)
    h = tops.create(cg, sp, 'split')
    try:
        torch.ops.bx.set_membrane_diffusivity(h, torch.as_tensor(Dm))
        cc = torch.as_tensor(st['cc_cells']).clone()
        cc[0, 3] = float('nan')              # a poisoned input, not a device fault
        torch.ops.bx.state_upload(h, torch.as_tensor(st['vm']), cc, torch.as_tensor(st['cc_at_mem']),
                                  torch.as_tensor(st['cc_env'][:, 0]))
        torch.ops.bx.step(h, 2, False)
        with pytest.raises(BetseSimUnstableException):
            tops.check_stable(h)
    finally:
        tops.release(h)


def test_torch_ops_network_equals_engine():
    """The molecule network through torch.ops.bx.network_* (state in CUDA
    tensors) gives the ctypes Network's state bit for bit."""
    import torch
    import betse_gb300.torch_ops as tops
    from betse_gb300.engine import ClusterEngine
    from betse_gb300.network import Network, NetworkSpec
    from test_oracle_network import network_inputs
    d = gi.load('net_r50_s21')
    cfg, names, targets, mods = network_inputs(d)
    cg, sp, Dm, st, _ = gi.engine_inputs(d)
    g = gi.geometry(d)
    spec = NetworkSpec.from_config(cfg['substances'], cfg['reactions'], cfg['time_dilation'],
                                   n_cells=len(g.cell_vol), profiles={'spot': targets['B']},
                                   growth_mod={'A': mods['A']}, ion_names=[str(x) for x in d['par_ion_names']],
                                   mem_vol=d['net_mem_vol'], R_rads=g.R_rads)
    dev = torch.device('cuda', 0)
    torch.cuda.set_device(0)
    h = tops.create(cg, sp, 'fp64')
    try:
        torch.ops.bx.set_membrane_diffusivity(h, torch.as_tensor(Dm, device=dev))
        cuda = {k: torch.as_tensor(np.ascontiguousarray(v), device=dev) for k, v in st.items()}
        torch.ops.bx.state_upload(h, cuda['vm'], cuda['cc_cells'], cuda['cc_at_mem'], cuda['cc_env'][:, 0].contiguous())
        n = tops.create_network(h, spec, sp)
        try:
            torch.ops.bx.network_upload(n, torch.as_tensor(d['init_net_c_cells'], device=dev),
                                        torch.as_tensor(d['init_net_cc_at_mem'], device=dev),
                                        torch.as_tensor(d['init_net_c_env'][:, 0], device=dev))
            torch.ops.bx.network_step(n, 50, True, False)
            tops.check_network_stable(n)
            cc, cm, ce = torch.ops.bx.network_download(n)
        finally:
            torch.ops.bx.network_destroy(n)
    finally:
        tops.release(h)
    with ClusterEngine(cg, sp, 'fp64') as e:
        e.set_membrane_diffusivity(Dm)
        e.upload(**st)
        with Network(e, spec) as net:
            net.upload(d['init_net_c_cells'], d['init_net_cc_at_mem'], d['init_net_c_env'])
            net.step(50, with_ions=True)
            ref = net.download()
    assert np.array_equal(cc.cpu().numpy(), ref['c_cells'])
    assert np.array_equal(cm.cpu().numpy(), ref['cc_at_mem'])
    assert np.array_equal(ce.cpu().numpy(), ref['c_env'])
