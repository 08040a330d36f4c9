"""The PyTorch operator boundary (torch.ops.bx.*) registers with the schemas
callers bind to; no GPU needed (the GPU test steps a cluster through them)."""
import pytest

torch = pytest.importorskip('torch')


def test_bx_ops_are_registered():
    import betse_gb300.torch_ops  # noqa: F401
    names = ['cluster_create', 'destroy', 'set_membrane_diffusivity', 'state_upload', 'step', 'state_download',
             'status', 'outputs', 'env_fields', 'set_lap_env_inv']
    for n in names:
        op = getattr(torch.ops.bx, n)
        assert op.default._schema.name == f'bx::{n}'
    s = str(torch.ops.bx.step.default._schema)
    assert 'n_steps' in s and 'outputs' in s
    s = str(torch.ops.bx.state_download.default._schema)
    assert s.endswith('(Tensor, Tensor, Tensor, Tensor)')


def test_params_tensor_round_trips_the_c_struct():
    import ctypes as ct
    from betse_gb300 import _lib
    from betse_gb300.torch_ops import params_tensor
    import golden_io as gi
    _, sp, _, _, _ = gi.engine_inputs(gi.load('noecm_r20_s2'))
    t = params_tensor(sp)
    assert t.dtype == torch.uint8 and t.numel() == ct.sizeof(_lib.BxParams)
    back = _lib.BxParams.from_buffer_copy(bytes(t.numpy()))
    assert back.n_ions == sp.n_ions and back.dt == sp.dt and back.F == sp.F
