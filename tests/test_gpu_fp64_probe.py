"""The FP64 throughput probe (bx_fp64_fma_probe) computes what it claims:
with b = c = 1 every chain adds `iters` to its start, so thread g of the grid
writes sum_j (g + j + iters) = 8 g + 28 + 8 iters, exactly."""
import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_probe_chains_are_exact():
    import torch
    from betse_gb300 import _lib
    from betse_gb300.build import build
    build()
    lib = _lib.load()
    n_blocks, iters = 3, 37
    out = torch.zeros(n_blocks * 256, dtype=torch.float64, device='cuda')
    s = torch.cuda.current_stream()
    assert lib.bx_fp64_fma_probe(n_blocks, iters, 1.0, 1.0, ct.c_void_p(out.data_ptr()),
                                 ct.c_void_p(s.cuda_stream)) == _lib.BX_OK
    torch.cuda.synchronize()
    g = np.arange(n_blocks * 256, dtype=np.float64)
    assert np.array_equal(out.cpu().numpy(), 8 * g + 28 + 8 * iters)
