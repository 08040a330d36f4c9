"""The no-allocation step against the handle-based step.

Some callers cannot allocate GPU memory while they step (their device memory
belongs to another framework's pool, or allocation is forbidden where they
run). ``bx_step_fp64_noalloc`` serves them: it steps the caller's own device
buffers and keeps its scratch in a fixed device array inside the library.
This test is the caller: it allocates its buffers with torch, calls the entry
point through the C ABI twice in a row, and compares each result with the
handle-based ``bx_step`` on the same cluster, at the tolerances of the FP64
parity tests. It sits in a file of its own, collected last.
"""
import ctypes as ct

import numpy as np
import pytest

import golden_io as gi

pytestmark = pytest.mark.gpu

TOL = 1e-10


def test_no_alloc_step_matches_handle_step():
    torch = pytest.importorskip('torch')
    from betse_gb300 import _lib
    from betse_gb300.engine import ClusterEngine
    lib = _lib.load()
    d = gi.load('noecm_r80_s1')
    cg, sp, Dm, st, _ = gi.engine_inputs(d)
    dev = torch.device('cuda', 0)
    torch.cuda.set_device(0)

    def t(a, dtype):
        return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device=dev)

    keep = dict(ptr=t(cg.cell_mem_ptr, torch.int32), nn=t(cg.nn_i, torch.int32),
                bflag=t(cg.bflag, torch.uint8), mp=t(cg.map_mem2ecm, torch.int32),
                sa=t(cg.mem_sa, torch.float64), nx=t(cg.mem_nx, torch.float64),
                ny=t(cg.mem_ny, torch.float64), gw=t(cg.gj_weight, torch.float64),
                swm=t(cg.smooth_weight_mem, torch.float64), swo=t(cg.smooth_weight_o, torch.float64),
                vol=t(cg.cell_vol, torch.float64), csa=t(cg.cell_sa, torch.float64),
                div=t(cg.diviterm, torch.float64))
    g = _lib.BxGeom()
    g.n_cells, g.n_mems = cg.n_cells, cg.n_mems
    g.grid_ny, g.grid_nx = cg.grid_shape
    cast = lambda x, T: ct.cast(ct.c_void_p(x.data_ptr()), T)  # noqa: E731
    g.cell_mem_ptr = cast(keep['ptr'], _lib._ip)
    g.nn_i = cast(keep['nn'], _lib._ip)
    g.bflag = cast(keep['bflag'], _lib._u8p)
    g.map_mem2ecm = cast(keep['mp'], _lib._ip)
    for f, k in (('mem_sa', 'sa'), ('mem_nx', 'nx'), ('mem_ny', 'ny'), ('gj_weight', 'gw'),
                 ('smooth_weight_mem', 'swm'), ('smooth_weight_o', 'swo'), ('cell_vol', 'vol'),
                 ('cell_sa', 'csa'), ('diviterm', 'div')):
        setattr(g, f, cast(keep[k], _lib._dp))
    g.mem_sa_per_env = None
    g.gj_len, g.delta = cg.gj_len, cg.delta
    p = sp.to_c()
    I, C, M = sp.n_ions, cg.n_cells, cg.n_mems
    ptr = cg.cell_mem_ptr
    Dm_d = t(Dm, torch.float64)
    vm = t(st['vm'], torch.float64)
    vm_w = torch.empty_like(vm)
    cc = t(st['cc_cells'], torch.float64)
    ccm = t(st['cc_at_mem'][:, ptr[:-1]], torch.float64)
    ccm_w = torch.empty_like(ccm)
    cenv = t(st['cc_env'][:, 0], torch.float64)

    ref = ClusterEngine(cg, sp, 'fp64')
    ref.set_membrane_diffusivity(Dm)
    ref.upload(**st)
    n = 25
    for call in range(2):
        rc = lib.bx_step_fp64_noalloc(ct.byref(g), ct.byref(p), Dm_d.data_ptr(), vm.data_ptr(),
                                      vm_w.data_ptr(), cc.data_ptr(), ccm.data_ptr(),
                                      ccm_w.data_ptr(), cenv.data_ptr(), n, None)
        assert rc == 0, lib.bx_last_error()
        torch.cuda.synchronize()
        ref.step(n)
        r = ref.download()
        assert gi.rel_err(vm.cpu().numpy(), r['vm']) < TOL, call
        assert gi.rel_err(cc.cpu().numpy(), r['cc_cells']) < TOL, call
        assert gi.rel_err(ccm.cpu().numpy(), r['cc_at_mem'][:, ptr[:-1]]) < TOL, call
        assert gi.rel_err(cenv.cpu().numpy(), r['cc_env']) < TOL, call
    ref.close()


def test_no_alloc_step_rejects_oversize():
    from betse_gb300 import _lib
    lib = _lib.load()
    g = _lib.BxGeom()
    g.n_cells, g.n_mems = 20000, 120000
    p = _lib.BxParams()
    p.n_ions, p.iNa, p.iK = 6, 0, 1
    one = ct.c_void_p(1)
    rc = lib.bx_step_fp64_noalloc(ct.byref(g), ct.byref(p), one, one, one, one, one, one, one, 1, None)
    assert rc == _lib.BX_EINVAL
    assert b'16384' in lib.bx_last_error()
