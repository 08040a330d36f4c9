"""The no-allocation step against the handle-based step.

Some callers cannot allocate GPU memory while they step (their device memory
belongs to another framework's pool, or allocation is forbidden where they
run). ``bx_step_fp64_noalloc`` serves them: it steps the caller's own device
buffers and keeps its scratch in a fixed device array inside the library.
This test is the caller: it allocates its buffers with torch, calls the entry
point through the C ABI twice in a row, and compares each result with the
handle-based ``bx_step`` on the same cluster, at the tolerances of the FP64
parity tests. It also checks the refusals (sizes, malformed maps, a
16-cell run over 256 membranes) and that a NaN comes back as BX_EUNSTABLE,
as check_v raises in BETSE. It sits in a file of its own, collected last.
"""
import ctypes as ct

import numpy as np
import pytest

import golden_io as gi

pytestmark = pytest.mark.gpu

TOL = 1e-10


class _Caller:
    """A caller's device copies of one cluster (torch allocates them) and the
    bx_geom / bx_params that point at them."""

    def __init__(self, cg, sp, Dm, st, torch, ptr=None, nn=None):
        from betse_gb300 import _lib
        self.torch = torch
        self.lib = _lib.load()
        dev = torch.device('cuda', 0)
        torch.cuda.set_device(0)

        def t(a, dtype):
            return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device=dev)

        ptr = cg.cell_mem_ptr if ptr is None else ptr
        nn = cg.nn_i if nn is None else nn
        self.keep = dict(ptr=t(ptr, torch.int32), nn=t(nn, torch.int32),
                         bflag=t(cg.bflag, torch.uint8), mp=t(cg.map_mem2ecm, torch.int32),
                         sa=t(cg.mem_sa, torch.float64), nx=t(cg.mem_nx, torch.float64),
                         ny=t(cg.mem_ny, torch.float64), gw=t(cg.gj_weight, torch.float64),
                         swm=t(cg.smooth_weight_mem, torch.float64),
                         swo=t(cg.smooth_weight_o, torch.float64),
                         vol=t(cg.cell_vol, torch.float64), csa=t(cg.cell_sa, torch.float64),
                         div=t(cg.diviterm, torch.float64))
        g = _lib.BxGeom()
        g.n_cells, g.n_mems = cg.n_cells, cg.n_mems
        g.grid_ny, g.grid_nx = cg.grid_shape
        cast = lambda x, T: ct.cast(ct.c_void_p(x.data_ptr()), T)  # noqa: E731
        g.cell_mem_ptr = cast(self.keep['ptr'], _lib._ip)
        g.nn_i = cast(self.keep['nn'], _lib._ip)
        g.bflag = cast(self.keep['bflag'], _lib._u8p)
        g.map_mem2ecm = cast(self.keep['mp'], _lib._ip)
        for f, k in (('mem_sa', 'sa'), ('mem_nx', 'nx'), ('mem_ny', 'ny'), ('gj_weight', 'gw'),
                     ('smooth_weight_mem', 'swm'), ('smooth_weight_o', 'swo'), ('cell_vol', 'vol'),
                     ('cell_sa', 'csa'), ('diviterm', 'div')):
            setattr(g, f, cast(self.keep[k], _lib._dp))
        g.mem_sa_per_env = None
        g.gj_len, g.delta = cg.gj_len, cg.delta
        self.g, self.p = g, sp.to_c()
        first = np.asarray(cg.cell_mem_ptr)[:-1]
        self.Dm = t(Dm, torch.float64)
        self.vm = t(st['vm'], torch.float64)
        self.vm_w = torch.empty_like(self.vm)
        self.cc = t(st['cc_cells'], torch.float64)
        self.ccm = t(st['cc_at_mem'][:, first], torch.float64)
        self.ccm_w = torch.empty_like(self.ccm)
        self.cenv = t(st['cc_env'][:, 0], torch.float64)

    def step(self, n, stream=None):
        return self.lib.bx_step_fp64_noalloc(
            ct.byref(self.g), ct.byref(self.p), self.Dm.data_ptr(), self.vm.data_ptr(),
            self.vm_w.data_ptr(), self.cc.data_ptr(), self.ccm.data_ptr(), self.ccm_w.data_ptr(),
            self.cenv.data_ptr(), n, stream)


def _check_against_handle(caller, ref, ptr, call):
    r = ref.download()
    assert gi.rel_err(caller.vm.cpu().numpy(), r['vm']) < TOL, call
    assert gi.rel_err(caller.cc.cpu().numpy(), r['cc_cells']) < TOL, call
    assert gi.rel_err(caller.ccm.cpu().numpy(), r['cc_at_mem'][:, ptr[:-1]]) < TOL, call
    assert gi.rel_err(caller.cenv.cpu().numpy(), r['cc_env']) < TOL, call


def test_no_alloc_step_matches_handle_step():
    torch = pytest.importorskip('torch')
    from betse_gb300.engine import ClusterEngine
    d = gi.load('noecm_r80_s1')
    cg, sp, Dm, st, _ = gi.engine_inputs(d)
    caller = _Caller(cg, sp, Dm, st, torch)
    ref = ClusterEngine(cg, sp, 'fp64')
    ref.set_membrane_diffusivity(Dm)
    ref.upload(**st)
    n = 25
    for call in range(2):
        rc = caller.step(n)
        assert rc == 0, caller.lib.bx_last_error()
        torch.cuda.synchronize()
        ref.step(n)
        _check_against_handle(caller, ref, np.asarray(cg.cell_mem_ptr), call)
    ref.close()


def test_no_alloc_step_on_a_side_stream():
    """The caller's own (non-default) stream, an even step count (no copy-back)."""
    torch = pytest.importorskip('torch')
    from betse_gb300.engine import ClusterEngine
    d = gi.load('noecm_r50_s7')
    cg, sp, Dm, st, _ = gi.engine_inputs(d)
    caller = _Caller(cg, sp, Dm, st, torch)
    side = torch.cuda.Stream()
    torch.cuda.synchronize()
    rc = caller.step(30, ct.c_void_p(side.cuda_stream))
    assert rc == 0, caller.lib.bx_last_error()
    side.synchronize()
    with ClusterEngine(cg, sp, 'fp64') as ref:
        ref.set_membrane_diffusivity(Dm)
        ref.upload(**st)
        ref.step(30)
        _check_against_handle(caller, ref, np.asarray(cg.cell_mem_ptr), 'side stream')


def test_no_alloc_step_reports_nan_as_unstable():
    """check_v: a NaN in a cell concentration (a poisoned input, not a device
    fault) makes the call return BX_EUNSTABLE."""
    torch = pytest.importorskip('torch')
    from betse_gb300 import _lib
    d = gi.load('noecm_r20_s2')
    cg, sp, Dm, st, _ = gi.engine_inputs(d)
    st = dict(st)
    cc = st['cc_cells'].copy()
    cc[0, 3] = np.nan
    st['cc_cells'] = cc
    caller = _Caller(cg, sp, Dm, st, torch)
    rc = caller.step(2)
    assert rc == _lib.BX_EUNSTABLE, caller.lib.bx_last_error()
    assert b'NaN' in caller.lib.bx_last_error()
    # the next call on clean buffers of another cluster is stable again
    d2 = gi.load('noecm_r80_s1')
    cg2, sp2, Dm2, st2, _ = gi.engine_inputs(d2)
    clean = _Caller(cg2, sp2, Dm2, st2, torch)
    assert clean.step(3) == 0, clean.lib.bx_last_error()


def test_no_alloc_step_rejects_malformed_maps():
    """cell_mem_ptr must end at n_mems and partners must be membranes: checked
    on the device before any step, refused with BX_EINVAL."""
    torch = pytest.importorskip('torch')
    from betse_gb300 import _lib
    d = gi.load('noecm_r20_s2')
    cg, sp, Dm, st, _ = gi.engine_inputs(d)
    ptr = np.asarray(cg.cell_mem_ptr).copy()
    ptr[-1] -= 1                                  # ptr[C] != M
    bad_ptr = _Caller(cg, sp, Dm, st, torch, ptr=ptr)
    vm0 = bad_ptr.vm.clone()
    assert bad_ptr.step(2) == _lib.BX_EINVAL
    assert b'row pointer' in bad_ptr.lib.bx_last_error()
    assert torch.equal(bad_ptr.vm, vm0)           # nothing was stepped
    nn = np.asarray(cg.nn_i).copy()
    nn[5] = cg.n_mems + 7                         # a partner past the last membrane
    bad_nn = _Caller(cg, sp, Dm, st, torch, nn=nn)
    assert bad_nn.step(2) == _lib.BX_EINVAL
    assert b'nn_i' in bad_nn.lib.bx_last_error()


def test_no_alloc_step_rejects_a_crowded_tile():
    """Sixteen consecutive cells of 20 membranes each (320 > 256)."""
    torch = pytest.importorskip('torch')
    from types import SimpleNamespace
    from betse_gb300 import _lib
    d = gi.load('noecm_r20_s2')
    cg0, sp, _, st0, _ = gi.engine_inputs(d)
    C, per = 16, 20
    M = C * per
    m2c = np.repeat(np.arange(C), per)
    cg = SimpleNamespace(n_cells=C, n_mems=M, grid_shape=cg0.grid_shape, gj_len=cg0.gj_len,
                         delta=cg0.delta, cell_mem_ptr=np.arange(0, M + 1, per),
                         nn_i=np.arange(M), bflag=np.ones(M, np.uint8),
                         map_mem2ecm=np.zeros(M, np.int32), mem_sa=np.full(M, 5e-11),
                         mem_nx=np.ones(M), mem_ny=np.zeros(M), gj_weight=np.zeros(M),
                         smooth_weight_mem=np.full(M, 0.5), smooth_weight_o=np.full(M, 0.5),
                         cell_vol=np.full(C, 5e-16), cell_sa=np.full(C, per * 5e-11),
                         diviterm=np.full(C, 5e-16 / (per * 5e-11)))
    I = sp.n_ions
    cc = np.repeat(np.asarray(st0['cc_cells'])[:, :1], C, axis=1)
    st = {'vm': np.zeros(M), 'cc_cells': cc, 'cc_at_mem': cc[:, m2c],
          'cc_env': np.repeat(np.asarray(st0['cc_env'])[:, :1], M, axis=1)}
    caller = _Caller(cg, sp, np.full((I, M), 1e-18), st, torch)
    assert caller.step(1) == _lib.BX_EINVAL
    assert b'256 membranes' in caller.lib.bx_last_error()


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
