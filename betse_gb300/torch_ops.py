"""The step as PyTorch custom operators: ``torch.ops.bx.*``.

A thin layer over the C ABI (``include/bx.h``, ``libbx.so``): every operator
calls one entry point, so a caller that holds its state in CUDA tensors can
step it without host arrays.  It replaces the same reference interface as the
C ABI -- ``Simulator._run_sim_core_loop`` (``betse/science/sim.py:1132-1390``)
with its state attributes ``vm``, ``cc_cells``, ``cc_at_mem``, ``cc_env``.

A cluster is an opaque integer handle returned by ``bx::cluster_create`` and
released by ``bx::destroy``; the handle carries the device copies of the
cluster, so the operators mutate state that PyTorch does not see (they are
eager operators, not graph-traceable).  State crosses as tensors in BETSE's
layouts: ``vm [M]``, ``cc_cells [I, C]``, ``cc_at_mem [I, M]`` and
``cc_env [I]`` (well mixed) -- CUDA or CPU tensors on upload (copied with
unified addressing), CUDA tensors on download.  ``bx::step`` runs on the
current CUDA stream.  Errors raise ``BxLibraryError``; a NaN state raises
``BetseSimUnstableException`` from ``check_stable(h)`` (check_v,
``sim_toolbox.py:332-344``).

    import betse_gb300.torch_ops  # registers torch.ops.bx.*
    h = betse_gb300.torch_ops.create(geom, params, 'split')
    torch.ops.bx.set_membrane_diffusivity(h, Dm)
    torch.ops.bx.state_upload(h, vm, cc_cells, cc_at_mem, cc_env)
    torch.ops.bx.step(h, 1000, False)
    vm, cc_cells, cc_at_mem, cc_env = torch.ops.bx.state_download(h)
"""
from __future__ import annotations

import ctypes as ct
from typing import List, Optional, Tuple

import numpy as np
import torch

from . import _lib
from .engine import PRECISIONS
from .exceptions import BetseSimUnstableException

Tensor = torch.Tensor


def _f64(t: Tensor) -> Tensor:
    return t.detach().to(torch.float64).contiguous()


def _host(t: Tensor, dtype) -> np.ndarray:
    return np.ascontiguousarray(t.detach().to('cpu', dtype).numpy())


def _p(t: Optional[Tensor]):
    return None if t is None else ct.c_void_p(t.data_ptr())


def _stream() -> ct.c_void_p:
    return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


@torch.library.custom_op('bx::cluster_create', mutates_args=())
def cluster_create(cell_mem_ptr: Tensor, nn_i: Tensor, bflag: Tensor, map_mem2ecm: Tensor, mem_sa: Tensor,
                   mem_nx: Tensor, mem_ny: Tensor, gj_weight: Tensor, smooth_weight_mem: Tensor,
                   smooth_weight_o: Tensor, cell_vol: Tensor, cell_sa: Tensor, diviterm: Tensor,
                   grid_shape: List[int], gj_len: float, delta: float, params: Tensor, precision: int,
                   mem_sa_per_env: Optional[Tensor] = None, R_rads: Optional[Tensor] = None) -> int:
    """bx_cluster_create: the geometry and index maps (BETSE's Cells arrays,
    any device; the library reads them on the host and keeps device copies)
    and the parameters as the bytes of a bx_params (``params_tensor``)."""
    lib = _lib.load()
    keep = dict(ptr=_host(cell_mem_ptr, torch.int32), nn=_host(nn_i, torch.int32),
                bflag=_host(bflag, torch.uint8), mp=_host(map_mem2ecm, torch.int32))
    for k, t in (('sa', mem_sa), ('nx', mem_nx), ('ny', mem_ny), ('gw', gj_weight), ('swm', smooth_weight_mem),
                 ('swo', smooth_weight_o), ('vol', cell_vol), ('csa', cell_sa), ('div', diviterm),
                 ('spe', mem_sa_per_env), ('rr', R_rads)):
        keep[k] = None if t is None else _host(t, torch.float64)
    g = _lib.BxGeom()
    g.n_cells, g.n_mems = len(keep['vol']), len(keep['sa'])
    g.grid_ny, g.grid_nx = int(grid_shape[0]), int(grid_shape[1])
    g.cell_mem_ptr, g.nn_i = _lib.iptr(keep['ptr']), _lib.iptr(keep['nn'])
    g.bflag, g.map_mem2ecm = _lib.u8ptr(keep['bflag']), _lib.iptr(keep['mp'])
    for f, k in (('mem_sa', 'sa'), ('mem_nx', 'nx'), ('mem_ny', 'ny'), ('gj_weight', 'gw'),
                 ('smooth_weight_mem', 'swm'), ('smooth_weight_o', 'swo'), ('cell_vol', 'vol'),
                 ('cell_sa', 'csa'), ('diviterm', 'div'), ('mem_sa_per_env', 'spe'), ('R_rads', 'rr')):
        setattr(g, f, _lib.dptr(keep[k]))
    g.gj_len, g.delta = float(gj_len), float(delta)
    raw = _host(params, torch.uint8).tobytes()
    if len(raw) != ct.sizeof(_lib.BxParams):
        raise ValueError(f'params: expected the {ct.sizeof(_lib.BxParams)} bytes of a bx_params')
    p = _lib.BxParams.from_buffer_copy(raw)
    h = ct.c_void_p()
    _lib.check(lib.bx_cluster_create(ct.byref(g), ct.byref(p), int(precision), ct.byref(h)), 'bx::cluster_create')
    return int(h.value)


@torch.library.custom_op('bx::destroy', mutates_args=())
def destroy(h: int) -> None:
    _lib.load().bx_destroy(ct.c_void_p(h))


@torch.library.custom_op('bx::set_membrane_diffusivity', mutates_args=())
def set_membrane_diffusivity(h: int, Dm: Tensor) -> None:
    """sim.Dm_cells [I, M] (any device)."""
    a = _host(Dm, torch.float64)
    _lib.check(_lib.load().bx_set_membrane_diffusivity(ct.c_void_p(h), _lib.dptr(a)), 'bx::set_membrane_diffusivity')


@torch.library.custom_op('bx::state_upload', mutates_args=())
def state_upload(h: int, vm: Tensor, cc_cells: Tensor, cc_at_mem: Tensor, cc_env: Tensor,
                 gjopen: Optional[Tensor] = None) -> None:
    """The Simulator state in BETSE's layouts, CUDA or CPU float64 tensors.
    Work queued on the current stream is finished first (the copy runs on the
    handle's own stream)."""
    ts = [_f64(t) for t in (vm, cc_cells, cc_at_mem, cc_env)]
    go = None if gjopen is None else _f64(gjopen)
    if any(t.is_cuda for t in ts):
        torch.cuda.current_stream().synchronize()
    s = _lib.BxState()
    s.vm, s.cc_cells, s.cc_at_mem, s.cc_env = (ct.cast(_p(t), _lib._dp) for t in ts)
    s.gjopen = None if go is None else ct.cast(_p(go), _lib._dp)
    _lib.check(_lib.load().bx_state_upload(ct.c_void_p(h), ct.byref(s)), 'bx::state_upload')


@torch.library.custom_op('bx::step', mutates_args=())
def step(h: int, n_steps: int, outputs: bool = False) -> None:
    """bx_step on the current CUDA stream (asynchronous)."""
    _lib.check(_lib.load().bx_step(ct.c_void_p(h), int(n_steps), int(bool(outputs)), _stream()), 'bx::step')


def _info(h: int):
    """(n_clusters, n_cells, n_mems, n_ions, grid_ny, grid_nx, is_ecm, precision)."""
    v = np.zeros(8, np.int32)
    _lib.check(_lib.load().bx_cluster_info(ct.c_void_p(h), _lib.iptr(v)), 'bx_cluster_info')
    return [int(x) for x in v]


@torch.library.custom_op('bx::state_download', mutates_args=())
def state_download(h: int) -> Tuple[Tensor, Tensor, Tensor, Tensor]:
    """(vm [M], cc_cells [I, C], cc_at_mem [I, M], cc_env [I]) as new CUDA
    float64 tensors (a batch handle's cc_env is [clusters * I])."""
    ncl, C, M, I, ny, nx, ecm, _ = _info(h)
    n_env = I * ny * nx if ecm else ncl * I
    dev = torch.device('cuda', torch.cuda.current_device())
    vm = torch.empty(M, dtype=torch.float64, device=dev)
    cc = torch.empty((I, C), dtype=torch.float64, device=dev)
    cam = torch.empty((I, M), dtype=torch.float64, device=dev)
    env = torch.empty(n_env, dtype=torch.float64, device=dev)
    s = _lib.BxState()
    s.vm, s.cc_cells, s.cc_at_mem, s.cc_env = (ct.cast(_p(t), _lib._dp) for t in (vm, cc, cam, env))
    torch.cuda.current_stream().synchronize()
    _lib.check(_lib.load().bx_state_download(ct.c_void_p(h), ct.byref(s)), 'bx::state_download')
    return vm, cc, cam, env


@torch.library.custom_op('bx::status', mutates_args=())
def status(h: int) -> Tensor:
    """int64 [5]: steps done, NaN Vmem count, NaN concentration count,
    clamped negatives (no_negs), unstable flag."""
    st = _lib.BxStepStatus()
    _lib.check(_lib.load().bx_status(ct.c_void_p(h), ct.byref(st)), 'bx::status')
    return torch.tensor([st.steps_done, st.nan_vm, st.nan_conc, st.neg_clamped, st.unstable], dtype=torch.int64)


@torch.library.custom_op('bx::outputs', mutates_args=())
def outputs(h: int) -> List[Tensor]:
    """The last output step's write2storage quantities (sim.py:1789-1884), as
    CUDA float64 tensors in the order of ``_lib.OUTPUT_FIELDS`` (fields a
    configuration does not compute are empty)."""
    ncl, C, M, I, ny, nx, ecm, _ = _info(h)
    G = ny * nx
    sizes = {'fluxes_mem': I * M, 'fluxes_gj': I * M, 'rho_cells': C, 'J_cell_x': C, 'J_cell_y': C,
             'vm_ave': C, 'E_cell_x': C, 'E_cell_y': C, 'sigma_cell': C, 'fluxes_env_x': I * G,
             'fluxes_env_y': I * G, 'rho_env': G, 'v_env': G}
    ecm_only = ('fluxes_env_x', 'fluxes_env_y', 'rho_env', 'v_env')
    dev = torch.device('cuda', torch.cuda.current_device())
    out = []
    o = _lib.BxOutputs()
    for name in _lib.OUTPUT_FIELDS:
        n = sizes.get(name, M) if (name not in ecm_only or ecm) else 0
        t = torch.empty(n, dtype=torch.float64, device=dev)
        out.append(t)
        setattr(o, name, ct.cast(_p(t), _lib._dp) if n else None)
    torch.cuda.current_stream().synchronize()
    _lib.check(_lib.load().bx_outputs_download(ct.c_void_p(h), ct.byref(o)), 'bx::outputs')
    return out


@torch.library.custom_op('bx::env_fields', mutates_args=())
def env_fields(h: int, D_env_weight: Optional[Tensor] = None) -> Tuple[Tensor, Tensor, Tensor, Tensor, Tensor,
                                                                      Tensor]:
    """get_current's environment fields (ion_current.py:50-171) of the last
    output step: (v_env, E_env_x, E_env_y, J_env_x, J_env_y, B_field), each
    [grid] on the GPU; needs ``bx::set_lap_env_inv`` first."""
    _, _, _, _, ny, nx, _, _ = _info(h)
    G = ny * nx
    dev = torch.device('cuda', torch.cuda.current_device())
    outs = [torch.empty(G, dtype=torch.float64, device=dev) for _ in range(6)]
    w = None if D_env_weight is None else _f64(D_env_weight)
    torch.cuda.current_stream().synchronize()
    _lib.check(_lib.load().bx_env_fields(ct.c_void_p(h), None if w is None else ct.cast(_p(w), _lib._dp),
                                         *(ct.cast(_p(t), _lib._dp) for t in outs)), 'bx::env_fields')
    return tuple(outs)


@torch.library.custom_op('bx::set_lap_env_inv', mutates_args=())
def set_lap_env_inv(h: int, lap_env_inv: Tensor) -> None:
    """cells.lapENVinv [grid, grid] (any device; read on the host once)."""
    a = _host(lap_env_inv, torch.float64)
    _lib.check(_lib.load().bx_set_lap_env_inv(ct.c_void_p(h), _lib.dptr(a)), 'bx::set_lap_env_inv')



# ---- molecule / gene regulatory networks (bx_network_*) ----------------------
def _net_info(n: int):
    """(substances, reactions, n_cells, n_mems)."""
    v = np.zeros(4, np.int32)
    _lib.check(_lib.load().bx_network_info(ct.c_void_p(n), _lib.iptr(v)), 'bx_network_info')
    return [int(x) for x in v]


@torch.library.custom_op('bx::network_upload', mutates_args=())
def network_upload(n: int, c_cells: Tensor, cc_at_mem: Tensor, c_env: Tensor) -> None:
    """Molecule.c_cells [S, C], cc_at_mem [S, M], c_env [S] (CUDA or CPU
    float64). Work queued on the current stream is finished first."""
    S, _, C, M = _net_info(n)
    ts = [_f64(c_cells).reshape(S, C), _f64(cc_at_mem).reshape(S, M), _f64(c_env).reshape(S)]
    if any(t.is_cuda for t in ts):
        torch.cuda.current_stream().synchronize()
    _lib.check(_lib.load().bx_network_upload(ct.c_void_p(n), *(_p(t) for t in ts)), 'bx::network_upload')


@torch.library.custom_op('bx::network_step', mutates_args=())
def network_step(n: int, n_steps: int, with_ions: bool = True, outputs: bool = False) -> None:
    """bx_network_step: the ion step then the network (or the network alone),
    on the cluster's stream after the current stream's queued work."""
    torch.cuda.current_stream().synchronize()
    _lib.check(_lib.load().bx_network_step(ct.c_void_p(n), int(n_steps), int(bool(with_ions)), int(bool(outputs))),
               'bx::network_step')


@torch.library.custom_op('bx::network_download', mutates_args=())
def network_download(n: int) -> Tuple[Tensor, Tensor, Tensor]:
    """(c_cells [S, C], cc_at_mem [S, M], c_env [S]) as new CUDA float64 tensors."""
    S, _, C, M = _net_info(n)
    dev = torch.device('cuda', torch.cuda.current_device())
    out = (torch.empty((S, C), dtype=torch.float64, device=dev), torch.empty((S, M), dtype=torch.float64, device=dev),
           torch.empty(S, dtype=torch.float64, device=dev))
    torch.cuda.current_stream().synchronize()
    _lib.check(_lib.load().bx_network_download(ct.c_void_p(n), *(_p(t) for t in out)), 'bx::network_download')
    return out


@torch.library.custom_op('bx::network_status', mutates_args=())
def network_status(n: int) -> Tensor:
    """int64 [1]: negative substance concentrations seen since the upload."""
    v = ct.c_int64()
    _lib.check(_lib.load().bx_network_status(ct.c_void_p(n), ct.byref(v)), 'bx::network_status')
    return torch.tensor([v.value], dtype=torch.int64)


@torch.library.custom_op('bx::network_destroy', mutates_args=())
def network_destroy(n: int) -> None:
    _lib.load().bx_network_destroy(ct.c_void_p(n))


def create_network(h: int, spec, params) -> int:
    """bx_network_create on cluster handle ``h`` (plain FP64) from a
    ``NetworkSpec`` (``betse_gb300.network``) and the cluster's
    ``StepParams`` (R and T give each reaction's equilibrium constant);
    returns the network's integer handle, released by ``bx::network_destroy``."""
    c = spec.to_c(params.R, params.T)
    out = ct.c_void_p()
    _lib.check(_lib.load().bx_network_create(ct.c_void_p(h), ct.byref(c), ct.byref(out)), 'bx_network_create')
    return int(out.value)


def check_network_stable(n: int) -> Tensor:
    """Raise BetseSimUnstableException on a negative substance concentration
    (sim_toolbox.py:1132-1151)."""
    st = torch.ops.bx.network_status(n)
    if int(st[0]):
        raise BetseSimUnstableException('Network concentration below zero! Your simulation has become unstable.')
    return st


def params_tensor(params) -> Tensor:
    """The bytes of a bx_params (from a ``StepParams``) as a uint8 tensor."""
    p = params.to_c()
    return torch.frombuffer(bytearray(bytes(p)), dtype=torch.uint8).clone()


def create(geom, params, precision='split') -> int:
    """bx::cluster_create from a ``ClusterGeometry`` and ``StepParams``."""
    t = lambda a: None if a is None else torch.as_tensor(np.ascontiguousarray(a))  # noqa: E731
    prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    h = torch.ops.bx.cluster_create(
        t(geom.cell_mem_ptr), t(geom.nn_i), t(geom.bflag), t(geom.map_mem2ecm), t(geom.mem_sa), t(geom.mem_nx),
        t(geom.mem_ny), t(geom.gj_weight), t(geom.smooth_weight_mem), t(geom.smooth_weight_o), t(geom.cell_vol),
        t(geom.cell_sa), t(geom.diviterm), list(geom.grid_shape), float(geom.gj_len), float(geom.delta),
        params_tensor(params), prec, t(getattr(geom, 'mem_sa_per_env', None)), t(getattr(geom, 'R_rads', None)))
    return h


def check_stable(h: int) -> Tensor:
    """check_v: raise BetseSimUnstableException if a NaN was seen."""
    st = torch.ops.bx.status(h)
    if int(st[4]):
        raise BetseSimUnstableException('Your simulation has become unstable. Please try a smaller time step,'
                                        'reduce gap junction radius, and/or reduce rate coefficients.')
    return st


def release(h: int) -> None:
    torch.ops.bx.destroy(h)
