"""The warm-start graph network on the GPU (``bx_gnn_*`` in libbx.so).

``GraphNet`` owns the network's parameters (FP32 master weights with BF16
copies) and the cell-adjacency graph of the clusters it runs on.  Inputs and
targets are FP32 arrays ``[nodes, n_in]`` / ``[nodes, n_out]`` (PyTorch CUDA
tensors or NumPy, copied to the GPU); every call acts on a node range
``[lo, hi)`` holding whole clusters.  The layout of the flat parameter vector
is given by the ``OFF_*`` constants below.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib

WIDTH = 64
N_LAYERS = 3
OFF_W0, OFF_B0 = 0, WIDTH * WIDTH
OFF_MP = OFF_B0 + WIDTH
MP_STRIDE = 2 * WIDTH * WIDTH + WIDTH
OFF_WD = OFF_MP + N_LAYERS * MP_STRIDE
OFF_BD = OFF_WD + WIDTH * WIDTH
N_PARAMS = OFF_BD + WIDTH


def init_params(n_in, n_out, seed=0):
    """He-uniform weights on the used rows/columns; biases and padding zero.
    The message-passing matrices are halved (two summed inputs) and the decoder
    scaled by 0.1 so the untrained network predicts close to the targets' mean."""
    rng = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, np.float32)
    W = WIDTH

    def block(off, fan_in, rows=W, cols=W, scale=1.0):
        lim = np.sqrt(6.0 / fan_in)
        m = p[off:off + W * W].reshape(W, W)
        m[:rows, :cols] = scale * rng.uniform(-lim, lim, (rows, cols))

    block(OFF_W0, n_in, cols=n_in)
    for l in range(N_LAYERS):
        o = OFF_MP + l * MP_STRIDE
        block(o, 2 * W, scale=0.5)
        block(o + W * W, 2 * W, scale=0.5)
    block(OFF_WD, W, rows=n_out, scale=0.1)
    return p


def _dev(a):
    import torch
    if isinstance(a, torch.Tensor):
        return a.to(device='cuda', dtype=torch.float32).contiguous()
    return torch.as_tensor(np.ascontiguousarray(a, np.float32), device='cuda')


class GraphNet:
    def __init__(self, params=None, n_in=None, n_out=None, seed=0):
        self.lib = _lib.load()
        if int(self.lib.bx_gnn_n_params()) != N_PARAMS:
            raise RuntimeError('parameter layout of libbx.so differs from this module')
        h = ct.c_void_p()
        _lib.check(self.lib.bx_gnn_create(ct.byref(h)), 'bx_gnn_create')
        self.h = h
        if params is None:
            params = init_params(n_in, n_out, seed)
        self.set_params(params)
        self.n_nodes = 0

    def set_params(self, params):
        p = np.ascontiguousarray(params, np.float32)
        if p.shape != (N_PARAMS,):
            raise ValueError(f'expected {N_PARAMS} parameters')
        _lib.check(self.lib.bx_gnn_set_params(self.h, p.ctypes.data_as(_lib._fp)), 'bx_gnn_set_params')

    def params(self):
        p = np.empty(N_PARAMS, np.float32)
        _lib.check(self.lib.bx_gnn_get_params(self.h, p.ctypes.data_as(_lib._fp)), 'bx_gnn_get_params')
        return p

    def set_graph(self, ptr, nbr):
        ptr = np.ascontiguousarray(ptr, np.int32)
        nbr = np.ascontiguousarray(nbr, np.int32)
        n = len(ptr) - 1
        _lib.check(self.lib.bx_gnn_set_graph(self.h, n, _lib.iptr(ptr), _lib.iptr(nbr)), 'bx_gnn_set_graph')
        self.n_nodes = n

    def forward(self, x, n_out, lo=0, hi=None):
        import torch
        hi = self.n_nodes if hi is None else hi
        xd = _dev(x)
        y = torch.empty((hi - lo, n_out), dtype=torch.float32, device='cuda')
        torch.cuda.synchronize()
        _lib.check(self.lib.bx_gnn_forward(self.h, int(lo), int(hi), ct.c_void_p(xd.data_ptr()), xd.shape[1],
                                           ct.c_void_p(y.data_ptr()), int(n_out)), 'bx_gnn_forward')
        return y

    def gradients(self, x, y, lo=0, hi=None):
        hi = self.n_nodes if hi is None else hi
        xd, yd = _dev(x), _dev(y)
        g = np.empty(N_PARAMS, np.float32)
        loss = ct.c_float()
        import torch
        torch.cuda.synchronize()
        _lib.check(self.lib.bx_gnn_gradients(self.h, int(lo), int(hi), ct.c_void_p(xd.data_ptr()), xd.shape[1],
                                             ct.c_void_p(yd.data_ptr()), yd.shape[1],
                                             g.ctypes.data_as(_lib._fp), ct.byref(loss)), 'bx_gnn_gradients')
        return float(loss.value), g

    def train_step(self, x, y, lr, lo=0, hi=None):
        """One Adam step on nodes [lo, hi); x, y device tensors of those rows."""
        hi = self.n_nodes if hi is None else hi
        loss = ct.c_float()
        import torch
        torch.cuda.current_stream().synchronize()  # inputs written on PyTorch's stream
        _lib.check(self.lib.bx_gnn_train_step(self.h, int(lo), int(hi), ct.c_void_p(x.data_ptr()), x.shape[1],
                                              ct.c_void_p(y.data_ptr()), y.shape[1], float(lr),
                                              ct.byref(loss)), 'bx_gnn_train_step')
        return float(loss.value)

    def close(self):
        if getattr(self, 'h', None) is not None and self.h.value:
            self.lib.bx_gnn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
