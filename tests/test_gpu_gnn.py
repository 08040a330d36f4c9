"""Warm-start network kernels (bx_gnn_*) against the NumPy reference.

The reference (oracle/gnn.py, pinned by finite differences) rounds to BF16
where the GPU stores BF16, so outputs and gradients differ only through FP32
summation order -- and the BF16 rounding flips that order can cause (one BF16
ulp, 2^-8, on a few activations).  Tolerances: outputs 2e-2 of their max and
1e-3 in the mean; each gradient block 5e-2 of its max.
"""
import numpy as np
import pytest

import golden_io as gi
from oracle import gnn as ref

pytestmark = pytest.mark.gpu


def _graph():
    ptrs, nbrs, off = [0], [], 0
    for name in ('noecm_r50_s7', 'noecm_r20_s2'):
        d = gi.load(name)
        p, f = d['geom_cell_nn_ptr'].astype(np.int64), d['geom_cell_nn_flat'].astype(np.int64)
        nbrs.append(f + off)
        ptrs.extend((p[1:] + ptrs[-1]).tolist())
        off += len(p) - 1
    return np.array(ptrs, np.int64), np.concatenate(nbrs), off


def _net(n_in, n_out):
    from betse_gb300.gnn import GraphNet, init_params
    p = init_params(n_in, n_out, seed=4)
    p[ref.OFF_B0:ref.OFF_B0 + 64] = 0.1
    return GraphNet(p), p


def test_forward_and_gradients_match_reference():
    ptr, nbr, n = _graph()
    rng = np.random.default_rng(2)
    n_in, n_out = 11, 5
    X = rng.standard_normal((n, n_in)).astype(np.float32)
    Y = rng.standard_normal((n, n_out)).astype(np.float32)
    net, p = _net(n_in, n_out)
    net.set_graph(ptr, nbr)
    yg = net.forward(X, n_out).cpu().numpy()
    yr, c = ref.forward(p, X, ptr, nbr, bf16=True)
    err = np.abs(yg - yr[:, :n_out])
    assert err.max() < 2e-2 * np.abs(yr).max() and err.mean() < 1e-3 * np.abs(yr).max()
    loss_g, g = net.gradients(X, Y)
    loss_r, gr = ref.backward(p, c, yr, Y, ptr, nbr)
    assert abs(loss_g - loss_r) < 1e-3 * loss_r
    for off, size in ((ref.OFF_W0, 4096), (ref.OFF_B0, 64), (ref.OFF_MP, 4096), (ref.OFF_MP + 4096, 4096),
                      (ref.OFF_MP + 8192, 64), (ref.OFF_MP + 2 * ref.MP_STRIDE + 4096, 4096),
                      (ref.OFF_WD, 4096), (ref.OFF_BD, 64)):
        a, b = g[off:off + size], gr[off:off + size]
        assert np.abs(a - b).max() <= 5e-2 * np.abs(b).max() + 1e-12, (off, np.abs(a - b).max(), np.abs(b).max())
    net.close()


def test_sub_range_equals_cluster_alone():
    ptr, nbr, n = _graph()
    n0 = gi.load('noecm_r50_s7')['geom_cell_nn_ptr'].shape[0] - 1
    rng = np.random.default_rng(3)
    X = rng.standard_normal((n, 11)).astype(np.float32)
    net, _ = _net(11, 5)
    net.set_graph(ptr, nbr)
    full = net.forward(X, 5).cpu().numpy()
    part = net.forward(X[n0:], 5, lo=n0, hi=n).cpu().numpy()
    assert np.array_equal(full[n0:], part)
    from betse_gb300 import _lib
    with pytest.raises(_lib.BxLibraryError):
        net.forward(X[5:], 5, lo=5, hi=n)   # cuts the first cluster
    net.close()


def test_training_reduces_loss():
    import torch
    ptr, nbr, n = _graph()
    rng = np.random.default_rng(4)
    X = rng.standard_normal((n, 11)).astype(np.float32)
    # a target the network can represent: neighbourhood averages of input features
    agg = np.zeros_like(X)
    deg = np.diff(ptr)
    rows = np.repeat(np.arange(n), deg)
    np.add.at(agg, rows, X[nbr])
    agg[deg > 0] /= deg[deg > 0, None]
    Y = np.tanh(agg[:, :5] + 0.5 * X[:, 5:10]).astype(np.float32)
    net, _ = _net(11, 5)
    net.set_graph(ptr, nbr)
    xd, yd = torch.as_tensor(X, device='cuda'), torch.as_tensor(Y, device='cuda')
    losses = [net.train_step(xd, yd, 3e-3) for _ in range(300)]
    assert losses[-1] < 0.2 * losses[0], (losses[0], losses[-1])
    assert np.all(np.isfinite(losses))
    net.close()
