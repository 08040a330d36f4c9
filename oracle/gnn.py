"""NumPy reference of the warm-start graph network (TEST INFRASTRUCTURE ONLY).

The network the library trains on the GPU (``betse_gb300/csrc/bx_gnn.cu``):
every layer is 64 wide (inputs zero-padded to 64 columns, outputs read from
the first ``n_out`` columns).

    H0 = relu(X W0^T + b0)
    A_l = mean_{j in nbr(i)} H_{l-1,j}                      (0 without neighbours)
    R_l = relu(H_{l-1} Ws_l^T + A_l Wn_l^T + b_l);  H_l = H_{l-1} + R_l,  l = 1..3
    Yhat = H3 Wd^T + bd
    loss = sum over nodes and the first n_out columns of (Yhat - Y)^2 / (N n_out)

With ``bf16=True`` it rounds where the GPU stores BF16 (weights used in the
products; X, H_l, A_l, R_l), so the CUDA kernels can be checked to FP32
accumulation-order differences; with ``bf16=False`` it runs in FP64 and is
checked against finite differences.
"""
from __future__ import annotations

import numpy as np

W = 64
N_MP = 3
# flat parameter layout (floats): W0, b0, (Ws, Wn, b) x 3, Wd, bd
OFF_W0, OFF_B0 = 0, W * W
OFF_MP = OFF_B0 + W
MP_STRIDE = 2 * W * W + W
OFF_WD = OFF_MP + N_MP * MP_STRIDE
OFF_BD = OFF_WD + W * W
N_PARAMS = OFF_BD + W


def bf16_round(x):
    """Round float32 values to the nearest BF16 (ties to even), as float32."""
    x = np.asarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def unpack(p):
    p = np.asarray(p)
    d = {'W0': p[OFF_W0:OFF_W0 + W * W].reshape(W, W), 'b0': p[OFF_B0:OFF_B0 + W],
         'Wd': p[OFF_WD:OFF_WD + W * W].reshape(W, W), 'bd': p[OFF_BD:OFF_BD + W]}
    for l in range(N_MP):
        o = OFF_MP + l * MP_STRIDE
        d[f'Ws{l + 1}'] = p[o:o + W * W].reshape(W, W)
        d[f'Wn{l + 1}'] = p[o + W * W:o + 2 * W * W].reshape(W, W)
        d[f'b{l + 1}'] = p[o + 2 * W * W:o + 2 * W * W + W]
    return d


def _agg(H, ptr, nbr):
    A = np.zeros_like(H)
    deg = np.diff(ptr)
    rows = np.repeat(np.arange(len(deg)), deg)
    np.add.at(A, rows, H[nbr])
    nz = deg > 0
    A[nz] /= deg[nz, None]
    return A


def _aggT(G, ptr, nbr):
    """Adjoint of _agg: out_j = sum over i with j in nbr(i) of G_i / deg_i."""
    deg = np.diff(ptr)
    w = np.zeros(len(deg))
    w[deg > 0] = 1.0 / deg[deg > 0]
    rows = np.repeat(np.arange(len(deg)), deg)
    out = np.zeros_like(G)
    np.add.at(out, nbr, G[rows] * w[rows, None])
    return out


def forward(p, X, ptr, nbr, bf16=True):
    dt = np.float32 if bf16 else np.float64
    r = bf16_round if bf16 else (lambda a: np.asarray(a, np.float64))
    q = {k: r(v) if k.startswith('W') else np.asarray(v, dt) for k, v in unpack(p).items()}
    Xp = np.zeros((X.shape[0], W), dt)
    Xp[:, :X.shape[1]] = X
    Xp = r(Xp)
    c = {'X': Xp, 'q': q}
    H = r(np.maximum(Xp @ q['W0'].T + q['b0'], 0))
    c['H0'] = H
    for l in range(N_MP):
        A = r(_agg(H, ptr, nbr))
        R = r(np.maximum(H @ q[f'Ws{l + 1}'].T + A @ q[f'Wn{l + 1}'].T + q[f'b{l + 1}'], 0))
        c[f'A{l}'], c[f'R{l}'] = A, R
        H = r(H + R)
        c[f'H{l + 1}'] = H
    Y = H @ q['Wd'].T + q['bd']
    return Y, c


def backward(p, c, Yhat, Y, ptr, nbr):
    """Loss and the flat gradient of every parameter."""
    N, n_out = Y.shape
    q = c['q']
    g = np.zeros(N_PARAMS, Yhat.dtype)
    d = np.zeros_like(Yhat)
    d[:, :n_out] = 2.0 * (Yhat[:, :n_out] - Y) / (N * n_out)
    loss = float(np.sum((Yhat[:, :n_out] - Y) ** 2) / (N * n_out))
    H = c[f'H{N_MP}']
    g[OFF_WD:OFF_WD + W * W] = (d.T @ H).ravel()
    g[OFF_BD:OFF_BD + W] = d.sum(0)
    dH = d @ q['Wd']
    for l in reversed(range(N_MP)):
        Hp, A, R = c[f'H{l}'], c[f'A{l}'], c[f'R{l}']
        dZ = dH * (R > 0)
        o = OFF_MP + l * MP_STRIDE
        g[o:o + W * W] = (dZ.T @ Hp).ravel()
        g[o + W * W:o + 2 * W * W] = (dZ.T @ A).ravel()
        g[o + 2 * W * W:o + 2 * W * W + W] = dZ.sum(0)
        dH = dH + dZ @ q[f'Ws{l + 1}'] + _aggT(dZ @ q[f'Wn{l + 1}'], ptr, nbr)
    dZ0 = dH * (c['H0'] > 0)
    g[OFF_W0:OFF_W0 + W * W] = (dZ0.T @ c['X']).ravel()
    g[OFF_B0:OFF_B0 + W] = dZ0.sum(0)
    return loss, g


def init_params(n_in, n_out, seed=0):
    """He-uniform weights on the live rows/columns, zero biases and padding."""
    rng = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, np.float32)
    d = unpack(p)

    def fill(M, fan_in, rows=W, cols=W):
        lim = np.sqrt(6.0 / fan_in)
        M[:rows, :cols] = rng.uniform(-lim, lim, (rows, cols))

    fill(d['W0'], n_in, cols=n_in)
    for l in range(1, N_MP + 1):
        fill(d[f'Ws{l}'], 2 * W)
        d[f'Ws{l}'] *= 0.5
        fill(d[f'Wn{l}'], 2 * W)
        d[f'Wn{l}'] *= 0.5
    fill(d['Wd'], W, rows=n_out)
    d['Wd'] *= 0.1
    return p
