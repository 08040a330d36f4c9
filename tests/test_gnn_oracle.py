"""The NumPy reference of the warm-start network, pinned by finite differences."""
import numpy as np

from oracle import gnn


def _graph(n, rng):
    # random symmetric graph with a few isolated nodes
    pairs = set()
    for i in range(n):
        for j in rng.choice(n, size=3, replace=False):
            if i != j and i % 11 != 5 and j % 11 != 5:
                pairs.add((i, j))
                pairs.add((j, i))
    nb = [[] for _ in range(n)]
    for i, j in sorted(pairs):
        nb[i].append(j)
    ptr = np.concatenate([[0], np.cumsum([len(x) for x in nb])]).astype(np.int64)
    return ptr, np.array([j for x in nb for j in x], np.int64)


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    n, n_in, n_out = 40, 9, 5
    ptr, nbr = _graph(n, rng)
    p = gnn.init_params(n_in, n_out, seed=1).astype(np.float64)
    p[gnn.OFF_B0:gnn.OFF_B0 + 64] = 0.05  # keep units away from the relu kink
    X = rng.standard_normal((n, n_in))
    Y = rng.standard_normal((n, n_out))
    Yh, c = gnn.forward(p, X, ptr, nbr, bf16=False)
    loss, g = gnn.backward(p, c, Yh, Y, ptr, nbr)
    idx = np.concatenate([rng.choice(np.arange(o, o + 64 * 64), 12, replace=False)
                          for o in (gnn.OFF_W0, gnn.OFF_MP, gnn.OFF_MP + 4096,
                                    gnn.OFF_MP + 2 * gnn.MP_STRIDE, gnn.OFF_WD)])
    idx = np.concatenate([idx, [gnn.OFF_B0 + 3, gnn.OFF_BD + 1, gnn.OFF_MP + 8192 + 7]])
    def loss_at(q):
        Yq, cq = gnn.forward(q, X, ptr, nbr, bf16=False)
        return gnn.backward(q, cq, Yq, Y, ptr, nbr)[0]

    h = 1e-6
    for k in idx:
        e = np.zeros_like(p)
        e[k] = h
        fd = (loss_at(p + e) - loss_at(p - e)) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9, (k, fd, g[k])


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 1e-30], np.float32)
    r = gnn.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0            # tie to even (mantissa 0)
    assert r[2] == np.float32(1.0 + 2 ** -6)       # tie rounds up to even
    assert r[3] == -2.5
    assert abs(r[4] - 1e-30) < 1e-32
