"""Learned warm start of BETSE's init phase.

BETSE's init phase (``Simulator.run_sim_core`` with ``SimPhaseKind.INIT``,
``betse/science/sim.py:1016-1128``) starts every cell at the same
concentrations and steps until the cluster settles.  Here a graph network
(``gnn.GraphNet``, trained by ``train``) predicts each cell's steady-state
Na, K, Cl, Ca and Vmem from its channel diffusivities, pump rate and
gap-junction conductance; ``warm_state`` turns the prediction into a
consistent state -- the charge-balancing anion M set so that the charge sum
gives the predicted Vmem exactly, the well-mixed environment adjusted so that
every ion's total amount equals the initial one -- and the ordinary time
stepping runs from there until its own residual test passes (max |dVm/dt| below
a tolerance, ``sim.dvm``, sim.py:2083).  The network only chooses the starting
point; the time stepping alone decides when the cluster has settled.

``python -m betse_gb300.warmstart train --out FILE`` generates the training
steady states with the GPU step itself (the split form on batches of
clusters) and trains the network on the GPU; ``evaluate`` measures the
init time-to-steady with and without the warm start.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import generator as gen
from .engine import BatchEngine
from .gnn import GraphNet

ION_NAMES = gen.ION_NAMES
TARGET_IONS = ('Na', 'K', 'Cl', 'Ca', 'M')   # the mobile ions (P has Dm = 0)
N_OUT = len(TARGET_IONS) + 1            # + Vmem
LOG_CLIP = 10.0                         # |log(c / c_init)| bound of the targets
FALLBACK_BLEND = 0.8                    # damping of the prediction after an unstable warm start
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'data', 'warmstart_gnn.npz')
DT = 1e-2
# per-cluster multipliers of the Na/K diffusivities and of the pump rate; Na/K
# above ~3x makes BETSE's explicit step diverge at dt = 1e-2 s with Dm up to 1e-17
MULT_RANGE = (0.1, 3.0)
PUMP_RANGE = (0.1, 10.0)


# ---------------------------------------------------------------------------
# features and targets
# ---------------------------------------------------------------------------
def cell_features(g, p, Dm):
    """Per-cell inputs [C, 10]: log10 of the membrane-mean Dm of Na, K, Cl, Ca, M;
    log10 of the pump rate; mean gap-junction weight; boundary-membrane
    fraction; membrane count; log10 of vol/area (diviterm)."""
    ptr = np.asarray(g.cell_mem_ptr)
    starts = ptr[:-1]
    cnt = np.diff(ptr).astype(np.float64)
    feats = []
    for ion in ('Na', 'K', 'Cl', 'Ca', 'M'):
        d = np.add.reduceat(Dm[ION_NAMES.index(ion)], starts) / cnt
        feats.append(np.log10(np.maximum(d, 1e-30)))
    feats.append(np.full(len(cnt), np.log10(p.alpha_NaK)))
    bflag = np.asarray(g.bflag).astype(np.float64)
    gw = np.asarray(g.gj_weight) * (1.0 - bflag)
    feats.append(np.add.reduceat(gw, starts) / cnt)
    feats.append(np.add.reduceat(bflag, starts) / cnt)
    feats.append(cnt)
    feats.append(np.log10(np.asarray(g.diviterm)))
    return np.stack(feats, axis=1)


def _cell_vm(g, vm):
    return np.asarray(vm)[np.asarray(g.cell_mem_ptr)[:-1]]


def cell_targets(g, st, st0):
    """[C, 6]: log(c / c_init) of Na, K, Cl, Ca, M and Vmem (V) of state st."""
    cc, cc0 = np.asarray(st['cc_cells']), np.asarray(st0['cc_cells'])
    cols = [np.clip(np.log(np.maximum(cc[ION_NAMES.index(n)], 1e-300) / cc0[ION_NAMES.index(n)]),
                    -LOG_CLIP, LOG_CLIP) for n in TARGET_IONS]
    cols.append(_cell_vm(g, st['vm']))
    return np.stack(cols, axis=1)


def warm_state(g, p, st0, pred):
    """A consistent state from predicted targets pred [C, 6] (``cell_targets``
    units), or None when the prediction is unusable (the caller then starts
    that cluster cold).

    The predicted concentrations do not in general carry exactly the charge of
    the predicted Vmem (Vmem is a small difference of large charges,
    sim.py:2027-2029), so the charge difference dq is spread over the mobile
    ions as c_i <- c_i (1 + a z_i) with a = dq / (F sum z_i^2 c_i): the same
    relative change for every ion, signed by its charge.  P is unchanged; the
    well-mixed environment keeps each ion's total amount (cells plus
    environment) equal to st0's."""
    cc0 = np.asarray(st0['cc_cells'], np.float64)
    cc = cc0.copy()
    mob = [ION_NAMES.index(n) for n in TARGET_IONS]
    for k, i in enumerate(mob):
        cc[i] = cc0[i] * np.exp(pred[:, k])
    V = pred[:, len(TARGET_IONS)]
    zs = np.asarray(p.zs, np.float64)
    rho_target = p.cm * V / np.asarray(g.diviterm)
    dq = rho_target - (zs * p.F) @ cc
    zm = zs[mob][:, None]
    a = dq / (p.F * np.sum(zm ** 2 * cc[mob], axis=0))
    cc[mob] = cc[mob] * (1.0 + a[None, :] * zm)
    if not (np.all(np.isfinite(cc)) and np.all(cc[mob] > 0) and np.all(np.abs(a) < 0.5)
            and np.all(np.abs(V) < 0.5)):
        return None
    rho = (zs * p.F) @ cc
    m2c = np.asarray(g.mem_to_cells)
    vm = (1.0 / p.cm) * (rho * np.asarray(g.diviterm))[m2c]
    # no-ECM environment: d(env) = -(moles into cells) / (n_mems * vol_env)
    moved = (cc - cc0) @ np.asarray(g.cell_vol)
    env = np.asarray(st0['cc_env'], np.float64) - moved / (g.n_mems * p.vol_env)
    if not np.all(env > 0):
        return None
    return dict(vm=vm, cc_cells=cc, cc_at_mem=cc[:, m2c].copy(), cc_env=env)


def warm_states(geoms, params, states0, pred, y0, blend=1.0):
    """warm_state for each cluster with y = y0 + blend (pred - y0); clusters
    whose prediction gives no usable state keep states0.  Returns (states,
    fallback flags)."""
    out, fb = [], []
    for g, p, s, y, a in zip(geoms, params, states0, pred, y0):
        w = warm_state(g, p, s, a + blend * (y - a))
        fb.append(w is None)
        out.append(s if w is None else w)
    return out, np.array(fb)


def graph_of(geoms):
    """Concatenated cell adjacency (CSR, global node ids) of a list of clusters."""
    ptrs, nbrs, off = [np.zeros(1, np.int64)], [], 0
    for g in geoms:
        p = np.asarray(g.cell_nn_ptr, np.int64)
        nbrs.append(np.asarray(g.cell_nn, np.int64) + off)
        ptrs.append(p[1:] + ptrs[-1][-1])
        off += len(p) - 1
    return np.concatenate(ptrs), np.concatenate(nbrs) if nbrs else np.zeros(0, np.int64)


# ---------------------------------------------------------------------------
# stepping to steady state
# ---------------------------------------------------------------------------
def run_to_steady(geoms, params, Dms, states, tol=1e-6, chunk=1000, max_steps=400_000, precision='split',
                  restart_states=(), compact=True, autotune=True):
    """Step a batch of clusters until every cluster's max |dVm/dt| < tol.

    Returns (final states, steps at which each cluster first passed -- -1 if
    never, -2 if it went unstable (NaN) --, wall s of the stepping, restarts
    per cluster).  Clusters are checked every ``chunk`` steps on the device
    (``bx_max_abs_dvm``); an unstable cluster does not affect the others
    (clusters share no data).  ``restart_states`` is a sequence of fallback
    state lists: a cluster that goes unstable restarts from the next one in
    turn, and its count of steps keeps running (steps before a restart count
    against it).  With ``compact``, once half of the clusters still stepping
    have passed (or given up), the batch is rebuilt from the others, so the
    last slow clusters do not carry the finished ones; a retired cluster's
    final state is the one it had when it left the batch."""
    import torch
    n = len(geoms)
    passed = np.full(n, -1, np.int64)
    level = np.zeros(n, np.int64)
    final = [None] * n

    def make(idx, sts):
        e = BatchEngine([geoms[i] for i in idx], [params[i] for i in idx], precision)
        e.set_membrane_diffusivity([Dms[i] for i in idx])
        e.upload_states(sts)
        if autotune:
            e.autotune(64)          # the kernel and tile size for this batch; the state is kept
        return e

    active = np.arange(n)
    eng = make(active, list(states))
    done = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    while done < max_steps:
        eng.step(chunk, outputs=True)
        done += chunk
        worst = eng.max_abs_dvm()                      # per cluster of the engine
        nonfinite = ~np.isfinite(worst)
        bad = (passed[active] == -1) & nonfinite
        fresh = bad & (level[active] < len(restart_states))
        passed[active[bad & ~fresh]] = -2
        if np.any(fresh):
            cur = eng.download_states()
            for j in np.nonzero(nonfinite)[0]:
                g = active[j]
                if fresh[j]:
                    cur[j] = restart_states[level[g]][g]
                    level[g] += 1
                else:   # given up or already recorded: any finite state keeps the upload valid
                    cur[j] = (restart_states[-1] if restart_states else states)[g]
            eng.upload_states(cur)
        newly = (passed[active] == -1) & (worst < tol)
        passed[active[newly]] = done
        still = np.nonzero(passed[active] == -1)[0]
        if len(still) == 0:
            break
        if compact and len(active) > 1 and len(still) <= len(active) // 2:
            cur = eng.download_states()
            for j, g in enumerate(active):
                final[g] = cur[j]
            eng.close()
            active = active[still]
            eng = make(active, [cur[j] for j in still])
    wall = time.perf_counter() - t0
    cur = eng.download_states()
    for j, g in enumerate(active):
        final[g] = cur[j]
    eng.close()
    return final, passed, wall, level


# ---------------------------------------------------------------------------
# training
# ---------------------------------------------------------------------------
def make_dataset(n_clusters, seed, cells_range=(500, 2000), batch=512, tol=3e-7, max_steps=1_200_000, log=print):
    """Features and steady-state targets of n_clusters fresh clusters.  Each
    batch steps (split form) until every cluster's residual is below tol or
    max_steps ran; clusters that went unstable are dropped."""
    X, Y, geoms_all = [], [], []
    for b0 in range(0, n_clusters, batch):
        nb = min(batch, n_clusters - b0)
        t = time.perf_counter()
        gs, ps, Dms, sts = gen.sweep_workload(nb, seed + 7919 * (b0 // batch + 1), cells_range=cells_range,
                                              dt=DT, dm_range=(1e-19, 1e-17), mult_range=MULT_RANGE,
                                              pump_range=PUMP_RANGE)
        t_gen = time.perf_counter() - t
        fin, passed, wall, _ = run_to_steady(gs, ps, Dms, sts, tol=tol, chunk=2000, max_steps=max_steps)
        keep = passed != -2
        ok = passed[passed >= 0]
        for k in np.nonzero(keep)[0]:
            X.append(cell_features(gs[k], ps[k], Dms[k]))
            Y.append(cell_targets(gs[k], fin[k], sts[k]))
            geoms_all.append(gs[k])
        log(f'batch {b0 // batch}: {nb} clusters, generated in {t_gen:.1f} s, stepped {wall:.1f} s; '
            f'{len(ok)} passed {tol:g} V/s (steps median {np.median(ok) if len(ok) else -1:.0f}), '
            f'{int(np.sum(passed == -1))} capped at {max_steps}, {int(np.sum(passed == -2))} unstable')
    return X, Y, geoms_all


def train(out, n_clusters=2048, seed=101, epochs=60, lr=2e-3, clusters_per_step=32, max_steps=1_200_000,
          log=print):
    import torch
    t_all = time.perf_counter()
    X, Y, geoms = make_dataset(n_clusters, seed, max_steps=max_steps, log=log)
    n_val = max(1, len(X) // 20)
    Xc, Yc = np.concatenate(X), np.concatenate(Y)
    x_mean, x_std = Xc.mean(0), Xc.std(0) + 1e-6
    y_mean, y_std = Yc.mean(0), Yc.std(0) + 1e-12
    sizes = np.array([len(x) for x in X])
    offs = np.concatenate([[0], np.cumsum(sizes)])
    ptr, nbr = graph_of(geoms)
    xd = torch.as_tensor(((Xc - x_mean) / x_std).astype(np.float32), device='cuda')
    yd = torch.as_tensor(((Yc - y_mean) / y_std).astype(np.float32), device='cuda')
    net = GraphNet(n_in=Xc.shape[1], n_out=N_OUT, seed=seed)
    net.set_graph(ptr, nbr)
    n_tr = len(X) - n_val
    rng = np.random.default_rng(seed)
    steps_per_epoch = max(1, n_tr // clusters_per_step)
    total = epochs * steps_per_epoch
    it = 0
    t0 = time.perf_counter()
    for ep in range(epochs):
        order = rng.permutation(n_tr // clusters_per_step) if n_tr >= clusters_per_step else np.zeros(1, int)
        tl = []
        for s in order:
            c0, c1 = s * clusters_per_step, min(n_tr, (s + 1) * clusters_per_step)
            lo, hi = int(offs[c0]), int(offs[c1])
            lr_t = lr * 0.5 * (1 + np.cos(np.pi * it / total))
            tl.append(net.train_step(xd[lo:hi], yd[lo:hi], lr_t, lo=lo, hi=hi))
            it += 1
        lo, hi = int(offs[n_tr]), int(offs[-1])
        with torch.no_grad():
            yv = net.forward(xd[lo:hi], N_OUT, lo=lo, hi=hi)
            vl = float(((yv - yd[lo:hi]) ** 2).mean())
        log(f'epoch {ep}: train loss {np.mean(tl):.4f}, validation loss {vl:.4f}')
    t_train = time.perf_counter() - t0
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    np.savez(out, params=net.params(), x_mean=x_mean, x_std=x_std, y_mean=y_mean, y_std=y_std,
             meta=json.dumps({'clusters': len(X), 'validation_clusters': n_val, 'cells': int(offs[-1]),
                              'epochs': epochs, 'train_s': t_train, 'total_s': time.perf_counter() - t_all,
                              'validation_loss': vl, 'dt': DT, 'tol': 3e-7, 'max_steps': max_steps}))
    net.close()
    return out


class WarmStart:
    """A trained network with its input/target normalisation."""

    def __init__(self, path=DEFAULT_WEIGHTS):
        d = np.load(path)
        self.params = d['params']
        self.x_mean, self.x_std = d['x_mean'], d['x_std']
        self.y_mean, self.y_std = d['y_mean'], d['y_std']
        self.meta = json.loads(str(d['meta']))

    def predict(self, geoms, params, Dms, net=None):
        """Predicted targets per cluster (list of [C, 5]); the forward pass runs
        on the GPU over all clusters at once.  Returns (list, seconds)."""
        import torch
        X = np.concatenate([cell_features(g, p, D) for g, p, D in zip(geoms, params, Dms)])
        own = net is None
        if own:
            net = GraphNet(self.params)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ptr, nbr = graph_of(geoms)
        net.set_graph(ptr, nbr)
        y = net.forward(((X - self.x_mean) / self.x_std).astype(np.float32), N_OUT).cpu().numpy()
        dt = time.perf_counter() - t0
        if own:
            net.close()
        y = y * self.y_std + self.y_mean
        offs = np.cumsum([0] + [g.n_cells for g in geoms])
        return [y[offs[k]:offs[k + 1]] for k in range(len(geoms))], dt


def evaluate(ws, n_clusters=256, n_cells=5000, seed=9001, tol=1e-6, chunk=500, max_steps=2_000_000, log=print,
             details=False, blend=(1.0,)):
    """Init time-to-steady on fresh clusters, cold (uniform initial profile)
    against warm (network prediction), same stepping and residual test.

    ``blend`` lists factors b of the warm start y = y_init + b (y_pred - y_init)
    to measure (1 = the prediction itself).  A warm-started cluster that goes
    unstable restarts from the prediction damped by FALLBACK_BLEND, then cold,
    and its steps keep counting; a prediction that gives no usable state
    starts cold."""
    gs, ps, Dms, sts = gen.sweep_workload(n_clusters, seed, cells_range=(n_cells, n_cells * 1.0001), dt=DT,
                                          dm_range=(1e-19, 1e-17), mult_range=MULT_RANGE, pump_range=PUMP_RANGE)
    cold_fin, cold_steps, cold_wall, _ = run_to_steady(gs, ps, Dms, sts, tol=tol, chunk=chunk,
                                                       max_steps=max_steps)
    # the comparison is on the clusters the plain method itself brings to steady
    # state; a cluster whose explicit step diverges from the uniform start is
    # reported and left out of both arms
    keep = np.nonzero(cold_steps > 0)[0]
    dropped = int(len(gs) - len(keep))
    gs, ps, Dms, sts = [gs[k] for k in keep], [ps[k] for k in keep], [Dms[k] for k in keep], [sts[k] for k in keep]
    cold_steps = cold_steps[keep]
    pred, t_pred = ws.predict(gs, ps, Dms)
    y0 = [cell_targets(g, s, s) for g, s in zip(gs, sts)]
    res = {'clusters': n_clusters, 'cells_per_cluster': n_cells, 'tol_V_per_s': tol, 'check_every': chunk,
           'dt': DT, 'precision': 'split',
           'cold': {'steps_median': float(np.median(cold_steps)), 'steps_max': int(cold_steps.max()),
                    'steps_mean': float(np.mean(cold_steps)), 'wall_s': cold_wall,
                    'passed': int(len(keep)), 'not_passed_left_out': dropped},
           'warm': []}
    for b in blend:
        t0 = time.perf_counter()
        warm, fallback = warm_states(gs, ps, sts, pred, y0, b)
        damped, _ = warm_states(gs, ps, sts, pred, y0, b * FALLBACK_BLEND)
        t_state = time.perf_counter() - t0
        _, warm_steps, warm_wall, restarted = run_to_steady(gs, ps, Dms, warm, tol=tol, chunk=chunk,
                                                            max_steps=max_steps, restart_states=(damped, sts))
        w = {'blend': b, 'steps_median': float(np.median(warm_steps)), 'steps_max': int(warm_steps.max()),
             'steps_mean': float(np.mean(warm_steps)),
             'wall_s': warm_wall + t_pred + t_state, 'predict_s': t_pred, 'state_s': t_state,
             'passed': int(np.sum(warm_steps > 0)), 'unstable': int(np.sum(warm_steps == -2)),
             'restarted_damped': int(np.sum(restarted >= 1)), 'restarted_cold': int(np.sum(restarted >= 2)),
             'cold_fallbacks': int(fallback.sum())}
        ok = (cold_steps > 0) & (warm_steps > 0)
        if np.any(ok):
            w['speedup_mean_steps'] = float(np.mean(cold_steps[ok]) / np.mean(warm_steps[ok]))
            w['speedup_median_steps'] = float(np.median(cold_steps[ok]) / np.median(warm_steps[ok]))
            w['speedup_max_steps'] = float(cold_steps[ok].max() / warm_steps[ok].max())
        w['speedup_wall'] = cold_wall / w['wall_s']
        if details:
            w['per_cluster'] = [[int(a), int(c), int(r)] for a, c, r in zip(cold_steps, warm_steps, restarted)]
        res['warm'].append(w)
    log(json.dumps(res))
    return res


def main():
    ap = argparse.ArgumentParser(prog='python -m betse_gb300.warmstart')
    sub = ap.add_subparsers(dest='cmd', required=True)
    t = sub.add_parser('train')
    t.add_argument('--out', default=DEFAULT_WEIGHTS)
    t.add_argument('--clusters', type=int, default=2048)
    t.add_argument('--epochs', type=int, default=60)
    t.add_argument('--max-steps', type=int, default=1_200_000)
    t.add_argument('--seed', type=int, default=101)
    e = sub.add_parser('evaluate')
    e.add_argument('--weights', default=DEFAULT_WEIGHTS)
    e.add_argument('--clusters', type=int, default=256)
    e.add_argument('--cells', type=int, default=5000)
    a = ap.parse_args()
    from .build import build
    build()
    if a.cmd == 'train':
        train(a.out, n_clusters=a.clusters, epochs=a.epochs, seed=a.seed, max_steps=a.max_steps)
    else:
        evaluate(WarmStart(a.weights), n_clusters=a.clusters, n_cells=a.cells)


if __name__ == '__main__':
    main()
