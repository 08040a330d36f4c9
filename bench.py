#!/usr/bin/env python3
"""Benchmark of the GB300 electrodiffusion step (one JSON line on rank 0).

Metric: membrane-updates/s (membranes x time steps / second) of BETSE's full
solver step, FP32/FP64-split form against the plain FP64 GPU form at Vmem
error below 1e-6 V.

Default workload (``--workload cluster100k``): one jittered-hex Voronoi cluster
of ~100k cells (~600k membranes), no extracellular spaces, diffusivities
log-uniform in [1e-19, 1e-16] m^2/s, dt 5e-3 s. One bench step is one run of
1000 time steps of that cluster (the run length of the workload); W warm-up
runs, then K timed runs bracketed by synchronisation, with the L2 flushed
(a 256 MiB write) before every run. The split form runs the kernel the
autotuner picks (its table is in the line). The plain FP64 form is timed on
the same cluster, and both are stepped side by side from the same start to
give the split form's Vmem error curve over the run.

``value``: device-resident throughput of the split form. ``e2e``: the same
metric through the C ABI with host buffers: every run uploads the state from
pinned host memory, steps, and downloads the state.

``configs``: the other workloads, each with its value, roofline and CPU
baseline -- the ~250-cell plain FP64 case, the ~20k-cell case with
extracellular spaces, the 512-cluster sweep, and the learned warm start.

``--impl reference`` times the CPU restatement of BETSE's step (C with
OpenMP on every host thread; the NumPy oracle where no C compiler exists) on
a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'membrane-updates/s vs plain FP64 GPU at Vmem err<1e-6 V; init time-to-steady'
UNIT = 'membrane-updates/s'

WORKLOADS = {
    # configs of the benchmark: radius (m) of the disc the hex lattice is clipped to
    # dt 5e-3: with Dm up to 1e-16 BETSE's explicit step diverges at dt 1e-2
    'cluster100k': dict(radius=1450e-6, seed=3, is_ecm=False, dt=5e-3, dm=(1e-19, 1e-16),
                        time_steps=1000, grid_size=20,
                        desc='precision variant: ~100k-cell jittered-hex Voronoi cluster '
                             '(~600k membranes), no ECM, Dm log-uniform [1e-19,1e-16], '
                             'dt 5e-3 s, 1000 steps per run; split step vs plain FP64'),
    'plain250': dict(radius=80e-6, seed=1, is_ecm=False, dt=1e-2, dm=(1e-19, 1e-17),
                     time_steps=2000, grid_size=20,
                     desc='plain FP64 reference step, ~250 cells, no ECM, 2000 steps'),
    'ecm20k': dict(radius=662e-6, seed=11, is_ecm=True, dt=5e-3, dm=(1e-19, 1e-17),
                   time_steps=500, grid_size=200, cell_space=25e-9,
                   desc='extracellular spaces: ~20k-cell jittered-hex Voronoi cluster (~123k '
                        'membranes), 199x200 environment grid, cell_space 25 nm, Dm log-uniform '
                        '[1e-19,1e-17], dt 5e-3 s, 500 steps per run'),
    'sweep512': dict(sweep=True, n_clusters=512, seed=7, dt=5e-3, dm=(1e-19, 1e-17),
                     time_steps=1000,
                     desc='batched sweep: 512 independent clusters, cells log-uniform [200,5000], '
                          'per-cluster Na/K Dm and pump multipliers log-uniform [0.1,10], '
                          'Dm log-uniform [1e-19,1e-17], dt 5e-3 s, 1000 steps per run, split step'),
}


def _env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def job_throughput(t_local, units_per_rank, world, dist=None, device=None):
    """Whole-job throughput of N replicas: every rank processed units_per_rank in
    t_local seconds; the job time is the maximum over ranks.  Returns (t_max,
    units of all ranks / t_max)."""
    t_max = t_local
    if dist is not None:
        import torch
        tt = torch.tensor([t_local], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max = float(tt.item())
    return t_max, units_per_rank * world / t_max


def bf16_peak():
    path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(path):
        return float(json.load(open(path))['bf16_tflops']), 'measured (burst)'
    return 1900.0, 'fallback'


def peaks():
    path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d['hbm_gbs']), 'measured'
    return 6800.0, 'fallback'


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index=0):
        self.f = tempfile.NamedTemporaryFile('w+', suffix='.csv', delete=False)
        self.p = None
        self.idx = gpu_index

    def start(self):
        try:
            self.p = subprocess.Popen(['nvidia-smi', '-i', str(self.idx), f'--query-gpu={self.Q}',
                                       '--format=csv,noheader,nounits', '-lms', '200'],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = [r.split(',') for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for r in rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == 'active':
                    reasons.add(n)
        if not sm:
            return None
        return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': smax, 'reasons': sorted(reasons),
                'samples': len(sm)}


def build_workload(name):
    from betse_gb300 import generator as gen
    w = WORKLOADS[name]
    if w.get('sweep'):
        gs, ps, Dms, sts = gen.sweep_workload(w['n_clusters'], w['seed'], dt=w['dt'],
                                              dm_range=w['dm'])
        return w, gs, ps, Dms, sts, None
    g, p, Dm, st, D_env = gen.workload(w['radius'], w['seed'], is_ecm=w['is_ecm'], dt=w['dt'],
                                       dm_range=w['dm'], grid_size=w['grid_size'],
                                       cell_space=w.get('cell_space', 26e-9))
    return w, g, p, Dm, st, D_env


class Sweep:
    """Adapter giving a batch the single-cluster calls bench.py uses."""

    def __init__(self, gs, ps, Dms, sts, precision):
        from betse_gb300.engine import BatchEngine
        self.e = BatchEngine(gs, ps, precision)
        self.e.set_membrane_diffusivity(Dms)
        self.sts = sts
        self.e.upload_states(sts)
        self.n_mems = self.e.M
        self.n_cells = self.e.C

    def __getattr__(self, k):
        return getattr(self.e, k)

    def upload(self, **_):
        self.e.upload_states(self.sts)

    def download(self):
        d = self.e.download_states()
        return {'vm': np.concatenate([x['vm'] for x in d]),
                'cc_cells': np.concatenate([x['cc_cells'] for x in d], axis=1),
                'cc_at_mem': np.concatenate([x['cc_at_mem'] for x in d], axis=1),
                'cc_env': np.concatenate([x['cc_env'] for x in d])}


def _c_steppers(clusters, D_env=None):
    """C restatements (oracle/c, OpenMP) of the clusters, or None when the C
    oracle cannot be built or does not cover the configuration."""
    try:
        from oracle import cstep
        from oracle.adapt import from_workload
        return ([cstep.Stepper(*from_workload(g, p, Dm, st, D_env)) for g, p, Dm, st in clusters],
                cstep.max_threads())
    except Exception as e:
        print(f'C restatement unavailable, timing the NumPy oracle: {e}', file=sys.stderr)
        return None, 1


def cpu_baseline(g, p, Dm, st, budget_s=12.0, D_env=None):
    """BETSE's step restated for the CPU, on a bounded sample: the whole
    cluster, as many time steps as fit in about budget_s seconds, with the C
    restatement on every host thread (OpenMP); the NumPy oracle on one thread
    if the C one cannot be built."""
    steppers, threads = _c_steppers([(g, p, Dm, st)], D_env)
    if steppers:
        s0 = steppers[0]
        s0.step(1)                   # the thread pool and first touches
        t0 = time.perf_counter()
        s0.step(2)
        one = (time.perf_counter() - t0) / 2
        n = max(1, int(budget_s / max(one, 1e-4)) - 1)
        t0 = time.perf_counter()
        s0.step(n)
        dt = time.perf_counter() - t0
        return {'value': g.n_mems * n / dt, 'unit': UNIT, 'cores': threads, 'kind': 'port',
                'sample': f'{n} time steps of the full {g.n_cells}-cell / {g.n_mems}-membrane '
                          f'cluster ({dt:.1f} s), C restatement of the step (oracle/c), {threads} OpenMP threads'}
    import oracle
    from oracle.adapt import from_workload
    geo, par, s = from_workload(g, p, Dm, st, D_env)
    t0 = time.perf_counter()
    oracle.step(geo, par, s)
    one = time.perf_counter() - t0
    n = max(1, int(budget_s / max(one, 1e-3)) - 1)
    t0 = time.perf_counter()
    for _ in range(n):
        oracle.step(geo, par, s)
    dt = time.perf_counter() - t0
    return {'value': g.n_mems * n / dt, 'unit': UNIT, 'cores': 1, 'kind': 'port',
            'sample': f'{n} time steps of the full {g.n_cells}-cell / {g.n_mems}-membrane '
                      f'cluster ({dt:.1f} s), NumPy oracle, one thread'}


def cpu_baseline_sweep(gs, ps, Dms, sts, budget_s=12.0):
    """The sweep on the C restatement: every cluster, as many time steps as
    fit in about budget_s seconds (each step visits all clusters in turn, each
    on every host thread)."""
    steppers, threads = _c_steppers(list(zip(gs, ps, Dms, sts)))
    if not steppers:
        return cpu_baseline(gs[0], ps[0], Dms[0], sts[0], budget_s)
    M = sum(g.n_mems for g in gs)
    steppers[0].step(1)              # the thread pool and first touches
    t0 = time.perf_counter()
    for s in steppers:
        s.step(1)
    one = time.perf_counter() - t0
    n = max(1, int(budget_s / max(one, 1e-4)) - 1)
    t0 = time.perf_counter()
    for s in steppers:
        s.step(n)
    dt = time.perf_counter() - t0
    return {'value': M * n / dt, 'unit': UNIT, 'cores': threads, 'kind': 'port',
            'sample': f'{n} time steps of all {len(gs)} clusters ({M} membranes, {dt:.1f} s), '
                      f'C restatement of the step (oracle/c), {threads} OpenMP threads'}


def init_time_to_steady(n_clusters=256, n_cells=5000):
    """The learned warm start against the plain init on fresh clusters."""
    from betse_gb300 import warmstart as ws
    r = ws.evaluate(ws.WarmStart(), n_clusters=n_clusters, n_cells=n_cells, seed=9001, max_steps=1_500_000,
                    log=lambda s: None)
    w = r['warm'][0]
    return {'metric': 'init steps to max|dVm/dt| < 1e-6 V/s per cluster, warm start vs uniform start',
            'value': w.get('speedup_mean_steps'), 'unit': 'x (mean steps per cluster, cold / warm)',
            'speedup_median_steps': w.get('speedup_median_steps'),
            'speedup_wall_lockstep_batch': w['speedup_wall'],
            'workload': f'{n_clusters} fresh clusters x {n_cells} cells, dt {ws.DT} s, split step, '
                        f'residual checked every {r["check_every"]} steps',
            'cold': r['cold'], 'warm': w}


# A four-substance network in BETSE's configuration format ('general network'
# -> 'biomolecules', 'reactions'): gene products with Hill activation and
# inhibition, a charged substance crossing the membrane and gap junctions, a
# neutral one with intracellular transport, two cell-zone reactions.
def _bench_substance(name, z, Dm, Dgj, env, cell, gad, ui=False, gj_imp=False):
    return {'name': name, 'Dm': Dm, 'Do': 1.0e-11, 'Dgj': Dgj, 'z': z, 'env conc': env, 'cell conc': cell,
            'update intracellular': ui, 'use time dilation': False, 'TJ permeable': False,
            'GJ impermeable': gj_imp, 'TJ factor': 1.0, 'growth and decay': gad,
            'plotting': {'plot 2D': False, 'animate': False}}


def _bench_gad(prod, decay, acts=None, inhs=None, apply_to='all', mod='None'):
    a = acts or ([], [], [])
    i = inhs or ([], [], [])
    return {'production rate': prod, 'decay rate': decay, 'apply to': apply_to, 'modulator function': mod,
            'activators': a[0] or 'None', 'Km activators': a[1] or 'None', 'n activators': a[2] or 'None',
            'inhibitors': i[0] or 'None', 'Km inhibitors': i[1] or 'None', 'n inhibitors': i[2] or 'None'}


BENCH_NETWORK = dict(
    substances=[
        _bench_substance('g1', 0, 0.0, 1e-15, 0.0, 0.1, _bench_gad(0.5, 0.2, inhs=(['g3'], [0.3], [2.0]),
                                                                    mod='gradient_x')),
        _bench_substance('g2', 0, 0.0, 1e-15, 0.0, 0.05, _bench_gad(1.0, 0.5, acts=(['g1', 'g3!'], [0.2, 0.5],
                                                                                     [2.0, 1.0]),
                                                                     apply_to=['spot']), gj_imp=True),
        _bench_substance('g3', -1, 1e-18, 1e-14, 0.5, 0.2, _bench_gad(0.2, 0.1, acts=(['g2'], [0.1], [1.0]))),
        _bench_substance('g4', 0, 5e-19, 1e-15, 1.0, 0.1, _bench_gad(0.05, 0.05, inhs=(['g3'], [0.4], [1.0])),
                         ui=True),
    ],
    reactions=[
        {'name': 'r1', 'reaction zone': 'cell', 'reactants': ['g1', 'g3'], 'reactant multipliers': [1, 1],
         'Km reactants': [0.1, 0.2], 'products': ['g4'], 'product multipliers': [1], 'Km products': [0.5],
         'max rate': 0.01, 'standard free energy': 'None', 'reaction activators': ['g2'], 'activator Km': [0.1],
         'activator n': [2.0]},
        {'name': 'r2', 'reaction zone': 'cell', 'reactants': ['g4'], 'reactant multipliers': [1],
         'Km reactants': [0.3], 'products': ['g2'], 'product multipliers': [2], 'Km products': [0.4],
         'max rate': 0.02, 'standard free energy': -5000.0},
    ])


def network_step(g, p, Dm, st, stream, flush, n_steps=200, cpu=True):
    """The molecule / gene-regulatory-network step (MasterOfNetworks.run_loop)
    with the plain FP64 ion step on the headline cluster: the network kernels
    alone and the coupled step, ms per time step (CUDA events), and the
    network kernels' roofline on their algorithmic bytes."""
    from betse_gb300.engine import ClusterEngine
    from betse_gb300.network import Network, NetworkSpec
    C, M = g.n_cells, g.n_mems
    rng = np.random.default_rng(17)
    spot = np.sort(rng.choice(C, size=C // 3, replace=False))
    gmod = rng.uniform(0.2, 1.2, size=C)
    R_rads = np.asarray(g.R_rads)
    mem_vol = 0.5 * R_rads * np.asarray(g.mem_sa)
    spec = NetworkSpec.from_config(BENCH_NETWORK['substances'], BENCH_NETWORK['reactions'], 1.0, n_cells=C,
                                   profiles={'spot': spot}, growth_mod={'g1': gmod}, ion_names=p.ion_names,
                                   mem_vol=mem_vol, R_rads=R_rads)
    out = {'workload': f'4-substance network (2 cell-zone reactions, Hill activators and inhibitors) on the '
                       f'{C}-cell / {M}-membrane cluster, plain FP64 ion step',
           'substances': 4, 'reactions': 2, 'unit': 'ms per time step'}
    with ClusterEngine(g, p, 'fp64') as eng:
        eng.set_membrane_diffusivity(Dm)
        eng.upload(**st)
        with Network(eng, spec) as net:
            net.upload_initial()
            net.step(2 * 32 + 3, with_ions=True)     # warm-up, graphs captured
            flush.fill_(1)
            torch_sync()
            ms_net = net.time_step(n_steps, with_ions=False)
            flush.fill_(1)
            torch_sync()
            ms_both = net.time_step(n_steps, with_ions=True)
            net.check_stable()
            eng.check_stable()
            nbytes = net.algorithmic_bytes()
    out.update({'ms_network_alone': ms_net, 'ms_with_ion_step': ms_both,
                'cell_substance_updates_per_s': C * 4 / (ms_net / 1e3),
                'roofline': roofline_entry(nbytes, ms_net / 1e3, 'k_net_cell + k_net_gj',
                                           note='algorithmic bytes of one network step (both kernels; '
                                                'Network.algorithmic_bytes) / its time per step, network alone. '
                                                'The plain FP64 network is bound by the FP64 pipe (about 80% '
                                                'of active cycles under ncu), not by HBM')})
    if cpu:
        out['cpu_baseline'] = cpu_baseline_network(g, p, Dm, st, spec_args=(spot, gmod, mem_vol, R_rads))
    return out


def torch_sync():
    import torch
    torch.cuda.synchronize()


def cpu_baseline_network(g, p, Dm, st, spec_args, budget_s=8.0):
    """The network oracle (oracle/network.py, NumPy, one thread) on the same
    cluster with Vmem frozen, a bounded number of steps."""
    from oracle.adapt import from_workload
    from oracle.network import Network as OracleNetwork
    spot, gmod, mem_vol, R_rads = spec_args
    og, op, os_ = from_workload(g, p, Dm, st)
    og.R_rads = R_rads
    onet = OracleNetwork(BENCH_NETWORK['substances'], BENCH_NETWORK['reactions'], og, op, mem_vol, 1.0,
                         {'g2': spot}, {'g1': gmod})
    ost = onet.initial_state()
    vm = os_.vm
    vgj = vm[og.nn_i] - vm
    gjo = op.gj_block * og.gj_weight
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < budget_s or n < 2:
        onet.step(ost, vm, vgj, gjo, op.gj_block)
        n += 1
    dt = time.perf_counter() - t0
    return {'value': 1e3 * dt / n, 'unit': 'ms per time step', 'cores': 1, 'kind': 'port',
            'sample': f'{n} network-alone steps of the full cluster, oracle/network.py (NumPy, one thread)'}


def batch_fields_timing(n_clusters=128):
    """Environment fields of a sweep at a sampled step: one tensor-core GEMM per
    grid shape for all clusters (host wall time of bx_batch_env_fields, the
    fields copied to the host)."""
    from betse_gb300 import generator as gen
    from betse_gb300.fields import lap_env_inverse
    from betse_gb300.engine import BatchEngine
    gs, ps, Dms, sts = gen.sweep_workload(n_clusters, 7, dt=5e-3)
    b = BatchEngine(gs, ps, 'split')
    b.set_membrane_diffusivity(Dms)
    b.upload_states(sts)
    b.step(2, outputs=True)
    shapes = {}
    for g in gs:
        shapes.setdefault(tuple(g.grid_shape), g.delta)
    for shp, d in shapes.items():
        b.set_lap_env_inv_shape(lap_env_inverse(*shp, d), shp, d)
    b.env_fields()
    t = []
    for _ in range(5):
        t0 = time.perf_counter()
        b.env_fields()
        t.append(time.perf_counter() - t0)
    b.close()
    return {'clusters': n_clusters, 'grid_shapes': len(shapes), 'grid_cells': int(sum(g.n_grid for g in gs)),
            'ms_per_sampled_step': 1e3 * min(t),
            'gemms_per_sampled_step': 2 * len(shapes) * 2,
            'note': 'all clusters of one grid shape share lapENVinv = delta^2 K(shape): their products run as one '
                    'BF16x3 tcgen05 GEMM with a per-column delta^2 and one FP64 refinement'}


def step_bytes(form, C, M, G=0, ecm=False):
    """Algorithmic bytes of one time step by the per-array count BETSE's step
    implies (each array once at its stored width, reads plus writes): plain
    FP64 104 B per membrane + 124 B per cell; split form 64 + 112; with
    extracellular spaces 4 B more per membrane (map_mem2ecm) and 160 B per
    grid cell (six ions' concentrations read and written, D, E_x, E_y)."""
    b = (104 * M + 124 * C) if form == 'fp64' else (64 * M + 112 * C)
    if ecm:
        b += 4 * M + 160 * G
    return b


def roofline_entry(bytes_per_step, s_per_step, kernel, note=None, step=None):
    """achieved = algorithmic bytes per time step / time per step.  With
    `step` (the per-membrane count of step_bytes, the step's algorithmic
    bytes by definition) that count is the one `achieved` and `frac` use;
    the bytes the chosen kernel's own layout reads and writes stand beside
    it (kernel_bytes_per_step, frac_on_kernel_bytes)."""
    hbm, src = peaks()
    algo = bytes_per_step if step is None else step
    a = algo / s_per_step / 1e9
    r = {'bound': 'hbm', 'achieved': a, 'peak': hbm, 'unit': 'GB/s', 'frac': a / hbm,
         'algorithmic_bytes_per_step': int(algo), 'kernel': kernel, 'peak_source': src}
    if step is not None:
        r['kernel_bytes_per_step'] = int(bytes_per_step)
        r['frac_on_kernel_bytes'] = bytes_per_step / s_per_step / 1e9 / hbm
    if note:
        r['note'] = note
    return r


_FP64_PEAK = {}


def fp64_peak(stream, best_of=5):
    """The FP64 pipe's measured peak on this GPU: the probe kernel
    (bx_fp64_fma_probe: 8 CTAs of 256 threads per SM, 8 independent FMA
    chains per thread) timed with CUDA events on `stream`, best of `best_of`
    launches after two warm-ups.  Cached per process."""
    if 'peak' in _FP64_PEAK:
        return _FP64_PEAK['peak']
    import ctypes as ct
    import torch
    from betse_gb300 import _lib
    lib = _lib.load()
    n_sm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    n_blocks, iters = 8 * n_sm, 2048
    out = torch.empty(n_blocks * 256, dtype=torch.float64, device='cuda')

    def run():
        rc = lib.bx_fp64_fma_probe(n_blocks, iters, 1.0, 1.0, ct.c_void_p(out.data_ptr()),
                                   ct.c_void_p(stream.cuda_stream))
        if rc != _lib.BX_OK:
            raise RuntimeError('bx_fp64_fma_probe: ' + lib.bx_last_error().decode())
    for _ in range(2):
        run()
    best = float('inf')
    for _ in range(best_of):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        run()
        b.record(stream)
        b.synchronize()
        best = min(best, a.elapsed_time(b))
    warp_fma = n_blocks * 64 * iters
    _FP64_PEAK['peak'] = {'warp_inst_per_s': warp_fma / (best / 1e3),
                          'fma_tflops': warp_fma * 32 * 2 / (best / 1e3) / 1e12, 'ms': best,
                          'launch': f'{n_blocks} CTAs x 256 threads, 8 FMA chains x {iters} per thread'}
    return _FP64_PEAK['peak']


def fp64_roofline(kernel_ms, n_mems, peak, kernel, workload):
    """The FP64-pipe roofline of a plain-form kernel: its FP64 warp
    instructions per launch (ncu's sm__inst_executed_pipe_fp64.sum, from the
    committed capture in profiles/fp64_counts.json, per membrane, scaled to
    this workload's membranes) over its measured time per launch, against
    the probe's FP64 warp-instruction rate.  An FP64 warp instruction holds
    the pipe the same whatever the number of active lanes, so `frac` is the
    share of the kernel's time its FP64 work needs at the pipe's peak."""
    r = {'bound': 'fp64', 'unit': 'G FP64 warp-instructions/s', 'peak': peak['warp_inst_per_s'] / 1e9,
         'peak_fma_tflops': peak['fma_tflops'], 'peak_source': 'measured: ' + peak['launch'],
         'kernel': kernel, 'ms_per_launch': kernel_ms}
    path = os.path.join(ROOT, 'profiles', 'fp64_counts.json')
    counts = json.load(open(path)).get('kernels', {}).get(workload, {}) if os.path.exists(path) else {}
    entry, counted = counts.get(kernel), kernel
    if entry is None and kernel.startswith('k_cell_step<double>'):
        # another tile size of the same kernel: every thread runs the same
        # code per membrane slot, so its count per membrane stands in
        for name, e in counts.items():
            if name.startswith('k_cell_step<double>'):
                entry, counted = e, name
                break
    if entry is None:
        r.update(achieved=None, frac=None, note='no FP64 instruction count captured for this kernel')
        return r
    per_mem = entry['fp64_warp_inst_per_launch'] / entry['membranes']
    inst = per_mem * n_mems
    a = inst / (kernel_ms / 1e3) / 1e9
    r.update(achieved=a, frac=a / r['peak'], fp64_warp_inst_per_launch=int(inst),
             fp64_warp_inst_per_membrane=per_mem, count_source='profiles/fp64_counts.json')
    if counted != kernel:
        r['count_of'] = counted + ' (per membrane)'
    return r


def timed_run_ms(eng, T, stream, flush, reps=3):
    """Best of `reps` runs of T time steps on `stream` (CUDA events), the L2
    flushed before each; one untimed run first."""
    import torch
    eng.step(T, stream=stream.cuda_stream)
    ms = []
    for _ in range(reps):
        flush.fill_(1)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.step(T, stream=stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    eng.check_stable()
    return min(ms)


def config_plain250(wl, stream, flush, cpu=True):
    """Config 1: the plain FP64 step on the ~250-cell cluster, 2000 steps."""
    from betse_gb300.engine import ClusterEngine
    w, g, p, Dm, st, D_env = wl
    T = w['time_steps']
    with ClusterEngine(g, p, 'fp64') as e:
        e.set_membrane_diffusivity(Dm)
        e.upload(**st)
        table = e.autotune_table(20)
        launch = e.launch_config()
        ms = timed_run_ms(e, T, stream, flush)
        e.upload(**st)
        kms = e.time_cell_kernel(200)
        kb = e.cell_kernel_bytes()
    out = {'workload': w['desc'], 'cells': g.n_cells, 'membranes': g.n_mems, 'time_steps_per_run': T,
           'form': 'plain FP64', 'value': g.n_mems * T / (ms / 1e3), 'unit': UNIT, 'ms_per_run': ms,
           'roofline': roofline_entry(kb, kms / 1e3, 'k_cell_step<double>',
                                      note='a 1.4k-membrane cluster fills a few dozen CTAs: bound by '
                                           'the dependent FP64 instruction chain of a lane, not by HBM',
                                      step=step_bytes('fp64', g.n_cells, g.n_mems)),
           'kernel_launches_per_step': 1 if launch[1] == 5 else 2,   # the ion kernel mixes the environment
           'autotuned_launch': {'cta_slots': launch[0], 'kernel': 'k_cell_step_ion' if launch[1] == 5
                                else 'k_cell_step<double>'},
           'autotune_table': table}
    out['roofline']['kernel'] = out['autotuned_launch']['kernel']
    kname = f"k_cell_step_ion<{launch[0]}>" if launch[1] == 5 else f"k_cell_step<double> ({launch[0]} slots)"
    out['roofline_fp64'] = fp64_roofline(kms, g.n_mems, fp64_peak(stream), kname, 'plain250')
    if cpu:
        out['cpu_baseline'] = cpu_baseline(g, p, Dm, st, budget_s=6.0)
    return out


def config_ecm20k(wl, stream, flush, cpu=True):
    """Config 2: extracellular spaces, ~20k cells on a 199x200 grid, 500
    steps; the plain FP64 form (the config's) and the split form."""
    from betse_gb300.engine import ClusterEngine
    w, g, p, Dm, st, D_env = wl
    T = w['time_steps']
    G = g.n_grid
    out = {'workload': w['desc'], 'cells': g.n_cells, 'membranes': g.n_mems, 'grid': list(g.grid_shape),
           'time_steps_per_run': T}
    for prec in ('fp64', 'split'):
        with ClusterEngine(g, p, prec) as e:
            e.set_membrane_diffusivity(Dm)
            e.set_env_diffusivity(D_env)
            e.upload(**st)
            e.autotune(5)
            ms = timed_run_ms(e, T, stream, flush)
        sv = step_bytes(prec, g.n_cells, g.n_mems, G, ecm=True)
        out[prec] = {'value': g.n_mems * T / (ms / 1e3), 'unit': UNIT, 'ms_per_run': ms,
                     'ms_per_time_step': ms / T,
                     'roofline': roofline_entry(sv, ms / 1e3 / T, 'whole step (cell kernel + grid stencils)',
                                                note='bytes by the per-array count with the grid terms; the '
                                                     'per-kernel shares are in profiles/ecm_step_kernels_ecm20k.md')}
    out['value'] = out['fp64']['value']
    out['unit'] = UNIT
    out['form'] = 'plain FP64 (split form beside it)'
    if cpu:
        out['cpu_baseline'] = cpu_baseline(g, p, Dm, st, budget_s=6.0, D_env=D_env)
    return out


def config_sweep512(wl, stream, flush, cpu=True):
    """Config 4: 512 clusters of uneven size in one batch, split form, the
    kernel the autotuner picks, 1000 steps per run."""
    w, gs, ps, Dms, sts, _ = wl
    T = w['time_steps']
    S = Sweep(gs, ps, Dms, sts, 'split')
    table = S.e.autotune_table(64)
    tpb, kind = S.launch_config()
    ms = timed_run_ms(S, T, stream, flush)
    S.upload()
    kms = S.time_cell_kernel(50)
    kb = S.cell_kernel_bytes()
    M, C = S.n_mems, S.n_cells
    kname = KERNEL_NAMES.get(kind, str(kind))
    out = {'workload': w['desc'], 'clusters': len(gs), 'cells': C, 'membranes': M, 'time_steps_per_run': T,
           'form': 'split', 'value': M * T / (ms / 1e3), 'unit': UNIT, 'ms_per_run': ms,
           'autotuned': {'tpb': tpb, 'kernel': kname}, 'autotune_table': table,
           'roofline': roofline_entry(kb, kms / 1e3, kname, step=step_bytes('split', C, M),
                                      note='algorithmic bytes of the split step (64 B per membrane + 112 B per '
                                           'cell); kernel_bytes_per_step is what the factored layout moves (one '
                                           'sum of Dm*mem_sa per cell instead of Dm per membrane)')}
    S.close()
    if cpu:
        out['cpu_baseline'] = cpu_baseline_sweep(gs, ps, Dms, sts, budget_s=8.0)
    return out


def dense_products(stream, flush, wl_ecm):
    """Output-side dense products: lapENVinv at the ECM workload's full grid
    (double-float streaming GEMV) and the BF16x3 tcgen05 GEMM of a
    lapGJinv-sized operator."""
    from betse_gb300.engine import ClusterEngine
    w, g, p, Dm, st, D_env = wl_ecm
    out = {}
    G = g.n_grid
    phys = os.sysconf('SC_PHYS_PAGES') * os.sysconf('SC_PAGE_SIZE')
    if phys < 4 * 8 * G * G:
        out['env_fields'] = {'skipped': f'host memory {phys >> 30} GiB too small for the operator'}
    else:
        with ClusterEngine(g, p, 'fp64') as fields_eng:
            fields_eng.set_membrane_diffusivity(Dm)
            fields_eng.set_env_diffusivity(D_env)
            fields_eng.upload(**st)
            t0 = time.perf_counter()
            fields_eng.build_lap_env_inv()       # the real operator, built on the GPU
            build_s = time.perf_counter() - t0
            fields_eng.step(1, outputs=True)
            ms_f, ms_p = fields_eng.time_env_fields(5)
        hbm, src = peaks()
        gbs = 8.0 * G * G / (ms_p / 1e3) / 1e9
        out['env_fields'] = {
            'operator': f'cells.lapENVinv of the {g.grid_shape[0]}x{g.grid_shape[1]} grid ({G}x{G}), built on the '
                        f'GPU from the sine-transform eigenvectors (no dense inversion), double-float storage; '
                        f'equal to an FP64 sine-transform solve within 1.7e-14 relative (tests/test_gpu_lapinv.py)',
            'build_s': build_s,
            'ms_per_sampled_step': ms_f, 'product_ms': ms_p, 'products_per_sample': 1,
            'roofline': {'bound': 'hbm', 'achieved': gbs, 'peak': hbm, 'unit': 'GB/s',
                         'frac': gbs / hbm, 'algorithmic_bytes_per_launch': 8 * G * G,
                         'kernel': 'k_dense_rows2_df', 'peak_source': src}}
    from betse_gb300.dense import DenseOperator
    n = 20480
    A = np.empty((n, n))
    A.fill(1e-3)  # timing only
    with DenseOperator(A) as op:
        del A
        res = []
        for nrhs in (256, 1024):
            ms = op.time(nrhs, 10)
            flops = 3 * 2.0 * n * n * nrhs
            res.append({'nrhs': nrhs, 'ms': ms, 'tflops': flops / (ms / 1e3) / 1e12})
    bf16 = bf16_peak()
    best = max(res, key=lambda r: r['tflops'])
    out['dense_op_gemm'] = {
        'operator': f'synthetic dense {n}x{n} (lapGJinv of a {n}-cell cluster), BF16 hi/lo tiles',
        'runs': res,
        'roofline': {'bound': 'tensor', 'achieved': best['tflops'], 'peak': bf16[0], 'unit': 'TFLOP/s',
                     'frac': best['tflops'] / bf16[0], 'flops_per_launch': 3 * 2.0 * n * n * best['nrhs'],
                     'kernel': 'k_gemm_bf16x3 (tcgen05.mma kind::f16, 3 products per K step)',
                     'peak_source': bf16[1]}}
    return out


def generator_timing(radius=1450e-6, seed=3, cpu=True):
    """Cluster generation (Cells.make_world's seeding): bx_generate_cluster on
    the GPU, the whole make_cluster call (generation, download, host
    assembly), against its NumPy/SciPy restatement on one host thread."""
    import torch
    from betse_gb300 import generator as gen
    gen.make_cluster(radius, seed)              # module load, first allocations
    ts = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gc = gen.make_cluster(radius, seed)
        ts.append(time.perf_counter() - t0)
    out = {'cells': gc.geom.n_cells, 'membranes': gc.geom.n_mems, 'gpu_ms': min(ts) * 1e3,
           'note': 'lattice (MT19937), two Voronoi passes, Z order, membranes, pairs, grid map, adjacency; '
                   'includes the download and ClusterGeometry assembly on the host'}
    if cpu:
        from oracle.generator import make_cluster as make_ref
        t0 = time.perf_counter()
        ref = make_ref(radius, seed)
        dt = time.perf_counter() - t0
        out['cpu_baseline'] = {'value': dt * 1e3, 'unit': 'ms', 'cores': 1, 'kind': 'port',
                               'sample': f'oracle/generator.py (NumPy/SciPy Delaunay) on the same radius and seed, '
                                         f'{ref.geom.n_cells} cells'}
        out['speedup'] = dt * 1e3 / out['gpu_ms']
    return out


def lap_gj_timing(wl_full, wl_ecm, dense_full=False):
    """cells.lapGJinv (Cells.graphLaplacian) of the generated clusters:
    the matrix-free FP64 product (two multigrid-preconditioned CG solves,
    bx_lap_gj_apply) at 100k cells for one right-hand side (pressures.py:59
    applies it to one vector per step) and for a block of 32; the dense
    operator built on the GPU from it and applied as a BF16x3 tcgen05 GEMM,
    with its error against the FP64 product, at 20k cells (and at 100k cells
    with dense_full: a build of several minutes)."""
    import torch
    from betse_gb300.dense import LapGJ, lap_gj_inputs

    def sync():
        torch.cuda.synchronize()

    out = {}
    g = wl_full[1]
    gen = torch.Generator('cuda').manual_seed(11)
    with LapGJ(*lap_gj_inputs(g, g.extra['cell_centres']), max_rhs=32) as op:
        res = {'cells': g.n_cells, 'levels': op.level_sizes, 'tol': 1e-10}
        for K in (1, 32):
            X = torch.randn(g.n_cells, K, dtype=torch.float64, device='cuda', generator=gen)
            op.apply(X, tol=1e-10)
            sync()
            t0 = time.perf_counter()
            for _ in range(3):
                op.apply(X, tol=1e-10)
            sync()
            res[f'ms_apply_{K}_rhs'] = (time.perf_counter() - t0) / 3 * 1e3
            res[f'cg_iterations_{K}_rhs'] = op.last_iters
        out['matrix_free_fp64'] = res
    cases = [wl_ecm] + ([wl_full] if dense_full else [])
    for wl in cases:
        g = wl[1]
        with LapGJ(*lap_gj_inputs(g, g.extra['cell_centres']), max_rhs=1024) as op:
            sync()
            t0 = time.perf_counter()
            dense = op.dense(tol=1e-10)
            sync()
            build_s = time.perf_counter() - t0
            try:
                X = torch.randn(g.n_cells, 256, dtype=torch.float64, device='cuda', generator=gen)
                ref = op.apply(X, tol=1e-13)
                Y = dense.apply(X)
                err = float((Y - ref).abs().max() / ref.abs().max())
                ms = dense.time(256, 5)
            finally:
                dense.close()
        n = g.n_cells
        tf = 3 * 2.0 * n * n * 256 / (ms / 1e3) / 1e12
        out[f'dense_bf16x3_{n}_cells'] = {
            'build_s': build_s, 'build': 'bx_lap_gj_dense: FP64 CG on blocks of 1024 identity columns, '
                                          'split into BF16 hi/lo tiles; no n x n FP64 matrix',
            'gemm_ms_256_rhs': ms, 'tflops': tf, 'rel_err_vs_fp64': err}
    return out


def run_reference(args, rank, world):
    """--impl reference: the CPU restatement of BETSE's step on the host cores
    (the C restatement on every OpenMP thread without extracellular spaces,
    the NumPy oracle with them); each step is a bounded sample of the
    workload, about BX_REF_BUDGET_S seconds."""
    if rank != 0:
        return
    w, g, p, Dm, st, D_env = build_workload(args.workload)
    budget = float(os.environ.get('BX_REF_BUDGET_S', '6'))
    n_cells, n_mems = (sum(x.n_cells for x in g), sum(x.n_mems for x in g)) if w.get('sweep') \
        else (g.n_cells, g.n_mems)
    samples = []
    for k in range(args.warmup + args.steps):
        if w.get('sweep'):
            r = cpu_baseline_sweep(g, p, Dm, st, budget_s=budget)
        else:
            r = cpu_baseline(g, p, Dm, st, budget_s=budget, D_env=D_env)
        if k >= args.warmup:
            samples.append(r['value'])
    v = statistics.mean(samples)
    line = {'metric': METRIC, 'value': v, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
            # one step of the workload is time_steps time steps of it, as in our arm
            'warmup': args.warmup, 'ms_per_step': 1e3 * n_mems * w['time_steps'] / v,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
            'data': 'synthetic', 'impl': 'reference',
            'config': {'workload': w['desc'], 'cells': n_cells, 'membranes': n_mems,
                       'time_steps_per_step': w['time_steps']},
            'cpu_baseline': {'value': v, 'unit': UNIT, 'cores': r['cores'], 'kind': 'port',
                             'sample': r['sample']},
            'e2e': {'value': v, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def profile_kernel(which):
    """One small launch sequence of a dense-product kernel for ncu captures:
    'gemm' -- k_gemm_bf16x3 on an 8192 x 8192 operator with 1024 right-hand
    sides (two warm-up launches, then the captured one); 'fields' --
    k_dense_rows2_df on a 12000 x 12000 double-float operator; 'network' --
    the four-substance network alone on the 100k-cell cluster (three warm-up
    steps, then k_net_cell and k_net_gj once each); 'fp64' -- the FP64 probe
    kernel as fp64_peak launches it (two warm-ups, five timed)."""
    from betse_gb300.build import build
    build()
    if which == 'fp64':
        import torch
        s = torch.cuda.Stream()
        pk = fp64_peak(s)
        print(f"FP64 probe: {pk['fma_tflops']:.3f} TFLOP/s ({pk['launch']}, {pk['ms']:.3f} ms)")
    elif which == 'network':
        from betse_gb300.engine import ClusterEngine
        from betse_gb300.network import Network, NetworkSpec
        w, g, p, Dm, st, _ = build_workload('cluster100k')
        C = g.n_cells
        rng = np.random.default_rng(17)
        R_rads = np.asarray(g.R_rads)
        spec = NetworkSpec.from_config(BENCH_NETWORK['substances'], BENCH_NETWORK['reactions'], 1.0, n_cells=C,
                                       profiles={'spot': np.sort(rng.choice(C, size=C // 3, replace=False))},
                                       growth_mod={'g1': rng.uniform(0.2, 1.2, size=C)}, ion_names=p.ion_names,
                                       mem_vol=0.5 * R_rads * np.asarray(g.mem_sa), R_rads=R_rads)
        with ClusterEngine(g, p, 'fp64') as eng:
            eng.set_membrane_diffusivity(Dm)
            eng.upload(**st)
            with Network(eng, spec) as net:
                net.upload_initial()
                net.step(4, with_ions=False)
                net.check_stable()
    elif which == 'gemm':
        from betse_gb300.dense import DenseOperator
        n = 8192
        A = np.empty((n, n))
        A.fill(1e-3)
        with DenseOperator(A) as op:
            op.time(1024, 3)
    else:
        from betse_gb300 import generator as gen
        from betse_gb300.engine import ClusterEngine
        g, p, Dm, st, _ = gen.workload(400e-6, 5, dt=1e-2, grid_size=110)
        G = g.n_grid
        e = ClusterEngine(g, p, 'fp64')
        e.set_membrane_diffusivity(Dm)
        e.upload(**st)
        A = np.empty((G, G))
        A.fill(1e-12)
        e.set_lap_env_inv(A)
        e.step(1, outputs=True)
        e.time_env_fields(2)
        e.close()
    print('profile kernel done:', which)


# kernels, by the number bx_set_launch_config takes (5: the plain form's)
KERNEL_NAMES = {0: 'k_split_step', 1: 'k_split_persist', 2: 'k_split_fact', 3: 'k_split_resident',
                4: 'k_split_fact_pipe', 5: 'k_cell_step_ion'}
LAUNCH_SUFFIX = {'': 0, 'p': 1, 'f': 2, 'r': 3, 'q': 4, 'i': 5}


def parse_launch(text):
    """'192' tile kernel, '192p' persistent, '192f' factored, '256r' resident,
    '256q' pipelined factored, '32i' the plain form's one-lane-per-ion
    kernel; a number after 'f' picks the factored kernel's
    variant ('256f12': two junctions per round, entries prefetched)."""
    head = text.lstrip('0123456789')
    tpb = int(text[:len(text) - len(head)])
    suffix = head.rstrip('0123456789')
    variant = head[len(suffix):]
    return tpb, LAUNCH_SUFFIX[suffix], int(variant) if variant else 0


def profile_run(args):
    """A short, deterministic launch sequence for ncu captures."""
    from betse_gb300.build import build
    build()
    w, g, p, Dm, st, D_env = build_workload(args.workload)
    if w.get('sweep'):
        e = Sweep(g, p, Dm, st, args.precision)
    else:
        from betse_gb300.engine import ClusterEngine
        e = ClusterEngine(g, p, args.precision)
        e.set_membrane_diffusivity(Dm)
        if D_env is not None:
            e.set_env_diffusivity(D_env)
        e.upload(**st)
    if args.launch:
        # the launch configuration the autotuner picks for this workload, pinned
        e.set_launch_config(*parse_launch(args.launch))
    e.step(args.time_steps or 4)
    e.check_stable()
    e.close()
    print('profile run done:', args.workload, args.precision, args.launch or 'default launch')


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--workload', default='cluster100k', choices=sorted(WORKLOADS))
    ap.add_argument('--time-steps', type=int, default=None)
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--no-secondary', action='store_true',
                    help='skip the ECM workload and environment-field measurements')
    ap.add_argument('--profile-run', action='store_true',
                    help='for ncu: build the workload, upload it, run 4 steps (or --time-steps), exit')
    ap.add_argument('--precision', default='split', choices=['split', 'fp64'])
    ap.add_argument('--lapgj-dense-full', action='store_true',
                    help='also build the dense lapGJinv of the 100k-cell cluster (several minutes)')
    ap.add_argument('--launch', default=None,
                    help='with --profile-run: membrane slots per tile, suffix p persistent, f factored '
                         '(optionally followed by its variant, e.g. 256f12), r resident, q pipelined (e.g. 192r)')
    ap.add_argument('--profile-kernel', choices=['gemm', 'fields', 'network', 'fp64'],
                    help='for ncu: run a small case of one dense-product kernel and exit')
    args = ap.parse_args()
    if args.profile_kernel:
        return profile_kernel(args.profile_kernel)
    world = _env_int('WORLD_SIZE', 1)
    if args.profile_run:
        return profile_run(args)
    rank = _env_int('RANK', 0)
    local = _env_int('LOCAL_RANK', 0)
    if args.impl == 'reference':
        return run_reference(args, rank, world)

    w, g, p, Dm, st, D_env = build_workload(args.workload)
    sweep = bool(w.get('sweep'))
    full = rank == 0 and world == 1 and args.workload == 'cluster100k' and not args.no_secondary
    # the other configurations' workloads (generated on the GPU), built first
    others = {n: build_workload(n) for n in ('plain250', 'ecm20k', 'sweep512')} if full else {}
    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group('nccl')
    else:
        torch.cuda.set_device(0)
    from betse_gb300.build import build
    build()
    from betse_gb300.engine import ClusterEngine

    T = args.time_steps or w['time_steps']
    dev = torch.device('cuda', torch.cuda.current_device())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    # a non-default stream: bx_step launches on it and the events bracket exactly it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    def make(prec):
        if sweep:
            return Sweep(g, p, Dm, st, prec)
        e = ClusterEngine(g, p, prec)
        e.set_membrane_diffusivity(Dm)
        if D_env is not None:
            e.set_env_diffusivity(D_env)
        e.upload(**st)
        return e

    split = make('split')
    plain = make('fp64')
    n_mems = split.n_mems if sweep else g.n_mems
    n_cells = split.n_cells if sweep else g.n_cells
    tune_table = split.autotune_table(64)
    plain.autotune(3)
    tune_split = split.launch_config()
    tune_plain = plain.launch_config()
    kname = KERNEL_NAMES.get(tune_split[1], str(tune_split[1]))

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    def timed_runs(eng, n_runs, runs_warm):
        for _ in range(runs_warm):
            flush.fill_(1)
            eng.step(T, stream=stream.cuda_stream)
        barrier()
        ev = []
        l0 = eng.launch_count()
        for _ in range(n_runs):
            flush.fill_(1)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            eng.step(T, stream=stream.cuda_stream)
            b.record(stream)
            ev.append((a, b))
        barrier()
        ms = [a.elapsed_time(b) for a, b in ev]
        return ms, eng.launch_count() - l0

    clocks = ClockSampler(local)
    clocks.start()
    ms_split, launches = timed_runs(split, args.steps, args.warmup)
    clk = clocks.stop()
    ms_plain, _ = timed_runs(plain, 1, 1)
    split.check_stable()
    plain.check_stable()
    # the plain kernel alone, for its FP64 roofline (the state is re-uploaded below)
    kms_plain = None if sweep else plain.time_cell_kernel(10)

    t_max, value = job_throughput(sum(ms_split) / 1e3, n_mems * T * args.steps, world, dist, dev)
    plain_value = n_mems * T * len(ms_plain) / (sum(ms_plain) / 1e3)

    # ---- Vmem error of the split form against the plain FP64 form (which
    # matches the FP64 oracle at 1e-10), stepped side by side from the same
    # start, at checkpoints up to the run length (the autotuned handles
    # themselves, back at the initial state)
    e_s, e_p = split, plain
    for e_ in (e_s, e_p):
        e_.upload(**({} if sweep else st))
    curve, done = [], 0
    for cp in sorted({c for c in (1, 10, 100, 250, 500, 1000, T) if c <= T}):
        e_s.step(cp - done)
        e_p.step(cp - done)
        done = cp
        curve.append([cp, float(np.max(np.abs(e_s.download()['vm'] - e_p.download()['vm'])))])
    vm_err = curve[-1][1]

    # ---- roofline of the split kernel the autotuner chose, events on its stream
    e_s.upload(**({} if sweep else st))
    kern_ms = e_s.time_cell_kernel(200)
    kbytes = e_s.cell_kernel_bytes()
    traffic = None
    tp = os.path.join(ROOT, 'profiles', f'{kname}_{args.workload}.traffic.json')
    if os.path.exists(tp):
        tj = json.load(open(tp))
        traffic = int(tj.get('dram_bytes_per_step', tj.get('dram_bytes_per_launch')) * n_mems / tj['membranes'])
    roof = roofline_entry(kbytes, kern_ms / 1e3, kname, step=step_bytes('split', n_cells, n_mems),
                          note='achieved = the split step\'s algorithmic bytes per time step (64 B per membrane '
                               '+ 112 B per cell: each per-membrane and per-cell array once at its stored width) '
                               '/ the chosen kernel\'s time per step; kernel_bytes_per_step is what the factored '
                               'layout itself moves (one sum of Dm*mem_sa per cell instead of Dm per membrane); '
                               'the resident kernel keeps its data in shared memory across steps, so HBM does '
                               'not bound it')
    roof['traffic'] = traffic
    roof['ms_per_step'] = kern_ms

    # ---- end to end through the C ABI with host buffers (pinned)
    def pinned(a):
        return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    if sweep:
        cat = {'vm': np.concatenate([s_['vm'] for s_ in st]),
               'cc_cells': np.concatenate([s_['cc_cells'] for s_ in st], axis=1),
               'cc_at_mem': np.concatenate([s_['cc_at_mem'] for s_ in st], axis=1),
               'cc_env': np.stack([np.asarray(s_['cc_env']) for s_ in st])}
        pin = {k: pinned(v) for k, v in cat.items()}
        up = lambda: e_s.e.upload_concat(**pin)  # noqa: E731
    else:
        pin = {k: pinned(v) for k, v in st.items()}
        up = lambda: e_s.upload(**pin)  # noqa: E731
    h2d = sum(v.nbytes for v in pin.values())
    up()
    e_s.step(T)
    torch.cuda.synchronize()
    # the result is read back into page-locked arrays the caller allocates once
    # and reuses, as a host loop over sampled steps would
    first = e_s.e.download_concat() if sweep else e_s.download()
    pin_out = {k: pinned(v) for k, v in first.items()}
    d2h = 0
    t_e2e = []
    for k in range(args.warmup + args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        up()
        e_s.step(T)
        out = e_s.e.download_concat(out=pin_out) if sweep else e_s.download(out=pin_out)
        t1 = time.perf_counter()
        d2h = sum(v.nbytes for v in out.values())
        if k >= args.warmup:
            t_e2e.append(t1 - t0)
    e2e_val = n_mems * T * len(t_e2e) * world / sum(t_e2e)
    for e in (split, plain):
        e.close()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        if sweep:
            cpu = cpu_baseline_sweep(g, p, Dm, st)
        else:
            cpu = cpu_baseline(g, p, Dm, st, D_env=D_env)
    configs = extra = None
    if full:
        cpu_on = not args.no_cpu_baseline
        configs = {'plain250': config_plain250(others['plain250'], stream, flush, cpu_on),
                   'ecm20k': config_ecm20k(others['ecm20k'], stream, flush, cpu_on),
                   'sweep512': config_sweep512(others['sweep512'], stream, flush, cpu_on),
                   'warm_start': init_time_to_steady()}
        extra = dense_products(stream, flush, others['ecm20k'])
        extra['batch_env_fields'] = batch_fields_timing()
        extra['network'] = network_step(g, p, Dm, st, stream, flush, cpu=cpu_on)
        extra['generator'] = generator_timing(cpu=cpu_on)
        extra['lap_gj'] = lap_gj_timing((w, g, p, Dm, st, D_env), others['ecm20k'],
                                        dense_full=args.lapgj_dense_full)

    if rank == 0:
        line = {
            'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': t_max * 1e3 / args.steps,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f32 fluxes and pumps; compensated-f32 (hi+lo) concentrations and charge; f32 Vmem record',
            'data': 'synthetic',
            'config': {'workload': w['desc'], 'cells': n_cells, 'membranes': n_mems,
                       'time_steps_per_step': T, 'precision': 'split',
                       'l2': 'flushed (256 MiB write) before every timed run',
                       'parallelism': f'replicas x{world}',
                       'autotuned_launch': {'split': {'tpb': tune_split[0], 'kernel': kname},
                                            'plain_fp64': {'cta_threads': tune_plain[0]}},
                       'autotune_table': tune_table},
            'plain_fp64': {'value': plain_value, 'unit': UNIT,
                           'ms_per_step': sum(ms_plain) / len(ms_plain),
                           'speedup_split_vs_plain': value / world / plain_value,
                           'vm_max_abs_err_V': vm_err, 'vm_err_after_steps': T,
                           'vm_err_curve_V': curve,
                           'roofline_fp64': None if kms_plain is None else fp64_roofline(
                               kms_plain, n_mems, fp64_peak(stream),
                               f'k_cell_step<double> ({tune_plain[0]} slots)', args.workload)},
            'roofline': roof,
            'cpu_baseline': cpu,
            'e2e': {'value': e2e_val, 'unit': UNIT, 'h2d_bytes_per_step': int(h2d),
                    'd2h_bytes_per_step': int(d2h)},
            'gpu_launches': int(launches),
            'clocks': clk,
        }
        if configs is not None:
            line['configs'] = configs
        if extra is not None:
            line['secondary'] = extra
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
