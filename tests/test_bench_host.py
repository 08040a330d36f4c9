"""bench.py's roofline arithmetic on CPU (no GPU): the per-array step bytes,
the HBM entry on the step's bytes with the kernel's own bytes beside it, and
the FP64 entry from the committed instruction counts, including the fallback
to another tile size of the same kernel and the refusal to invent a count."""
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

PEAK = {'warp_inst_per_s': 16.0e9, 'fma_tflops': 1.024, 'ms': 10.0, 'launch': 'probe'}


def test_step_bytes_counts_each_array_once():
    C, M, G = 100, 600, 400
    assert bench.step_bytes('fp64', C, M) == 104 * M + 124 * C
    assert bench.step_bytes('split', C, M) == 64 * M + 112 * C
    assert bench.step_bytes('fp64', C, M, G, ecm=True) == 104 * M + 124 * C + 4 * M + 160 * G


def test_hbm_entry_uses_the_step_bytes():
    hbm, _ = bench.peaks()
    r = bench.roofline_entry(25.0e6, 10e-6, 'k', step=50.0e6)
    assert r['algorithmic_bytes_per_step'] == 50_000_000
    assert r['achieved'] == pytest.approx(50.0e6 / 10e-6 / 1e9)
    assert r['frac'] == pytest.approx(r['achieved'] / hbm)
    assert r['frac_on_kernel_bytes'] == pytest.approx(r['frac'] / 2)


def test_fp64_entry_from_the_committed_counts():
    counts = json.load(open(os.path.join(ROOT, 'profiles', 'fp64_counts.json')))['kernels']
    e = counts['cluster100k']['k_cell_step<double> (128 slots)']
    per_mem = e['fp64_warp_inst_per_launch'] / e['membranes']
    r = bench.fp64_roofline(0.5, 1000, PEAK, 'k_cell_step<double> (128 slots)', 'cluster100k')
    assert r['bound'] == 'fp64' and 'count_of' not in r
    assert r['fp64_warp_inst_per_launch'] == int(per_mem * 1000)
    assert r['achieved'] == pytest.approx(per_mem * 1000 / 0.5e-3 / 1e9)
    assert r['frac'] == pytest.approx(r['achieved'] / 16.0)
    # another tile size of the tile kernel takes the same count per membrane
    r2 = bench.fp64_roofline(0.5, 1000, PEAK, 'k_cell_step<double> (256 slots)', 'cluster100k')
    assert r2['achieved'] == pytest.approx(r['achieved'])
    assert r2['count_of'].startswith('k_cell_step<double> (128 slots)')


def test_fp64_entry_without_a_count_reports_none():
    r = bench.fp64_roofline(0.02, 1426, PEAK, 'k_cell_step_ion<8>', 'plain250')
    assert r['achieved'] is None and r['frac'] is None and 'no FP64 instruction count' in r['note']
    r = bench.fp64_roofline(0.02, 1426, PEAK, 'k_cell_step_ion<16>', 'no-such-workload')
    assert r['achieved'] is None
