"""The GPU cluster generator (bx_generate_cluster) against its NumPy/SciPy
restatement (oracle/generator.py, itself pinned to BETSE's Cells in
test_generator_betse.py) and against BETSE's own seed lattice.

* the seed lattice is BETSE's bit for bit (tests/golden/cells_lattice.npz);
* on the same radius and seed the GPU and the restatement build the same
  cluster: cell count, membrane count, CSR row pointers, gap-junction
  partners, boundary membranes, grid map and cell adjacency identical; the
  geometry (areas, normals, volumes, centres, R_rads, grid areas) within
  1e-12 relative (the restatement's hypot and atan2 are libm's, the GPU's
  CUDA's: they differ in the last bit now and then).
"""
import os
import time

import numpy as np
import pytest

import golden_io as gi

pytestmark = pytest.mark.gpu

LATTICE = {'r80_s1': (80e-6, 1), 'r50_s7': (50e-6, 7), 'r50_s3': (50e-6, 3)}
CLUSTERS = [(50e-6, 3), (80e-6, 1), (300e-6, 5), (662e-6, 11), (1450e-6, 3)]


@pytest.mark.parametrize('key', sorted(LATTICE))
def test_gpu_lattice_is_betse_bit_for_bit(key):
    from betse_gb300.generator import seed_lattice
    fx = np.load(os.path.join(gi.GOLDEN, 'cells_lattice.npz'))
    radius, seed = LATTICE[key]
    assert np.array_equal(seed_lattice(radius, seed), fx[f'{key}_xypts'])


def test_gpu_lattice_matches_numpy_at_size():
    from betse_gb300.generator import seed_lattice, world_size
    from oracle.generator import hex_lattice
    radius, seed = 1450e-6, 3
    wsx = world_size(radius)[1]
    ref = hex_lattice(wsx, wsx, 10e-6, 0.4, np.random.RandomState(seed))
    assert np.array_equal(seed_lattice(radius, seed), ref)


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize('radius,seed', CLUSTERS)
def test_gpu_cluster_equals_restatement(radius, seed):
    from betse_gb300.generator import make_cluster
    from oracle.generator import make_cluster as make_ref
    grid = 200 if radius == 662e-6 else 20
    t0 = time.perf_counter()
    got = make_cluster(radius, seed, grid_size=grid)
    t_gpu = time.perf_counter() - t0
    t0 = time.perf_counter()
    ref = make_ref(radius, seed, grid_size=grid)
    t_cpu = time.perf_counter() - t0
    g, r = got.geom, ref.geom
    print(f'\nR = {radius * 1e6:.0f} um seed {seed}: {g.n_cells} cells, {g.n_mems} membranes; '
          f'GPU {t_gpu * 1e3:.1f} ms (with host assembly), NumPy/SciPy {t_cpu * 1e3:.1f} ms')
    assert (g.n_cells, g.n_mems, g.grid_shape) == (r.n_cells, r.n_mems, r.grid_shape)
    for name in ('cell_mem_ptr', 'mem_to_cells', 'nn_i', 'bflag', 'map_mem2ecm', 'cell_nn_ptr', 'cell_nn'):
        assert np.array_equal(getattr(g, name), getattr(r, name)), name
    for name in ('mem_sa', 'mem_nx', 'mem_ny', 'cell_vol', 'cell_sa', 'diviterm', 'R_rads',
                 'smooth_weight_mem', 'mem_sa_per_env'):
        assert _rel(getattr(g, name), getattr(r, name)) < 1e-12, name
    assert _rel(got.cell_centres, ref.cell_centres) < 1e-12
    assert _rel(got.mem_mids, ref.mem_mids) < 1e-12
    for k in ('xmin', 'xmax', 'ymin', 'ymax', 'world'):
        assert getattr(got, k) == getattr(ref, k), k
    assert g.delta == r.delta


def test_gpu_generator_rejects_a_bad_spec():
    from betse_gb300 import _lib
    from betse_gb300.generator import gen_spec, _Generated
    spec = gen_spec(80e-6, 1)
    spec.grid_size = 1
    with pytest.raises(_lib.BxLibraryError, match='bad specification'):
        _Generated(spec)
