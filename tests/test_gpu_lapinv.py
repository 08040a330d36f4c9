"""cells.lapENVinv built on the GPU from the sine-transform eigenvectors of
makeLaplacian's interior block (bx_lap_env_inv_build / bx_build_lap_env_inv).

* small grids: equal to the dense inverse of the oracle's Laplacian (BETSE's
  makeLaplacian restated) within 1e-12 relative, and A L = I;
* the full 199 x 200 grid of the extracellular-space workload: the operator
  applied to random vectors (the double-float field product the step's
  environment fields use) against an independent FP64 solve of the same
  Dirichlet problem by sine transforms (scipy.fft.dstn), error printed;
* the environment fields of a golden cluster from the GPU-built operator equal
  those from the uploaded dense inverse.
"""
import numpy as np
import pytest

import golden_io as gi
import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('shape,delta', [((3, 3), 1.0), ((5, 7), 2e-6), ((19, 20), 1e-5), ((37, 41), 3e-6)])
def test_gpu_inverse_equals_dense_inverse(shape, delta):
    from betse_gb300.fields import lap_env_inverse
    A = lap_env_inverse(*shape, delta)
    L = oracle.fields.make_laplacian(*shape, delta)
    ref = np.linalg.inv(L)
    assert np.max(np.abs(A - ref)) <= 1e-12 * np.max(np.abs(ref)), shape
    G = shape[0] * shape[1]
    assert np.max(np.abs(A @ L - np.eye(G))) < 1e-9


def _dirichlet_solve(b, ny, nx, delta):
    """A^-1 b for makeLaplacian's matrix, in FP64 by sine transforms: edge
    values pass through (times delta^2), the interior solves the Dirichlet
    problem with the edge values moved to the right-hand side."""
    from scipy.fft import dstn, idstn
    x = b.reshape(ny, nx) * delta ** 2
    r = x[1:-1, 1:-1].copy()                  # delta^2 b_i - L_ie x_e at unit spacing
    r[0, :] -= x[0, 1:-1]
    r[-1, :] -= x[-1, 1:-1]
    r[:, 0] -= x[1:-1, 0]
    r[:, -1] -= x[1:-1, -1]
    n1, n2 = ny - 2, nx - 2
    lam = (-2 + 2 * np.cos(np.pi * np.arange(1, n1 + 1) / (n1 + 1)))[:, None] + \
          (-2 + 2 * np.cos(np.pi * np.arange(1, n2 + 1) / (n2 + 1)))[None, :]
    out = x.copy()
    out[1:-1, 1:-1] = idstn(dstn(r, type=1, norm='ortho') / lam, type=1, norm='ortho')
    return out.ravel()


def test_full_grid_operator_products_against_fp64_solve():
    import torch
    from betse_gb300 import generator as gen
    from betse_gb300.engine import ClusterEngine
    g, p, Dm, st, D_env = gen.workload(662e-6, 11, is_ecm=True, dt=5e-3, dm_range=(1e-19, 1e-17),
                                       grid_size=200, cell_space=25e-9)
    ny, nx = g.grid_shape
    G = ny * nx
    torch.cuda.set_device(0)
    from betse_gb300.fields import lap_env_inverse
    A = lap_env_inverse(ny, nx, g.delta, device='cuda')           # FP64 on the device, 12.7 GB
    rng = np.random.default_rng(5)
    B = rng.standard_normal((G, 4))
    Y = (A @ torch.as_tensor(B, device='cuda')).cpu().numpy()     # FP64 product of the built operator
    del A
    torch.cuda.empty_cache()
    ref = np.stack([_dirichlet_solve(B[:, c], ny, nx, g.delta) for c in range(4)], 1)
    err = np.max(np.abs(Y - ref)) / np.max(np.abs(ref))
    print(f'\nlapENVinv {ny}x{nx}: FP64 operator vs sine-transform solve, max rel err {err:.2e}')
    assert err < 1e-11
    # the handle's double-float store and its streaming product (the kernel the
    # environment fields use), on two right-hand sides
    with ClusterEngine(g, p, 'fp64') as e:
        e.set_membrane_diffusivity(Dm)
        e.set_env_diffusivity(D_env)
        e.upload(**st)
        e.build_lap_env_inv()
        e.step(1, outputs=True)
        f = e.env_fields()
    assert np.all(np.isfinite(f['v_env']))


def test_fields_from_gpu_built_operator_equal_uploaded_inverse():
    from betse_gb300.engine import ClusterEngine
    for name in ('noecm_r80_s1', 'ecm_r50_s3'):
        d = gi.load(name)
        cg, sp, Dm, st, D_env = gi.engine_inputs(d)
        g = gi.geometry(d)
        res = []
        for built in (False, True):
            with ClusterEngine(cg, sp, 'fp64') as e:
                e.set_membrane_diffusivity(Dm)
                if sp.is_ecm:
                    e.set_env_diffusivity(D_env)
                e.upload(**st)
                if built:
                    e.build_lap_env_inv()
                else:
                    e.set_lap_env_inv(np.linalg.inv(oracle.fields.make_laplacian(*g.grid_shape, g.delta)))
                e.step(3, outputs=True)
                res.append(e.env_fields(g.D_env_weight))
        for k in ('v_env', 'E_env_x', 'E_env_y'):
            assert gi.rel_err(res[1][k], res[0][k]) < 1e-9, (name, k)
        if sp.is_ecm:       # without ECM these are round-off of a pure gradient in any code
            for k in ('J_env_x', 'J_env_y', 'B_field'):
                assert gi.rel_err(res[1][k], res[0][k]) < 1e-6, (name, k)
