// bx_env.cuh -- environment-grid kernels (extracellular spaces and fields).
//
// The grid is row-major (ny, nx), k = i*nx + j, as FiniteDiffSolver.cell_grid
// lays it out (betse/science/math/finitediff.py:158-250).  Each kernel is one
// thread per grid cell; the work is a few hundred bytes per cell, HBM- or
// launch-bound, and runs inside the step's CUDA graph.
#pragma once
#include "bx_kernels.cuh"

namespace bx {

struct EnvConst {
  int I, ny, nx, G;
  double delta, inv_delta, inv_2delta, dt, sharpness;
  double np_alpha[kMaxIons];   // z q / (kb T)  (times D_env per cell)
  double zF[kMaxIons];
  double c_bound[kMaxIons];
  double surf_scale;           // cell_height delta^2 / mean(memSa_per_envSquare[map])
  double inv_koeoer;           // 1 / (ko_env eo er)
  double screen;               // (2/(ko_env delta)) (cell_radius/true_cell_size)
  double inv_h_d2;             // 1 / (cell_height delta^2)
  double gw[9];                // Gaussian taps, sigma 1, radius 4
};

__device__ __forceinline__ bool on_edge(int i, int j, int ny, int nx) {
  return i == 0 || j == 0 || i == ny - 1 || j == nx - 1;
}

// Boundary-set concentration (update_ecm sets the four edges, sim.py:2214-2217)
__device__ __forceinline__ double cb_at(const double* c, const EnvConst& e, int ion, int i, int j) {
  return on_edge(i, j, e.ny, e.nx) ? e.c_bound[ion] : c[(size_t)ion * e.G + i * e.nx + j];
}

// Nernst-Planck flux on the grid (update_ecm, sim.py:2219-2242;
// stb.nernst_planck_flux, sim_toolbox.py:385-413) with fd.gradient
// (finitediff.py:1236-1266).  E_env is the previous update_V's field.
// The grid kernels multiply by 1/delta and 1/(2 delta) where the reference
// divides (a difference of at most one rounding): an FP64 division costs
// GB300 several FP64-pipe operations, and the stencils are otherwise cheap.
// R = float is the split form's stencil: the concentration differences are
// taken in FP64 (the state) and scaled, with the drift term, in FP32.
// One thread per (ion, grid cell): t = ion*G + k.
template <typename R>
__global__ void k_env_np_flux(const double* __restrict__ cenv, const double* __restrict__ Denv,
                              const double* __restrict__ Ex, const double* __restrict__ Ey,
                              double* fx, double* fy, EnvConst e) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= e.I * e.G) return;
  const int ion = t / e.G, k = t - ion * e.G;
  const int i = k / e.nx, j = k - i * e.nx;
  {
    const double c0 = cb_at(cenv, e, ion, i, j);
    const R inv_d = (R)e.inv_delta, inv_2d = (R)e.inv_2delta;
    R gcx, gcy;
    if (j == 0) gcx = (R)(cb_at(cenv, e, ion, i, 1) - c0) * inv_d;
    else if (j == e.nx - 1) gcx = (R)(c0 - cb_at(cenv, e, ion, i, j - 1)) * inv_d;
    else gcx = -(R)(cb_at(cenv, e, ion, i, j - 1) - cb_at(cenv, e, ion, i, j + 1)) * inv_2d;
    if (i == 0) gcy = (R)(cb_at(cenv, e, ion, 1, j) - c0) * inv_d;
    else if (i == e.ny - 1) gcy = (R)(c0 - cb_at(cenv, e, ion, i - 1, j)) * inv_d;
    else gcy = -(R)(cb_at(cenv, e, ion, i - 1, j) - cb_at(cenv, e, ion, i + 1, j)) * inv_2d;
    const R D = (R)Denv[(size_t)ion * e.G + k];
    const R alpha = D * (R)e.np_alpha[ion];
    const R gvx = -(R)Ex[k], gvy = -(R)Ey[k];
    fx[(size_t)ion * e.G + k] = (double)(-D * gcx - alpha * gvx * (R)c0);
    fy[(size_t)ion * e.G + k] = (double)(-D * gcy - alpha * gvy * (R)c0);
  }
}

// fd.diff with the reference's flipped one-sided edge signs (finitediff.py:1268-1303)
template <typename R = double>
__device__ __forceinline__ R ddx_neg(const double* f, const EnvConst& e, int i, int j) {
  // diff(-f, axis=0)
  const double* r = f + i * e.nx;
  const R inv_d = (R)e.inv_delta, inv_2d = (R)e.inv_2delta;
  if (j == 0) return ((-(R)r[0]) - (-(R)r[1])) * inv_d;
  if (j == e.nx - 1) return ((-(R)r[j - 1]) - (-(R)r[j])) * inv_d;
  return -((-(R)r[j - 1]) - (-(R)r[j + 1])) * inv_2d;
}
template <typename R = double>
__device__ __forceinline__ R ddy_neg(const double* f, const EnvConst& e, int i, int j) {
  // diff(-f, axis=1)
  const int nx = e.nx;
  const R inv_d = (R)e.inv_delta, inv_2d = (R)e.inv_2delta;
  if (i == 0) return -((-(R)f[nx + j]) - (-(R)f[j])) * inv_d;
  if (i == e.ny - 1) return -((-(R)f[i * nx + j]) - (-(R)f[(i - 1) * nx + j])) * inv_d;
  return -((-(R)f[(i - 1) * nx + j]) - (-(R)f[(i + 1) * nx + j])) * inv_2d;
}

// Environment charge of grid cell k from its new concentrations, for
// get_current's ECM branch (ion_current.py:82-92): rho = sum_i F z_i c_i (ions
// in order) and, on the membrane-touched cells, the surface-charge potential
// source v = (rho surf_scale) / (ko_env eo er); written by the kernel that
// produces the cell's final concentrations.
__device__ __forceinline__ void env_charge_out(int k, double rho, const uint8_t* touched, double* vsrc,
                                               double* rho_env, const EnvConst& e) {
  vsrc[k] = touched[k] ? (rho * e.surf_scale) * e.inv_koeoer : 0.0;
  if (rho_env) rho_env[k] = rho;
}

// c <- cb + div(-f) dt  [+ membrane exchange if FUSE_SCATTER]
// (update_ecm sim.py:2247-2254, then update_Co's ECM term sim_toolbox.py:1189-1195
//  with div_env = M_divmap_mem2ecm @ (-flux) / (cell_height delta^2), :1229-1232).
// One thread per (ion, grid cell); while the new concentration is written in
// place, the kernel reads only fluxes and its own cell's value.
template <bool FUSE_SCATTER>
__global__ void k_env_update(double* cenv, double* tmp, const double* __restrict__ fx,
                             const double* __restrict__ fy, const int* __restrict__ env_ptr,
                             const int* __restrict__ env_mem, const double* __restrict__ mem_flux_sa,
                             int M, EnvConst e) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= e.I * e.G) return;
  const int ion = t / e.G, k = t - ion * e.G;
  const int i = k / e.nx, j = k - i * e.nx;
  {
    const double* fxi = fx + (size_t)ion * e.G;
    const double* fyi = fy + (size_t)ion * e.G;
    const double div = ddx_neg(fxi, e, i, j) + ddy_neg(fyi, e, i, j);
    double c = cb_at(cenv, e, ion, i, j) + div * e.dt;
    if (FUSE_SCATTER) {
      double s = 0.0;
      for (int q = env_ptr[k]; q < env_ptr[k + 1]; ++q) s += -mem_flux_sa[(size_t)ion * M + env_mem[q]];
      c = c + (s * e.inv_h_d2) * e.dt;
      cenv[(size_t)ion * e.G + k] = c;
    } else {
      tmp[(size_t)ion * e.G + k] = c;
    }
  }
}

// The environment charge of each grid cell from its final concentrations
// (ions in order), for get_current's ECM branch.
__global__ void k_env_charge(const double* __restrict__ cenv, const uint8_t* __restrict__ touched, double* vsrc,
                             double* rho_env, EnvConst e) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= e.G) return;
  double rho = 0.0;
  for (int ion = 0; ion < e.I; ++ion) rho += e.zF[ion] * cenv[(size_t)ion * e.G + k];
  env_charge_out(k, rho, touched, vsrc, rho_env, e);
}

// fd.integrator (finitediff.py:1479-1512) when sharpness < 1, then the membrane
// exchange (SCATTER; without it the smoothed grid is written to cenv, which is
// then a separate buffer).  One thread per (ion, grid cell).
template <bool SCATTER = true>
__global__ void k_env_integrate_scatter(double* cenv, const double* __restrict__ tmp,
                                        const int* __restrict__ env_ptr, const int* __restrict__ env_mem,
                                        const double* __restrict__ mem_flux_sa, int M, EnvConst e) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= e.I * e.G) return;
  const int ion = t / e.G, k = t - ion * e.G;
  const int i = k / e.nx, j = k - i * e.nx;
  const double sides = (1 - e.sharpness) / 4;
  {
    const double* P = tmp + (size_t)ion * e.G;
    double F;
    if (on_edge(i, j, e.ny, e.nx)) {
      F = P[k];
    } else {
      F = e.sharpness * P[k];
      F += sides * P[k + e.nx];
      F += sides * P[k - e.nx];
      F += sides * P[k + 1];
      F += sides * P[k - 1];
    }
    if (!SCATTER) {
      cenv[(size_t)ion * e.G + k] = F;
      return;
    }
    double s = 0.0;
    for (int q = env_ptr[k]; q < env_ptr[k + 1]; ++q) s += -mem_flux_sa[(size_t)ion * M + env_mem[q]];
    cenv[(size_t)ion * e.G + k] = F + (s * e.inv_h_d2) * e.dt;
  }
}

// The membrane exchange onto an environment already advanced by the
// Nernst-Planck update (and smoothing): update_Co's ECM term
// (sim_toolbox.py:1185-1200), the same arithmetic as the fused kernels.
__global__ void k_env_scatter_add(double* cenv, const double* __restrict__ src,
                                  const int* __restrict__ env_ptr, const int* __restrict__ env_mem,
                                  const double* __restrict__ mem_flux_sa, int M, EnvConst e) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= e.I * e.G) return;
  const int ion = t / e.G, k = t - ion * e.G;
  double s = 0.0;
  for (int q = env_ptr[k]; q < env_ptr[k + 1]; ++q) s += -mem_flux_sa[(size_t)ion * M + env_mem[q]];
  cenv[t] = src[t] + (s * e.inv_h_d2) * e.dt;
}

// get_current ECM branch (ion_current.py:79-110): the axis-0 pass of a
// sigma=1 Gaussian with zero padding (scipy mode='constant') over the
// potential source the concentration kernel left in vsrc.
__global__ void k_env_gauss_y(const double* __restrict__ vsrc, double* tmp, EnvConst e) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= e.G) return;
  const int i = k / e.nx, j = k - i * e.nx;
  double acc = 0.0;
#pragma unroll
  for (int q = -4; q <= 4; ++q) {
    const int ii = i + q;
    if (ii < 0 || ii >= e.ny) continue;
    acc += e.gw[q + 4] * vsrc[ii * e.nx + j];
  }
  tmp[k] = acc;
}

// axis-1 pass of the Gaussian (+ Phi_b) -> v_env
__global__ void k_env_gauss_x(const double* __restrict__ tmp, const double* __restrict__ phib,
                              double* venv, EnvConst e) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= e.G) return;
  const int i = k / e.nx, j = k - i * e.nx;
  double acc = 0.0;
  for (int q = -4; q <= 4; ++q) {
    const int jj = j + q;
    if (jj < 0 || jj >= e.nx) continue;
    acc += e.gw[q + 4] * tmp[i * e.nx + jj];
  }
  venv[k] = acc + (phib ? phib[k] : 0.0);
}

// E = -gradient(scale * F)  (fd.gradient, finitediff.py:1236-1266)
__global__ void k_env_neg_grad(const double* __restrict__ F, double scale, double* Ex, double* Ey,
                               EnvConst e) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= e.G) return;
  const int i = k / e.nx, j = k - i * e.nx;
  const int nx = e.nx;
  auto f = [&](int a, int bb) { return scale * F[a * nx + bb]; };
  double gx, gy;
  if (j == 0) gx = (f(i, 1) - f(i, 0)) * e.inv_delta;
  else if (j == nx - 1) gx = (f(i, j) - f(i, j - 1)) * e.inv_delta;
  else gx = -(f(i, j - 1) - f(i, j + 1)) * e.inv_2delta;
  if (i == 0) gy = (f(1, j) - f(0, j)) * e.inv_delta;
  else if (i == e.ny - 1) gy = (f(i, j) - f(i - 1, j)) * e.inv_delta;
  else gy = -(f(i - 1, j) - f(i + 1, j)) * e.inv_2delta;
  Ex[k] = -gx;
  Ey[k] = -gy;
}

// ---------------------------------------------------------------------------
// Fused forms of the sequences above, for the common configuration (no
// Ca-ATPase, sharpness >= 1): fewer launches on a grid that is small against
// the GPU, the same arithmetic term by term.
// ---------------------------------------------------------------------------

// k_env_update<true> and k_env_charge in one launch.  Eight lanes per grid
// cell (lane = ion, I <= 8): each lane advances its ion's concentration in
// place (it reads only fluxes and its own cell's value), then the cell's
// group sums F z_i c_i over the ions in order through shuffles.
// R = float (split form): the divergence of the FP32 fluxes in FP32; the
// concentration, the membrane exchange and the charge stay FP64.
template <typename R>
__global__ void __launch_bounds__(256) k_env_update_charge(double* cenv, const double* __restrict__ fx,
                                                           const double* __restrict__ fy,
                                                           const int* __restrict__ env_ptr,
                                                           const int* __restrict__ env_mem,
                                                           const double* __restrict__ mem_flux_sa, int M,
                                                           const uint8_t* __restrict__ touched, double* vsrc,
                                                           double* rho_env, EnvConst e) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = t >> 3, ion = t & 7;
  const bool live = k < e.G && ion < e.I;
  double zc = 0.0;
  if (live) {
    const int i = k / e.nx, j = k - i * e.nx;
    const double* fxi = fx + (size_t)ion * e.G;
    const double* fyi = fy + (size_t)ion * e.G;
    const R div = ddx_neg<R>(fxi, e, i, j) + ddy_neg<R>(fyi, e, i, j);
    double c = cb_at(cenv, e, ion, i, j) + (double)(div * (R)e.dt);
    // the membrane exchange: indices, then values, four at a time (the
    // loads of a batch are independent), added in list order
    double s = 0.0;
    const int q1 = env_ptr[k + 1];
    const double* mf = mem_flux_sa + (size_t)ion * M;
    for (int q0 = env_ptr[k]; q0 < q1; q0 += 4) {
      int mm[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) mm[u] = q0 + u < q1 ? env_mem[q0 + u] : -1;
      double fv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) fv[u] = mm[u] >= 0 ? mf[mm[u]] : 0.0;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (mm[u] >= 0) s += -fv[u];
    }
    c = c + (s * e.inv_h_d2) * e.dt;
    cenv[(size_t)ion * e.G + k] = c;
    zc = e.zF[ion] * c;
  }
  // the group of cell k: lanes 8 (k mod 4) .. +7 of this warp
  const int base = threadIdx.x & 24;
  double rho = 0.0;
  for (int q = 0; q < e.I; ++q) {
    const double v = __shfl_sync(0xffffffffu, zc, base + q);
    rho += v;
  }
  if (live && ion == 0) env_charge_out(k, rho, touched, vsrc, rho_env, e);
}

// k_env_gauss_y, k_env_gauss_x (+ Phi_b) and k_env_neg_grad in one launch:
// each CTA computes a kEnvTX x kEnvTY tile of E_env (and v_env) from the
// potential source in shared memory, with the halos the two Gaussian passes
// (4 cells) and the gradient (1 cell) need.
constexpr int kEnvTX = 32, kEnvTY = 16;
constexpr int kEnvVX = kEnvTX + 2, kEnvVY = kEnvTY + 2;        // v_env tile (gradient halo)
constexpr int kEnvSX = kEnvVX + 8, kEnvSY = kEnvVY + 8;        // source tile (Gaussian halo)
// R = float (split form): both passes and the gradient in FP32.
template <typename R>
__global__ void __launch_bounds__(kEnvTX * kEnvTY) k_env_fields_tile(const double* __restrict__ vsrc,
                                                                     const double* __restrict__ phib,
                                                                     double* venv, double scale, double* Ex,
                                                                     double* Ey, EnvConst e) {
  __shared__ R src[kEnvSY][kEnvSX];
  __shared__ R gy[kEnvVY][kEnvSX];
  __shared__ R v[kEnvVY][kEnvVX];
  const int i0 = blockIdx.y * kEnvTY - 1 - 4, j0 = blockIdx.x * kEnvTX - 1 - 4;   // src tile origin
  const int nt = blockDim.x;
  for (int q = threadIdx.x; q < kEnvSY * kEnvSX; q += nt) {
    const int a = q / kEnvSX, b = q - a * kEnvSX, i = i0 + a, j = j0 + b;
    src[a][b] = (i >= 0 && i < e.ny && j >= 0 && j < e.nx) ? (R)vsrc[i * e.nx + j] : (R)0;
  }
  __syncthreads();
  // axis-0 pass (zero padding: taps outside the grid are skipped, as k_env_gauss_y does)
  for (int q = threadIdx.x; q < kEnvVY * kEnvSX; q += nt) {
    const int a = q / kEnvSX, b = q - a * kEnvSX, i = i0 + 4 + a;
    R acc = 0;
#pragma unroll
    for (int w = -4; w <= 4; ++w) {
      const int ii = i + w;
      if (ii < 0 || ii >= e.ny) continue;
      acc += (R)e.gw[w + 4] * src[a + 4 + w][b];
    }
    gy[a][b] = acc;
  }
  __syncthreads();
  // axis-1 pass + Phi_b -> v_env on the tile and its one-cell halo
  for (int q = threadIdx.x; q < kEnvVY * kEnvVX; q += nt) {
    const int a = q / kEnvVX, b = q - a * kEnvVX, i = i0 + 4 + a, j = j0 + 4 + b;
    R acc = 0;
    for (int w = -4; w <= 4; ++w) {
      const int jj = j + w;
      if (jj < 0 || jj >= e.nx) continue;
      acc += (R)e.gw[w + 4] * gy[a][b + 4 + w];
    }
    const bool in = i >= 0 && i < e.ny && j >= 0 && j < e.nx;
    v[a][b] = in ? acc + (phib ? (R)phib[i * e.nx + j] : (R)0) : (R)0;
  }
  __syncthreads();
  // E = -gradient(scale * v_env), one-sided on the grid edges
  const int a = threadIdx.x / kEnvTX + 1, b = threadIdx.x % kEnvTX + 1;
  const int i = blockIdx.y * kEnvTY + a - 1, j = blockIdx.x * kEnvTX + b - 1;
  if (i >= e.ny || j >= e.nx) return;
  const int k = i * e.nx + j;
  venv[k] = (double)v[a][b];
  const R sc = (R)scale, inv_d = (R)e.inv_delta, inv_2d = (R)e.inv_2delta;
  auto f = [&](int da, int db) { return sc * v[a + da][b + db]; };
  R gx, gyy;
  if (j == 0) gx = (f(0, 1) - f(0, 0)) * inv_d;
  else if (j == e.nx - 1) gx = (f(0, 0) - f(0, -1)) * inv_d;
  else gx = -(f(0, -1) - f(0, 1)) * inv_2d;
  if (i == 0) gyy = (f(1, 0) - f(0, 0)) * inv_d;
  else if (i == e.ny - 1) gyy = (f(0, 0) - f(-1, 0)) * inv_d;
  else gyy = -(f(-1, 0) - f(1, 0)) * inv_2d;
  Ex[k] = (double)(-gx);
  Ey[k] = (double)(-gyy);
}

// ---------------------------------------------------------------------------
// Dense FP64 products Y[n x R] = A[n x n] X[n x R], R <= 4 (row-major).
// One warp per row; the row streams from HBM with 16-byte loads, X is
// L2-resident.  The HBM-bound form of np.dot(lapENVinv, .).
// ---------------------------------------------------------------------------
template <int R>
__global__ void __launch_bounds__(256) k_dense_rows(const double* __restrict__ A, const double* __restrict__ X,
                                                    double* __restrict__ Y, int n) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const double* row = A + (size_t)warp * n;
  double acc[R];
#pragma unroll
  for (int r = 0; r < R; ++r) acc[r] = 0.0;
  const bool al16 = ((reinterpret_cast<uintptr_t>(row) & 15) == 0);
  int k0 = 0;
  if (al16) {
    const int n2 = n >> 1;
    const double2* row2 = reinterpret_cast<const double2*>(row);
    for (int q = lane; q < n2; q += 32) {
      const double2 a = __ldcs(row2 + q);
      const int kk = 2 * q;
#pragma unroll
      for (int r = 0; r < R; ++r) acc[r] += a.x * X[(size_t)kk * R + r] + a.y * X[(size_t)(kk + 1) * R + r];
    }
    k0 = 2 * n2;
  }
  for (int kk = k0 + lane; kk < n; kk += 32) {
    const double a = row[kk];
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] += a * X[(size_t)kk * R + r];
  }
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const double s = warp_sum(acc[r]);
    if (lane == 0) Y[(size_t)warp * R + r] = s;
  }
}

}  // namespace bx
