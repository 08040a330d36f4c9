// bx_fields.cuh -- the environment fields of get_current, computed on demand.
//
// get_current (betse/science/physics/ion_current.py:50-171) ends every step
// with environment fields that no later step reads (apart from E_env with
// extracellular spaces, which the step itself keeps): v_env, E_env, J_env and
// B_field.  They are observed only where a caller stores them (write2storage,
// betse/science/sim.py:1789-1884), so the library computes them when asked,
// from the state the last step left: no per-step cost, and the two dense
// lapENVinv products per Helmholtz-Hodge split run only at sampled steps.
//
// The products y = lapENVinv @ x are streaming matrix-vector products with two
// right-hand sides.  GB300's FP64 pipe cannot keep up with HBM on them (two
// FP64 FMAs per 8-byte element need ~3.4 TFLOP/s at full bandwidth), so the
// matrix is stored once as a double-float pair per element -- (hi, lo) FP32,
// the same 8 bytes as FP64 and ~48 significand bits -- and the products run on
// the FP32 pipe with error-free transformations (TwoProduct via FMA, TwoSum;
// Dekker 1971, Knuth TAOCP vol. 2 4.2.2), accumulating in double-float.
#pragma once
#include "bx_kernels.cuh"

namespace bx {

// ---------------------------------------------------------------------------
// double-float operator storage
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 split_df(double a) {
  const float hi = __double2float_rn(a);
  const float lo = __double2float_rn(a - (double)hi);
  return make_float2(hi, lo);
}

// (sh, sl) += (ah + al) * (xh + xl), dropping al*xl (below 2^-48 relative).
__device__ __forceinline__ void df_dot_acc(float& sh, float& sl, float ah, float al, float xh, float xl) {
  const float p = __fmul_rn(ah, xh);
  float e = __fmaf_rn(ah, xh, -p);  // exact low part of ah*xh
  e = __fmaf_rn(ah, xl, e);
  e = __fmaf_rn(al, xh, e);
  const float s = __fadd_rn(sh, p);  // TwoSum(sh, p)
  const float bb = __fsub_rn(s, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  sh = s;
  sl = __fadd_rn(sl, __fadd_rn(err, e));
}

// rows of src (n doubles each) -> double-float rows of pitch ld >= n, the
// columns [n, ld) zeroed
__global__ void k_to_df_rows(const double* __restrict__ src, int nrows, int n, float2* __restrict__ dst, int ld) {
  const size_t tot = (size_t)nrows * ld;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const size_t r = e / ld;
    const int c = (int)(e - r * ld);
    dst[e] = c < n ? split_df(src[r * n + c]) : make_float2(0.f, 0.f);
  }
}

// Y[n x 2] = A X with A [n][ld] double-float (ld even, zero-padded columns, so
// every row is 16-byte aligned and holds ld/2 element pairs) and X [ld][2]
// double-float (zero-padded rows).  ROWS rows per warp: each 16-byte load of X
// feeds all of them, dividing X traffic per operator byte by ROWS; four
// pieces of each row in flight per lane.
template <int ROWS>
__global__ void __launch_bounds__(256) k_dense_rows2_df(const float2* __restrict__ A, int ld,
                                                        const float2* __restrict__ X, double* __restrict__ Y,
                                                        int n) {
  const int warp = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  const int r0 = ROWS * warp;
  if (r0 >= n) return;
  const float4* ap[ROWS];
#pragma unroll
  for (int rr = 0; rr < ROWS; ++rr)
    ap[rr] = reinterpret_cast<const float4*>(A + (size_t)(r0 + rr < n ? r0 + rr : r0) * ld);
  const float4* x4 = reinterpret_cast<const float4*>(X);   // x4[k] = (hi0, lo0, hi1, lo1) of element k
  float sh[ROWS][2], sl[ROWS][2];
#pragma unroll
  for (int rr = 0; rr < ROWS; ++rr) sh[rr][0] = sh[rr][1] = sl[rr][0] = sl[rr][1] = 0.f;
  const int npair = ld >> 1;
  auto consume = [&](const float4 (&a)[ROWS], int q) {
    const float4 xa = __ldg(x4 + 2 * q);       // element 2q
    const float4 xb = __ldg(x4 + 2 * q + 1);   // element 2q + 1
#pragma unroll
    for (int rr = 0; rr < ROWS; ++rr) {
      df_dot_acc(sh[rr][0], sl[rr][0], a[rr].x, a[rr].y, xa.x, xa.y);
      df_dot_acc(sh[rr][1], sl[rr][1], a[rr].x, a[rr].y, xa.z, xa.w);
      df_dot_acc(sh[rr][0], sl[rr][0], a[rr].z, a[rr].w, xb.x, xb.y);
      df_dot_acc(sh[rr][1], sl[rr][1], a[rr].z, a[rr].w, xb.z, xb.w);
    }
  };
  int q = lane;
  for (; q + 96 < npair; q += 128) {
    float4 a[4][ROWS];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int rr = 0; rr < ROWS; ++rr) a[u][rr] = __ldcs(ap[rr] + q + 32 * u);
#pragma unroll
    for (int u = 0; u < 4; ++u) consume(a[u], q + 32 * u);
  }
  for (; q < npair; q += 32) {
    float4 a[ROWS];
#pragma unroll
    for (int rr = 0; rr < ROWS; ++rr) a[rr] = __ldcs(ap[rr] + q);
    consume(a, q);
  }
#pragma unroll
  for (int rr = 0; rr < ROWS; ++rr) {
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const double v = warp_sum((double)sh[rr][c] + (double)sl[rr][c]);
      if (lane == 0 && r0 + rr < n) Y[(size_t)(r0 + rr) * 2 + c] = v;
    }
  }
}
constexpr int kDenseRows = 4;   // rows per warp of the lapENVinv product

// ---------------------------------------------------------------------------
// field stencils on the (ny, nx) grid, k = i*nx + j
// ---------------------------------------------------------------------------
struct ZF {
  double v[kMaxIons];  // F z_i per ion
};

struct FieldGrid {
  int ny, nx, G;
  double delta;
  double gw[9];  // Gaussian taps, sigma 1, radius 4 (scipy.ndimage.gaussian_filter)
};

// Local field potential source without extracellular spaces
// (ion_current.py:118-124): vce[map_mem2ecm] = (vm/2)[mem_to_cells] -- the
// membrane vector vm/2 indexed with the CELL index of each membrane, numpy's
// repeated-index assignment keeping the last membrane of a grid cell
// (last_mem[k], -1 if none).  Writes Phi = -vce.
__global__ void k_fields_vce(int G, const int* __restrict__ last_mem, const int* __restrict__ m2c,
                             const double* __restrict__ vm, double* __restrict__ neg_vce) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= G) return;
  const int m = last_mem[k];
  neg_vce[k] = (m >= 0) ? -(vm[m2c[m]] / 2) : 0.0;
}

// One axis of the sigma = 1 Gaussian.  REFLECT: scipy mode 'reflect'
// (half-sample symmetric, repeated for axes shorter than the radius);
// otherwise mode 'constant' with zeros.  Taps are summed from -4 to +4.
template <bool REFLECT>
__global__ void k_fields_gauss(const double* __restrict__ in, double* __restrict__ out, int axis, FieldGrid g) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.G) return;
  const int i = k / g.nx, j = k - i * g.nx;
  const int n = axis == 0 ? g.ny : g.nx;
  const int pos = axis == 0 ? i : j;
  double acc = 0.0;
#pragma unroll
  for (int t = -4; t <= 4; ++t) {
    int r = pos + t;
    if (REFLECT) {
      while (r < 0 || r >= n) r = (r < 0) ? -r - 1 : 2 * n - r - 1;
    } else if (r < 0 || r >= n) {
      continue;
    }
    acc += g.gw[t + 4] * in[axis == 0 ? r * g.nx + j : i * g.nx + r];
  }
  out[k] = acc;
}

// fd.gradient (finitediff.py:1236-1266) of scale*F at (i, j), stride-s reads
__device__ __forceinline__ void fd_grad(const double* F, int s, double scale, int i, int j, const FieldGrid& g,
                                        double& gx, double& gy) {
  auto f = [&](int a, int b) { return scale * F[(size_t)(a * g.nx + b) * s]; };
  const double d = g.delta;
  if (j == 0) gx = (f(i, 1) - f(i, 0)) / d;
  else if (j == g.nx - 1) gx = (f(i, j) - f(i, j - 1)) / d;
  else gx = -(f(i, j - 1) - f(i, j + 1)) / (2 * d);
  if (i == 0) gy = (f(1, j) - f(0, j)) / d;
  else if (i == g.ny - 1) gy = (f(i, j) - f(i - 1, j)) / d;
  else gy = -(f(i - 1, j) - f(i + 1, j)) / (2 * d);
}

// (gx, gy) = gradient(scale * F)
__global__ void k_fields_grad(const double* __restrict__ F, double scale, double* __restrict__ gx,
                              double* __restrict__ gy, FieldGrid g) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.G) return;
  double a, b;
  fd_grad(F, 1, scale, k / g.nx, k % g.nx, g, a, b);
  gx[k] = a;
  gy[k] = b;
}

// fd.diff along x / y at an interior point (edges are overwritten by the
// caller: HH_Decomp zeroes them, sim_toolbox.py:1256-1259, 1276-1280)
__device__ __forceinline__ double ddx_in(const double* F, double s, int i, int j, const FieldGrid& g) {
  return -(s * F[i * g.nx + j - 1] - s * F[i * g.nx + j + 1]) / (2 * g.delta);
}
__device__ __forceinline__ double ddy_in(const double* F, double s, int i, int j, const FieldGrid& g) {
  return -(s * F[(i - 1) * g.nx + j] - s * F[(i + 1) * g.nx + j]) / (2 * g.delta);
}

// Right-hand sides of HH_Decomp (sim_toolbox.py:1236-1290) as a two-column
// double-float operand: column 0 = -div(-Jy, Jx), column 1 = div(Jx, Jy), both
// zero on the grid edge (no applied boundary voltage: bound_V = 0,
// sim.py:702-706).
__global__ void k_fields_hh_rhs(const double* __restrict__ Jx, const double* __restrict__ Jy,
                                float2* __restrict__ X, FieldGrid g) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.G) return;
  const int i = k / g.nx, j = k - i * g.nx;
  double r0 = 0.0, r1 = 0.0;
  if (!(i == 0 || j == 0 || i == g.ny - 1 || j == g.nx - 1)) {
    const double divJr = ddx_in(Jy, -1.0, i, j, g) + ddy_in(Jx, 1.0, i, j, g);
    const double divJd = ddx_in(Jx, 1.0, i, j, g) + ddy_in(Jy, 1.0, i, j, g);
    r0 = -divJr;
    r1 = divJd;
  }
  X[2 * k] = split_df(r0);
  X[2 * k + 1] = split_df(r1);
}

// From Y[k] = (AA, BB): AA_out = aa_scale*AA (if asked), (Fx, Fy) =
// (-dAA/dy, dAA/dx), (Gx, Gy) = grad BB (if asked).
__global__ void k_fields_hh_out(const double* __restrict__ Y, double aa_scale, double* __restrict__ AA_out,
                                double* __restrict__ Fx, double* __restrict__ Fy, double* __restrict__ Gx,
                                double* __restrict__ Gy, FieldGrid g) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.G) return;
  const int i = k / g.nx, j = k - i * g.nx;
  double ax, ay;
  fd_grad(Y, 2, 1.0, i, j, g, ax, ay);
  if (AA_out) AA_out[k] = aa_scale * Y[2 * k];
  Fx[k] = -ay;
  Fy[k] = ax;
  if (Gx) {
    double bx_, by_;
    fd_grad(Y + 1, 2, 1.0, i, j, g, bx_, by_);
    Gx[k] = bx_;
    Gy[k] = by_;
  }
}

// smooth_flux reconstruction and the environment current without
// extracellular spaces (ion_current.py:133-145):
// E = -(Fr + Fd); J = sigma * E * D_env_weight.
__global__ void k_fields_e_and_j(int G, const double* __restrict__ Frx, const double* __restrict__ Fry,
                                 const double* __restrict__ Fdx, const double* __restrict__ Fdy,
                                 const double* __restrict__ w, double sigma, double* __restrict__ Ex,
                                 double* __restrict__ Ey, double* __restrict__ Jx, double* __restrict__ Jy) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= G) return;
  const double ex = -(Frx[k] + Fdx[k]);
  const double ey = -(Fry[k] + Fdy[k]);
  Ex[k] = ex;
  Ey[k] = ey;
  const double wk = w ? w[k] : 1.0;
  Jx[k] = sigma * ex * wk;
  Jy[k] = sigma * ey * wk;
}

// Environment current from the grid fluxes with extracellular spaces
// (ion_current.py:55-56): J = sum_i F z_i flux_i, ions in order.
__global__ void k_fields_zf_sum(int G, int I, const double* __restrict__ fx, const double* __restrict__ fy,
                                ZF zf, double* __restrict__ Jx, double* __restrict__ Jy) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= G) return;
  double sx = 0.0, sy = 0.0;
#pragma unroll
  for (int i = 0; i < kMaxIons; ++i) {
    if (i < I) {
      sx += zf.v[i] * fx[(size_t)i * G + k];
      sy += zf.v[i] * fy[(size_t)i * G + k];
    }
  }
  Jx[k] = sx;
  Jy[k] = sy;
}

}  // namespace bx

namespace bx {

// ---------------------------------------------------------------------------
// Batched environment fields: one CTA per cluster of a batch (each cluster
// has its own, small grid), the two dense products per Helmholtz-Hodge split
// done for all clusters of one grid shape as one GEMM (bx_dense_op_apply).
// Per-cluster descriptor ci[c*kCi + .]: grid offset, ny, nx, X offset of the
// cluster's shape, first column of the cluster in that shape's operand,
// columns of that operand, first membrane, first cell; cd[c*2 + .]: grid
// spacing, sigma.
// ---------------------------------------------------------------------------
constexpr int kCi = 8;

__device__ __forceinline__ FieldGrid cluster_grid(const int* ci, const double* cd, int c, const FieldGrid& base) {
  FieldGrid g = base;
  g.ny = ci[c * kCi + 1];
  g.nx = ci[c * kCi + 2];
  g.G = g.ny * g.nx;
  g.delta = cd[c * 2];
  return g;
}

__global__ void kb_vce(const int* __restrict__ ci, const double* __restrict__ cd, FieldGrid base,
                       const int* __restrict__ last_mem, const int* __restrict__ m2c, const double* __restrict__ vm,
                       double* __restrict__ neg_vce) {
  const int c = blockIdx.x;
  const FieldGrid g = cluster_grid(ci, cd, c, base);
  const int off = ci[c * kCi];
  const int m0 = ci[c * kCi + 6], c0 = ci[c * kCi + 7];
  for (int k = threadIdx.x; k < g.G; k += blockDim.x) {
    // (vm/2)[mem_to_cells] within the cluster: its membrane vector indexed by
    // its own cell indices (ion_current.py:120-122)
    const int m = last_mem[off + k];
    neg_vce[off + k] = (m >= 0) ? -(vm[m0 + (m2c[m] - c0)] / 2) : 0.0;
  }
}

template <bool REFLECT>
__global__ void kb_gauss(const int* __restrict__ ci, const double* __restrict__ cd, FieldGrid base,
                         const double* __restrict__ in, double* __restrict__ out, int axis) {
  const int c = blockIdx.x;
  const FieldGrid g = cluster_grid(ci, cd, c, base);
  const int off = ci[c * kCi];
  for (int k = threadIdx.x; k < g.G; k += blockDim.x) {
    const int i = k / g.nx, j = k - i * g.nx;
    const int n = axis == 0 ? g.ny : g.nx;
    const int pos = axis == 0 ? i : j;
    double acc = 0.0;
#pragma unroll
    for (int t = -4; t <= 4; ++t) {
      int r = pos + t;
      if (REFLECT) {
        while (r < 0 || r >= n) r = (r < 0) ? -r - 1 : 2 * n - r - 1;
      } else if (r < 0 || r >= n) {
        continue;
      }
      acc += g.gw[t + 4] * in[off + (axis == 0 ? r * g.nx + j : i * g.nx + r)];
    }
    out[off + k] = acc;
  }
}

// (gx, gy) = gradient(delta_c * F) per cluster (ion_current.py:133)
__global__ void kb_grad_delta(const int* __restrict__ ci, const double* __restrict__ cd, FieldGrid base,
                              const double* __restrict__ F, double* __restrict__ gx, double* __restrict__ gy) {
  const int c = blockIdx.x;
  const FieldGrid g = cluster_grid(ci, cd, c, base);
  const int off = ci[c * kCi];
  for (int k = threadIdx.x; k < g.G; k += blockDim.x) {
    double a, b;
    fd_grad(F + off, 1, g.delta, k / g.nx, k % g.nx, g, a, b);
    gx[off + k] = a;
    gy[off + k] = b;
  }
}

// HH_Decomp right-hand sides of each cluster into its two columns of its
// shape's operand X[k][ncols] (FP64, row-major)
__global__ void kb_hh_rhs(const int* __restrict__ ci, const double* __restrict__ cd, FieldGrid base,
                          const double* __restrict__ Jx, const double* __restrict__ Jy, double* __restrict__ X) {
  const int c = blockIdx.x;
  const FieldGrid g = cluster_grid(ci, cd, c, base);
  const int off = ci[c * kCi], xo = ci[c * kCi + 3], col = ci[c * kCi + 4], nc = ci[c * kCi + 5];
  for (int k = threadIdx.x; k < g.G; k += blockDim.x) {
    const int i = k / g.nx, j = k - i * g.nx;
    double r0 = 0.0, r1 = 0.0;
    if (!(i == 0 || j == 0 || i == g.ny - 1 || j == g.nx - 1)) {
      r0 = -(ddx_in(Jy + off, -1.0, i, j, g) + ddy_in(Jx + off, 1.0, i, j, g));
      r1 = ddx_in(Jx + off, 1.0, i, j, g) + ddy_in(Jy + off, 1.0, i, j, g);
    }
    X[xo + (size_t)k * nc + col] = r0;
    X[xo + (size_t)k * nc + col + 1] = r1;
  }
}

// from each cluster's two columns (AA, BB) of Y: AA_out = aa_scale AA (if
// asked), (Fx, Fy) = (-dAA/dy, dAA/dx), (Gx, Gy) = grad BB (if asked)
__global__ void kb_hh_out(const int* __restrict__ ci, const double* __restrict__ cd, FieldGrid base,
                          const double* __restrict__ Y, double aa_scale, double* __restrict__ AA_out,
                          double* __restrict__ Fx, double* __restrict__ Fy, double* __restrict__ Gx,
                          double* __restrict__ Gy) {
  const int c = blockIdx.x;
  const FieldGrid g = cluster_grid(ci, cd, c, base);
  const int off = ci[c * kCi], xo = ci[c * kCi + 3], col = ci[c * kCi + 4], nc = ci[c * kCi + 5];
  const double* Ya = Y + xo + col;
  for (int k = threadIdx.x; k < g.G; k += blockDim.x) {
    const int i = k / g.nx, j = k - i * g.nx;
    double ax, ay;
    fd_grad(Ya, nc, 1.0, i, j, g, ax, ay);
    if (AA_out) AA_out[off + k] = aa_scale * Ya[(size_t)k * nc];
    Fx[off + k] = -ay;
    Fy[off + k] = ax;
    if (Gx) {
      double bx_, by_;
      fd_grad(Ya + 1, nc, 1.0, i, j, g, bx_, by_);
      Gx[off + k] = bx_;
      Gy[off + k] = by_;
    }
  }
}

__global__ void kb_e_and_j(const int* __restrict__ ci, const double* __restrict__ cd, FieldGrid base,
                           const double* __restrict__ Frx, const double* __restrict__ Fry,
                           const double* __restrict__ Fdx, const double* __restrict__ Fdy,
                           const double* __restrict__ w, double* __restrict__ Ex, double* __restrict__ Ey,
                           double* __restrict__ Jx, double* __restrict__ Jy) {
  const int c = blockIdx.x;
  const FieldGrid g = cluster_grid(ci, cd, c, base);
  const int off = ci[c * kCi];
  const double sigma = cd[c * 2 + 1];
  for (int k = off + threadIdx.x; k < off + g.G; k += blockDim.x) {
    const double ex = -(Frx[k] + Fdx[k]);
    const double ey = -(Fry[k] + Fdy[k]);
    Ex[k] = ex;
    Ey[k] = ey;
    const double wk = w ? w[k] : 1.0;
    Jx[k] = sigma * ex * wk;
    Jy[k] = sigma * ey * wk;
  }
}

}  // namespace bx
