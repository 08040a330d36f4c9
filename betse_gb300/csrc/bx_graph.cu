// bx_graph.cu -- BETSE's cell-network Poisson operators at any cluster size.
//
// Cells.graphLaplacian (betse/science/cells.py:1845-1894) forms, from the
// incidence matrix D of the cluster's triangulation (one row per edge),
//     lapGJinv = pinv(D) diag(tri_len / vor_len) (-pinv(D)^T) diag(vor_sa)
//              = -L+ Lw L+ A,
// with L = D^T D the graph Laplacian, L+ its pseudo-inverse (pinv(D) =
// L+ D^T for a connected graph), Lw = D^T diag(tri_len / vor_len) D and
// A = diag(vor_sa); physics/pressures.py:59 applies it with np.dot.  BETSE
// builds it densely with an SVD, O(n^3); here L+ is applied to a block of
// right-hand sides by conjugate gradients in FP64, one independent CG per
// column, preconditioned by an aggregation multigrid V-cycle:
//   * level l+1 aggregates consecutive groups of four nodes of level l
//     (node i -> i / 4); the caller orders the cells so that consecutive
//     cells are neighbours (the generator's Z curve), and passes each
//     level's Galerkin operator P^T L P (again a graph Laplacian);
//   * two damped Jacobi sweeps (omega 2/3) before and after the coarse
//     correction, which is over-weighted by 1.8 (unsmoothed aggregation
//     under-corrects smooth errors); the coarsest level is solved with its
//     pseudo-inverse;
//   * every right-hand side and every preconditioned residual is projected
//     orthogonal to the constants (the null space of L), so the iterate
//     stays in the range of L+.
// At 100k cells this takes ~60 iterations to a relative residual of 1e-10
// (plain Jacobi-preconditioned CG: ~1300).
//
// Layout: every block of vectors is [n][nrhs] row-major (the nrhs values of
// a node contiguous), so one warp reads 32 consecutive columns of a row.
// Column reductions are deterministic (fixed partition, fixed order).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/bx.h"

void bx_record_error(const char* msg);

namespace {

constexpr int kAgg = 4;             // nodes per aggregate
constexpr double kOmega = 2.0 / 3.0;
constexpr double kCoarseWeight = 1.8;
constexpr int kRedRows = 256;       // row partitions of a column reduction

int gfail(int code, const std::string& msg) {
  bx_record_error(msg.c_str());
  return code;
}

#define GCK(call)                                                                          \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return gfail(BX_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Kernels over [rows][K] blocks: a CTA covers kt columns (a power of two up
// to 256, so that wide blocks read long runs of each row) times 256 / kt
// rows, and strides over the rows.
struct Shape {
  dim3 grid, block;
};

Shape shape_for(int rows, int K) {
  int kt = 1;
  while (kt < K && kt < 256) kt <<= 1;
  const int rpb = 256 / kt;
  const int gx = (K + kt - 1) / kt;
  // about 16 CTAs per SM in all, each striding over rows: short-lived CTAs
  // of one row each cost more to schedule than their work
  const int gy = std::max(1, std::min((rows + rpb - 1) / rpb, std::max(1, 152 * 16 / gx)));
  return {dim3((unsigned)gx, (unsigned)gy), dim3((unsigned)kt, (unsigned)rpb)};
}

#define FOR_RC(rows, K)                                       \
  const int k = blockIdx.x * blockDim.x + threadIdx.x;        \
  if (k >= (K)) return;                                       \
  for (int i = blockIdx.y * blockDim.y + threadIdx.y; i < (rows); i += gridDim.y * blockDim.y)

#define LAUNCH(kern, rows, K, s, ...)                          \
  do {                                                        \
    const Shape sh_ = shape_for((rows), (K));                 \
    kern<<<sh_.grid, sh_.block, 0, (s)>>>(__VA_ARGS__);       \
  } while (0)

// sum over row i's entries p of val[p] * xv(col[p]), in entry order
template <class F>
__device__ __forceinline__ double row_dot(const int* __restrict__ ptr, const int* __restrict__ col,
                                          const double* __restrict__ val, int i, F xv) {
  double sum = 0.0;
  for (int p = ptr[i]; p < ptr[i + 1]; ++p) sum += val[p] * xv(col[p]);
  return sum;
}

// out = L in (CSR, rows of K values)
__global__ void k_spmv(int n, int K, const int* __restrict__ ptr, const int* __restrict__ col,
                       const double* __restrict__ val, const double* __restrict__ in, double* __restrict__ out) {
  FOR_RC(n, K) {
    out[(long long)i * K + k] = row_dot(ptr, col, val, i, [&](int j) { return in[(long long)j * K + k]; });
  }
}

// two damped Jacobi sweeps from x = 0: x1 = w D^-1 b, x = x1 + w D^-1 (b - L x1)
__global__ void k_smooth_pre(int n, int K, const int* __restrict__ ptr, const int* __restrict__ col,
                             const double* __restrict__ val, const double* __restrict__ dinv,
                             const double* __restrict__ b, double* __restrict__ x) {
  FOR_RC(n, K) {
    const double sum =
        row_dot(ptr, col, val, i, [&](int j) { return kOmega * dinv[j] * b[(long long)j * K + k]; });
    const double bi = b[(long long)i * K + k];
    x[(long long)i * K + k] = kOmega * dinv[i] * bi + kOmega * dinv[i] * (bi - sum);
  }
}

// the coarse correction and one sweep: xp = x + w_c xc[aggregate],
// out = xp + w D^-1 (b - L xp)
__global__ void k_smooth_post(int n, int K, const int* __restrict__ ptr, const int* __restrict__ col,
                              const double* __restrict__ val, const double* __restrict__ dinv,
                              const double* __restrict__ b, const double* __restrict__ x,
                              const double* __restrict__ xc, double* __restrict__ out) {
  FOR_RC(n, K) {
    const double sum = row_dot(ptr, col, val, i, [&](int j) {
      return x[(long long)j * K + k] + kCoarseWeight * xc[(long long)(j / kAgg) * K + k];
    });
    const double xi = x[(long long)i * K + k] + kCoarseWeight * xc[(long long)(i / kAgg) * K + k];
    out[(long long)i * K + k] = xi + kOmega * dinv[i] * (b[(long long)i * K + k] - sum);
  }
}

// x_out = x_in + w D^-1 (b - L x_in)
__global__ void k_jacobi(int n, int K, const int* __restrict__ ptr, const int* __restrict__ col,
                         const double* __restrict__ val, const double* __restrict__ dinv,
                         const double* __restrict__ b, const double* __restrict__ xin, double* __restrict__ xout) {
  FOR_RC(n, K) {
    const double sum = row_dot(ptr, col, val, i, [&](int j) { return xin[(long long)j * K + k]; });
    const long long t = (long long)i * K + k;
    xout[t] = xin[t] + kOmega * dinv[i] * (b[t] - sum);
  }
}

// bc[a] = sum over the aggregate's nodes of (b - L x)
__global__ void k_restrict(int n, int nc, int K, const int* __restrict__ ptr, const int* __restrict__ col,
                           const double* __restrict__ val, const double* __restrict__ b,
                           const double* __restrict__ x, double* __restrict__ bc) {
  FOR_RC(nc, K) {
    double r = 0.0;
    for (int m = i * kAgg; m < min(i * kAgg + kAgg, n); ++m) {
      const double sum = row_dot(ptr, col, val, m, [&](int j) { return x[(long long)j * K + k]; });
      r += b[(long long)m * K + k] - sum;
    }
    bc[(long long)i * K + k] = r;
  }
}

// x = Pinv b on the coarsest level
__global__ void k_coarse(int nc, int K, const double* __restrict__ pinv, const double* __restrict__ b,
                         double* __restrict__ x) {
  FOR_RC(nc, K) {
    double sum = 0.0;
    for (int j = 0; j < nc; ++j) sum += pinv[(long long)i * nc + j] * b[(long long)j * K + k];
    x[(long long)i * K + k] = sum;
  }
}

// per-column partial sums of a*b (or of a when b is null) over gridDim.y
// row partitions (blocks shaped as shape_for's; smem: one double a thread)
__global__ void k_colsum(int n, int K, const double* __restrict__ a, const double* __restrict__ b,
                         double* __restrict__ part) {
  extern __shared__ double sh[];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double sum = 0.0;
  if (k < K) {
#pragma unroll 4
    for (int i = blockIdx.y * blockDim.y + threadIdx.y; i < n; i += gridDim.y * blockDim.y) {
      const double v = a[(long long)i * K + k];
      sum += b ? v * b[(long long)i * K + k] : v;
    }
  }
  sh[threadIdx.y * blockDim.x + threadIdx.x] = sum;
  __syncthreads();
  if (threadIdx.y == 0 && k < K) {
    double r = 0.0;
    for (int j = 0; j < (int)blockDim.y; ++j) r += sh[j * blockDim.x + threadIdx.x];
    part[(long long)blockIdx.y * K + k] = r;
  }
}

// out[k] = scale * sum of the nparts partials of column k: 8 lanes per
// column take every 8th partial, then add up in lane order (fixed order)
__global__ void k_colfinish(int K, int nparts, const double* __restrict__ part, double scale, double* __restrict__ out) {
  __shared__ double sh[8][33];
  const int k = blockIdx.x * 32 + threadIdx.x;
  double r = 0.0;
  if (k < K) {
#pragma unroll 8
    for (int j = threadIdx.y; j < nparts; j += 8) r += part[(long long)j * K + k];
  }
  sh[threadIdx.y][threadIdx.x] = r;
  __syncthreads();
  if (threadIdx.y == 0 && k < K) {
    double t = 0.0;
    for (int j = 0; j < 8; ++j) t += sh[j][threadIdx.x];
    out[k] = scale * t;
  }
}

// dst = src - mean (per column; src may be dst)
__global__ void k_sub_mean(int n, int K, const double* __restrict__ mean, const double* src, double* dst) {
  FOR_RC(n, K) dst[(long long)i * K + k] = src[(long long)i * K + k] - mean[k];
}

// num / den, 0 where either vanishes (a converged column stops moving)
__device__ __forceinline__ double guarded_ratio(double num, double den) {
  return (den != 0.0 && num != 0.0) ? num / den : 0.0;
}

// X += alpha P, R -= alpha Q with alpha = rz / pq
__global__ void k_xr_update(int n, int K, const double* __restrict__ rz, const double* __restrict__ pq,
                            const double* __restrict__ P, const double* __restrict__ Q, double* __restrict__ X,
                            double* __restrict__ R) {
  const int kk = blockIdx.x * blockDim.x + threadIdx.x;
  const double a = kk < K ? guarded_ratio(rz[kk], pq[kk]) : 0.0;
  FOR_RC(n, K) {
    const long long t = (long long)i * K + k;
    X[t] += a * P[t];
    R[t] -= a * Q[t];
  }
}

// P = Z + beta P with beta = rz_new / rz_old
__global__ void k_p_update(int n, int K, const double* __restrict__ rz_new, const double* __restrict__ rz_old,
                           const double* __restrict__ Z, double* __restrict__ P) {
  const int kk = blockIdx.x * blockDim.x + threadIdx.x;
  const double be = kk < K ? guarded_ratio(rz_new[kk], rz_old[kk]) : 0.0;
  FOR_RC(n, K) {
    const long long t = (long long)i * K + k;
    P[t] = Z[t] + be * P[t];
  }
}

// Y = sign * diag(s) X (s null: 1)
__global__ void k_row_scale(int n, int K, const double* __restrict__ s, const double* __restrict__ X,
                            double* __restrict__ Y, double sign) {
  FOR_RC(n, K) Y[(long long)i * K + k] = sign * (s ? s[i] : 1.0) * X[(long long)i * K + k];
}

// the scaled identity columns col0 .. col0+K-1: E[i][k] = s_i where i == col0 + k
__global__ void k_scaled_identity(int n, int K, int col0, const double* __restrict__ s, double* __restrict__ E) {
  FOR_RC(n, K) E[(long long)i * K + k] = (i == col0 + k) ? s[i] : 0.0;
}

struct Level {
  int n = 0, nnz = 0;
  int *ptr = nullptr, *col = nullptr;
  double *val = nullptr, *dinv = nullptr;
  double *x = nullptr, *t = nullptr, *b = nullptr;   // [n][max_rhs] (coarse levels)
};

}  // namespace

struct bx_graph_solver {
  int n = 0, max_rhs = 0, nc = 0;
  std::vector<Level> lv;
  double* pinv = nullptr;
  int *w_ptr = nullptr, *w_col = nullptr;
  double *w_val = nullptr, *area = nullptr;
  double *R = nullptr, *Z = nullptr, *P = nullptr, *Q = nullptr, *T0 = nullptr, *T1 = nullptr, *T2 = nullptr;
  double *part = nullptr, *rz = nullptr, *rz2 = nullptr, *rr = nullptr, *bb = nullptr, *pq = nullptr,
         *mean = nullptr;
  std::vector<void*> owned;
  ~bx_graph_solver() {
    for (void* p : owned) cudaFree(p);
  }
  template <class T>
  T* alloc(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
    owned.push_back(p);
    return static_cast<T*>(p);
  }
};

namespace {

int colsum(bx_graph_solver* h, int n, int K, const double* a, const double* b, double scale, double* out,
           cudaStream_t s) {
  Shape sh = shape_for(n, K);
  sh.grid.y = kRedRows;
  k_colsum<<<sh.grid, sh.block, 256 * sizeof(double), s>>>(n, K, a, b, h->part);
  k_colfinish<<<(K + 31) / 32, dim3(32, 8), 0, s>>>(K, kRedRows, h->part, scale, out);
  GCK(cudaGetLastError());
  return BX_OK;
}

// x = V-cycle(b) on level l; returns the buffer holding x (x or t of the level)
double* vcycle(bx_graph_solver* h, int l, const double* b, double* x, double* t, int K, cudaStream_t s) {
  const Level& L = h->lv[l];
  if (l + 1 == (int)h->lv.size()) {
    LAUNCH(k_coarse, L.n, K, s, L.n, K, h->pinv, b, x);
    return x;
  }
  LAUNCH(k_smooth_pre, L.n, K, s, L.n, K, L.ptr, L.col, L.val, L.dinv, b, x);
  const Level& C = h->lv[l + 1];
  LAUNCH(k_restrict, C.n, K, s, L.n, C.n, K, L.ptr, L.col, L.val, b, x, C.b);
  const double* xc = vcycle(h, l + 1, C.b, C.x, C.t, K, s);
  LAUNCH(k_smooth_post, L.n, K, s, L.n, K, L.ptr, L.col, L.val, L.dinv, b, x, xc, t);
  LAUNCH(k_jacobi, L.n, K, s, L.n, K, L.ptr, L.col, L.val, L.dinv, b, t, x);
  return x;
}

// X = L+ B for K columns (B and X device [n][K], distinct from the workspace)
int solve(bx_graph_solver* h, const double* B, double* X, int K, double tol, int max_iter, int* iters,
          double* rel_res, cudaStream_t s) {
  const int n = h->n;
  const long long tot = (long long)n * K;
  const Level& L0 = h->lv[0];
  int rc = colsum(h, n, K, B, nullptr, 1.0 / n, h->mean, s);
  if (rc != BX_OK) return rc;
  LAUNCH(k_sub_mean, n, K, s, n, K, h->mean, B, h->R);
  GCK(cudaMemsetAsync(X, 0, (size_t)tot * sizeof(double), s));
  if ((rc = colsum(h, n, K, h->R, h->R, 1.0, h->bb, s)) != BX_OK) return rc;
  // Z = M(R) projected orthogonal to the constants; rz2 = R . Z
  auto precondition = [&]() -> int {
    double* z = vcycle(h, 0, h->R, h->Z, h->T0, K, s);
    int r = colsum(h, n, K, z, nullptr, 1.0 / n, h->mean, s);
    if (r != BX_OK) return r;
    LAUNCH(k_sub_mean, n, K, s, n, K, h->mean, z, h->Z);
    return colsum(h, n, K, h->R, h->Z, 1.0, h->rz2, s);
  };
  if ((rc = precondition()) != BX_OK) return rc;
  GCK(cudaMemcpyAsync(h->P, h->Z, (size_t)tot * sizeof(double), cudaMemcpyDeviceToDevice, s));
  std::swap(h->rz, h->rz2);
  std::vector<double> hrr(K), hbb(K);
  GCK(cudaMemcpyAsync(hbb.data(), h->bb, (size_t)K * sizeof(double), cudaMemcpyDeviceToHost, s));
  double worst = 0.0;
  int it = 0;
  for (it = 1; it <= max_iter; ++it) {
    LAUNCH(k_spmv, n, K, s, n, K, L0.ptr, L0.col, L0.val, h->P, h->Q);
    if ((rc = colsum(h, n, K, h->P, h->Q, 1.0, h->pq, s)) != BX_OK) return rc;
    LAUNCH(k_xr_update, n, K, s, n, K, h->rz, h->pq, h->P, h->Q, X, h->R);
    if (it % 4 == 0 || it == max_iter) {
      if ((rc = colsum(h, n, K, h->R, h->R, 1.0, h->rr, s)) != BX_OK) return rc;
      GCK(cudaMemcpyAsync(hrr.data(), h->rr, (size_t)K * sizeof(double), cudaMemcpyDeviceToHost, s));
      GCK(cudaStreamSynchronize(s));
      worst = 0.0;
      for (int k = 0; k < K; ++k)
        if (hbb[k] > 0.0) worst = std::max(worst, std::sqrt(hrr[k] / hbb[k]));
      if (!(worst == worst)) return gfail(BX_EUNSTABLE, "graph Laplacian solve: NaN residual");
      if (worst <= tol) break;
    }
    if ((rc = precondition()) != BX_OK) return rc;
    LAUNCH(k_p_update, n, K, s, n, K, h->rz2, h->rz, h->Z, h->P);
    std::swap(h->rz, h->rz2);
    GCK(cudaGetLastError());
  }
  if (iters) *iters = std::min(it, max_iter);
  if (rel_res) *rel_res = worst;
  return BX_OK;
}

// Y = lapGJinv X = -L+ Lw L+ A X
int lap_gj(bx_graph_solver* h, const double* X, double* Y, int K, double tol, int max_iter, int* iters,
           double* rel_res, cudaStream_t s, bool identity_cols = false, int col0 = 0) {
  const int n = h->n;
  if (identity_cols)
    LAUNCH(k_scaled_identity, n, K, s, n, K, col0, h->area, h->T1);
  else
    LAUNCH(k_row_scale, n, K, s, n, K, h->area, X, h->T1, 1.0);
  int i1 = 0, i2 = 0;
  double r1 = 0.0, r2 = 0.0;
  int rc = solve(h, h->T1, h->T2, K, tol, max_iter, &i1, &r1, s);
  if (rc != BX_OK) return rc;
  LAUNCH(k_spmv, n, K, s, n, K, h->w_ptr, h->w_col, h->w_val, h->T2, h->T1);
  if ((rc = solve(h, h->T1, h->T2, K, tol, max_iter, &i2, &r2, s)) != BX_OK) return rc;
  LAUNCH(k_row_scale, n, K, s, n, K, nullptr, h->T2, Y, -1.0);
  GCK(cudaGetLastError());
  if (iters) *iters = std::max(i1, i2);
  if (rel_res) *rel_res = std::max(r1, r2);
  return BX_OK;
}

int check_csr(const bx_graph_level& L, int n, const char* what) {
  if (L.n != n || L.nnz < 0 || !L.row_ptr || !L.col || !L.val)
    return gfail(BX_EINVAL, std::string("bx_graph_create: bad ") + what);
  if (L.row_ptr[0] != 0 || L.row_ptr[n] != L.nnz)
    return gfail(BX_EINVAL, std::string("bx_graph_create: row pointers of ") + what);
  for (int i = 0; i < n; ++i)
    if (L.row_ptr[i + 1] < L.row_ptr[i]) return gfail(BX_EINVAL, std::string("bx_graph_create: row pointers of ") + what);
  for (int p = 0; p < L.nnz; ++p)
    if (L.col[p] < 0 || L.col[p] >= n) return gfail(BX_EINVAL, std::string("bx_graph_create: column out of range in ") + what);
  return BX_OK;
}

}  // namespace

extern "C" int bx_dense_op_create_empty(int n, bx_dense_op_handle* out);
extern "C" int bx_dense_op_set_columns(bx_dense_op_handle op, int col0, int ncols, const double* cols, void* stream);
extern "C" int bx_dense_op_destroy(bx_dense_op_handle op);

extern "C" int bx_graph_create(int n_levels, const bx_graph_level* levels, const double* coarse_pinv,
                               const bx_graph_level* weighted, const double* vor_sa, int max_rhs,
                               bx_graph_handle* out) {
  if (!out || !levels || !coarse_pinv || !weighted || !vor_sa || n_levels < 1 || max_rhs < 1)
    return gfail(BX_EINVAL, "bx_graph_create: bad arguments");
  *out = nullptr;
  const int n = levels[0].n;
  if (n < 2) return gfail(BX_EINVAL, "bx_graph_create: fewer than 2 nodes");
  int rc = BX_OK;
  for (int l = 0; l < n_levels; ++l) {
    const int expect = l == 0 ? n : (levels[l - 1].n + kAgg - 1) / kAgg;
    if ((rc = check_csr(levels[l], expect, "level operator")) != BX_OK) return rc;
  }
  if ((rc = check_csr(*weighted, n, "weighted Laplacian")) != BX_OK) return rc;
  auto* h = new bx_graph_solver();
  h->n = n;
  h->max_rhs = max_rhs;
  h->nc = levels[n_levels - 1].n;
  const size_t big = (size_t)n * max_rhs;
  bool ok = true;
  for (int l = 0; l < n_levels && ok; ++l) {
    const bx_graph_level& src = levels[l];
    Level L;
    L.n = src.n;
    L.nnz = src.nnz;
    L.ptr = h->alloc<int>(src.n + 1);
    L.col = h->alloc<int>(src.nnz);
    L.val = h->alloc<double>(src.nnz);
    L.dinv = h->alloc<double>(src.n);
    if (l > 0) {
      L.x = h->alloc<double>((size_t)src.n * max_rhs);
      L.t = h->alloc<double>((size_t)src.n * max_rhs);
      L.b = h->alloc<double>((size_t)src.n * max_rhs);
    }
    ok = L.ptr && L.col && L.val && L.dinv && (l == 0 || (L.x && L.t && L.b));
    if (!ok) break;
    std::vector<double> dinv(src.n, 0.0);
    for (int i = 0; i < src.n; ++i)
      for (int p = src.row_ptr[i]; p < src.row_ptr[i + 1]; ++p)
        if (src.col[p] == i && src.val[p] != 0.0) dinv[i] = 1.0 / src.val[p];
    ok = cudaMemcpy(L.ptr, src.row_ptr, (size_t)(src.n + 1) * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(L.col, src.col, (size_t)src.nnz * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(L.val, src.val, (size_t)src.nnz * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(L.dinv, dinv.data(), (size_t)src.n * 8, cudaMemcpyHostToDevice) == cudaSuccess;
    h->lv.push_back(L);
  }
  if (ok) {
    const int nc = h->nc;
    h->pinv = h->alloc<double>((size_t)nc * nc);
    h->w_ptr = h->alloc<int>(n + 1);
    h->w_col = h->alloc<int>(weighted->nnz);
    h->w_val = h->alloc<double>(weighted->nnz);
    h->area = h->alloc<double>(n);
    for (double** v : {&h->R, &h->Z, &h->P, &h->Q, &h->T0, &h->T1, &h->T2}) *v = h->alloc<double>(big);
    h->part = h->alloc<double>((size_t)kRedRows * max_rhs);
    for (double** v : {&h->rz, &h->rz2, &h->rr, &h->bb, &h->pq, &h->mean})
      *v = h->alloc<double>(max_rhs);
    ok = h->pinv && h->w_ptr && h->w_col && h->w_val && h->area && h->R && h->Z && h->P && h->Q && h->T0 &&
         h->T1 && h->T2 && h->part && h->rz && h->rz2 && h->rr && h->bb && h->pq && h->mean;
    ok = ok && cudaMemcpy(h->pinv, coarse_pinv, (size_t)nc * nc * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(h->w_ptr, weighted->row_ptr, (size_t)(n + 1) * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(h->w_col, weighted->col, (size_t)weighted->nnz * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(h->w_val, weighted->val, (size_t)weighted->nnz * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(h->area, vor_sa, (size_t)n * 8, cudaMemcpyHostToDevice) == cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    delete h;
    return gfail(BX_ENOMEM, "bx_graph_create: device allocation or upload failed");
  }
  *out = h;
  return BX_OK;
}

extern "C" int bx_graph_solve(bx_graph_handle h, const double* B, double* X, int nrhs, double tol, int max_iter,
                              int* iters, double* rel_res, void* stream) {
  if (!h || !B || !X || nrhs < 1 || nrhs > h->max_rhs || max_iter < 1)
    return gfail(BX_EINVAL, "bx_graph_solve: bad arguments (nrhs must be 1..max_rhs)");
  return solve(h, B, X, nrhs, tol, max_iter, iters, rel_res, static_cast<cudaStream_t>(stream));
}

extern "C" int bx_lap_gj_apply(bx_graph_handle h, const double* X, double* Y, int nrhs, double tol, int max_iter,
                               int* iters, double* rel_res, void* stream) {
  if (!h || !X || !Y || nrhs < 1 || nrhs > h->max_rhs || max_iter < 1)
    return gfail(BX_EINVAL, "bx_lap_gj_apply: bad arguments (nrhs must be 1..max_rhs)");
  return lap_gj(h, X, Y, nrhs, tol, max_iter, iters, rel_res, static_cast<cudaStream_t>(stream));
}

extern "C" int bx_lap_gj_dense(bx_graph_handle h, double tol, int max_iter, int* iters, double* rel_res,
                               void* stream, bx_dense_op_handle* out) {
  if (!h || !out || max_iter < 1) return gfail(BX_EINVAL, "bx_lap_gj_dense: bad arguments");
  *out = nullptr;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  bx_dense_op_handle op = nullptr;
  int rc = bx_dense_op_create_empty(h->n, &op);
  if (rc != BX_OK) return rc;
  // blocks of whole 64-column tiles
  const int K = std::max(64, h->max_rhs / 64 * 64);
  if (K > h->max_rhs) {
    bx_dense_op_destroy(op);
    return gfail(BX_EINVAL, "bx_lap_gj_dense: the solver needs max_rhs >= 64");
  }
  double* Y = nullptr;
  if (cudaMalloc(&Y, (size_t)h->n * K * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    bx_dense_op_destroy(op);
    return gfail(BX_ENOMEM, "bx_lap_gj_dense: column block");
  }
  int worst_it = 0;
  double worst_res = 0.0;
  for (int c0 = 0; c0 < h->n && rc == BX_OK; c0 += K) {
    const int k = std::min(K, h->n - c0);
    int it = 0;
    double res = 0.0;
    rc = lap_gj(h, nullptr, Y, k, tol, max_iter, &it, &res, s, true, c0);
    if (rc == BX_OK) rc = bx_dense_op_set_columns(op, c0, k, Y, s);
    worst_it = std::max(worst_it, it);
    worst_res = std::max(worst_res, res);
  }
  if (rc == BX_OK && cudaStreamSynchronize(s) != cudaSuccess) rc = gfail(BX_ECUDA, "bx_lap_gj_dense: build failed");
  cudaFree(Y);
  if (rc != BX_OK) {
    bx_dense_op_destroy(op);
    return rc;
  }
  if (iters) *iters = worst_it;
  if (rel_res) *rel_res = worst_res;
  *out = op;
  return BX_OK;
}

extern "C" int bx_graph_destroy(bx_graph_handle h) {
  delete h;
  return BX_OK;
}
