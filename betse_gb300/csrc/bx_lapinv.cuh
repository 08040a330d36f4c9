// bx_lapinv.cuh -- cells.lapENVinv built on the GPU from its eigenvectors.
//
// FiniteDiffSolver.makeLaplacian (finitediff.py:252-431) is, on the
// row-major (ny, nx) grid at unit spacing, the 5-point Laplacian on interior
// points and the identity on the four edges; cells.lapENVinv is the (p)inverse
// of that matrix over delta^2 (cells.py:503-504), i.e. delta^2 times the
// inverse at unit spacing.  BETSE inverts it densely, O(G^3).  In block form
// (edge rows e, interior rows i)
//
//   A = [[I, 0], [L_ie, L_ii]],   A^-1 = [[I, 0], [-L_ii^-1 L_ie, L_ii^-1]],
//
// and the interior block L_ii (Dirichlet Laplacian on n1 x n2 points,
// n1 = ny - 2, n2 = nx - 2) is diagonalised by the orthonormal sine matrices
// S1, S2 (S[i][a] = sqrt(2/(n+1)) sin(pi (i+1)(a+1)/(n+1))) with eigenvalues
// lam1_a + lam2_b, lam_a = -2 + 2 cos(pi (a+1)/(n+1)).  Hence
//
//   L_ii^-1[(i,j),(k,l)] = sum_a S1[i][a] S1[k][a] M_a[j][l],
//   M_a = S2 diag(1 / (lam1_a + lam2)) S2^T,
//
// one FP64 GEMM of (n1^2) x n1 x (n2^2) with rows (i,k) and columns (j,l)
// -- O(G^2 sqrt(G)) work instead of O(G^3).  Each edge point other than a
// corner has exactly one interior neighbour q, so its column of
// -L_ii^-1 L_ie is minus column q of L_ii^-1; corners give zero columns.
//
// Output: FP64, or double-float pairs (hi, lo) as the field products read
// them; row r of the operator at out + r * ld.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <vector>

namespace bx {

template <typename T> struct LapStore;
template <> struct LapStore<double> {
  __device__ static void put(double* p, double v) { *p = v; }
  __device__ static double get(const double* p) { return *p; }
};
template <> struct LapStore<float2> {
  __device__ static void put(float2* p, double v) {
    const float hi = __double2float_rn(v);
    *p = make_float2(hi, __double2float_rn(v - (double)hi));
  }
  __device__ static double get(const float2* p) { return (double)p->x + (double)p->y; }
};

// M[a][j][l] = sum_b S2[j][b] S2[l][b] / (lam1[a] + lam2[b])
__global__ void k_lapinv_M(const double* __restrict__ S2, const double* __restrict__ lam1,
                           const double* __restrict__ lam2, int n1, int n2, double* __restrict__ M) {
  const int jl = blockIdx.x * blockDim.x + threadIdx.x;
  const int a = blockIdx.y;
  if (jl >= n2 * n2) return;
  const int j = jl / n2, l = jl % n2;
  double s = 0.0;
  for (int b = 0; b < n2; ++b) s += S2[j * n2 + b] * S2[l * n2 + b] / (lam1[a] + lam2[b]);
  M[((size_t)a * n2 + j) * n2 + l] = s;
}

// The interior block: a 64 x 64 tile of the GEMM per CTA (rows: 8 values of
// i by 8 of k; columns: 8 of j by 8 of l), 16 values of a per stage, each
// thread a 4 x 4 register tile; scaled by delta^2 and written at the grid
// rows (i+1)*nx + j+1 and columns (k+1)*nx + l+1.
template <typename T>
__global__ void __launch_bounds__(256)
k_lapinv_inner(const double* __restrict__ S1, const double* __restrict__ M, int n1, int n2, int nx,
               double scale, T* __restrict__ out, size_t ld) {
  constexpr int KA = 16;
  __shared__ double As[KA][64];
  __shared__ double Bs[KA][64];
  const int nt2 = (n2 + 7) / 8;
  const int i0 = 8 * blockIdx.z, k0 = 8 * blockIdx.y;
  const int j0 = 8 * (blockIdx.x / nt2), l0 = 8 * (blockIdx.x % nt2);
  const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
  double acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.0;
  for (int a0 = 0; a0 < n1; a0 += KA) {
    for (int q = t; q < KA * 64; q += 256) {
      const int aa = q / 64, r = q % 64, a = a0 + aa;
      const int i = i0 + (r >> 3), k = k0 + (r & 7);
      As[aa][r] = (a < n1 && i < n1 && k < n1) ? S1[i * n1 + a] * S1[k * n1 + a] : 0.0;
      const int j = j0 + (r >> 3), l = l0 + (r & 7);
      Bs[aa][r] = (a < n1 && j < n2 && l < n2) ? M[((size_t)a * n2 + j) * n2 + l] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int aa = 0; aa < KA; ++aa) {
      double x[4], y[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) { x[u] = As[aa][ty * 4 + u]; y[u] = Bs[aa][tx * 4 + u]; }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(x[u], y[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int r = ty * 4 + u, i = i0 + (r >> 3), k = k0 + (r & 7);
    if (i >= n1 || k >= n1) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int c = tx * 4 + v, j = j0 + (c >> 3), l = l0 + (c & 7);
      if (j >= n2 || l >= n2) continue;
      const size_t row = (size_t)(i + 1) * nx + (j + 1), col = (size_t)(k + 1) * nx + (l + 1);
      LapStore<T>::put(out + row * ld + col, scale * acc[u][v]);
    }
  }
}

// Edge columns of the interior rows (minus the inward neighbour's column) and
// the edge rows (delta^2 on the diagonal); everything else was zeroed.
template <typename T>
__global__ void k_lapinv_edges(int ny, int nx, double scale, T* __restrict__ out, size_t ld) {
  const int ne = 2 * nx + 2 * (ny - 2);
  const int G = ny * nx;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)G * ne) return;
  const int row = (int)(idx / ne), q = (int)(idx % ne);
  // the q-th edge point and its inward neighbour (-1 at a corner)
  int ei, ej;
  if (q < nx) { ei = 0; ej = q; }
  else if (q < 2 * nx) { ei = ny - 1; ej = q - nx; }
  else { const int r = q - 2 * nx; ei = 1 + (r >> 1); ej = (r & 1) ? nx - 1 : 0; }
  const int e = ei * nx + ej;
  int in = -1;
  if (ei == 0 && ej > 0 && ej < nx - 1) in = nx + ej;
  else if (ei == ny - 1 && ej > 0 && ej < nx - 1) in = (ny - 2) * nx + ej;
  else if (ej == 0 && ei > 0 && ei < ny - 1) in = ei * nx + 1;
  else if (ej == nx - 1 && ei > 0 && ei < ny - 1) in = ei * nx + nx - 2;
  const int ri = row / nx, rj = row % nx;
  const bool row_edge = ri == 0 || rj == 0 || ri == ny - 1 || rj == nx - 1;
  if (row_edge) {
    if (row == e) LapStore<T>::put(out + (size_t)row * ld + e, scale);
  } else if (in >= 0) {
    LapStore<T>::put(out + (size_t)row * ld + e, -LapStore<T>::get(out + (size_t)row * ld + in));
  }
}

// Build delta^2 * A_unit^-1 into out ([ny*nx] rows of ld elements, device),
// on `stream`; allocates and frees its own small factors (S1, S2, the
// eigenvalues, M: n1 * n2^2 doubles).  The caller zeroes `out` first.
template <typename T>
cudaError_t build_lap_env_inv(int ny, int nx, double delta, T* out, size_t ld, cudaStream_t stream) {
  const int n1 = ny - 2, n2 = nx - 2;
  const double scale = delta * delta;
  const double pi = 3.14159265358979323846;
  std::vector<double> S1((size_t)n1 * n1), S2((size_t)n2 * n2), l1(n1), l2(n2);
  for (int a = 0; a < n1; ++a) {
    l1[a] = -2.0 + 2.0 * std::cos(pi * (a + 1) / (n1 + 1));
    for (int i = 0; i < n1; ++i) S1[(size_t)i * n1 + a] = std::sqrt(2.0 / (n1 + 1)) * std::sin(pi * (i + 1) * (a + 1) / (n1 + 1));
  }
  for (int b = 0; b < n2; ++b) {
    l2[b] = -2.0 + 2.0 * std::cos(pi * (b + 1) / (n2 + 1));
    for (int j = 0; j < n2; ++j) S2[(size_t)j * n2 + b] = std::sqrt(2.0 / (n2 + 1)) * std::sin(pi * (j + 1) * (b + 1) / (n2 + 1));
  }
  double *dS1 = nullptr, *dS2 = nullptr, *dl1 = nullptr, *dl2 = nullptr, *dM = nullptr;
  cudaError_t e = cudaSuccess;
  auto need = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
  need(cudaMalloc(&dS1, S1.size() * sizeof(double)));
  need(cudaMalloc(&dS2, S2.size() * sizeof(double)));
  need(cudaMalloc(&dl1, l1.size() * sizeof(double)));
  need(cudaMalloc(&dl2, l2.size() * sizeof(double)));
  need(cudaMalloc(&dM, (size_t)n1 * n2 * n2 * sizeof(double)));
  if (e == cudaSuccess) {
    need(cudaMemcpyAsync(dS1, S1.data(), S1.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
    need(cudaMemcpyAsync(dS2, S2.data(), S2.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
    need(cudaMemcpyAsync(dl1, l1.data(), l1.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
    need(cudaMemcpyAsync(dl2, l2.data(), l2.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
  }
  if (e == cudaSuccess) {
    k_lapinv_M<<<dim3((unsigned)((n2 * n2 + 255) / 256), (unsigned)n1), 256, 0, stream>>>(dS2, dl1, dl2, n1, n2, dM);
    need(cudaGetLastError());
    const unsigned nt1 = (unsigned)((n1 + 7) / 8), nt2 = (unsigned)((n2 + 7) / 8);
    k_lapinv_inner<T><<<dim3(nt2 * nt2, nt1, nt1), 256, 0, stream>>>(dS1, dM, n1, n2, nx, scale, out, ld);
    need(cudaGetLastError());
    const long long n_edge = (long long)ny * nx * (2 * nx + 2 * (ny - 2));
    k_lapinv_edges<T><<<(unsigned)((n_edge + 255) / 256), 256, 0, stream>>>(ny, nx, scale, out, ld);
    need(cudaGetLastError());
    need(cudaStreamSynchronize(stream));
  }
  cudaFree(dS1); cudaFree(dS2); cudaFree(dl1); cudaFree(dl2); cudaFree(dM);
  return e;
}

}  // namespace bx
