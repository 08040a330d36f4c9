// bx_gemm.cu -- dense operator products on the fifth-generation tensor cores.
//
// BETSE applies dense inverse Laplacians by matrix-vector products:
//   np.dot(cells.lapGJinv, rhs)    physics/pressures.py:59 (cells.py:1845-1891)
//   np.dot(cells.lapENVinv, rhs)   physics/ion_current.py:90,170,
//                                  sim_toolbox.py:1263,1284
// One right-hand side is a streaming GEMV (bx_env_fields does those).  Where
// right-hand sides batch -- many clusters sharing one grid-shape operator,
// or a block of source terms -- the product is a GEMM, and this file puts it
// on tcgen05:
//
//   * the FP64 operator A is split once into BF16 planes, A = A_hi + A_lo
//     (+ O(2^-17 |A|)), and stored in 128x64 tiles laid out in the canonical
//     no-swizzle K-major core-matrix order (8 rows x 16 bytes per core matrix,
//     K-adjacent cores 128 B apart, 8-row groups 1024 B apart), so each tile is
//     one contiguous 16 KB block;
//   * the right-hand sides X are split and packed the same way per call;
//   * one CTA per 128 x 128 output tile: a producer thread streams the four
//     tiles of each 64-wide K block with cp.async.bulk (TMA engine) into a
//     3-stage ring guarded by mbarriers; one thread issues
//     tcgen05.mma.kind::f16 (BF16 x BF16 -> FP32 in TMEM) for
//     A_hi.X_hi + A_hi.X_lo + A_lo.X_hi and commits each stage back to the
//     producer; four epilogue warps read the accumulator with tcgen05.ld and
//     write FP64;
//   * an optional refinement step with the forward operator L (CSR, FP64):
//     r = X - L.Y0, Y = Y0 + A.r, which squares the BF16-split error when A is
//     L's inverse.
// Every mbarrier wait is bounded (about two seconds of %globaltimer); a wait
// that runs out sets a timeout bit in an error word (bx_dense_op_status) and the CTA drains
// its copies, frees its TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/bx.h"
#include "bx_tc.cuh"

// error text for bx_last_error (defined with the other entry points)
void bx_record_error(const char* msg);

namespace bxg {

using namespace bxtc;

constexpr int BM = 128, BN = 128, BK = 64, STAGES = 3;
constexpr int TILE = BM * BK;                        // elements per 128x64 tile
constexpr int TILE_BYTES = TILE * 2;                 // 16 KB of BF16
constexpr int STAGE_BYTES = 4 * TILE_BYTES;          // A_hi, A_lo, B_hi, B_lo
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024;
constexpr int kThreads = 192;                        // producer, MMA, 4 epilogue warps
constexpr uint32_t kTmemCols = BN;                   // FP32 accumulator: 128 lanes x BN columns
constexpr unsigned int kErrTimeout = 1u;

// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both K-major
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                            ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accum) {
  mma_f16(d_tmem, a, b, kIdesc, accum);
}

struct GemmArgs {
  const __nv_bfloat16* a_hi;  // [Mt][Kt] tiles
  const __nv_bfloat16* a_lo;
  const __nv_bfloat16* b_hi;  // [Nt][Kt] tiles
  const __nv_bfloat16* b_lo;
  int Kt;
  int m, ncols;               // valid rows of A / columns of X
  double* Y;                  // row-major [m][ldy]
  int ldy;
  int accumulate;             // Y += A X instead of Y = A X
  unsigned int* err;
};

__global__ void __launch_bounds__(kThreads, 1) k_gemm_bf16x3(GemmArgs g) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], accum_full;
  __shared__ uint32_t tmem_base;
  __shared__ int failed;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nt = blockIdx.x, mt = blockIdx.y, Kt = g.Kt;  // N-tiles of one row block run together (A shared in L2)

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), 1);
    }
    mbar_init(smem_u32(&accum_full), 1);
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (warp == 0 && lane == 0) {
    // ---- producer: four 16 KB tiles per K block.  The right-hand sides (read
    // by every row block) are marked evict_last so the operator streaming
    // through L2 does not push them out between row blocks.
    const uint64_t keep = policy_evict_last();
    int issued = 0;
    for (int kb = 0; kb < Kt; ++kb) {
      const int s = kb % STAGES;
      const uint32_t use = (uint32_t)(kb / STAGES);
      if (kb >= STAGES && !mbar_wait(smem_u32(&empty[s]), (use & 1u) ^ 1u)) {
        failed = 1;
        break;
      }
      const uint32_t fb = smem_u32(&full[s]);
      const uint32_t dst = smem_u32(smem + (size_t)s * STAGE_BYTES);
      const size_t ao = ((size_t)mt * Kt + kb) * TILE, bo = ((size_t)nt * Kt + kb) * TILE;
      mbar_expect_tx(fb, STAGE_BYTES);
      bulk_g2s(dst, g.a_hi + ao, TILE_BYTES, fb);
      bulk_g2s(dst + TILE_BYTES, g.a_lo + ao, TILE_BYTES, fb);
      bulk_g2s_hint(dst + 2 * TILE_BYTES, g.b_hi + bo, TILE_BYTES, fb, keep);
      bulk_g2s_hint(dst + 3 * TILE_BYTES, g.b_lo + bo, TILE_BYTES, fb, keep);
      issued = kb + 1;
    }
    // drain: the last copies of each stage have landed before the CTA can exit
    for (int kb = (issued > STAGES ? issued - STAGES : 0); kb < issued; ++kb)
      if (!mbar_wait(smem_u32(&full[kb % STAGES]), (uint32_t)(kb / STAGES) & 1u)) failed = 1;
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer
    bool ok = true;
    for (int kb = 0; kb < Kt && ok; ++kb) {
      const int s = kb % STAGES;
      if (!mbar_wait(smem_u32(&full[s]), (uint32_t)(kb / STAGES) & 1u)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t base = smem_u32(smem + (size_t)s * STAGE_BYTES);
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk) {
        const uint32_t o = (uint32_t)kk * 256u;  // two K-adjacent core matrices per MMA (K = 16)
        const uint64_t ah = smem_desc(base + o, 128, 1024);
        const uint64_t al = smem_desc(base + TILE_BYTES + o, 128, 1024);
        const uint64_t bh = smem_desc(base + 2 * TILE_BYTES + o, 128, 1024);
        const uint64_t bl = smem_desc(base + 3 * TILE_BYTES + o, 128, 1024);
        mma_bf16(tmem, ah, bh, (kb > 0 || kk > 0) ? 1u : 0u);
        mma_bf16(tmem, ah, bl, 1u);
        mma_bf16(tmem, al, bh, 1u);
      }
      mma_commit(smem_u32(&empty[s]));  // stage free once these MMAs have read it
    }
    if (!ok) failed = 1;
    mma_commit(smem_u32(&accum_full));  // every MMA issued so far has completed
  } else if (warp >= 2) {
    // ---- epilogue: warp w reads TMEM lanes [32 (w%4), 32 (w%4) + 32)
    const int q = warp & 3;
    const bool ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&accum_full), 0u));  // warp-uniform
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok) {
      failed = 1;
    } else {
      const int row = mt * BM + q * 32 + lane;
      for (int c0 = 0; c0 < BN; c0 += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
        if (row < g.m) {
          double* yr = g.Y + (size_t)row * g.ldy;
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int col = nt * BN + c0 + i;
            if (col < g.ncols) yr[col] = g.accumulate ? yr[col] + (double)v[i] : (double)v[i];
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  }
  if (threadIdx.x == 0 && failed) atomicOr(g.err, kErrTimeout);
}

// Split src (FP64, element (r, k) at src[r*ld_r + k*ld_k]) into packed BF16
// hi/lo tiles [rows/128][cols/64], zero outside [0,rows) x [0,cols).
__global__ void k_pack_split(const double* __restrict__ src, int rows, int cols, long long ld_r, long long ld_k,
                             int Kt, long long n_el, __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n_el;
       e += (long long)gridDim.x * blockDim.x) {
    const long long tile = e / TILE;
    const int w = (int)(e - tile * TILE);
    const int core = w >> 6, in = w & 63;
    const int r = ((core >> 3) << 3) + (in >> 3), k = ((core & 7) << 3) + (in & 7);
    const int row = (int)(tile / Kt) * BM + r, col = (int)(tile % Kt) * BK + k;
    const double a = (row < rows && col < cols) ? src[(long long)row * ld_r + (long long)col * ld_k] : 0.0;
    const __nv_bfloat16 h = __double2bfloat16(a);
    hi[e] = h;
    lo[e] = __double2bfloat16(a - (double)__bfloat162float(h));
  }
}

// Split columns [col0, col0 + ncols) of an n x n operator, given as
// src[row * ncols + (col - col0)], into the hi/lo tiles of 64-column tile
// columns kt0 .. kt0 + nkt - 1 (col0 = kt0 * 64); zero outside the block.
__global__ void k_pack_cols(const double* __restrict__ src, int n, int col0, int ncols, int Mt, int Kt, int kt0,
                            int nkt, __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo) {
  const long long n_el = (long long)Mt * nkt * TILE;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n_el;
       e += (long long)gridDim.x * blockDim.x) {
    const long long tl = e / TILE;
    const int w = (int)(e - tl * TILE);
    const int mt = (int)(tl / nkt), kt = kt0 + (int)(tl % nkt);
    const int core = w >> 6, in = w & 63;
    const int r = ((core >> 3) << 3) + (in >> 3), k = ((core & 7) << 3) + (in & 7);
    const int row = mt * BM + r, col = kt * BK + k;
    const double a = (row < n && col < n && col - col0 < ncols) ? src[(long long)row * ncols + (col - col0)] : 0.0;
    const long long d = ((long long)mt * Kt + kt) * TILE + w;
    const __nv_bfloat16 h = __double2bfloat16(a);
    hi[d] = h;
    lo[d] = __double2bfloat16(a - (double)__bfloat162float(h));
  }
}

// R = X - L Y for a CSR operator L, all [n][nrhs] row-major
__global__ void k_csr_residual(int n, int nrhs, const int* __restrict__ ptr, const int* __restrict__ col,
                               const double* __restrict__ val, const double* __restrict__ X,
                               const double* __restrict__ Y, double* __restrict__ R) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * nrhs) return;
  const int i = (int)(t / nrhs), j = (int)(t - (long long)i * nrhs);
  double s = 0.0;
  for (int p = ptr[i]; p < ptr[i + 1]; ++p) s += val[p] * Y[(size_t)col[p] * nrhs + j];
  R[t] = X[t] - s;
}

__global__ void k_scale_cols(int n, int nrhs, const double* __restrict__ s, double* __restrict__ Y) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (long long)n * nrhs) Y[t] *= s[t % nrhs];
}

}  // namespace bxg

struct bx_dense_op {
  int n = 0, Mt = 0, Kt = 0;
  __nv_bfloat16 *a_hi = nullptr, *a_lo = nullptr;
  int *f_ptr = nullptr, *f_col = nullptr;
  double* f_val = nullptr;
  int cap_rhs = 0;                          // packed-X and residual capacity (columns)
  __nv_bfloat16 *b_hi = nullptr, *b_lo = nullptr;
  double* resid = nullptr;
  unsigned int* err = nullptr;
};

namespace {

int gfail(int code, const std::string& msg) {
  bx_record_error(msg.c_str());
  return code;
}
#define GX(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) return gfail(BX_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

int ensure_rhs(bx_dense_op* op, int nrhs) {
  if (nrhs <= op->cap_rhs) return BX_OK;
  cudaFree(op->b_hi);
  cudaFree(op->b_lo);
  cudaFree(op->resid);
  op->b_hi = op->b_lo = nullptr;
  op->resid = nullptr;
  op->cap_rhs = 0;
  const int Nt = (nrhs + bxg::BN - 1) / bxg::BN;
  const size_t el = (size_t)Nt * op->Kt * bxg::TILE;
  if (cudaMalloc(&op->b_hi, el * 2) != cudaSuccess || cudaMalloc(&op->b_lo, el * 2) != cudaSuccess ||
      cudaMalloc(&op->resid, (size_t)op->n * Nt * bxg::BN * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return gfail(BX_ENOMEM, "cudaMalloc dense-op right-hand sides");
  }
  op->cap_rhs = Nt * bxg::BN;
  return BX_OK;
}

unsigned grid_for(long long n_el) {
  return (unsigned)std::min<long long>((n_el + 255) / 256, 152LL * 32);
}

// Y (=|+=) A X on stream s, X and Y [n][nrhs] row-major on the device
int gemm(bx_dense_op* op, const double* X, double* Y, int nrhs, bool accumulate, cudaStream_t s) {
  const int Nt = (nrhs + bxg::BN - 1) / bxg::BN;
  const long long n_el = (long long)Nt * op->Kt * bxg::TILE;
  // B operand is X^T: element (j, k) = X[k][j]
  bxg::k_pack_split<<<grid_for(n_el), 256, 0, s>>>(X, nrhs, op->n, 1, nrhs, op->Kt, n_el, op->b_hi, op->b_lo);
  GX(cudaGetLastError());
  bxg::GemmArgs a{op->a_hi, op->a_lo, op->b_hi, op->b_lo, op->Kt, op->n, nrhs, Y, nrhs, accumulate ? 1 : 0,
                  op->err};
  bxg::k_gemm_bf16x3<<<dim3((unsigned)Nt, (unsigned)op->Mt), bxg::kThreads, bxg::SMEM_BYTES, s>>>(a);
  GX(cudaGetLastError());
  return BX_OK;
}

}  // namespace

extern "C" {

int bx_dense_op_create(const double* A, int n, bx_dense_op_handle* out) {
  if (!A || !out || n <= 0) return gfail(BX_EINVAL, "bx_dense_op_create: bad arguments");
  *out = nullptr;
  GX(cudaFuncSetAttribute(bxg::k_gemm_bf16x3, cudaFuncAttributeMaxDynamicSharedMemorySize, bxg::SMEM_BYTES));
  bx_dense_op* op = new bx_dense_op();
  op->n = n;
  op->Mt = (n + bxg::BM - 1) / bxg::BM;
  op->Kt = (n + bxg::BK - 1) / bxg::BK;
  const size_t el = (size_t)op->Mt * op->Kt * bxg::TILE;
  double* stage = nullptr;
  const size_t rows_per = std::max<size_t>(bxg::BM, ((size_t)256 << 20) / ((size_t)n * sizeof(double)) / bxg::BM * bxg::BM);
  int rc = BX_OK;
  if (cudaMalloc(&op->a_hi, el * 2) != cudaSuccess || cudaMalloc(&op->a_lo, el * 2) != cudaSuccess ||
      cudaMalloc(&op->err, sizeof(unsigned int)) != cudaSuccess ||
      cudaMalloc(&stage, std::min<size_t>(rows_per, (size_t)n) * n * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    rc = gfail(BX_ENOMEM, "cudaMalloc dense operator");
  }
  if (rc == BX_OK && cudaMemset(op->err, 0, sizeof(unsigned int)) != cudaSuccess)
    rc = gfail(BX_ECUDA, "cudaMemset");
  // split row blocks (whole 128-row tile rows) through a bounded staging buffer
  for (size_t r0 = 0; rc == BX_OK && r0 < (size_t)n; r0 += rows_per) {
    const size_t nr = std::min(rows_per, (size_t)n - r0);
    if (cudaMemcpy(stage, A + r0 * n, nr * n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
      rc = gfail(BX_ECUDA, "dense operator upload");
      break;
    }
    const int mt0 = (int)(r0 / bxg::BM), mtn = (int)((nr + bxg::BM - 1) / bxg::BM);
    const long long n_el = (long long)mtn * op->Kt * bxg::TILE;
    const size_t off = (size_t)mt0 * op->Kt * bxg::TILE;
    bxg::k_pack_split<<<grid_for(n_el), 256>>>(stage, (int)nr, n, n, 1, op->Kt, n_el, op->a_hi + off,
                                               op->a_lo + off);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess)
      rc = gfail(BX_ECUDA, "dense operator split");
  }
  cudaFree(stage);
  if (rc != BX_OK) {
    bx_dense_op_destroy(op);
    return rc;
  }
  *out = op;
  return BX_OK;
}

int bx_dense_op_create_empty(int n, bx_dense_op_handle* out) {
  if (!out || n <= 0) return gfail(BX_EINVAL, "bx_dense_op_create_empty: bad arguments");
  *out = nullptr;
  GX(cudaFuncSetAttribute(bxg::k_gemm_bf16x3, cudaFuncAttributeMaxDynamicSharedMemorySize, bxg::SMEM_BYTES));
  bx_dense_op* op = new bx_dense_op();
  op->n = n;
  op->Mt = (n + bxg::BM - 1) / bxg::BM;
  op->Kt = (n + bxg::BK - 1) / bxg::BK;
  const size_t el = (size_t)op->Mt * op->Kt * bxg::TILE;
  if (cudaMalloc(&op->a_hi, el * 2) != cudaSuccess || cudaMalloc(&op->a_lo, el * 2) != cudaSuccess ||
      cudaMalloc(&op->err, sizeof(unsigned int)) != cudaSuccess) {
    cudaGetLastError();
    bx_dense_op_destroy(op);
    return gfail(BX_ENOMEM, "cudaMalloc dense operator");
  }
  if (cudaMemset(op->a_hi, 0, el * 2) != cudaSuccess || cudaMemset(op->a_lo, 0, el * 2) != cudaSuccess ||
      cudaMemset(op->err, 0, sizeof(unsigned int)) != cudaSuccess) {
    bx_dense_op_destroy(op);
    return gfail(BX_ECUDA, "cudaMemset dense operator");
  }
  *out = op;
  return BX_OK;
}

int bx_dense_op_set_columns(bx_dense_op_handle op, int col0, int ncols, const double* cols, void* stream) {
  if (!op || !cols || col0 < 0 || ncols <= 0 || col0 + ncols > op->n || col0 % bxg::BK ||
      (ncols % bxg::BK && col0 + ncols != op->n))
    return gfail(BX_EINVAL, "bx_dense_op_set_columns: the block must start on a 64-column boundary and hold "
                            "whole 64-column tiles (or end at n)");
  const int kt0 = col0 / bxg::BK, nkt = (ncols + bxg::BK - 1) / bxg::BK;
  const long long n_el = (long long)op->Mt * nkt * bxg::TILE;
  bxg::k_pack_cols<<<grid_for(n_el), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      cols, op->n, col0, ncols, op->Mt, op->Kt, kt0, nkt, op->a_hi, op->a_lo);
  GX(cudaGetLastError());
  return BX_OK;
}

int bx_dense_op_set_forward(bx_dense_op_handle op, const int32_t* row_ptr, const int32_t* col,
                            const double* val) {
  if (!op || !row_ptr || !col || !val) return gfail(BX_EINVAL, "bx_dense_op_set_forward: null argument");
  const int n = op->n;
  const int nnz = row_ptr[n];
  if (row_ptr[0] != 0 || nnz < 0) return gfail(BX_EINVAL, "bx_dense_op_set_forward: bad row pointers");
  for (int i = 0; i < n; ++i)
    if (row_ptr[i + 1] < row_ptr[i]) return gfail(BX_EINVAL, "bx_dense_op_set_forward: row pointers decrease");
  for (int p = 0; p < nnz; ++p)
    if (col[p] < 0 || col[p] >= n) return gfail(BX_EINVAL, "bx_dense_op_set_forward: column out of range");
  cudaFree(op->f_ptr);
  cudaFree(op->f_col);
  cudaFree(op->f_val);
  op->f_ptr = op->f_col = nullptr;
  op->f_val = nullptr;
  if (cudaMalloc(&op->f_ptr, (size_t)(n + 1) * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&op->f_col, (size_t)std::max(nnz, 1) * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&op->f_val, (size_t)std::max(nnz, 1) * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return gfail(BX_ENOMEM, "cudaMalloc forward operator");
  }
  GX(cudaMemcpy(op->f_ptr, row_ptr, (size_t)(n + 1) * sizeof(int), cudaMemcpyHostToDevice));
  GX(cudaMemcpy(op->f_col, col, (size_t)nnz * sizeof(int), cudaMemcpyHostToDevice));
  GX(cudaMemcpy(op->f_val, val, (size_t)nnz * sizeof(double), cudaMemcpyHostToDevice));
  return BX_OK;
}

int bx_dense_op_apply(bx_dense_op_handle op, const double* X, double* Y, int nrhs, const double* col_scale,
                      int refine, void* stream) {
  if (!op || !X || !Y || nrhs <= 0) return gfail(BX_EINVAL, "bx_dense_op_apply: bad arguments");
  if (refine && !op->f_ptr) return gfail(BX_ESTATE, "bx_dense_op_apply: refinement needs bx_dense_op_set_forward");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = ensure_rhs(op, nrhs);
  if (rc != BX_OK) return rc;
  rc = gemm(op, X, Y, nrhs, false, s);
  if (rc != BX_OK) return rc;
  const long long tot = (long long)op->n * nrhs;
  if (refine) {
    bxg::k_csr_residual<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(op->n, nrhs, op->f_ptr, op->f_col,
                                                                      op->f_val, X, Y, op->resid);
    GX(cudaGetLastError());
    rc = gemm(op, op->resid, Y, nrhs, true, s);
    if (rc != BX_OK) return rc;
  }
  if (col_scale) {
    bxg::k_scale_cols<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(op->n, nrhs, col_scale, Y);
    GX(cudaGetLastError());
  }
  return BX_OK;
}

int bx_dense_op_status(bx_dense_op_handle op, int* timed_out) {
  if (!op || !timed_out) return gfail(BX_EINVAL, "null argument");
  unsigned int e = 0;
  GX(cudaDeviceSynchronize());
  GX(cudaMemcpy(&e, op->err, sizeof(e), cudaMemcpyDeviceToHost));
  *timed_out = (e & bxg::kErrTimeout) ? 1 : 0;
  return BX_OK;
}

int bx_dense_op_time(bx_dense_op_handle op, const double* X, double* Y, int nrhs, int n_iter, double* ms) {
  if (!op || !X || !Y || nrhs <= 0 || n_iter <= 0 || !ms) return gfail(BX_EINVAL, "bad arguments");
  int rc = ensure_rhs(op, nrhs);
  if (rc != BX_OK) return rc;
  rc = gemm(op, X, Y, nrhs, false, nullptr);  // warm-up (also packs X)
  if (rc != BX_OK) return rc;
  const int Nt = (nrhs + bxg::BN - 1) / bxg::BN;
  bxg::GemmArgs a{op->a_hi, op->a_lo, op->b_hi, op->b_lo, op->Kt, op->n, nrhs, Y, nrhs, 0, op->err};
  cudaEvent_t e0, e1;
  GX(cudaEventCreate(&e0));
  GX(cudaEventCreate(&e1));
  GX(cudaEventRecord(e0, nullptr));
  for (int i = 0; i < n_iter; ++i)
    bxg::k_gemm_bf16x3<<<dim3((unsigned)Nt, (unsigned)op->Mt), bxg::kThreads, bxg::SMEM_BYTES>>>(a);
  GX(cudaGetLastError());
  GX(cudaEventRecord(e1, nullptr));
  GX(cudaEventSynchronize(e1));
  float t = 0.f;
  GX(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = (double)t / n_iter;
  return BX_OK;
}

int bx_dense_op_destroy(bx_dense_op_handle op) {
  if (!op) return BX_OK;
  cudaFree(op->a_hi);
  cudaFree(op->a_lo);
  cudaFree(op->f_ptr);
  cudaFree(op->f_col);
  cudaFree(op->f_val);
  cudaFree(op->b_hi);
  cudaFree(op->b_lo);
  cudaFree(op->resid);
  cudaFree(op->err);
  delete op;
  return BX_OK;
}

}  // extern "C"
