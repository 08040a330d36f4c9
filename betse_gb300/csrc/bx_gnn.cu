// bx_gnn.cu -- the warm-start graph network: training and inference kernels.
//
// A 3-layer message-passing network on the cell adjacency (cells.cell_nn,
// betse/science/cells.py:1498-1533) predicts each cell's steady-state ion
// concentrations and Vmem from its channel diffusivities, pump rate and
// gap-junction conductance; the time stepping then runs from that prediction
// until its own residual test (max |dVm/dt|, sim.py:2083) passes.  BETSE has
// no counterpart: its init phase always starts from the uniform profile.
//
// Every layer is 64 wide (inputs zero-padded, the first n_out outputs used):
//   H0 = relu(X W0^T + b0)
//   A_l = mean over neighbours of H_{l-1}
//   R_l = relu(H_{l-1} Ws_l^T + A_l Wn_l^T + b_l),  H_l = H_{l-1} + R_l   (l = 1..3)
//   Yhat = H3 Wd^T + bd
// Training is BF16 with FP32 master weights: products read BF16 copies of the
// weights and BF16 activations and accumulate in FP32; gradients and Adam
// moments are FP32.  A forward layer is a tall product [nodes x 64] [64 x 64]
// (two of them for a message layer): it runs on the tensor cores, one CTA per
// 128 nodes, the activation tile and the weights staged in shared memory in
// the canonical K-major core-matrix layout, tcgen05.mma (BF16 x BF16 -> FP32
// in TMEM, M = 128, N = 64, K = 16 per instruction) issued by one thread, and
// four warps reading the accumulator back for the bias, activation and
// residual epilogue.  The backward products take FP32 gradients and stay on
// the FMA pipe: a warp per node, the weights in shared memory.  Weight
// gradients are per-block partial sums reduced in a fixed order
// (deterministic, no floating-point atomics).
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

namespace bxn {

using bf16 = __nv_bfloat16;
constexpr int W = 64, NMP = 3;
constexpr int OFF_W0 = 0, OFF_B0 = W * W, OFF_MP = OFF_B0 + W, MP_STRIDE = 2 * W * W + W;
constexpr int OFF_WD = OFF_MP + NMP * MP_STRIDE, OFF_BD = OFF_WD + W * W, NP = OFF_BD + W;
constexpr int kThreads = 256;
constexpr unsigned FULL = 0xffffffffu;

// activation planes, each [rows][W] BF16
enum Plane { P_X = 0, P_H0, P_H1, P_H2, P_H3, P_A1, P_A2, P_A3, P_R1, P_R2, P_R3, N_PLANES };

__device__ __forceinline__ float2 ld_bf2(const bf16* row, int lane) {
  return __bfloat1622float2(reinterpret_cast<const __nv_bfloat162*>(row)[lane]);
}

// x (FP32 [rows][n_in]) -> BF16 [rows][W], zero-padded
__global__ void k_pack_x(int rows, int n_in, const float* __restrict__ x, bf16* __restrict__ X) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)rows * W) return;
  const int i = (int)(t / W), f = (int)(t % W);
  X[t] = __float2bfloat16_rn(f < n_in ? x[(size_t)i * n_in + f] : 0.0f);
}

// ---- forward layers on the tensor cores
constexpr int kTcRows = 128;                         // nodes per CTA (the MMA's M)
constexpr int kTcThreads = 128;                      // four warps: TMEM lanes 32 w .. 32 w + 31
constexpr int kActTile = kTcRows * W * 2;            // 16 KB of BF16
constexpr int kWTile = W * W * 2;                    // 8 KB
constexpr int kTcSmem = 2 * (kActTile + kWTile) + 1024;   // two inputs (MODE 1)
constexpr int kTcSmem1 = kActTile + kWTile + 1024;        // one input (MODE 0, 2)
// kind::f16: FP32 accumulator, BF16 A and B, both K-major, N = 64, M = 128
constexpr uint32_t kIdescFwd = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(W >> 3) << 17) |
                               ((uint32_t)(kTcRows >> 4) << 24);

// A tile of ROWS rows of a row-major [*][64] BF16 array is ROWS * 8 pieces of
// 16 bytes; thread t holds pieces t, t + 128, ...  All of a thread's loads
// are issued before any store, so a tile costs one memory round trip.
template <int ROWS>
__device__ __forceinline__ void load_rows(uint4 (&v)[ROWS * 8 / kTcThreads], const bf16* __restrict__ src,
                                          int valid) {
  static_assert(ROWS * 8 % kTcThreads == 0, "whole pieces per thread");
#pragma unroll
  for (int j = 0; j < ROWS * 8 / kTcThreads; ++j) {
    const int e = (int)threadIdx.x + j * kTcThreads, r = e >> 3, c = e & 7;
    v[j] = r < valid ? reinterpret_cast<const uint4*>(src + (size_t)r * W)[c] : make_uint4(0u, 0u, 0u, 0u);
  }
}

// The pieces into the canonical no-swizzle K-major layout: 8 x 16-byte core
// matrices, the 8 K-adjacent cores of an 8-row group contiguous (128 B
// apart), 8-row groups 1024 B apart; rows at or past `valid` are zero.
template <int ROWS>
__device__ __forceinline__ void store_rows(uint8_t* tile, const uint4 (&v)[ROWS * 8 / kTcThreads]) {
#pragma unroll
  for (int j = 0; j < ROWS * 8 / kTcThreads; ++j) {
    const int e = (int)threadIdx.x + j * kTcThreads, r = e >> 3, c = e & 7;
    *reinterpret_cast<uint4*>(tile + ((r >> 3) * 8 + c) * 128 + (r & 7) * 16) = v[j];
  }
}

// MODE 0: encoder  H = relu(in1 W1^T + b)
// MODE 1: message  R = relu(in1 W1^T + in2 W2^T + b), H = in1 + R
// MODE 2: decoder  Y = in1 W1^T + b (FP32, first n_out columns)
// A wait that runs out (about two seconds) raises *err and leaves the rows
// unwritten; the TMEM is freed either way.
template <int MODE>
__global__ void __launch_bounds__(kTcThreads) k_fwd_tc(int n, const bf16* __restrict__ in1, const bf16* __restrict__ in2,
                                                       const bf16* __restrict__ wb, int off_w1, int off_w2,
                                                       const float* __restrict__ master, int off_b,
                                                       bf16* __restrict__ outR, bf16* __restrict__ outH,
                                                       float* __restrict__ outY, int n_out, unsigned* err) {
  using namespace bxtc;
  extern __shared__ uint8_t tc_smem_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* a1 = sm;
  uint8_t* b1 = a1 + kActTile;
  uint8_t* a2 = b1 + kWTile;
  uint8_t* b2 = a2 + kActTile;
  __shared__ __align__(8) uint64_t done;
  __shared__ uint32_t tmem_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r0 = blockIdx.x * kTcRows;
  const int valid = min(kTcRows, n - r0);

  if (MODE == 1) {
    // both activation tiles in one round trip, then both weight tiles (L2-resident)
    uint4 va[kTcRows * 8 / kTcThreads], vb[kTcRows * 8 / kTcThreads];
    load_rows<kTcRows>(va, in1 + (size_t)r0 * W, valid);
    load_rows<kTcRows>(vb, in2 + (size_t)r0 * W, valid);
    store_rows<kTcRows>(a1, va);
    store_rows<kTcRows>(a2, vb);
    uint4 w1[W * 8 / kTcThreads], w2[W * 8 / kTcThreads];
    load_rows<W>(w1, wb + off_w1, W);
    load_rows<W>(w2, wb + off_w2, W);
    store_rows<W>(b1, w1);
    store_rows<W>(b2, w2);
  } else {
    uint4 va[kTcRows * 8 / kTcThreads], w1[W * 8 / kTcThreads];
    load_rows<kTcRows>(va, in1 + (size_t)r0 * W, valid);
    load_rows<W>(w1, wb + off_w1, W);
    store_rows<kTcRows>(a1, va);
    store_rows<W>(b1, w1);
  }
  // the tensor core reads shared memory through the async proxy
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&done), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(W));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (threadIdx.x == 0) {
#pragma unroll
    for (int kk = 0; kk < W / 16; ++kk) {     // two K-adjacent core matrices per MMA (K = 16)
      const uint32_t o = (uint32_t)kk * 256u;
      mma_f16(tmem, smem_desc(smem_u32(a1) + o, 128, 1024), smem_desc(smem_u32(b1) + o, 128, 1024), kIdescFwd,
              kk > 0 ? 1u : 0u);
    }
    if (MODE == 1)
#pragma unroll
      for (int kk = 0; kk < W / 16; ++kk) {
        const uint32_t o = (uint32_t)kk * 256u;
        mma_f16(tmem, smem_desc(smem_u32(a2) + o, 128, 1024), smem_desc(smem_u32(b2) + o, 128, 1024), kIdescFwd,
                1u);
      }
    mma_commit(smem_u32(&done));
  }
  __syncwarp();
  const bool ok = __all_sync(FULL, mbar_wait(smem_u32(&done), 0u));
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    float v[W];
#pragma unroll
    for (int c0 = 0; c0 < W; c0 += 16) tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v + c0);
    const int r = r0 + warp * 32 + lane;
    if (r < n) {
      const size_t o = (size_t)r * W;
#pragma unroll
      for (int f = 0; f < W; ++f) v[f] += master[off_b + f];
      if (MODE == 2) {
#pragma unroll
        for (int f = 0; f < W; ++f)           // constant indices keep v in registers
          if (f < n_out) outY[(size_t)r * n_out + f] = v[f];
      } else {
#pragma unroll
        for (int f8 = 0; f8 < W; f8 += 8) {
          __align__(16) bf16 rr[8], hh[8];
          const uint4 x = reinterpret_cast<const uint4*>(in1 + o)[f8 / 8];
          const bf16* xb = reinterpret_cast<const bf16*>(&x);
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            rr[q] = __float2bfloat16_rn(fmaxf(v[f8 + q], 0.f));
            hh[q] = MODE == 1 ? __float2bfloat16_rn(__bfloat162float(xb[q]) + __bfloat162float(rr[q])) : rr[q];
          }
          if (MODE == 1) reinterpret_cast<uint4*>(outR + o)[f8 / 8] = *reinterpret_cast<const uint4*>(rr);
          reinterpret_cast<uint4*>(outH + o)[f8 / 8] = *reinterpret_cast<const uint4*>(hh);
        }
      }
    }
  } else if (lane == 0) {
    atomicOr(err, 1u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(W));
  }
}

// A_i = mean_{j in nbr(i)} H_j for local nodes i in [0, n) of a range starting at lo
__global__ void k_agg(int n, int lo, const int* __restrict__ ptr, const int* __restrict__ nbr,
                      const bf16* __restrict__ H, bf16* __restrict__ A) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < n; i += nw) {
    const int a = ptr[lo + i], b = ptr[lo + i + 1];
    float sx = 0.f, sy = 0.f;
    for (int p = a; p < b; ++p) {
      const float2 h = ld_bf2(H + (size_t)(nbr[p] - lo) * W, lane);
      sx += h.x;
      sy += h.y;
    }
    if (b > a) {
      sx /= (float)(b - a);
      sy /= (float)(b - a);
    }
    reinterpret_cast<__nv_bfloat162*>(A + (size_t)i * W)[lane] = __floats2bfloat162_rn(sx, sy);
  }
}

// dY = 2 (Yhat - Y) / (N n_out) in the first n_out columns; per-block sums of squares
__global__ void k_loss(int n, int n_out, const float* __restrict__ yhat, const float* __restrict__ y,
                       float* __restrict__ dY, float* __restrict__ part) {
  __shared__ float red[kThreads / 32];
  const float scale = 2.0f / ((float)n * (float)n_out);
  float s = 0.f;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < (long long)n * W;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t / W), f = (int)(t % W);
    float d = 0.f;
    if (f < n_out) {
      const float e = yhat[(size_t)i * n_out + f] - y[(size_t)i * n_out + f];
      s += e * e;
      d = scale * e;
    }
    dY[t] = d;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < kThreads / 32; ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}

// MODE 0 (decoder): dH = dIn W1 (dZ = dIn)
// MODE 1 (message): dZ = dIn * (R > 0); dHprev = dIn + dZ W1; G = dZ W2
// MODE 2 (encoder): dZ = dIn * (H0 > 0)
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_bwd(int n, const float* __restrict__ dIn, const bf16* __restrict__ mask,
                                                  const bf16* __restrict__ wb, int off_w1, int off_w2,
                                                  float* __restrict__ dZ, float* __restrict__ out1,
                                                  float* __restrict__ out2) {
  __shared__ float w1[MODE == 2 ? 1 : W * W];
  __shared__ float w2[MODE == 1 ? W * W : 1];
  if (MODE != 2) {
    for (int e = threadIdx.x; e < W * W; e += blockDim.x) {
      w1[e] = __bfloat162float(wb[off_w1 + e]);
      if (MODE == 1) w2[e] = __bfloat162float(wb[off_w2 + e]);
    }
    __syncthreads();
  }
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < n; i += nw) {
    const size_t o = (size_t)i * W;
    float d0 = dIn[o + lane], d1 = dIn[o + lane + 32];  // f = lane, lane + 32
    if (MODE != 0) {
      if (!(__bfloat162float(mask[o + lane]) > 0.f)) d0 = 0.f;
      if (!(__bfloat162float(mask[o + lane + 32]) > 0.f)) d1 = 0.f;
      dZ[o + lane] = d0;
      dZ[o + lane + 32] = d1;
    }
    if (MODE == 2) continue;
    float p0 = 0.f, p1 = 0.f, q0 = 0.f, q1 = 0.f;  // k = lane, lane + 32
#pragma unroll 8
    for (int src = 0; src < 32; ++src) {
      const float z0 = __shfl_sync(FULL, d0, src), z1 = __shfl_sync(FULL, d1, src);  // f = src, src + 32
      p0 = fmaf(w1[src * W + lane], z0, p0);
      p0 = fmaf(w1[(src + 32) * W + lane], z1, p0);
      p1 = fmaf(w1[src * W + lane + 32], z0, p1);
      p1 = fmaf(w1[(src + 32) * W + lane + 32], z1, p1);
      if (MODE == 1) {
        q0 = fmaf(w2[src * W + lane], z0, q0);
        q0 = fmaf(w2[(src + 32) * W + lane], z1, q0);
        q1 = fmaf(w2[src * W + lane + 32], z0, q1);
        q1 = fmaf(w2[(src + 32) * W + lane + 32], z1, q1);
      }
    }
    if (MODE == 0) {
      out1[o + lane] = p0;
      out1[o + lane + 32] = p1;
    } else {
      out1[o + lane] = dIn[o + lane] + p0;
      out1[o + lane + 32] = dIn[o + lane + 32] + p1;
      out2[o + lane] = q0;
      out2[o + lane + 32] = q1;
    }
  }
}

// dH_j += sum over i with j in nbr(i) of G_i / deg_i (transposed CSR, local ids)
__global__ void k_aggT_add(int n, int lo, const int* __restrict__ ptrT, const int* __restrict__ nbrT,
                           const float* __restrict__ inv_deg, const float* __restrict__ G, float* __restrict__ dH) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int j = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); j < n; j += nw) {
    float s0 = 0.f, s1 = 0.f;
    for (int p = ptrT[lo + j]; p < ptrT[lo + j + 1]; ++p) {
      const int i = nbrT[p] - lo;
      const float w = inv_deg[lo + i];
      s0 = fmaf(G[(size_t)i * W + lane], w, s0);
      s1 = fmaf(G[(size_t)i * W + lane + 32], w, s1);
    }
    dH[(size_t)j * W + lane] += s0;
    dH[(size_t)j * W + lane + 32] += s1;
  }
}

// part[b] = (sum over this block's nodes of dZ^T In  [W][W],  sum of dZ [W])
constexpr int kWgTile = 32;
__global__ void __launch_bounds__(kThreads) k_wgrad(int n, const float* __restrict__ dZ, const bf16* __restrict__ In,
                                                    float* __restrict__ part) {
  __shared__ float sz[kWgTile][W];
  __shared__ float si[kWgTile][W];
  const int f = threadIdx.x & (W - 1), kq = threadIdx.x >> 6;  // 4 groups of 16 inputs
  const int per = (n + gridDim.x - 1) / gridDim.x;
  const int i0 = blockIdx.x * per, i1 = min(n, i0 + per);
  float acc[16], bacc = 0.f;
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = 0.f;
  for (int t0 = i0; t0 < i1; t0 += kWgTile) {
    const int cnt = min(kWgTile, i1 - t0);
    for (int e = threadIdx.x; e < kWgTile * W; e += blockDim.x) {
      const int r = e / W, c = e - r * W;
      sz[r][c] = r < cnt ? dZ[(size_t)(t0 + r) * W + c] : 0.f;
      si[r][c] = r < cnt ? __bfloat162float(In[(size_t)(t0 + r) * W + c]) : 0.f;
    }
    __syncthreads();
    for (int r = 0; r < cnt; ++r) {
      const float d = sz[r][f];
      bacc += d;
#pragma unroll
      for (int q = 0; q < 16; ++q) acc[q] = fmaf(d, si[r][kq * 16 + q], acc[q]);
    }
    __syncthreads();
  }
  float* pb = part + (size_t)blockIdx.x * (W * W + W);
#pragma unroll
  for (int q = 0; q < 16; ++q) pb[f * W + kq * 16 + q] = acc[q];
  if (kq == 0) pb[W * W + f] = bacc;
}

// grad[off_w + e] (= or +=) sum_b part[b][e]; bias to grad[off_b + f] when off_b >= 0
__global__ void k_wgrad_reduce(int nblk, const float* __restrict__ part, float* __restrict__ grad, int off_w,
                               int off_b) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= W * W + W) return;
  float s = 0.f;
  for (int b = 0; b < nblk; ++b) s += part[(size_t)b * (W * W + W) + e];
  if (e < W * W) grad[off_w + e] = s;
  else if (off_b >= 0) grad[off_b + e - W * W] = s;
}

__global__ void k_sum_parts(int n, const float* __restrict__ part, float scale, float* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    float s = 0.f;
    for (int b = 0; b < n; ++b) s += part[b];
    *out = s * scale;
  }
}

__global__ void k_adam(int np, float* __restrict__ master, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, bf16* __restrict__ wb, float lr, float b1, float b2, float eps,
                       float bc1, float bc2) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= np) return;
  const float gg = g[e];
  const float mm = b1 * m[e] + (1.f - b1) * gg;
  const float vv = b2 * v[e] + (1.f - b2) * gg * gg;
  m[e] = mm;
  v[e] = vv;
  const float w = master[e] - lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
  master[e] = w;
  wb[e] = __float2bfloat16_rn(w);
}

__global__ void k_to_bf16(int np, const float* __restrict__ src, bf16* __restrict__ dst) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < np) dst[e] = __float2bfloat16_rn(src[e]);
}

}  // namespace bxn

struct bx_gnn {
  float *master = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr;
  __nv_bfloat16* wb = nullptr;
  int n_graph = 0;
  int *ptr = nullptr, *nbr = nullptr, *ptrT = nullptr, *nbrT = nullptr;
  float* inv_deg = nullptr;
  int cap = 0;                              // activation rows
  __nv_bfloat16* act = nullptr;             // N_PLANES x [cap][W]
  float *yhat = nullptr, *dY = nullptr, *dHa = nullptr, *dHb = nullptr, *dZ = nullptr, *G = nullptr;
  float *part = nullptr, *loss_part = nullptr, *loss = nullptr;
  unsigned* err = nullptr;                  // a tensor-core wait ran out (k_fwd_tc)
  int nblk_wg = 0, nblk_loss = 0;
  int step = 0;
  cudaStream_t stream = nullptr;
  std::vector<int> h_ptr, h_nbr;            // host copy: node ranges are checked for closure
  int ok_lo = -1, ok_hi = -1;               // last range found closed under adjacency
};

namespace {

using bxn::W;

int nfail(int code, const std::string& msg) {
  bx_record_error(msg.c_str());
  return code;
}
#define NX(call)                                                                            \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) return nfail(BX_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

unsigned node_grid(int n) {
  return (unsigned)std::max(1, std::min((n + 7) / 8, 152 * 8));
}

int ensure_cap(bx_gnn* h, int rows) {
  if (rows <= h->cap) return BX_OK;
  void* ptrs[] = {h->act, h->yhat, h->dY, h->dHa, h->dHb, h->dZ, h->G};
  for (void* p : ptrs) cudaFree(p);
  h->act = nullptr;
  h->yhat = h->dY = h->dHa = h->dHb = h->dZ = h->G = nullptr;
  h->cap = 0;
  const size_t r = (size_t)rows;
  if (cudaMalloc(&h->act, (size_t)bxn::N_PLANES * r * W * sizeof(__nv_bfloat16)) != cudaSuccess ||
      cudaMalloc(&h->yhat, r * W * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&h->dY, r * W * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&h->dHa, r * W * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&h->dHb, r * W * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&h->dZ, r * W * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&h->G, r * W * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    return nfail(BX_ENOMEM, "cudaMalloc network activations");
  }
  h->cap = rows;
  return BX_OK;
}

__nv_bfloat16* plane(bx_gnn* h, int p) { return h->act + (size_t)p * h->cap * W; }

// after a synchronisation: did a tensor-core wait run out?
int check_tc(bx_gnn* h) {
  unsigned e = 0;
  NX(cudaMemcpy(&e, h->err, 4, cudaMemcpyDeviceToHost));
  if (e) return nfail(BX_ECUDA, "network: a tensor-core wait timed out");
  return BX_OK;
}

int check_range(bx_gnn* h, int lo, int hi) {
  if (!h->ptr) return nfail(BX_ESTATE, "network: bx_gnn_set_graph first");
  if (lo < 0 || hi <= lo || hi > h->n_graph) return nfail(BX_EINVAL, "network: node range outside the graph");
  if (lo != h->ok_lo || hi != h->ok_hi) {
    // every neighbour of a node in [lo, hi) must lie in [lo, hi) (whole clusters)
    for (int p = h->h_ptr[lo]; p < h->h_ptr[hi]; ++p)
      if (h->h_nbr[p] < lo || h->h_nbr[p] >= hi)
        return nfail(BX_EINVAL, "network: node range cuts through a cluster (neighbour outside the range)");
    h->ok_lo = lo;
    h->ok_hi = hi;
  }
  return ensure_cap(h, hi - lo);
}

int forward(bx_gnn* h, int lo, int hi, const float* x, int n_in, int n_out) {
  using namespace bxn;
  const int n = hi - lo;
  cudaStream_t s = h->stream;
  const long long tot = (long long)n * W;
  k_pack_x<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(n, n_in, x, plane(h, P_X));
  const unsigned g = node_grid(n);
  const unsigned gt = (unsigned)((n + kTcRows - 1) / kTcRows);
  k_fwd_tc<0><<<gt, kTcThreads, kTcSmem1, s>>>(n, plane(h, P_X), nullptr, h->wb, OFF_W0, 0, h->master, OFF_B0,
                                              nullptr, plane(h, P_H0), nullptr, 0, h->err);
  for (int l = 0; l < NMP; ++l) {
    const int o = OFF_MP + l * MP_STRIDE;
    k_agg<<<g, kThreads, 0, s>>>(n, lo, h->ptr, h->nbr, plane(h, P_H0 + l), plane(h, P_A1 + l));
    k_fwd_tc<1><<<gt, kTcThreads, kTcSmem, s>>>(n, plane(h, P_H0 + l), plane(h, P_A1 + l), h->wb, o, o + W * W,
                                                h->master, o + 2 * W * W, plane(h, P_R1 + l), plane(h, P_H1 + l),
                                                nullptr, 0, h->err);
  }
  k_fwd_tc<2><<<gt, kTcThreads, kTcSmem1, s>>>(n, plane(h, P_H3), nullptr, h->wb, OFF_WD, 0, h->master, OFF_BD,
                                              nullptr, nullptr, h->yhat, n_out, h->err);
  NX(cudaGetLastError());
  return BX_OK;
}

int backward(bx_gnn* h, int lo, int hi, const float* y, int n_out) {
  using namespace bxn;
  const int n = hi - lo;
  cudaStream_t s = h->stream;
  const unsigned g = node_grid(n);
  k_loss<<<h->nblk_loss, kThreads, 0, s>>>(n, n_out, h->yhat, y, h->dY, h->loss_part);
  k_sum_parts<<<1, 32, 0, s>>>(h->nblk_loss, h->loss_part, 1.0f / ((float)n * (float)n_out), h->loss);
  auto wgrad = [&](const float* dz, const __nv_bfloat16* in, int off_w, int off_b) {
    k_wgrad<<<h->nblk_wg, kThreads, 0, s>>>(n, dz, in, h->part);
    k_wgrad_reduce<<<(W * W + W + 255) / 256, 256, 0, s>>>(h->nblk_wg, h->part, h->grad, off_w, off_b);
  };
  // decoder: dWd = dY^T H3, dbd = sum dY, dH3 = dY Wd
  wgrad(h->dY, plane(h, P_H3), OFF_WD, OFF_BD);
  k_bwd<0><<<g, kThreads, 0, s>>>(n, h->dY, nullptr, h->wb, OFF_WD, 0, nullptr, h->dHa, nullptr);
  float *dH = h->dHa, *dHn = h->dHb;
  for (int l = NMP - 1; l >= 0; --l) {
    const int o = OFF_MP + l * MP_STRIDE;
    k_bwd<1><<<g, kThreads, 0, s>>>(n, dH, plane(h, P_R1 + l), h->wb, o, o + W * W, h->dZ, dHn, h->G);
    k_aggT_add<<<g, kThreads, 0, s>>>(n, lo, h->ptrT, h->nbrT, h->inv_deg, h->G, dHn);
    wgrad(h->dZ, plane(h, P_H0 + l), o, o + 2 * W * W);
    wgrad(h->dZ, plane(h, P_A1 + l), o + W * W, -1);
    std::swap(dH, dHn);
  }
  k_bwd<2><<<g, kThreads, 0, s>>>(n, dH, plane(h, P_H0), nullptr, 0, 0, h->dZ, nullptr, nullptr);
  wgrad(h->dZ, plane(h, P_X), OFF_W0, OFF_B0);
  NX(cudaGetLastError());
  return BX_OK;
}

}  // namespace

extern "C" {

int bx_gnn_create(bx_gnn_handle* out) {
  if (!out) return nfail(BX_EINVAL, "null argument");
  bx_gnn* h = new bx_gnn();
  h->nblk_wg = 152 * 2;
  h->nblk_loss = 152 * 4;
  const size_t P = bxn::NP;
  if (cudaMalloc(&h->master, P * 4) != cudaSuccess || cudaMalloc(&h->m, P * 4) != cudaSuccess ||
      cudaMalloc(&h->v, P * 4) != cudaSuccess || cudaMalloc(&h->grad, P * 4) != cudaSuccess ||
      cudaMalloc(&h->wb, P * 2) != cudaSuccess ||
      cudaMalloc(&h->part, (size_t)h->nblk_wg * (W * W + W) * 4) != cudaSuccess ||
      cudaMalloc(&h->loss_part, (size_t)h->nblk_loss * 4) != cudaSuccess ||
      cudaMalloc(&h->loss, 4) != cudaSuccess || cudaMalloc(&h->err, 4) != cudaSuccess ||
      cudaStreamCreate(&h->stream) != cudaSuccess) {
    cudaGetLastError();
    bx_gnn_destroy(h);
    return nfail(BX_ENOMEM, "cudaMalloc network parameters");
  }
  if (cudaFuncSetAttribute(bxn::k_fwd_tc<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, bxn::kTcSmem) !=
          cudaSuccess ||
      cudaFuncSetAttribute(bxn::k_fwd_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, bxn::kTcSmem) !=
          cudaSuccess ||
      cudaFuncSetAttribute(bxn::k_fwd_tc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bxn::kTcSmem) !=
          cudaSuccess) {
    cudaGetLastError();
    bx_gnn_destroy(h);
    return nfail(BX_ECUDA, "network: shared memory attribute of the tensor-core layers");
  }
  cudaMemset(h->err, 0, 4);
  cudaMemset(h->master, 0, P * 4);
  cudaMemset(h->m, 0, P * 4);
  cudaMemset(h->v, 0, P * 4);
  cudaMemset(h->wb, 0, P * 2);
  *out = h;
  return BX_OK;
}

int bx_gnn_n_params(void) { return bxn::NP; }

int bx_gnn_set_params(bx_gnn_handle h, const float* params) {
  if (!h || !params) return nfail(BX_EINVAL, "null argument");
  NX(cudaMemcpy(h->master, params, bxn::NP * 4, cudaMemcpyHostToDevice));
  NX(cudaMemset(h->m, 0, bxn::NP * 4));
  NX(cudaMemset(h->v, 0, bxn::NP * 4));
  bxn::k_to_bf16<<<(bxn::NP + 255) / 256, 256, 0, h->stream>>>(bxn::NP, h->master, h->wb);
  NX(cudaGetLastError());
  NX(cudaStreamSynchronize(h->stream));
  h->step = 0;
  return BX_OK;
}

int bx_gnn_get_params(bx_gnn_handle h, float* params) {
  if (!h || !params) return nfail(BX_EINVAL, "null argument");
  NX(cudaStreamSynchronize(h->stream));
  NX(cudaMemcpy(params, h->master, bxn::NP * 4, cudaMemcpyDeviceToHost));
  return BX_OK;
}

int bx_gnn_set_graph(bx_gnn_handle h, int n_nodes, const int32_t* ptr, const int32_t* nbr) {
  if (!h || !ptr || n_nodes <= 0) return nfail(BX_EINVAL, "bad graph arguments");
  const int nnz = ptr[n_nodes];
  if (ptr[0] != 0 || nnz < 0 || (nnz > 0 && !nbr)) return nfail(BX_EINVAL, "bad row pointers");
  std::vector<int> cnt(n_nodes + 1, 0);
  std::vector<float> inv(n_nodes, 0.f);
  for (int i = 0; i < n_nodes; ++i) {
    if (ptr[i + 1] < ptr[i]) return nfail(BX_EINVAL, "row pointers decrease");
    const int d = ptr[i + 1] - ptr[i];
    inv[i] = d > 0 ? 1.0f / (float)d : 0.f;
    for (int p = ptr[i]; p < ptr[i + 1]; ++p) {
      if (nbr[p] < 0 || nbr[p] >= n_nodes) return nfail(BX_EINVAL, "neighbour index out of range");
      cnt[nbr[p] + 1]++;
    }
  }
  for (int j = 0; j < n_nodes; ++j) cnt[j + 1] += cnt[j];
  std::vector<int> ptrT(cnt), nbrT(std::max(nnz, 1));
  std::vector<int> fill(cnt.begin(), cnt.end() - 1);
  for (int i = 0; i < n_nodes; ++i)
    for (int p = ptr[i]; p < ptr[i + 1]; ++p) nbrT[fill[nbr[p]]++] = i;
  void* old[] = {h->ptr, h->nbr, h->ptrT, h->nbrT, h->inv_deg};
  for (void* p : old) cudaFree(p);
  h->ptr = h->nbr = h->ptrT = h->nbrT = nullptr;
  h->inv_deg = nullptr;
  const size_t nz = (size_t)std::max(nnz, 1);
  if (cudaMalloc(&h->ptr, (size_t)(n_nodes + 1) * 4) != cudaSuccess || cudaMalloc(&h->nbr, nz * 4) != cudaSuccess ||
      cudaMalloc(&h->ptrT, (size_t)(n_nodes + 1) * 4) != cudaSuccess ||
      cudaMalloc(&h->nbrT, nz * 4) != cudaSuccess || cudaMalloc(&h->inv_deg, (size_t)n_nodes * 4) != cudaSuccess) {
    cudaGetLastError();
    return nfail(BX_ENOMEM, "cudaMalloc graph");
  }
  NX(cudaMemcpy(h->ptr, ptr, (size_t)(n_nodes + 1) * 4, cudaMemcpyHostToDevice));
  if (nnz > 0) NX(cudaMemcpy(h->nbr, nbr, (size_t)nnz * 4, cudaMemcpyHostToDevice));
  NX(cudaMemcpy(h->ptrT, ptrT.data(), (size_t)(n_nodes + 1) * 4, cudaMemcpyHostToDevice));
  NX(cudaMemcpy(h->nbrT, nbrT.data(), nz * 4, cudaMemcpyHostToDevice));
  NX(cudaMemcpy(h->inv_deg, inv.data(), (size_t)n_nodes * 4, cudaMemcpyHostToDevice));
  h->n_graph = n_nodes;
  h->h_ptr.assign(ptr, ptr + n_nodes + 1);
  h->h_nbr.assign(nbr, nbr + nnz);
  h->ok_lo = h->ok_hi = -1;
  return BX_OK;
}

int bx_gnn_forward(bx_gnn_handle h, int lo, int hi, const float* x, int n_in, float* y, int n_out) {
  if (!h || !x || !y || n_in <= 0 || n_in > W || n_out <= 0 || n_out > W)
    return nfail(BX_EINVAL, "bx_gnn_forward: bad arguments");
  int rc = check_range(h, lo, hi);
  if (rc != BX_OK) return rc;
  rc = forward(h, lo, hi, x, n_in, n_out);
  if (rc != BX_OK) return rc;
  NX(cudaMemcpyAsync(y, h->yhat, (size_t)(hi - lo) * n_out * 4, cudaMemcpyDeviceToDevice, h->stream));
  NX(cudaStreamSynchronize(h->stream));
  return check_tc(h);
}

int bx_gnn_gradients(bx_gnn_handle h, int lo, int hi, const float* x, int n_in, const float* y, int n_out,
                     float* grad_host, float* loss_host) {
  if (!h || !x || !y || !grad_host || n_in <= 0 || n_in > W || n_out <= 0 || n_out > W)
    return nfail(BX_EINVAL, "bx_gnn_gradients: bad arguments");
  int rc = check_range(h, lo, hi);
  if (rc == BX_OK) rc = forward(h, lo, hi, x, n_in, n_out);
  if (rc == BX_OK) rc = backward(h, lo, hi, y, n_out);
  if (rc != BX_OK) return rc;
  NX(cudaStreamSynchronize(h->stream));
  NX(cudaMemcpy(grad_host, h->grad, bxn::NP * 4, cudaMemcpyDeviceToHost));
  if (loss_host) NX(cudaMemcpy(loss_host, h->loss, 4, cudaMemcpyDeviceToHost));
  return check_tc(h);
}

int bx_gnn_train_step(bx_gnn_handle h, int lo, int hi, const float* x, int n_in, const float* y, int n_out, float lr,
                      float* loss_host) {
  if (!h || !x || !y || n_in <= 0 || n_in > W || n_out <= 0 || n_out > W || !(lr > 0.f))
    return nfail(BX_EINVAL, "bx_gnn_train_step: bad arguments");
  int rc = check_range(h, lo, hi);
  if (rc == BX_OK) rc = forward(h, lo, hi, x, n_in, n_out);
  if (rc == BX_OK) rc = backward(h, lo, hi, y, n_out);
  if (rc != BX_OK) return rc;
  const float b1 = 0.9f, b2 = 0.999f;
  h->step += 1;
  const float bc1 = 1.f - powf(b1, (float)h->step), bc2 = 1.f - powf(b2, (float)h->step);
  bxn::k_adam<<<(bxn::NP + 255) / 256, 256, 0, h->stream>>>(bxn::NP, h->master, h->m, h->v, h->grad, h->wb, lr, b1,
                                                           b2, 1e-8f, bc1, bc2);
  NX(cudaGetLastError());
  if (loss_host) {
    NX(cudaMemcpyAsync(loss_host, h->loss, 4, cudaMemcpyDeviceToHost, h->stream));
    NX(cudaStreamSynchronize(h->stream));
    return check_tc(h);
  }
  return BX_OK;
}

int bx_gnn_destroy(bx_gnn_handle h) {
  if (!h) return BX_OK;
  void* ptrs[] = {h->master, h->m, h->v, h->grad, h->wb, h->ptr, h->nbr, h->ptrT, h->nbrT, h->inv_deg,
                  h->act, h->yhat, h->dY, h->dHa, h->dHb, h->dZ, h->G, h->part, h->loss_part, h->loss, h->err};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return BX_OK;
}

}  // extern "C"
