// bx_probe.cu -- the FP64 throughput probe behind the plain form's FP64 roofline.
//
// The plain FP64 step is bound by GB300's FP64 pipe rather than by HBM, so its
// roofline needs the pipe's peak rate on this part, measured rather than taken
// from a data sheet.  k_fp64_fma keeps the pipe saturated: every thread runs
// kChains independent FMA chains (enough independent work per warp to cover
// the FMA latency), so the launch issues exactly
//   n_blocks * kThreads / 32 * kChains * iters
// FP64 warp instructions in its loop, plus a final reduction of kChains - 1
// additions per thread.  The host times the launch with events on its stream.
#include <cuda_runtime.h>

#include "../../include/bx.h"

void bx_record_error(const char* msg);

namespace {

constexpr int kThreads = 256;
constexpr int kChains = 8;

__global__ void __launch_bounds__(kThreads) k_fp64_fma(int iters, double b, double c, double* __restrict__ out) {
  const int g = blockIdx.x * kThreads + threadIdx.x;
  double a[kChains];
#pragma unroll
  for (int j = 0; j < kChains; ++j) a[j] = (double)(g + j);
#pragma unroll 4
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int j = 0; j < kChains; ++j) a[j] = fma(a[j], b, c);
  }
  double s = a[0];
#pragma unroll
  for (int j = 1; j < kChains; ++j) s += a[j];
  out[g] = s;   // keeps every chain live
}

}  // namespace

extern "C" int bx_fp64_fma_probe(int n_blocks, int iters, double b, double c, double* out, void* stream) {
  // thread indices are int: at most 2^22 CTAs of 256 threads
  if (n_blocks <= 0 || n_blocks > (1 << 22) || iters <= 0 || !out) {
    bx_record_error("bx_fp64_fma_probe: bad arguments");
    return BX_EINVAL;
  }
  k_fp64_fma<<<n_blocks, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(iters, b, c, out);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    bx_record_error(cudaGetErrorString(e));
    return BX_ECUDA;
  }
  return BX_OK;
}
