// bx_noalloc.cu -- the plain FP64 step on caller-owned device memory, with no
// allocation of any kind.
//
// Who needs it: code that must not allocate device memory while it steps --
// a caller whose device memory is owned by another framework's pool, or one
// that steps from a context where cudaMalloc is forbidden or too slow (a
// real-time loop, an allocator-free embedding).  bx_cluster_create allocates
// every buffer a handle needs; this entry point instead takes the caller's
// device buffers and keeps the step's scratch (derived index maps, the CTA
// tiling, the per-CTA partial sums of the well-mixed environment and the
// check_v / no_negs counters) in one file-scope __device__ array of fixed size.
//
// Limits (checked before any step; BX_EINVAL beyond them):
//   n_cells <= 16384, n_mems <= 131072, n_ions <= 8, and every run of 16
//   consecutive cells has at most 256 membranes.
// The caller's cell_mem_ptr and nn_i are checked on the device before any
// step (cell_mem_ptr[0] == 0, cell_mem_ptr[C] == M, strictly increasing;
// 0 <= nn_i[m] < M); no index outside the array is written or read.
// The array lives on every GPU that loads the library until the process
// exits: 140,297 doubles, about 1.1 MB (kScratchDoubles).
//
// Sharing: every call uses the same array and leaves the last call's contents
// in it; each call rebuilds what it reads before it reads it.  Calls that
// overlap on the GPU (two streams, or two host threads) race on the array and
// corrupt each other's results: serialise them.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/bx.h"
#include "bx_launch.cuh"

namespace {

constexpr int kMaxCells = 16384;
constexpr int kMaxMems = 131072;
constexpr int kTileCells = 16;
constexpr int kTileThreads = 256;
constexpr int kMaxTiles = kMaxCells / kTileCells;
// layout of the scratch, in 8-byte words
constexpr size_t kOffM2c = 0;                                   // int32 [kMaxMems]
constexpr size_t kOffNnCell = kOffM2c + kMaxMems / 2;           // int32 [kMaxMems]
constexpr size_t kOffBlk = kOffNnCell + kMaxMems / 2;           // int32 [kMaxTiles + 1]
constexpr size_t kOffBlkCl = kOffBlk + (kMaxTiles + 2) / 2;     // int32 [kMaxTiles]
constexpr size_t kOffClBlk = kOffBlkCl + kMaxTiles / 2;         // int32 [2]
constexpr size_t kOffPart = kOffClBlk + 1;                      // double [kMaxTiles * 8]
constexpr size_t kOffPump = kOffPart + (size_t)kMaxTiles * BX_MAX_IONS;  // double [1]
constexpr size_t kOffEscale = kOffPump + 1;                     // double [1]
constexpr size_t kOffStatus = kOffEscale + 1;                   // u64 [4]
constexpr size_t kOffFlag = kOffStatus + 4;                     // int32 [2]: tile overflow, bad map
constexpr size_t kScratchDoubles = kOffFlag + 1;

static __device__ __align__(256) double g_scratch[kScratchDoubles];

}  // namespace

// error text for bx_last_error (defined with the other entry points)
void bx_record_error(const char* msg);

namespace {

int na_fail(int code, const char* msg) {
  bx_record_error(msg);
  return code;
}

// Set-up: the device address of the scratch array (its name in host code is
// only a host-side stand-in).  It is looked up once per CUDA context, with
// that context current, and cached under its context id: a context that was
// destroyed and created again (cudaDeviceReset) reloads the module, and the
// new context gets a new id, so a stale address is never reused.  The cache
// is guarded by a mutex, so host threads may call concurrently (their GPU
// work still races on the array, see above).
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);

bool current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_cur = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_cur = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  });
  void* ctx = nullptr;
  if (!get_cur || !get_id || get_cur(&ctx) != 0 || !ctx) return false;
  return get_id(ctx, id) == 0;
}

double* scratch_address(int* rc) {
  struct Entry { unsigned long long ctx; double* addr; };
  static std::mutex mu;
  static Entry cache[64];
  static int n_cache = 0;
  unsigned long long ctx = 0;
  if (!current_context_id(&ctx)) {
    // no context is current on this thread yet: make the current device's
    // primary context current (cudaSetDevice initialises it), then ask again
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaSetDevice(dev) != cudaSuccess) {
      *rc = na_fail(BX_ECUDA, "bx_step_fp64_noalloc: no usable CUDA device");
      return nullptr;
    }
  }
  if (!ctx && !current_context_id(&ctx)) {
    *rc = na_fail(BX_ECUDA, "bx_step_fp64_noalloc: cannot identify the current CUDA context");
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(mu);
  for (int k = 0; k < n_cache; ++k)
    if (cache[k].ctx == ctx) { *rc = BX_OK; return cache[k].addr; }
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) {
    *rc = na_fail(BX_ECUDA, "bx_step_fp64_noalloc: cudaGetSymbolAddress failed");
    return nullptr;
  }
  const Entry e{ctx, static_cast<double*>(p)};
  if (n_cache < 64) cache[n_cache++] = e;
  else cache[ctx % 64] = e;          // more contexts than slots: replace one
  *rc = BX_OK;
  return e.addr;
}

// Rebuild the derived maps in the scratch: mem_to_cells, the partner's cell,
// the fixed 16-cell tiling, the per-cluster constants; clear the counters.
// The caller's maps are checked as they are read: flag[0] is raised if a
// tile holds more than 256 membranes, flag[1] if cell_mem_ptr is not a CSR
// row pointer over M membranes or a partner index is out of range, and no
// write or read leaves the arrays.  The host clears both flags before this
// launch.
__global__ void k_noalloc_prep(const int* __restrict__ ptr, const int* __restrict__ nn, int C, int M,
                               double* scratch, double pump, double escale) {
  int* m2c = reinterpret_cast<int*>(scratch + kOffM2c);
  int* blk = reinterpret_cast<int*>(scratch + kOffBlk);
  int* blk_cl = reinterpret_cast<int*>(scratch + kOffBlkCl);
  int* cl_blk = reinterpret_cast<int*>(scratch + kOffClBlk);
  int* flag = reinterpret_cast<int*>(scratch + kOffFlag);
  const int ntile = (C + kTileCells - 1) / kTileCells;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int stride = gridDim.x * blockDim.x;
  if (tid == 0 && (ptr[0] != 0 || ptr[C] != M)) atomicExch(flag + 1, 1);
  for (int c = tid; c < C; c += stride) {
    const int a = ptr[c], e = ptr[c + 1];
    if (a >= e || a < 0 || e > M) { atomicExch(flag + 1, 1); continue; }
    for (int m = a; m < e; ++m) m2c[m] = c;
  }
  for (int m = tid; m < M; m += stride)
    if (nn[m] < 0 || nn[m] >= M) atomicExch(flag + 1, 1);
  for (int b = tid; b <= ntile; b += stride) {
    const int cb = min(b * kTileCells, C);
    blk[b] = cb;
    if (b < ntile) {
      blk_cl[b] = 0;
      const int ce = min(cb + kTileCells, C);
      if (ptr[ce] - ptr[cb] > kTileThreads) atomicExch(flag, 1);
    }
  }
  if (tid == 0) {
    cl_blk[0] = 0;
    cl_blk[1] = ntile;
    scratch[kOffPump] = pump;
    scratch[kOffEscale] = escale;
    unsigned long long* st = reinterpret_cast<unsigned long long*>(scratch + kOffStatus);
    st[0] = st[1] = st[2] = st[3] = 0ull;
  }
}

// The partner's cell; an out-of-range partner (flagged by the prep kernel) is
// skipped, and the call returns before any step reads the map.
__global__ void k_noalloc_nn_cell(const int* __restrict__ nn, int M, double* scratch) {
  const int* m2c = reinterpret_cast<const int*>(scratch + kOffM2c);
  int* nn_cell = reinterpret_cast<int*>(scratch + kOffNnCell);
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    const int q = nn[m];
    nn_cell[m] = (q >= 0 && q < M) ? m2c[q] : 0;
  }
}

int zc(double z) { return z == 1.0 ? 1 : z == -1.0 ? -1 : z == 2.0 ? 2 : z == -2.0 ? -2 : 0; }

}  // namespace

extern "C" int bx_step_fp64_noalloc(const bx_geom* g, const bx_params* p, const double* Dm,
                                    double* vm, double* vm_work, double* cc_cells, double* cc_mem,
                                    double* cc_mem_work, double* cc_env, int n_steps, void* stream) {
  if (!g || !p || !Dm || !vm || !vm_work || !cc_cells || !cc_mem || !cc_mem_work || !cc_env)
    return na_fail(BX_EINVAL, "bx_step_fp64_noalloc: null argument");
  const int C = g->n_cells, M = g->n_mems, I = p->n_ions;
  if (C <= 0 || M <= 0 || n_steps < 0) return na_fail(BX_EINVAL, "bx_step_fp64_noalloc: bad sizes");
  if (C > kMaxCells || M > kMaxMems)
    return na_fail(BX_EINVAL, "bx_step_fp64_noalloc: at most 16384 cells and 131072 membranes");
  if (I <= 0 || I > BX_MAX_IONS || p->iNa < 0 || p->iNa >= I || p->iK < 0 || p->iK >= I)
    return na_fail(BX_EINVAL, "bx_step_fp64_noalloc: bad ion indices");
  if (p->is_ecm) return na_fail(BX_EINVAL, "bx_step_fp64_noalloc: needs is_ecm == 0");
  if (p->v_sensitive_gj)
    return na_fail(BX_EINVAL, "bx_step_fp64_noalloc: needs v_sensitive_gj == 0 (the open fraction is state)");
  if (p->iCa >= 0 && p->alpha_Ca > 0.0)
    return na_fail(BX_EINVAL, "bx_step_fp64_noalloc: needs the Ca-ATPase off (alpha_Ca == 0 or iCa == -1)");
  if (p->cell_polarizability != 0.0)
    return na_fail(BX_EINVAL, "bx_step_fp64_noalloc: needs cell_polarizability == 0");
  if (!g->cell_mem_ptr || !g->nn_i || !g->bflag || !g->map_mem2ecm || !g->mem_sa || !g->gj_weight ||
      !g->cell_vol || !g->diviterm)
    return na_fail(BX_EINVAL, "bx_step_fp64_noalloc: missing geometry array");
  int rc = BX_OK;
  double* scratch = scratch_address(&rc);
  if (!scratch) return rc;
  if (n_steps == 0) return BX_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int ntile = (C + kTileCells - 1) / kTileCells;
  const double pump = -3.0 * p->nakatp_block * p->alpha_NaK;
  const double escale = p->dt / (p->vol_env * (double)M);

  if (cudaMemsetAsync(scratch + kOffFlag, 0, 2 * sizeof(int), s) != cudaSuccess)
    return na_fail(BX_ECUDA, "bx_step_fp64_noalloc: clearing the set-up flags failed");
  k_noalloc_prep<<<64, 256, 0, s>>>(g->cell_mem_ptr, g->nn_i, C, M, scratch, pump, escale);
  k_noalloc_nn_cell<<<64, 256, 0, s>>>(g->nn_i, M, scratch);
  int flag[2] = {0, 0};
  if (cudaMemcpyAsync(flag, scratch + kOffFlag, sizeof(flag), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return na_fail(BX_ECUDA, "bx_step_fp64_noalloc: set-up kernels failed");
  if (flag[1])
    return na_fail(BX_EINVAL, "bx_step_fp64_noalloc: cell_mem_ptr is not a row pointer over n_mems membranes "
                              "(ptr[0] == 0, ptr[n_cells] == n_mems, strictly increasing) or nn_i is out of range");
  if (flag[0]) return na_fail(BX_EINVAL, "bx_step_fp64_noalloc: 16 consecutive cells hold more than 256 membranes");

  bx::DevGeom dg{};
  dg.C = C; dg.M = M; dg.I = I; dg.G = g->grid_ny * g->grid_nx; dg.ny = g->grid_ny; dg.nx = g->grid_nx;
  dg.cell_ptr = g->cell_mem_ptr;
  dg.m2c = reinterpret_cast<const int*>(scratch + kOffM2c);
  dg.nn = g->nn_i;
  dg.nn_cell = reinterpret_cast<const int*>(scratch + kOffNnCell);
  dg.bflag = g->bflag; dg.map_env = g->map_mem2ecm; dg.mem_sa = g->mem_sa; dg.gj_w = g->gj_weight;
  dg.mem_nx = g->mem_nx; dg.mem_ny = g->mem_ny; dg.sw_mem = g->smooth_weight_mem; dg.sw_o = g->smooth_weight_o;
  dg.cell_vol = g->cell_vol; dg.cell_sa = g->cell_sa; dg.diviterm = g->diviterm;
  dg.blk_cell = reinterpret_cast<const int*>(scratch + kOffBlk);
  dg.blk_cluster = reinterpret_cast<const int*>(scratch + kOffBlkCl);

  bx::StepConst k{};
  k.I = I; k.iNa = p->iNa; k.iK = p->iK;
  k.iCa = -1;  // Ca-ATPase off
  const double RT = p->R * p->T;
  for (int i = 0; i < I; ++i) {
    k.z[i] = p->zs[i]; k.zcode[i] = zc(p->zs[i]); k.zF[i] = p->zs[i] * p->F;
    k.sig_coef[i] = ((p->zs[i] * p->zs[i]) * (p->F * p->F) * p->D_free[i] * 0.1) / RT;
    k.dgj_gs[i] = p->D_gj[i] * p->gj_surface;
  }
  k.F_RT = p->F / RT; k.dt = p->dt; k.inv_cm = 1.0 / p->cm; k.tm = p->tm; k.gj_len = g->gj_len;
  k.inv_tm = 1.0 / p->tm; k.inv_gj_len = 1.0 / g->gj_len;
  k.gj_block = p->gj_block; k.inv_KmNa = 1.0 / p->KmNK_Na; k.inv_KmK = 1.0 / p->KmNK_K;
  k.atp_term = p->cATP / p->KmNK_ATP; k.atp_den = 1.0 + p->cATP / p->KmNK_ATP;
  k.qnum_c = (p->cADP * 1e-3) * (p->cPi * 1e-3); k.qden_c = p->cATP * 1e-3;
  k.K0 = std::exp(-(p->deltaGATP / RT));

  double* vbuf[2] = {vm, vm_work};
  double* cbuf[2] = {cc_mem, cc_mem_work};
  int par = 0;
  for (int q = 0; q < n_steps; ++q) {
    bx::StepPtrs sp{};
    sp.vm_in = vbuf[par]; sp.vm_out = vbuf[par ^ 1];
    sp.ccm_in = cbuf[par]; sp.ccm_out = cbuf[par ^ 1];
    sp.cc = cc_cells; sp.Dm = Dm; sp.cenv = cc_env;
    sp.pump_coef = scratch + kOffPump;
    sp.phib = nullptr;
    sp.env_part = scratch + kOffPart;
    sp.status = reinterpret_cast<unsigned long long*>(scratch + kOffStatus);
    if (bx::launch_cell_step<double, kTileThreads>(false, false, false, ntile, s, dg, sp, k) != cudaSuccess)
      return na_fail(BX_ECUDA, "bx_step_fp64_noalloc: step launch failed");
    bx::k_env_mix<<<1, 256, 0, s>>>(scratch + kOffPart, reinterpret_cast<const int*>(scratch + kOffClBlk), I,
                                    cc_env, scratch + kOffEscale);
    par ^= 1;
  }
  if (par == 1) {   // the result sits in the work buffers: move it to the caller's primaries
    if (cudaMemcpyAsync(vm, vm_work, (size_t)M * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(cc_mem, cc_mem_work, (size_t)I * C * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return na_fail(BX_ECUDA, "bx_step_fp64_noalloc: copy-back failed");
  }
  if (cudaGetLastError() != cudaSuccess) return na_fail(BX_ECUDA, "bx_step_fp64_noalloc: launch failed");
  // check_v / no_negs (sim_toolbox.py:332-344, 475-503): the step kernels
  // count NaN Vmem, NaN concentrations and clamped negatives into the
  // scratch; a NaN is reported as BX_EUNSTABLE, as bx_status does for handles
  unsigned long long st[3] = {0ull, 0ull, 0ull};
  if (cudaMemcpyAsync(st, scratch + kOffStatus, sizeof(st), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return na_fail(BX_ECUDA, "bx_step_fp64_noalloc: reading the step status failed");
  if (st[0] || st[1]) {
    const std::string msg = "bx_step_fp64_noalloc: unstable: NaN in Vmem (" + std::to_string(st[0]) +
                            " membrane values) or in cell concentrations (" + std::to_string(st[1]) + ")";
    bx_record_error(msg.c_str());
    return BX_EUNSTABLE;
  }
  return BX_OK;
}
