// bx_api.cu -- the C ABI (include/bx.h): handle lifetime, validation of the
// CSR index maps, host<->device state transfer, CUDA-graph-captured stepping
// and the environment / dense-product entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bx.h"
#include "bx_env.cuh"
#include "bx_launch.cuh"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define BX_CU(call)                                                                   \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      return fail(BX_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));     \
  } while (0)

template <typename P>
cudaError_t dalloc(P** p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  return cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(P));
}

constexpr int kGraphChunk = 32;   // steps per captured graph (even: ping-pong parity returns)
constexpr int kEnvTPB = 256;

}  // namespace

struct bx_cluster {
  int dev = 0;
  cudaStream_t stream = nullptr;
  int C = 0, M = 0, I = 0, G = 0, ny = 0, nx = 0;
  int precision = BX_PLAIN_FP64;
  int tpb = 256;
  int nblk = 0;
  bool ecm = false;
  bx_params par{};
  // geometry
  int *d_cell_ptr = nullptr, *d_m2c = nullptr, *d_nn = nullptr, *d_nn_cell = nullptr,
      *d_map_env = nullptr, *d_blk = nullptr, *d_env_ptr = nullptr, *d_env_mem = nullptr;
  uint8_t *d_bflag = nullptr, *d_touched = nullptr;
  double *d_mem_sa = nullptr, *d_gj_w = nullptr, *d_nx = nullptr, *d_ny = nullptr,
         *d_swm = nullptr, *d_swo = nullptr, *d_cell_vol = nullptr, *d_cell_sa = nullptr,
         *d_diviterm = nullptr;
  float *d_mem_sa_f = nullptr, *d_gj_w_f = nullptr, *d_Dm_f = nullptr;
  double* d_Dm = nullptr;
  // state
  double *d_vm[2] = {nullptr, nullptr}, *d_ccm[2] = {nullptr, nullptr};
  double *d_cc = nullptr, *d_cenv = nullptr, *d_phib = nullptr, *d_env_part = nullptr,
         *d_mem_flux_sa = nullptr;
  double *d_Denv = nullptr, *d_Ex = nullptr, *d_Ey = nullptr, *d_fx = nullptr, *d_fy = nullptr,
         *d_tmp = nullptr, *d_tmp2 = nullptr, *d_venv = nullptr, *d_rho_env = nullptr;
  unsigned long long* d_status = nullptr;
  // outputs
  double *o_fmem = nullptr, *o_fgj = nullptr, *o_rate = nullptr, *o_rho = nullptr,
         *o_Jn = nullptr, *o_Imem = nullptr, *o_Jcx = nullptr, *o_Jcy = nullptr,
         *o_Jc = nullptr, *o_vmave = nullptr, *o_dvm = nullptr, *o_Ecx = nullptr,
         *o_Ecy = nullptr, *o_Emc = nullptr, *o_Egjx = nullptr, *o_Egjy = nullptr,
         *o_gjopen = nullptr, *o_sigma = nullptr;
  // field outputs
  double *d_lap = nullptr, *d_fld = nullptr;
  int parity = 0;
  bool have_state = false, have_dm = false, have_denv = false, have_outputs = false;
  bool phib_nonzero = false;
  int64_t steps_done = 0, launches = 0;
  cudaGraphExec_t graph = nullptr;
  bool graph_valid = false;
  int64_t neg_seen = 0;
  std::vector<int> h_cell_ptr;
  std::vector<int> h_m2c;
  double env_surf_scale = 0.0;
  double gj_len = 0.0, delta = 0.0;
};

using bx_cluster_ext = bx_cluster;

namespace {

void free_all(bx_cluster* h) {
  void* ptrs[] = {h->d_cell_ptr, h->d_m2c, h->d_nn, h->d_nn_cell, h->d_map_env, h->d_blk,
                  h->d_env_ptr, h->d_env_mem, h->d_bflag, h->d_touched, h->d_mem_sa, h->d_gj_w,
                  h->d_nx, h->d_ny, h->d_swm, h->d_swo, h->d_cell_vol, h->d_cell_sa,
                  h->d_diviterm, h->d_mem_sa_f, h->d_gj_w_f, h->d_Dm_f, h->d_Dm, h->d_vm[0],
                  h->d_vm[1], h->d_ccm[0], h->d_ccm[1], h->d_cc, h->d_cenv, h->d_phib,
                  h->d_env_part, h->d_mem_flux_sa, h->d_Denv, h->d_Ex, h->d_Ey, h->d_fx, h->d_fy,
                  h->d_tmp, h->d_tmp2, h->d_venv, h->d_rho_env, h->d_status, h->o_fmem, h->o_fgj,
                  h->o_rate, h->o_rho, h->o_Jn, h->o_Imem, h->o_Jcx, h->o_Jcy, h->o_Jc,
                  h->o_vmave, h->o_dvm, h->o_Ecx, h->o_Ecy, h->o_Emc, h->o_Egjx, h->o_Egjy,
                  h->o_gjopen, h->o_sigma, h->d_lap, h->d_fld};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (h->graph) cudaGraphExecDestroy(h->graph);
  if (h->stream) cudaStreamDestroy(h->stream);
}

int zcode_of(double z) {
  if (z == 1.0) return 1;
  if (z == -1.0) return -1;
  if (z == 2.0) return 2;
  if (z == -2.0) return -2;
  return 0;
}

bx::StepConst make_step_const(const bx_cluster* h) {
  const bx_params& p = h->par;
  bx::StepConst k{};
  k.I = h->I;
  k.iNa = p.iNa;
  k.iK = p.iK;
  const double RT = p.R * p.T;
  for (int i = 0; i < h->I; ++i) {
    k.z[i] = p.zs[i];
    k.zcode[i] = zcode_of(p.zs[i]);
    k.zF[i] = p.zs[i] * p.F;
    k.sig_coef[i] = ((p.zs[i] * p.zs[i]) * (p.F * p.F) * p.D_free[i] * 0.1) / RT;
    k.dgj_gs[i] = p.D_gj[i] * p.gj_surface;
  }
  k.F_RT = p.F / RT;
  k.dt = p.dt;
  k.inv_cm = 1.0 / p.cm;
  k.tm = p.tm;
  k.gj_len = 0.0;  // set by caller (geometry)
  k.gj_block = p.gj_block;
  k.pump_coef = -3.0 * p.nakatp_block * p.alpha_NaK;
  k.inv_KmNa = 1.0 / p.KmNK_Na;
  k.inv_KmK = 1.0 / p.KmNK_K;
  k.atp_term = p.cATP / p.KmNK_ATP;
  k.atp_den = 1.0 + p.cATP / p.KmNK_ATP;
  k.qnum_c = (p.cADP * 1e-3) * (p.cPi * 1e-3);
  k.qden_c = p.cATP * 1e-3;
  k.K0 = std::exp(-(p.deltaGATP / RT));
  k.pump_on = p.alpha_NaK > 0.0 ? 1.0 : 0.0;
  k.env_scale = p.dt / (p.vol_env * (double)h->M);
  return k;
}

bx::EnvConst make_env_const(const bx_cluster* h, double delta) {
  const bx_params& p = h->par;
  bx::EnvConst e{};
  e.I = h->I;
  e.ny = h->ny;
  e.nx = h->nx;
  e.G = h->G;
  e.delta = delta;
  e.inv_delta = 1.0 / delta;
  e.inv_2delta = 1.0 / (2.0 * delta);
  e.dt = p.dt;
  e.sharpness = p.sharpness;
  for (int i = 0; i < h->I; ++i) {
    e.np_alpha[i] = (p.zs[i] * p.q) / (p.kb * p.T);
    e.zF[i] = p.zs[i] * p.F;
    e.c_bound[i] = p.c_env_bound[i];
  }
  e.surf_scale = h->env_surf_scale;
  e.inv_koeoer = (p.ko_env != 0.0) ? 1.0 / (p.ko_env * p.eo * p.er) : 0.0;
  e.screen = (p.ko_env != 0.0) ? (2.0 / (p.ko_env * delta)) * (p.cell_radius / p.true_cell_size) : 0.0;
  e.inv_h_d2 = 1.0 / (p.cell_height * delta * delta);
  // sigma = 1, truncate = 4: the taps scipy.ndimage.gaussian_filter uses
  double w[9], s = 0.0;
  for (int q = -4; q <= 4; ++q) { w[q + 4] = std::exp(-0.5 * (double)(q * q)); s += w[q + 4]; }
  for (int q = 0; q < 9; ++q) e.gw[q] = w[q] / s;
  return e;
}

}  // namespace

namespace {

bx::DevGeom dev_geom(const bx_cluster_ext* h) {
  bx::DevGeom g{};
  g.C = h->C; g.M = h->M; g.I = h->I; g.G = h->G; g.ny = h->ny; g.nx = h->nx;
  g.cell_ptr = h->d_cell_ptr; g.m2c = h->d_m2c; g.nn = h->d_nn; g.nn_cell = h->d_nn_cell;
  g.bflag = h->d_bflag; g.map_env = h->d_map_env; g.mem_sa = h->d_mem_sa; g.mem_sa_f = h->d_mem_sa_f;
  g.gj_w = h->d_gj_w; g.gj_w_f = h->d_gj_w_f; g.mem_nx = h->d_nx; g.mem_ny = h->d_ny;
  g.sw_mem = h->d_swm; g.sw_o = h->d_swo; g.cell_vol = h->d_cell_vol; g.cell_sa = h->d_cell_sa;
  g.diviterm = h->d_diviterm; g.blk_cell = h->d_blk;
  return g;
}

bx::StepPtrs step_ptrs(bx_cluster_ext* h, int parity) {
  bx::StepPtrs p{};
  p.vm_in = h->d_vm[parity]; p.vm_out = h->d_vm[parity ^ 1];
  p.ccm_in = h->d_ccm[parity]; p.ccm_out = h->d_ccm[parity ^ 1];
  p.cc = h->d_cc; p.Dm = h->d_Dm; p.Dm_f = h->d_Dm_f; p.cenv = h->d_cenv;
  p.phib = h->d_phib; p.env_part = h->d_env_part; p.mem_flux_sa = h->d_mem_flux_sa;
  p.status = h->d_status;
  p.o_fmem = h->o_fmem; p.o_fgj = h->o_fgj; p.o_rate = h->o_rate; p.o_rho = h->o_rho;
  p.o_Jn = h->o_Jn; p.o_Imem = h->o_Imem; p.o_Jcx = h->o_Jcx; p.o_Jcy = h->o_Jcy;
  p.o_Jc = h->o_Jc; p.o_vmave = h->o_vmave; p.o_dvm = h->o_dvm; p.o_Ecx = h->o_Ecx;
  p.o_Ecy = h->o_Ecy; p.o_Emc = h->o_Emc; p.o_Egjx = h->o_Egjx; p.o_Egjy = h->o_Egjy;
  p.o_gjopen = h->o_gjopen; p.o_sigma = h->o_sigma;
  return p;
}

inline int env_grid(int G) { return (G + kEnvTPB - 1) / kEnvTPB; }

// Enqueue one time step (reads parity, writes parity^1).
cudaError_t enqueue_step(bx_cluster_ext* h, int parity, bool out, cudaStream_t s) {
  bx::DevGeom g = dev_geom(h);
  bx::StepConst k = make_step_const(h);
  k.gj_len = h->gj_len;
  bx::StepPtrs p = step_ptrs(h, parity);
  cudaError_t e;
  const bool split = h->precision == BX_SPLIT_FP32;
  if (split) {
    e = (h->tpb == 128) ? bx::launch_cell_step<float, 128>(h->ecm, out, h->phib_nonzero, h->nblk, s, g, p, k)
                        : bx::launch_cell_step<float, 256>(h->ecm, out, h->phib_nonzero, h->nblk, s, g, p, k);
  } else {
    e = (h->tpb == 128) ? bx::launch_cell_step<double, 128>(h->ecm, out, h->phib_nonzero, h->nblk, s, g, p, k)
                        : bx::launch_cell_step<double, 256>(h->ecm, out, h->phib_nonzero, h->nblk, s, g, p, k);
  }
  if (e != cudaSuccess) return e;
  h->launches++;
  if (!h->ecm) {
    bx::k_env_mix<<<1, 256, 0, s>>>(h->d_env_part, h->nblk, h->I, h->d_cenv, k.env_scale);
    h->launches++;
    return cudaGetLastError();
  }
  bx::EnvConst ec = make_env_const(h, h->delta);
  const int gg = env_grid(h->G);
  bx::k_env_np_flux<<<gg, kEnvTPB, 0, s>>>(h->d_cenv, h->d_Denv, h->d_Ex, h->d_Ey, h->d_fx, h->d_fy, ec);
  if (h->par.sharpness < 1.0) {
    bx::k_env_update<false><<<gg, kEnvTPB, 0, s>>>(h->d_cenv, h->d_tmp2, h->d_fx, h->d_fy, h->d_env_ptr,
                                                  h->d_env_mem, h->d_mem_flux_sa, h->M, ec);
    bx::k_env_integrate_scatter<<<gg, kEnvTPB, 0, s>>>(h->d_cenv, h->d_tmp2, h->d_env_ptr, h->d_env_mem,
                                                      h->d_mem_flux_sa, h->M, ec);
    h->launches += 2;
  } else {
    bx::k_env_update<true><<<gg, kEnvTPB, 0, s>>>(h->d_cenv, nullptr, h->d_fx, h->d_fy, h->d_env_ptr,
                                                 h->d_env_mem, h->d_mem_flux_sa, h->M, ec);
    h->launches += 1;
  }
  bx::k_env_charge_gauss_y<<<gg, kEnvTPB, 0, s>>>(h->d_cenv, h->d_touched, out ? h->d_rho_env : nullptr,
                                                 h->d_tmp, ec);
  bx::k_env_gauss_x<<<gg, kEnvTPB, 0, s>>>(h->d_tmp, h->phib_nonzero ? h->d_phib : nullptr, h->d_venv, ec);
  bx::k_env_neg_grad<<<gg, kEnvTPB, 0, s>>>(h->d_venv, ec.screen, h->d_Ex, h->d_Ey, ec);
  h->launches += 4;
  return cudaGetLastError();
}

}  // namespace

extern "C" {

int bx_abi_version(void) { return BX_ABI_VERSION; }
const char* bx_last_error(void) { return g_err.c_str(); }

int bx_cluster_create(const bx_geom* g, const bx_params* p, int precision, bx_handle* out) {
  if (!g || !p || !out) return fail(BX_EINVAL, "null argument");
  *out = nullptr;
  if (precision != BX_PLAIN_FP64 && precision != BX_SPLIT_FP32)
    return fail(BX_EINVAL, "precision must be BX_PLAIN_FP64 or BX_SPLIT_FP32");
  const int C = g->n_cells, M = g->n_mems, I = p->n_ions;
  if (C <= 0 || M <= 0) return fail(BX_EINVAL, "empty cluster (n_cells and n_mems must be > 0)");
  if (I <= 0 || I > BX_MAX_IONS) return fail(BX_EINVAL, "n_ions must be in [1, 8]");
  if (p->iNa < 0 || p->iNa >= I || p->iK < 0 || p->iK >= I || p->iNa == p->iK)
    return fail(BX_EINVAL, "iNa/iK out of range");
  if (g->grid_ny < 3 || g->grid_nx < 3) return fail(BX_EINVAL, "environment grid must be at least 3x3");
  if (!g->cell_mem_ptr || !g->nn_i || !g->bflag || !g->map_mem2ecm || !g->mem_sa || !g->gj_weight ||
      !g->cell_vol || !g->cell_sa || !g->diviterm || !g->mem_nx || !g->mem_ny ||
      !g->smooth_weight_mem || !g->smooth_weight_o)
    return fail(BX_EINVAL, "missing geometry array");
  if (!(g->gj_len > 0.0) || !(g->delta > 0.0)) return fail(BX_EINVAL, "gj_len and delta must be > 0");
  const int G = g->grid_ny * g->grid_nx;
  // ---- validate the CSR map (the bit-exact form of mem_to_cells / cell_to_mems)
  if (g->cell_mem_ptr[0] != 0 || g->cell_mem_ptr[C] != M)
    return fail(BX_EINVAL, "cell_mem_ptr must start at 0 and end at n_mems");
  std::vector<int> m2c(M);
  for (int c = 0; c < C; ++c) {
    const int a = g->cell_mem_ptr[c], b = g->cell_mem_ptr[c + 1];
    if (b < a) return fail(BX_EINVAL, "cell_mem_ptr must be non-decreasing");
    if (b - a > BX_MAX_MEMS_PER_CELL) return fail(BX_EINVAL, "a cell has more than 256 membranes");
    for (int m = a; m < b; ++m) m2c[m] = c;
  }
  std::vector<int> nn_cell(M);
  for (int m = 0; m < M; ++m) {
    const int n = g->nn_i[m];
    if (n < 0 || n >= M) return fail(BX_EINVAL, "nn_i out of range");
    nn_cell[m] = m2c[n];
    const int e = g->map_mem2ecm[m];
    if (e < 0 || e >= G) return fail(BX_EINVAL, "map_mem2ecm out of range");
  }
  for (int c = 0; c < C; ++c)
    if (!(g->cell_vol[c] > 0.0) || !(g->cell_sa[c] > 0.0))
      return fail(BX_EINVAL, "cell_vol and cell_sa must be > 0");
  if (p->is_ecm && !g->mem_sa_per_env) return fail(BX_EINVAL, "ECM needs mem_sa_per_env");

  bx_cluster_ext* h = new (std::nothrow) bx_cluster_ext();
  if (!h) return fail(BX_ENOMEM, "host allocation failed");
  h->C = C; h->M = M; h->I = I; h->G = G; h->ny = g->grid_ny; h->nx = g->grid_nx;
  h->precision = precision; h->par = *p; h->ecm = p->is_ecm != 0;
  h->gj_len = g->gj_len; h->delta = g->delta;
  h->h_cell_ptr.assign(g->cell_mem_ptr, g->cell_mem_ptr + C + 1);
  h->h_m2c = m2c;
  int rc = BX_OK;
  auto bail = [&](int code, const std::string& msg) {
    free_all(h);
    delete h;
    return fail(code, msg);
  };
  if (cudaGetDevice(&h->dev) != cudaSuccess) return bail(BX_ECUDA, "no CUDA device");
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(BX_ECUDA, "cudaStreamCreate failed");

  // ---- CTA partition: whole cells, at most tpb membranes each
  h->tpb = 256;
  std::vector<int> blk{0};
  {
    int acc = 0;
    for (int c = 0; c < C; ++c) {
      const int n = g->cell_mem_ptr[c + 1] - g->cell_mem_ptr[c];
      if (acc + n > h->tpb && acc > 0) { blk.push_back(c); acc = 0; }
      acc += n;
    }
    blk.push_back(C);
  }
  h->nblk = (int)blk.size() - 1;

  // ---- environment CSR (grid cell -> its membranes, ascending) for the ECM scatter
  std::vector<int> env_ptr(G + 1, 0), env_mem(M);
  std::vector<uint8_t> touched(G, 0);
  for (int m = 0; m < M; ++m) env_ptr[g->map_mem2ecm[m] + 1]++;
  for (int k = 0; k < G; ++k) env_ptr[k + 1] += env_ptr[k];
  {
    std::vector<int> fill(env_ptr.begin(), env_ptr.end() - 1);
    for (int m = 0; m < M; ++m) env_mem[fill[g->map_mem2ecm[m]]++] = m;
  }
  for (int k = 0; k < G; ++k) touched[k] = env_ptr[k + 1] > env_ptr[k];
  if (h->ecm) {
    double s = 0.0;
    for (int m = 0; m < M; ++m) s += g->mem_sa_per_env[g->map_mem2ecm[m]];
    const double mean = s / (double)M;  // memSa_per_envSquare[map_mem2ecm].mean()
    h->env_surf_scale = (p->cell_height * g->delta * g->delta) / mean;
  }

  std::vector<float> fsa(M), fgw(M);
  for (int m = 0; m < M; ++m) { fsa[m] = (float)g->mem_sa[m]; fgw[m] = (float)g->gj_weight[m]; }
  std::vector<double> gjw(g->gj_weight, g->gj_weight + M);

#define ALLOC(ptr, n) if (dalloc(&(ptr), (size_t)(n)) != cudaSuccess) return bail(BX_ENOMEM, "cudaMalloc " #ptr)
#define H2D(dst, src, n) if (cudaMemcpy((dst), (src), sizeof(*(dst)) * (size_t)(n), cudaMemcpyHostToDevice) != cudaSuccess) return bail(BX_ECUDA, "copy " #dst)
  ALLOC(h->d_cell_ptr, C + 1); H2D(h->d_cell_ptr, g->cell_mem_ptr, C + 1);
  ALLOC(h->d_m2c, M); H2D(h->d_m2c, m2c.data(), M);
  ALLOC(h->d_nn, M); H2D(h->d_nn, g->nn_i, M);
  ALLOC(h->d_nn_cell, M); H2D(h->d_nn_cell, nn_cell.data(), M);
  ALLOC(h->d_map_env, M); H2D(h->d_map_env, g->map_mem2ecm, M);
  ALLOC(h->d_blk, blk.size()); H2D(h->d_blk, blk.data(), blk.size());
  ALLOC(h->d_env_ptr, G + 1); H2D(h->d_env_ptr, env_ptr.data(), G + 1);
  ALLOC(h->d_env_mem, M); H2D(h->d_env_mem, env_mem.data(), M);
  ALLOC(h->d_touched, G); H2D(h->d_touched, touched.data(), G);
  ALLOC(h->d_bflag, M); H2D(h->d_bflag, g->bflag, M);
  ALLOC(h->d_mem_sa, M); H2D(h->d_mem_sa, g->mem_sa, M);
  ALLOC(h->d_mem_sa_f, M); H2D(h->d_mem_sa_f, fsa.data(), M);
  ALLOC(h->d_gj_w, M); H2D(h->d_gj_w, gjw.data(), M);
  ALLOC(h->d_gj_w_f, M); H2D(h->d_gj_w_f, fgw.data(), M);
  ALLOC(h->d_nx, M); H2D(h->d_nx, g->mem_nx, M);
  ALLOC(h->d_ny, M); H2D(h->d_ny, g->mem_ny, M);
  ALLOC(h->d_swm, M); H2D(h->d_swm, g->smooth_weight_mem, M);
  ALLOC(h->d_swo, M); H2D(h->d_swo, g->smooth_weight_o, M);
  ALLOC(h->d_cell_vol, C); H2D(h->d_cell_vol, g->cell_vol, C);
  ALLOC(h->d_cell_sa, C); H2D(h->d_cell_sa, g->cell_sa, C);
  ALLOC(h->d_diviterm, C); H2D(h->d_diviterm, g->diviterm, C);
  if (precision == BX_SPLIT_FP32) { ALLOC(h->d_Dm_f, (size_t)I * M); }
  else { ALLOC(h->d_Dm, (size_t)I * M); }
  ALLOC(h->d_vm[0], M); ALLOC(h->d_vm[1], M);
  ALLOC(h->d_ccm[0], (size_t)I * C); ALLOC(h->d_ccm[1], (size_t)I * C);
  ALLOC(h->d_cc, (size_t)I * C);
  ALLOC(h->d_cenv, h->ecm ? (size_t)I * G : (size_t)I);
  ALLOC(h->d_phib, G);
  ALLOC(h->d_env_part, (size_t)h->nblk * I);
  ALLOC(h->d_status, 4);
  if (cudaMemset(h->d_status, 0, 4 * sizeof(unsigned long long)) != cudaSuccess) return bail(BX_ECUDA, "memset");
  if (cudaMemset(h->d_phib, 0, G * sizeof(double)) != cudaSuccess) return bail(BX_ECUDA, "memset");
  if (h->ecm) {
    ALLOC(h->d_mem_flux_sa, (size_t)I * M);
    ALLOC(h->d_Denv, (size_t)I * G);
    ALLOC(h->d_Ex, G); ALLOC(h->d_Ey, G);
    ALLOC(h->d_fx, (size_t)I * G); ALLOC(h->d_fy, (size_t)I * G);
    ALLOC(h->d_tmp, G); ALLOC(h->d_tmp2, (size_t)I * G);
    ALLOC(h->d_venv, G); ALLOC(h->d_rho_env, G);
  }
  // outputs
  ALLOC(h->o_fmem, (size_t)I * M); ALLOC(h->o_fgj, (size_t)I * M);
  ALLOC(h->o_rate, M); ALLOC(h->o_rho, C); ALLOC(h->o_Jn, M); ALLOC(h->o_Imem, M);
  ALLOC(h->o_Jcx, C); ALLOC(h->o_Jcy, C); ALLOC(h->o_Jc, M); ALLOC(h->o_vmave, C);
  ALLOC(h->o_dvm, M); ALLOC(h->o_Ecx, C); ALLOC(h->o_Ecy, C); ALLOC(h->o_Emc, M);
  ALLOC(h->o_Egjx, M); ALLOC(h->o_Egjy, M); ALLOC(h->o_gjopen, M); ALLOC(h->o_sigma, C);
#undef ALLOC
#undef H2D
  (void)rc;
  *out = h;
  return BX_OK;
}

void bx_destroy(bx_handle hh) {
  if (!hh) return;
  bx_cluster_ext* h = static_cast<bx_cluster_ext*>(hh);
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_all(h);
  delete h;
}

int bx_set_params(bx_handle hh, const bx_params* p) {
  if (!hh || !p) return fail(BX_EINVAL, "null argument");
  bx_cluster_ext* h = static_cast<bx_cluster_ext*>(hh);
  if (p->n_ions != h->I || (p->is_ecm != 0) != h->ecm)
    return fail(BX_EINVAL, "n_ions / is_ecm cannot change after create");
  h->par = *p;
  h->graph_valid = false;
  return BX_OK;
}

int bx_set_membrane_diffusivity(bx_handle hh, const double* Dm) {
  if (!hh || !Dm) return fail(BX_EINVAL, "null argument");
  bx_cluster_ext* h = static_cast<bx_cluster_ext*>(hh);
  const size_t n = (size_t)h->I * h->M;
  for (size_t q = 0; q < n; ++q)
    if (!(Dm[q] >= 0.0)) return fail(BX_EINVAL, "Dm must be finite and >= 0");
  if (h->precision == BX_SPLIT_FP32) {
    std::vector<float> f(n);
    for (size_t q = 0; q < n; ++q) f[q] = (float)Dm[q];
    BX_CU(cudaMemcpyAsync(h->d_Dm_f, f.data(), n * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    BX_CU(cudaStreamSynchronize(h->stream));
  } else {
    BX_CU(cudaMemcpyAsync(h->d_Dm, Dm, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    BX_CU(cudaStreamSynchronize(h->stream));
  }
  h->have_dm = true;
  return BX_OK;
}

int bx_set_env_diffusivity(bx_handle hh, const double* D_env) {
  if (!hh || !D_env) return fail(BX_EINVAL, "null argument");
  bx_cluster_ext* h = static_cast<bx_cluster_ext*>(hh);
  if (!h->ecm) return fail(BX_EINVAL, "environment diffusivity needs is_ecm");
  BX_CU(cudaMemcpyAsync(h->d_Denv, D_env, (size_t)h->I * h->G * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  BX_CU(cudaStreamSynchronize(h->stream));
  h->have_denv = true;
  return BX_OK;
}

int bx_set_boundary_potential(bx_handle hh, const double* Phi_b) {
  if (!hh) return fail(BX_EINVAL, "null handle");
  bx_cluster_ext* h = static_cast<bx_cluster_ext*>(hh);
  bool nz = false;
  if (Phi_b) for (int k = 0; k < h->G; ++k) nz |= (Phi_b[k] != 0.0);
  if (nz) {
    BX_CU(cudaMemcpyAsync(h->d_phib, Phi_b, (size_t)h->G * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  } else {
    BX_CU(cudaMemsetAsync(h->d_phib, 0, (size_t)h->G * sizeof(double), h->stream));
  }
  BX_CU(cudaStreamSynchronize(h->stream));
  if (nz != h->phib_nonzero) h->graph_valid = false;
  h->phib_nonzero = nz;
  return BX_OK;
}

int bx_state_upload(bx_handle hh, const bx_state* s) {
  if (!hh || !s || !s->vm || !s->cc_cells || !s->cc_at_mem || !s->cc_env)
    return fail(BX_EINVAL, "null argument");
  bx_cluster_ext* h = static_cast<bx_cluster_ext*>(hh);
  const int C = h->C, M = h->M, I = h->I;
  std::vector<double> ccm((size_t)I * C);
  for (int i = 0; i < I; ++i)
    for (int c = 0; c < C; ++c) {
      const int a = h->h_cell_ptr[c], b = h->h_cell_ptr[c + 1];
      const double v = (b > a) ? s->cc_at_mem[(size_t)i * M + a] : s->cc_cells[(size_t)i * C + c];
      for (int m = a + 1; m < b; ++m)
        if (s->cc_at_mem[(size_t)i * M + m] != v)
          return fail(BX_EINVAL, "cc_at_mem must be constant over each cell's membranes");
      ccm[(size_t)i * C + c] = v;
    }
  if (h->ecm && (!s->E_env_x || !s->E_env_y)) return fail(BX_EINVAL, "ECM state needs E_env_x/E_env_y");
  h->parity = 0;
  BX_CU(cudaMemcpyAsync(h->d_vm[0], s->vm, (size_t)M * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  BX_CU(cudaMemcpyAsync(h->d_cc, s->cc_cells, (size_t)I * C * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  BX_CU(cudaMemcpyAsync(h->d_ccm[0], ccm.data(), (size_t)I * C * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  BX_CU(cudaMemcpyAsync(h->d_cenv, s->cc_env, (h->ecm ? (size_t)I * h->G : (size_t)I) * sizeof(double),
                        cudaMemcpyHostToDevice, h->stream));
  if (h->ecm) {
    BX_CU(cudaMemcpyAsync(h->d_Ex, s->E_env_x, (size_t)h->G * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    BX_CU(cudaMemcpyAsync(h->d_Ey, s->E_env_y, (size_t)h->G * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  }
  BX_CU(cudaStreamSynchronize(h->stream));
  h->have_state = true;
  h->have_outputs = false;
  return BX_OK;
}

int bx_state_download(bx_handle hh, bx_state* s) {
  if (!hh || !s) return fail(BX_EINVAL, "null argument");
  bx_cluster_ext* h = static_cast<bx_cluster_ext*>(hh);
  if (!h->have_state) return fail(BX_ESTATE, "no state uploaded");
  const int C = h->C, M = h->M, I = h->I;
  BX_CU(cudaStreamSynchronize(h->stream));
  if (s->vm) BX_CU(cudaMemcpy(s->vm, h->d_vm[h->parity], (size_t)M * sizeof(double), cudaMemcpyDeviceToHost));
  if (s->cc_cells) BX_CU(cudaMemcpy(s->cc_cells, h->d_cc, (size_t)I * C * sizeof(double), cudaMemcpyDeviceToHost));
  if (s->cc_at_mem) {
    std::vector<double> ccm((size_t)I * C);
    BX_CU(cudaMemcpy(ccm.data(), h->d_ccm[h->parity], ccm.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int i = 0; i < I; ++i)
      for (int m = 0; m < M; ++m) s->cc_at_mem[(size_t)i * M + m] = ccm[(size_t)i * C + h->h_m2c[m]];
  }
  if (s->cc_env)
    BX_CU(cudaMemcpy(s->cc_env, h->d_cenv, (h->ecm ? (size_t)I * h->G : (size_t)I) * sizeof(double),
                     cudaMemcpyDeviceToHost));
  if (h->ecm) {
    if (s->E_env_x) BX_CU(cudaMemcpy(s->E_env_x, h->d_Ex, (size_t)h->G * sizeof(double), cudaMemcpyDeviceToHost));
    if (s->E_env_y) BX_CU(cudaMemcpy(s->E_env_y, h->d_Ey, (size_t)h->G * sizeof(double), cudaMemcpyDeviceToHost));
  }
  return BX_OK;
}

int bx_step(bx_handle hh, int n_steps, int want_outputs, void* stream) {
  if (!hh) return fail(BX_EINVAL, "null handle");
  bx_cluster_ext* h = static_cast<bx_cluster_ext*>(hh);
  if (n_steps < 0) return fail(BX_EINVAL, "n_steps must be >= 0");
  if (!h->have_state) return fail(BX_ESTATE, "bx_step before bx_state_upload");
  if (!h->have_dm) return fail(BX_ESTATE, "bx_step before bx_set_membrane_diffusivity");
  if (h->ecm && !h->have_denv) return fail(BX_ESTATE, "ECM step before bx_set_env_diffusivity");
  if (n_steps == 0) return BX_OK;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : h->stream;
  if (s != h->stream) {
    // order the caller's stream after the handle's pending work
    cudaEvent_t ev;
    BX_CU(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    BX_CU(cudaEventRecord(ev, h->stream));
    BX_CU(cudaStreamWaitEvent(s, ev, 0));
    cudaEventDestroy(ev);
  }
  int left = n_steps;
  const int tail_out = want_outputs ? 1 : 0;
  // graph-captured chunks of kGraphChunk steps from parity 0
  if (left - tail_out >= kGraphChunk) {
    if (h->parity != 0) {
      if (enqueue_step(h, h->parity, false, s) != cudaSuccess) return fail(BX_ECUDA, cudaGetErrorString(cudaGetLastError()));
      h->parity ^= 1; --left;
    }
    if (!h->graph_valid) {
      if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
      cudaStream_t cs;
      BX_CU(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      cudaGraph_t graph;
      const int64_t l0 = h->launches;
      BX_CU(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      int par = 0;
      for (int q = 0; q < kGraphChunk; ++q) { enqueue_step(h, par, false, cs); par ^= 1; }
      cudaError_t ce = cudaStreamEndCapture(cs, &graph);
      cudaStreamDestroy(cs);
      h->launches = l0;  // captured launches are counted on replay
      if (ce != cudaSuccess) return fail(BX_ECUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
      ce = cudaGraphInstantiate(&h->graph, graph, 0);
      cudaGraphDestroy(graph);
      if (ce != cudaSuccess) return fail(BX_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
      h->graph_valid = true;
    }
    const int per_step_launches = h->ecm ? ((h->par.sharpness < 1.0) ? 7 : 6) : 2;
    while (left - tail_out >= kGraphChunk) {
      BX_CU(cudaGraphLaunch(h->graph, s));
      h->launches += (int64_t)kGraphChunk * per_step_launches;
      left -= kGraphChunk;
    }
  }
  while (left > 0) {
    const bool out = want_outputs && left == 1;
    cudaError_t e = enqueue_step(h, h->parity, out, s);
    if (e != cudaSuccess) return fail(BX_ECUDA, std::string("step launch: ") + cudaGetErrorString(e));
    h->parity ^= 1;
    --left;
  }
  h->steps_done += n_steps;
  if (want_outputs) h->have_outputs = true;
  if (s != h->stream) {
    cudaEvent_t ev;
    BX_CU(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    BX_CU(cudaEventRecord(ev, s));
    BX_CU(cudaStreamWaitEvent(h->stream, ev, 0));
    cudaEventDestroy(ev);
  }
  return BX_OK;
}

int bx_status(bx_handle hh, bx_step_status* st) {
  if (!hh || !st) return fail(BX_EINVAL, "null argument");
  bx_cluster_ext* h = static_cast<bx_cluster_ext*>(hh);
  unsigned long long v[4];
  BX_CU(cudaStreamSynchronize(h->stream));
  BX_CU(cudaMemcpy(v, h->d_status, sizeof(v), cudaMemcpyDeviceToHost));
  st->steps_done = h->steps_done;
  st->nan_vm = (int32_t)std::min<unsigned long long>(v[0], 0x7fffffff);
  st->nan_conc = (int32_t)std::min<unsigned long long>(v[1], 0x7fffffff);
  st->neg_clamped = (int64_t)v[2];
  st->unstable = (v[0] || v[1]) ? 1 : 0;
  st->precision = h->precision;
  return BX_OK;
}

int bx_outputs_download(bx_handle hh, bx_outputs* o) {
  if (!hh || !o) return fail(BX_EINVAL, "null argument");
  bx_cluster_ext* h = static_cast<bx_cluster_ext*>(hh);
  if (!h->have_outputs) return fail(BX_ESTATE, "no step with want_outputs has run");
  BX_CU(cudaStreamSynchronize(h->stream));
  const size_t M = h->M, C = h->C, I = h->I, G = h->G;
  struct Pair { double* dst; const double* src; size_t n; };
  Pair pairs[] = {
      {o->fluxes_mem, h->o_fmem, I * M}, {o->fluxes_gj, h->o_fgj, I * M}, {o->rate_NaKATP, h->o_rate, M},
      {o->rho_cells, h->o_rho, C}, {o->Jn, h->o_Jn, M}, {o->I_mem, h->o_Imem, M},
      {o->J_cell_x, h->o_Jcx, C}, {o->J_cell_y, h->o_Jcy, C}, {o->Jc, h->o_Jc, M},
      {o->vm_ave, h->o_vmave, C}, {o->dvm, h->o_dvm, M}, {o->E_cell_x, h->o_Ecx, C},
      {o->E_cell_y, h->o_Ecy, C}, {o->Emc, h->o_Emc, M}, {o->E_gj_x, h->o_Egjx, M},
      {o->E_gj_y, h->o_Egjy, M}, {o->gjopen, h->o_gjopen, M}, {o->sigma_cell, h->o_sigma, C},
      {o->fluxes_env_x, h->ecm ? h->d_fx : nullptr, I * G}, {o->fluxes_env_y, h->ecm ? h->d_fy : nullptr, I * G},
      {o->rho_env, h->ecm ? h->d_rho_env : nullptr, G}, {o->v_env, h->ecm ? h->d_venv : nullptr, G},
  };
  for (const Pair& p : pairs)
    if (p.dst && p.src) BX_CU(cudaMemcpy(p.dst, p.src, p.n * sizeof(double), cudaMemcpyDeviceToHost));
  return BX_OK;
}

int bx_time_cell_kernel(bx_handle hh, int n, double* ms_per_launch) {
  if (!hh || !ms_per_launch || n <= 0) return fail(BX_EINVAL, "bad arguments");
  bx_cluster_ext* h = static_cast<bx_cluster_ext*>(hh);
  if (!h->have_state || !h->have_dm) return fail(BX_ESTATE, "upload state and Dm first");
  bx::DevGeom g = dev_geom(h);
  bx::StepConst k = make_step_const(h);
  k.gj_len = h->gj_len;
  cudaEvent_t e0, e1;
  BX_CU(cudaEventCreate(&e0));
  BX_CU(cudaEventCreate(&e1));
  double tot = 0.0;
  const bool split = h->precision == BX_SPLIT_FP32;
  for (int q = 0; q < n; ++q) {
    bx::StepPtrs p = step_ptrs(h, h->parity);
    BX_CU(cudaEventRecord(e0, h->stream));
    cudaError_t e = split ? bx::launch_cell_step<float, 256>(h->ecm, false, h->phib_nonzero, h->nblk, h->stream, g, p, k)
                          : bx::launch_cell_step<double, 256>(h->ecm, false, h->phib_nonzero, h->nblk, h->stream, g, p, k);
    if (e != cudaSuccess) return fail(BX_ECUDA, cudaGetErrorString(e));
    BX_CU(cudaEventRecord(e1, h->stream));
    BX_CU(cudaEventSynchronize(e1));
    float ms = 0.f;
    BX_CU(cudaEventElapsedTime(&ms, e0, e1));
    tot += ms;
    h->parity ^= 1;
    h->launches++;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms_per_launch = tot / n;
  return BX_OK;
}

int64_t bx_cell_kernel_bytes(bx_handle hh) {
  if (!hh) return -1;
  bx_cluster_ext* h = static_cast<bx_cluster_ext*>(hh);
  const int64_t M = h->M, C = h->C, I = h->I;
  const int64_t w = (h->precision == BX_SPLIT_FP32) ? 4 : 8;   // Dm, mem_sa, gj_w width
  // per membrane: Dm, vm in+out, m2c, nn, nn_cell, bflag, mem_sa, gj_w (+ map_env with ECM,
  // + f*sa export with ECM); per cell: cc in+out, cc_mem in+out, cell_vol, diviterm, ptr
  int64_t mem = I * w + 16 + 12 + 1 + 2 * w + (h->ecm ? 4 + I * 8 : 0);
  int64_t cell = 4 * I * 8 + 16 + 4;
  int64_t blk = h->ecm ? 0 : (int64_t)h->nblk * I * 8;
  return M * mem + C * cell + blk;
}

int64_t bx_launch_count(bx_handle hh) {
  if (!hh) return -1;
  return static_cast<bx_cluster_ext*>(hh)->launches;
}

int bx_dense_apply_f64(const double* A, const double* x, double* y, int n, int nrhs, void* stream) {
  if (!A || !x || !y || n <= 0 || nrhs <= 0 || nrhs > 4) return fail(BX_EINVAL, "bad dense_apply arguments");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int threads = 256;
  const long long blocks = ((long long)n * 32 + threads - 1) / threads;
  switch (nrhs) {
    case 1: bx::k_dense_rows<1><<<(unsigned)blocks, threads, 0, s>>>(A, x, y, n); break;
    case 2: bx::k_dense_rows<2><<<(unsigned)blocks, threads, 0, s>>>(A, x, y, n); break;
    case 3: bx::k_dense_rows<3><<<(unsigned)blocks, threads, 0, s>>>(A, x, y, n); break;
    default: bx::k_dense_rows<4><<<(unsigned)blocks, threads, 0, s>>>(A, x, y, n); break;
  }
  BX_CU(cudaGetLastError());
  return BX_OK;
}

int bx_env_fields(bx_handle hh, const double* lap_env_inv, double* v_env, double* E_env_x,
                  double* E_env_y, double* J_env_x, double* J_env_y, double* B_field) {
  (void)lap_env_inv; (void)v_env; (void)E_env_x; (void)E_env_y; (void)J_env_x; (void)J_env_y; (void)B_field;
  if (!hh) return fail(BX_EINVAL, "null handle");
  return fail(BX_EINVAL, "bx_env_fields: not available in this build");
}

}  // extern "C"
