// bx_api.cu -- the C ABI (include/bx.h): handle lifetime, validation of the
// CSR index maps, host<->device state transfer, CUDA-graph-captured stepping
// and the environment / dense-product entry points.
//
// A handle holds one cluster or a batch of clusters (a parameter sweep).  The
// clusters' cells and membranes are concatenated; CTAs never straddle two
// clusters, so per-cluster quantities (the well-mixed environment, the pump
// rate) are looked up by CTA.
//
// Three step paths:
//   plain      BX_PLAIN_FP64: k_cell_step<double> (bx_kernels.cuh)
//   split      BX_SPLIT_FP32 without ECM: k_split_step (bx_split.cuh), no FP64
//              arithmetic per step
//   split+ECM  BX_SPLIT_FP32 with ECM: k_cell_step<float> + the FP64 grid
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/bx.h"
#include "bx_env.cuh"
#include "bx_factored.cuh"
#include "bx_fields.cuh"
#include "bx_launch.cuh"
#include "bx_lapinv.cuh"
#include "bx_network.cuh"
#include "bx_split.cuh"
#include "bx_state.cuh"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define BX_CU(call)                                                               \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess)                                                        \
      return fail(BX_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <typename P>
cudaError_t dalloc(P** p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  return cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(P));
}

template <typename P>
cudaError_t h2d(P* dst, const P* src, size_t n) {
  return cudaMemcpy(dst, src, n * sizeof(P), cudaMemcpyHostToDevice);
}

constexpr int kGraphChunk = 32;  // steps per captured graph (even: ping-pong parity returns)
constexpr int kEnvTPB = 256;
constexpr int kTPB = 256;        // membrane slots per CTA of the cell kernels
constexpr int kRec = 8;          // floats per cell record of the split form (<= 7 ions + Vmem)

enum Mode { MODE_PLAIN = 0, MODE_SPLIT = 1 };
// kernels of the split form (bx_set_launch_config's `kernel`)
enum Kind { KIND_TILE = 0, KIND_PERSIST = 1, KIND_FACT = 2, KIND_RESIDENT = 3, KIND_FACT_PIPE = 4, KIND_ION = 5 };
constexpr long long kResTimeoutNs = 2000000000LL;   // grid-barrier wait limit of k_split_resident

}  // namespace

struct bx_cluster {
  int dev = 0;
  cudaStream_t stream = nullptr;
  int ncl = 1;
  int C = 0, M = 0, I = 0, G = 0, ny = 0, nx = 0;
  int precision = BX_PLAIN_FP64;
  int mode = MODE_PLAIN;
  int nblk = 0;
  int tpb = kTPB;                  // membrane slots per CTA (autotuned)
  int kind = KIND_TILE;            // split form: tile, persistent, factored or resident kernel (autotuned)
  int fact_unroll = 4;             // factored kernel: gap junctions loaded per round (2 or 4; +10 with the
                                   // first entries prefetched before the dependency wait), autotuned
  double tune_ms = -1.0;           // ms per step of the configuration the last autotune chose
  int sm_count = 0;
  bool ecm = false;
  bool ca = false;                 // Ca-ATPase on (iCa >= 0 and alpha_Ca > 0)
  bool polar = false;              // cell polarizability: per-membrane Vmem (plain form)
  // state transfers: the caller's arrays staged on the device (BETSE layouts)
  double* st_vm = nullptr;         // [M]
  double* st_cc = nullptr;         // [I][C]
  double* st_cam = nullptr;        // [I][M]
  double* st_go = nullptr;         // [M]
  int* d_flag = nullptr;           // [2] upload checks
  int* t_slot_of_mem = nullptr;    // [M] split form: membrane slot of each membrane
  void* t_blob = nullptr;          // [nblk] PersistGeo: the persistent kernel's static tile data
  size_t t_blob_bytes = 0;
  double* d_Rrads = nullptr;       // [M] membrane distance from the cell centre
  double* d_cnew = nullptr;        // [I][G] ECM with the Ca-ATPase: environment after the
                                   // Nernst-Planck update and smoothing, before the membrane scatter
  bool vgj = false;                // voltage-gated gap junctions: the open fraction is state
  double* d_gjo = nullptr;         // [M] plain form
  float* t_gjo = nullptr;          // [Q] split form, per membrane slot
  bx_params par{};                 // parameters of cluster 0 (the shared ones)
  std::vector<bx_params> cl_par;   // per-cluster parameters
  std::vector<int> cl_cell, cl_mem, cl_blk;   // offsets [ncl+1]
  double gj_len = 0.0, delta = 0.0, env_surf_scale = 0.0;
  // ---- geometry (device)
  int *d_cell_ptr = nullptr, *d_m2c = nullptr, *d_nn = nullptr, *d_nn_cell = nullptr,
      *d_map_env = nullptr, *d_blk = nullptr, *d_blk_cl = nullptr, *d_cl_blk = nullptr,
      *d_env_ptr = nullptr, *d_env_mem = nullptr;
  uint8_t *d_bflag = nullptr, *d_touched = nullptr, *d_lcell = nullptr;
  double *d_mem_sa = nullptr, *d_gj_w = nullptr, *d_nx = nullptr, *d_ny = nullptr, *d_swm = nullptr,
         *d_swo = nullptr, *d_cell_vol = nullptr, *d_cell_sa = nullptr, *d_diviterm = nullptr;
  float *d_mem_sa_f = nullptr, *d_gj_w_f = nullptr, *d_gjw0_f = nullptr, *d_dtv = nullptr,
        *d_dvc = nullptr;
  // ---- per-membrane channel data
  double* d_Dm = nullptr;
  float* d_Dm_f = nullptr;
  // ---- state: plain / split+ECM
  double *d_vm[2] = {nullptr, nullptr}, *d_ccm[2] = {nullptr, nullptr}, *d_cc = nullptr;
  // ---- split form: tile-major slots (Q membrane slots, S cell slots)
  int Q = 0, S = 0;
  uint8_t* t_lcell = nullptr;
  int *t_nn = nullptr, *t_map_env = nullptr, *t_nn_env = nullptr, *t_c0 = nullptr, *t_m0 = nullptr,
      *t_slot_of_cell = nullptr;
  float *t_sa = nullptr, *t_gw = nullptr, *t_dtv = nullptr, *t_dvc = nullptr;
  short2* t_rng = nullptr;
  std::vector<int> h_slot_of_cell, h_slot_of_mem;
  std::vector<double> h_Dm, h_msa, h_gjw, h_vol, h_div;
  std::vector<uint8_t> h_bflag;
  std::vector<int> h_nn;
  float2* s_cc2 = nullptr;                  // [I][S]
  float* s_rec[2] = {nullptr, nullptr};     // [S][kRec]: membrane-side concentrations + Vmem
  float *s_cenv_f = nullptr, *s_pump = nullptr, *s_part = nullptr, *s_phib = nullptr;
  unsigned int* s_count = nullptr;
  // ---- environment
  double *d_cenv = nullptr, *d_phib = nullptr, *d_env_part = nullptr, *d_mem_flux_sa = nullptr,
         *d_pump = nullptr, *d_env_scale = nullptr;
  double *d_Denv = nullptr, *d_Ex = nullptr, *d_Ey = nullptr, *d_fx = nullptr, *d_fy = nullptr,
         *d_tmp = nullptr, *d_tmp2 = nullptr, *d_venv = nullptr, *d_rho_env = nullptr, *d_vsrc = nullptr;
  unsigned long long* d_status = nullptr;
  unsigned* d_env_ticket = nullptr;   // [ncl] k_cell_step_ion's last-CTA counters (zero between steps)
  // ---- outputs
  double *o_fmem = nullptr, *o_fgj = nullptr, *o_rate = nullptr, *o_rho = nullptr, *o_Jn = nullptr,
         *o_Imem = nullptr, *o_Jcx = nullptr, *o_Jcy = nullptr, *o_Jc = nullptr, *o_vmave = nullptr,
         *o_dvm = nullptr, *o_Ecx = nullptr, *o_Ecy = nullptr, *o_Emc = nullptr, *o_Egjx = nullptr,
         *o_Egjy = nullptr, *o_gjopen = nullptr, *o_sigma = nullptr, *o_vmc = nullptr, *o_drho = nullptr,
         *o_vm_mem = nullptr;
  int parity = 0;
  bool have_state = false, have_dm = false, have_denv = false, have_outputs = false;
  bool phib_nonzero = false;
  int64_t steps_done = 0, launches = 0;
  cudaGraphExec_t graph = nullptr;
  bool graph_valid = false;
  std::vector<int> h_cell_ptr, h_m2c, h_map_env;
  std::vector<double> h_phib;
  // ---- environment fields on demand (bx_env_fields)
  float2* f_lap = nullptr;         // lapENVinv as double-float pairs [G][f_ld], columns >= G zero
  int f_ld = 0;                    // row pitch of f_lap (G rounded up to even)
  float2* f_X = nullptr;           // two-column right-hand side [G][2]
  double* f_buf = nullptr;         // field scratch, kFieldBufs x [G]
  int* f_last = nullptr;           // last membrane of each grid cell (-1: none)
  bool last_step_outputs = false;  // the latest bx_step computed outputs
  int* d_cl_mem = nullptr;         // membrane offsets of the clusters [ncl+1] (residual test)
  double* d_resid = nullptr;       // [ncl]
  // ---- batched environment fields (bx_batch_env_fields)
  std::vector<int> cl_ny, cl_nx, cl_goff;   // grid shape and offset in the concatenated grids
  std::vector<double> cl_delta;
  struct FieldShape {
    int ny = 0, nx = 0, xoff = 0, ncols = 0, soff = 0;
    std::vector<int> clusters;
    bx_dense_op_handle op = nullptr;
  };
  std::vector<FieldShape> fshapes;
  int Gtot = 0, Xtot = 0;
  int *bf_ci = nullptr, *bf_last = nullptr;
  double *bf_cd = nullptr, *bf_buf = nullptr, *bf_X = nullptr, *bf_Y = nullptr, *bf_scale = nullptr;
  // ---- factored split form (bx_factored.cuh), per cell slot
  float* f_dsa = nullptr;          // [I][S] sum of Dm_i * mem_sa over the cell's membranes
  float4* f_cst = nullptr;         // [S] {sum mem_sa, dt/cell_vol, diviterm/cm, gap-junction count | -1}
  int* f_gbeg = nullptr;           // [S] first gap-junction entry
  int2* f_gj = nullptr;            // [P + 2] {partner cell slot, bits of gj_weight*mem_sa} (+2: aligned copies)
  int f_P = 0;
  int* f_tile_e0 = nullptr;        // [nblk + 1] first gap-junction entry of each tile
  int f_max_ent = 0;               // entries of the largest tile
  std::vector<float> h_fsa;        // [S] sum of mem_sa (host, for f_cst)
  std::vector<int> h_gbeg, h_gcnt; // [S] (gcnt -1 = padding slot)
  std::vector<int2> h_gj;          // [P]
  // ---- resident cooperative kernel: built on first use, dropped with the layout
  int r_state = 0;                 // 0 not built, 1 ready, -1 does not fit (r_why)
  std::string r_why;
  int r_grid = 0, r_threads = 0, r_ntile_max = 0, r_nent_max = 0, r_nhalo_max = 0;
  size_t r_smem = 0;
  bx::ResCta* r_cta = nullptr;
  int2* r_gj = nullptr;
  int2* r_gbeg = nullptr;
  int* r_halo = nullptr;
  float2* r_cpart = nullptr;
  unsigned* r_ctl = nullptr;       // [0] barrier counter, [1] timeout flag
};

namespace {

void free_all(bx_cluster* h) {
  void* ptrs[] = {
      h->d_cell_ptr, h->d_m2c, h->d_nn, h->d_nn_cell, h->d_map_env, h->d_blk, h->d_blk_cl, h->d_cl_blk,
      h->d_env_ptr, h->d_env_mem, h->d_bflag, h->d_touched, h->d_lcell, h->d_mem_sa, h->d_gj_w, h->d_nx,
      h->d_ny, h->d_swm, h->d_swo, h->d_cell_vol, h->d_cell_sa, h->d_diviterm, h->d_mem_sa_f,
      h->d_gj_w_f, h->d_gjw0_f, h->d_dtv, h->d_dvc, h->d_Dm, h->d_Dm_f, h->d_vm[0], h->d_vm[1],
      h->d_ccm[0], h->d_ccm[1], h->d_cc, h->s_cc2, h->s_rec[0], h->s_rec[1], h->s_count,
      h->t_lcell, h->t_nn, h->t_map_env, h->t_nn_env, h->t_c0, h->t_m0, h->t_slot_of_cell, h->t_sa,
      h->t_gw, h->t_dtv, h->t_dvc, h->t_rng,
      h->s_cenv_f, h->s_pump, h->s_part, h->s_phib, h->d_cenv, h->d_phib, h->d_env_part,
      h->d_mem_flux_sa, h->d_pump, h->d_env_scale, h->d_Denv, h->d_Ex, h->d_Ey, h->d_fx, h->d_fy,
      h->d_tmp, h->d_tmp2, h->d_venv, h->d_rho_env, h->d_vsrc, h->d_status, h->d_env_ticket, h->o_fmem, h->o_fgj, h->o_rate,
      h->o_rho, h->o_Jn, h->o_Imem, h->o_Jcx, h->o_Jcy, h->o_Jc, h->o_vmave, h->o_dvm, h->o_Ecx,
      h->o_Ecy, h->o_Emc, h->o_Egjx, h->o_Egjy, h->o_gjopen, h->o_sigma, h->o_vmc, h->o_vm_mem,
      h->o_drho, h->f_lap, h->f_X, h->f_buf, h->f_last, h->d_cl_mem, h->d_resid,
      h->bf_ci, h->bf_last, h->bf_cd, h->bf_buf, h->bf_X, h->bf_Y, h->bf_scale, h->d_gjo, h->t_gjo, h->d_cnew, h->d_Rrads,
      h->st_vm, h->st_cc, h->st_cam, h->st_go, h->d_flag, h->t_slot_of_mem, h->t_blob,
      h->f_dsa, h->f_cst, h->f_gbeg, h->f_gj, h->f_tile_e0, h->r_cta, h->r_gj, h->r_gbeg, h->r_halo, h->r_cpart, h->r_ctl};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (auto& fs : h->fshapes)
    if (fs.op) bx_dense_op_destroy(fs.op);
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

// ca_handler runs its pump when Ca2+ is an ion and alpha_Ca > 0 (sim.py:1282-1283, 2129)
bool ca_pump_on(const bx_params& p) { return p.iCa >= 0 && p.iCa < p.n_ions && p.alpha_Ca > 0.0; }

// ECM with the Ca-ATPase: the Ca2+ row of the environment the pump reads
// (after the Nernst-Planck update and smoothing, before the scatter)
const double* ca_env_ptr(const bx_cluster* h) {
  if (!(h->ca && h->ecm)) return nullptr;
  const double* src = (h->par.sharpness < 1.0) ? h->d_cnew : h->d_tmp2;
  return src + (size_t)h->par.iCa * h->G;
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
  k.gj_len = h->gj_len;
  k.inv_tm = 1.0 / p.tm;
  k.inv_gj_len = 1.0 / h->gj_len;
  k.gj_block = p.gj_block;
  k.vgj = h->vgj ? 1 : 0;
  k.gj_vth = p.gj_vthresh;
  k.gj_min = p.gj_min;
  k.gj_dt_ms = p.dt * 1e3;
  k.iCa = h->ca ? p.iCa : -1;
  k.polar = h->polar ? 1 : 0;
  k.cm = p.cm;
  k.true_ratio = p.true_cell_size / p.cell_radius;
  k.ca_alpha = p.alpha_Ca;
  k.ca_inv_Km = 1.0 / p.KmCa_Ca;
  k.ca_atp_term = p.cATP / p.KmCa_ATP;
  k.ca_atp_den = 1.0 + p.cATP / p.KmCa_ATP;
  k.ca_qnum_c = p.cADP * p.cPi;
  k.ca_qden_c = p.cATP;
  k.inv_KmNa = 1.0 / p.KmNK_Na;
  k.inv_KmK = 1.0 / p.KmNK_K;
  k.atp_term = p.cATP / p.KmNK_ATP;
  k.atp_den = 1.0 + p.cATP / p.KmNK_ATP;
  k.qnum_c = (p.cADP * 1e-3) * (p.cPi * 1e-3);
  k.qden_c = p.cATP * 1e-3;
  k.K0 = std::exp(-(p.deltaGATP / RT));
  return k;
}

bx::SplitConst make_split_const(const bx_cluster* h) {
  const bx::StepConst d = make_step_const(h);
  bx::SplitConst k{};
  k.I = d.I;
  k.iNa = d.iNa;
  k.iK = d.iK;
  for (int i = 0; i < d.I; ++i) {
    k.zcode[i] = d.zcode[i];
    k.z[i] = (float)d.z[i];
    k.zF_hi[i] = (float)d.zF[i];
    k.zF_lo[i] = (float)(d.zF[i] - (double)k.zF_hi[i]);
    k.dgj_gs[i] = (float)d.dgj_gs[i];
  }
  k.F_RT = (float)d.F_RT;
  k.inv_tm = (float)(1.0 / d.tm);
  k.inv_gjl = (float)(1.0 / d.gj_len);
  k.gj_block = (float)d.gj_block;
  k.vgj = d.vgj;
  k.gj_vth = (float)d.gj_vth;
  k.gj_min = (float)d.gj_min;
  k.gj_dt_ms = (float)d.gj_dt_ms;
  k.iCa = d.iCa;
  k.ca_alpha = (float)d.ca_alpha;
  k.ca_inv_Km = (float)d.ca_inv_Km;
  k.ca_atp_term = (float)d.ca_atp_term;
  k.ca_atp_den = (float)d.ca_atp_den;
  k.ca_qnum_c = (float)d.ca_qnum_c;
  k.ca_qden_c = (float)d.ca_qden_c;
  k.inv_KmNa = (float)d.inv_KmNa;
  k.inv_KmK = (float)d.inv_KmK;
  k.atp_term = (float)d.atp_term;
  k.atp_den = (float)d.atp_den;
  k.qnum_c = (float)d.qnum_c;
  k.qden_c = (float)d.qden_c;
  k.K0 = (float)d.K0;
  return k;
}

bx::EnvConst make_env_const(const bx_cluster* h) {
  const bx_params& p = h->par;
  bx::EnvConst e{};
  e.I = h->I;
  e.ny = h->ny;
  e.nx = h->nx;
  e.G = h->G;
  e.delta = h->delta;
  e.inv_delta = 1.0 / h->delta;
  e.inv_2delta = 1.0 / (2.0 * h->delta);
  e.dt = p.dt;
  e.sharpness = p.sharpness;
  for (int i = 0; i < h->I; ++i) {
    e.np_alpha[i] = (p.zs[i] * p.q) / (p.kb * p.T);
    e.zF[i] = p.zs[i] * p.F;
    e.c_bound[i] = p.c_env_bound[i];
  }
  e.surf_scale = h->env_surf_scale;
  e.inv_koeoer = (p.ko_env != 0.0) ? 1.0 / (p.ko_env * p.eo * p.er) : 0.0;
  e.screen = (p.ko_env != 0.0) ? (2.0 / (p.ko_env * h->delta)) * (p.cell_radius / p.true_cell_size) : 0.0;
  e.inv_h_d2 = 1.0 / (p.cell_height * h->delta * h->delta);
  // sigma = 1, truncate = 4: the taps scipy.ndimage.gaussian_filter uses
  double w[9], s = 0.0;
  for (int q = -4; q <= 4; ++q) {
    w[q + 4] = std::exp(-0.5 * (double)(q * q));
    s += w[q + 4];
  }
  for (int q = 0; q < 9; ++q) e.gw[q] = w[q] / s;
  return e;
}

bx::DevGeom dev_geom(const bx_cluster* h) {
  bx::DevGeom g{};
  g.C = h->C; g.M = h->M; g.I = h->I; g.G = h->G; g.ny = h->ny; g.nx = h->nx;
  g.cell_ptr = h->d_cell_ptr; g.m2c = h->d_m2c; g.nn = h->d_nn; g.nn_cell = h->d_nn_cell;
  g.bflag = h->d_bflag; g.map_env = h->d_map_env; g.mem_sa = h->d_mem_sa; g.mem_sa_f = h->d_mem_sa_f;
  g.gj_w = h->d_gj_w; g.gj_w_f = h->d_gj_w_f; g.mem_nx = h->d_nx; g.mem_ny = h->d_ny;
  g.sw_mem = h->d_swm; g.sw_o = h->d_swo; g.cell_vol = h->d_cell_vol; g.cell_sa = h->d_cell_sa;
  g.diviterm = h->d_diviterm; g.blk_cell = h->d_blk; g.blk_cluster = h->d_blk_cl;
  g.R_rads = h->d_Rrads;
  return g;
}

bx::StepPtrs step_ptrs(bx_cluster* h, int parity) {
  bx::StepPtrs p{};
  p.vm_in = h->d_vm[parity]; p.vm_out = h->d_vm[parity ^ 1];
  p.ccm_in = h->d_ccm[parity]; p.ccm_out = h->d_ccm[parity ^ 1];
  p.cc = h->d_cc; p.Dm = h->d_Dm; p.Dm_f = h->d_Dm_f; p.cenv = h->d_cenv; p.pump_coef = h->d_pump;
  p.phib = h->d_phib; p.env_part = h->d_env_part; p.mem_flux_sa = h->d_mem_flux_sa;
  p.status = h->d_status;
  p.o_fmem = h->o_fmem; p.o_fgj = h->o_fgj; p.o_rate = h->o_rate; p.o_rho = h->o_rho;
  p.o_Jn = h->o_Jn; p.o_Imem = h->o_Imem; p.o_Jcx = h->o_Jcx; p.o_Jcy = h->o_Jcy;
  p.o_Jc = h->o_Jc; p.o_vmave = h->o_vmave; p.o_dvm = h->o_dvm; p.o_Ecx = h->o_Ecx;
  p.o_Ecy = h->o_Ecy; p.o_Emc = h->o_Emc; p.o_Egjx = h->o_Egjx; p.o_Egjy = h->o_Egjy;
  p.o_gjopen = h->o_gjopen; p.o_sigma = h->o_sigma;
  p.gjo = h->d_gjo;
  p.ca_env = ca_env_ptr(h);
  return p;
}

bx::SplitGeom split_geom(const bx_cluster* h) {
  bx::SplitGeom g{};
  g.C = h->C; g.M = h->M; g.I = h->I; g.G = h->G; g.Q = h->Q; g.S = h->S;
  g.lcell = h->t_lcell; g.nn_slot = h->t_nn; g.mem_sa = h->t_sa; g.gjw = h->t_gw;
  g.cell_rng = h->t_rng; g.dtv = h->t_dtv; g.dvc = h->t_dvc; g.blk_cluster = h->d_blk_cl;
  g.tile_c0 = h->t_c0; g.tile_m0 = h->t_m0; g.map_env = h->t_map_env; g.nn_env = h->t_nn_env;
  g.geo_blob = h->t_blob;
  return g;
}

bx::SplitPtrs split_ptrs(bx_cluster* h, int parity) {
  bx::SplitPtrs p{};
  p.rec_in = h->s_rec[parity]; p.rec_out = h->s_rec[parity ^ 1];
  p.cc2 = h->s_cc2; p.Dm = h->d_Dm_f; p.cenv_f = h->s_cenv_f;
  p.pump_coef = h->s_pump; p.phib = h->s_phib;
  p.env_part = h->s_part; p.status = h->d_status;
  p.o_fmem = h->o_fmem; p.o_fgj = h->o_fgj; p.o_rate = h->o_rate; p.o_rho = h->o_rho;
  p.o_vmem = h->o_vmc;
  p.o_drho = h->o_drho;
  p.cenv_grid = h->ecm ? h->d_cenv : nullptr;
  p.mfs = h->d_mem_flux_sa;
  p.gjo = h->t_gjo;
  p.o_gjopen = h->o_gjopen;
  p.ca_env = ca_env_ptr(h);
  return p;
}

// BETSE's six-ion set compiled as constants (bx_split.cuh IonSet<1>)
bx::FactGeom fact_geom(const bx_cluster* h) {
  bx::FactGeom g{};
  g.S = h->S; g.ntile = h->nblk;
  g.dsa = h->f_dsa; g.cst = h->f_cst; g.gbeg = h->f_gbeg; g.gj = h->f_gj; g.blk_cluster = h->d_blk_cl;
  return g;
}

// The factored and resident kernels need one Vmem and one environment per
// cell: no Phi_b, no extracellular spaces, no per-membrane gating state, no
// Ca-ATPase (which reads the cell concentration per membrane), no outputs.
bool fact_eligible(const bx_cluster* h, bool out) {
  return h->mode == MODE_SPLIT && !out && !h->phib_nonzero && !h->ecm && !h->vgj && !h->ca;
}

// The plain form's one-lane-per-ion kernel covers the same configuration
// without polarizability, on CTAs of 8 to 64 membrane slots.
bool ion_eligible(const bx_cluster* h, bool out) {
  return h->mode != MODE_SPLIT && !out && !h->phib_nonzero && !h->ecm && !h->vgj && !h->ca && !h->polar &&
         (h->tpb == 8 || h->tpb == 16 || h->tpb == 32 || h->tpb == 64);
}

bool is_betse_six_ions(const bx_cluster* h) {
  const double z6[6] = {1, 1, -1, 2, -1, -1};
  if (h->I != 6 || h->par.iNa != 0 || h->par.iK != 1) return false;
  for (int i = 0; i < 6; ++i)
    if (h->par.zs[i] != z6[i]) return false;
  return true;
}

inline int env_grid(int G) { return (G + kEnvTPB - 1) / kEnvTPB; }

// The persistent kernel's contiguous per-tile static data (PersistGeo), for
// the instantiation that will read it; rebuilt after every layout or Dm change.
template <int TPB, int NI>
cudaError_t build_geo_blob_t(bx_cluster* h) {
  using PG = bx::PersistGeo<TPB, NI>;
  const size_t bytes = sizeof(PG) * (size_t)h->nblk;
  if (h->t_blob_bytes != bytes) {
    if (h->t_blob) cudaFree(h->t_blob);
    h->t_blob = nullptr;
    h->t_blob_bytes = 0;
    cudaError_t e = cudaMalloc(&h->t_blob, bytes);
    if (e != cudaSuccess) return e;
    h->t_blob_bytes = bytes;
  }
  bx::k_split_blob<TPB, NI><<<h->nblk, TPB, 0, h->stream>>>(static_cast<PG*>(h->t_blob), h->d_Dm_f, h->t_sa,
                                                            h->t_gw, h->t_nn, h->t_lcell, h->d_blk_cl, h->I,
                                                            h->Q);
  return cudaGetLastError();
}

cudaError_t build_geo_blob(bx_cluster* h) {
  if (h->mode != MODE_SPLIT || !h->t_lcell) return cudaSuccess;
  const bool six = is_betse_six_ions(h);
  if (h->tpb == 192) return six ? build_geo_blob_t<192, 6>(h) : build_geo_blob_t<192, bx::kMaxIons>(h);
  return six ? build_geo_blob_t<256, 6>(h) : build_geo_blob_t<256, bx::kMaxIons>(h);
}

// launch with programmatic dependent launch: the kernel's prologue overlaps
// the previous kernel; cudaGridDependencySynchronize orders the state accesses
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl_smem(void (*kern)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t s,
                            Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, args...);
}

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kern)(KArgs...), unsigned grid, unsigned block, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, args...);
}

template <int TPB, bool OUT, bool PHIB, bool ECM>
cudaError_t launch_split_t(bx_cluster* h, int parity, cudaStream_t s) {
  if (is_betse_six_ions(h))
    return launch_pdl(bx::k_split_step<TPB, kRec, 1, OUT, PHIB, ECM>, (unsigned)h->nblk, TPB, s, split_geom(h),
                      split_ptrs(h, parity), make_split_const(h));
  return launch_pdl(bx::k_split_step<TPB, kRec, 0, OUT, PHIB, ECM>, (unsigned)h->nblk, TPB, s, split_geom(h),
                    split_ptrs(h, parity), make_split_const(h));
}

template <int TPB, bool OUT, bool PHIB>
cudaError_t launch_split_e(bx_cluster* h, int parity, cudaStream_t s) {
  return h->ecm ? launch_split_t<TPB, OUT, PHIB, true>(h, parity, s)
                : launch_split_t<TPB, OUT, PHIB, false>(h, parity, s);
}

// the persistent kernel: one wave of CTAs walking the tiles
template <int TPB, int ZP>
cudaError_t launch_persist_t(bx_cluster* h, int parity, cudaStream_t s) {
  auto kern = bx::k_split_persist<TPB, ZP>;
  const size_t smem = sizeof(bx::PersistSmem<TPB, bx::IonSet<ZP>::NI>);
  static bool attr_set = false;   // per instantiation
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TPB, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int grid = std::max(1, std::min(h->nblk, per_sm * h->sm_count));
  return launch_pdl_smem(kern, (unsigned)grid, TPB, smem, s, split_geom(h), split_ptrs(h, parity),
                         make_split_const(h), h->nblk);
}

// the factored step: 8 tiles (warps) per CTA
constexpr int kFactWarps = 8;
template <int U, int PF>
cudaError_t launch_fact_u(bx_cluster* h, int parity, cudaStream_t s) {
  const unsigned grid = (unsigned)((h->nblk + kFactWarps - 1) / kFactWarps);
  if (is_betse_six_ions(h))
    return launch_pdl(bx::k_split_fact<kFactWarps, 1, U, PF>, grid, kFactWarps * 32, s, fact_geom(h),
                      split_ptrs(h, parity), make_split_const(h));
  return launch_pdl(bx::k_split_fact<kFactWarps, 0, U, PF>, grid, kFactWarps * 32, s, fact_geom(h),
                    split_ptrs(h, parity), make_split_const(h));
}

// the pipelined factored step: one warp per CTA, as many CTAs as fit an SM
template <int ZP>
cudaError_t launch_fact_pipe_t(bx_cluster* h, int parity, cudaStream_t s) {
  auto kern = bx::k_split_fact_pipe<1, ZP>;
  const bx::FactPipeSmem L(h->f_max_ent, bx::IonSet<ZP>::NI);
  const size_t smem = L.warp_bytes;
  static int attr_set = 0;      // per instantiation: the largest size set so far
  if ((int)smem > attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = (int)smem;
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int grid = std::max(1, std::min(h->nblk, per_sm * h->sm_count));
  return launch_pdl_smem(kern, (unsigned)grid, 32, smem, s, fact_geom(h), split_ptrs(h, parity),
                         make_split_const(h), (const int*)h->f_tile_e0, h->f_max_ent);
}

cudaError_t launch_fact(bx_cluster* h, int parity, cudaStream_t s) {
  if (h->kind == KIND_FACT_PIPE)
    return is_betse_six_ions(h) ? launch_fact_pipe_t<1>(h, parity, s) : launch_fact_pipe_t<0>(h, parity, s);
  // fact_unroll: gap junctions per load round (2, 4); +10 with the first
  // entries prefetched before the grid dependency wait (2, 3, 6 per round
  // with 6 prefetched; 4 per round with 8)
  switch (h->fact_unroll) {
    case 2: return launch_fact_u<2, 0>(h, parity, s);
    case 12: return launch_fact_u<2, 6>(h, parity, s);
    case 13: return launch_fact_u<3, 6>(h, parity, s);
    case 14: return launch_fact_u<4, 8>(h, parity, s);
    case 16: return launch_fact_u<6, 6>(h, parity, s);
    default: return launch_fact_u<4, 0>(h, parity, s);
  }
}

void drop_resident(bx_cluster* h) {
  void* ptrs[] = {h->r_cta, h->r_gj, h->r_gbeg, h->r_halo, h->r_cpart, h->r_ctl};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  h->r_cta = nullptr; h->r_gj = nullptr; h->r_gbeg = nullptr; h->r_halo = nullptr; h->r_cpart = nullptr;
  h->r_ctl = nullptr;
  h->r_state = 0;
}

template <int ZP>
void* resident_kernel() { return reinterpret_cast<void*>(bx::k_split_resident<ZP>); }

// Partition of the tiles over one CTA per SM for k_split_resident, each CTA's
// gap-junction entries re-indexed into its record table (own cells, then
// the halo of partner cells it does not own), and the shared-memory size.
// Marks the handle "does not fit" (r_state = -1, reason in r_why) when a
// CTA's cells and entries exceed the shared memory of one SM, when more than
// 32 tiles would share a CTA, or for a batch of clusters.
int build_resident(bx_cluster* h) {
  drop_resident(h);
  auto refuse = [&](const std::string& why) {
    h->r_state = -1;
    h->r_why = why;
    return BX_OK;
  };
  if (h->ncl != 1) return refuse("the resident kernel steps one cluster (its environment is one sum)");
  const int nblk = h->nblk, nsm = h->sm_count;
  const int grid = std::min(nblk, nsm);
  const int ntile_max = (nblk + grid - 1) / grid;
  // one thread per cell, at most two cells per thread (1024 threads)
  if (ntile_max > 64) return refuse("more than 64 tiles per SM");
  std::vector<bx::ResCta> cta(grid);
  std::vector<int2> ent;
  std::vector<int2> gbeg(h->S, make_int2(0, 0));
  std::vector<int> halo;
  int nent_max = 0, nhalo_max = 0;
  for (int j = 0; j < grid; ++j) {
    const int t0 = (int)((long long)j * nblk / grid), t1 = (int)((long long)(j + 1) * nblk / grid);
    const int slot0 = 32 * t0, n_own = 32 * (t1 - t0);
    bx::ResCta& c = cta[j];
    c.tile0 = t0; c.ntile = t1 - t0; c.ent0 = (int)ent.size(); c.halo0 = (int)halo.size();
    c.pad[0] = c.pad[1] = 0;
    std::vector<int> hl;                       // this CTA's halo, sorted
    for (int ls = 0; ls < n_own; ++ls) {
      const int sl = slot0 + ls;
      for (int q = 0; q < std::max(0, h->h_gcnt[sl]); ++q) {
        const int p = h->h_gj[h->h_gbeg[sl] + q].x;
        if (p < slot0 || p >= slot0 + n_own) hl.push_back(p);
      }
    }
    std::sort(hl.begin(), hl.end());
    hl.erase(std::unique(hl.begin(), hl.end()), hl.end());
    // each cell's entries: partners this CTA owns first (in membrane order),
    // then halo partners (in membrane order); gbeg = {first, owned count}
    for (int ls = 0; ls < n_own; ++ls) {
      const int sl = slot0 + ls;
      const int first = (int)ent.size() - c.ent0;
      int nloc = 0;
      for (int pass = 0; pass < 2; ++pass)
        for (int q = 0; q < std::max(0, h->h_gcnt[sl]); ++q) {
          const int2 e = h->h_gj[h->h_gbeg[sl] + q];
          const bool local = e.x >= slot0 && e.x < slot0 + n_own;
          if (local != (pass == 0)) continue;
          int loc;
          if (local) { loc = e.x - slot0; ++nloc; }
          else loc = n_own + (int)(std::lower_bound(hl.begin(), hl.end(), e.x) - hl.begin());
          ent.push_back(make_int2(loc, e.y));
        }
      gbeg[sl] = make_int2(first, nloc);
    }
    c.nent = (int)ent.size() - c.ent0;
    c.nhalo = (int)hl.size();
    halo.insert(halo.end(), hl.begin(), hl.end());
    nent_max = std::max(nent_max, c.nent);
    nhalo_max = std::max(nhalo_max, c.nhalo);
  }
  const bool six = is_betse_six_ions(h);
  const int NI = six ? 6 : bx::kMaxIons;
  const bx::ResSmem L(ntile_max, nent_max, nhalo_max, NI);
  int optin = 0;
  BX_CU(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->dev));
  if (L.total > (size_t)optin)
    return refuse("the cells of one SM need " + std::to_string(L.total) + " bytes of shared memory (" +
                  std::to_string(optin) + " available)");
  const void* kern = six ? resident_kernel<1>() : resident_kernel<0>();
  // the device's limit, so handles of different sizes never undercut each other
  BX_CU(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
  const int threads = 32 * std::min(ntile_max, 32);
  int per_sm = 0;
  BX_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, L.total));
  if (per_sm < 1) return refuse("one CTA of the resident kernel does not fit an SM");
  int coop = 0;
  BX_CU(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, h->dev));
  if (!coop) return refuse("the device has no cooperative launch");
  BX_CU(dalloc(&h->r_cta, cta.size())); BX_CU(h2d(h->r_cta, cta.data(), cta.size()));
  BX_CU(dalloc(&h->r_gj, std::max<size_t>(1, ent.size())));
  if (!ent.empty()) BX_CU(h2d(h->r_gj, ent.data(), ent.size()));
  BX_CU(dalloc(&h->r_gbeg, gbeg.size())); BX_CU(h2d(h->r_gbeg, gbeg.data(), gbeg.size()));
  BX_CU(dalloc(&h->r_halo, std::max<size_t>(1, halo.size())));
  if (!halo.empty()) BX_CU(h2d(h->r_halo, halo.data(), halo.size()));
  BX_CU(dalloc(&h->r_cpart, (size_t)2 * grid * h->I));
  BX_CU(dalloc(&h->r_ctl, 2));
  BX_CU(cudaMemset(h->r_ctl, 0, 2 * sizeof(unsigned)));
  h->r_grid = grid; h->r_threads = threads; h->r_smem = L.total;
  h->r_ntile_max = ntile_max; h->r_nent_max = nent_max; h->r_nhalo_max = nhalo_max;
  h->r_state = 1;
  return BX_OK;
}

// n_steps time steps in one cooperative launch of k_split_resident (reads
// parity, leaves the state at parity ^ (n_steps & 1)).
cudaError_t launch_resident(bx_cluster* h, int parity, int n_steps, cudaStream_t s,
                            long long timeout_ns = kResTimeoutNs, unsigned bias = 0) {
  cudaError_t e = cudaMemsetAsync(h->r_ctl, 0, sizeof(unsigned), s);   // the barrier counter
  if (e != cudaSuccess) return e;
  bx::ResArrays ra{};
  ra.cta = h->r_cta; ra.gj = h->r_gj; ra.gbeg = h->r_gbeg; ra.halo = h->r_halo; ra.cpart = h->r_cpart;
  ra.ctl = h->r_ctl; ra.cenv64 = h->d_cenv; ra.cenv_f = h->s_cenv_f; ra.env_scale = h->d_env_scale;
  ra.rec_glob[0] = h->s_rec[parity]; ra.rec_glob[1] = h->s_rec[parity ^ 1];
  ra.ntile_max = h->r_ntile_max; ra.nent_max = h->r_nent_max; ra.nhalo_max = h->r_nhalo_max;
  ra.timeout_ns = timeout_ns;
  ra.barrier_bias = bias;
  bx::FactGeom fg = fact_geom(h);
  bx::SplitPtrs sp = split_ptrs(h, parity);
  bx::SplitConst k = make_split_const(h);
  void* args[] = {&fg, &sp, &k, &ra, &n_steps};
  const void* kern = is_betse_six_ions(h) ? resident_kernel<1>() : resident_kernel<0>();
  return cudaLaunchCooperativeKernel(kern, dim3(h->r_grid), dim3(h->r_threads), args, h->r_smem, s);
}

cudaError_t launch_split(bx_cluster* h, int parity, bool out, cudaStream_t s) {
  if ((h->kind == KIND_FACT || h->kind == KIND_RESIDENT || h->kind == KIND_FACT_PIPE) && fact_eligible(h, out))
    return launch_fact(h, parity, s);
  if (h->kind == KIND_PERSIST && !out && !h->phib_nonzero && !h->ecm && !h->vgj && !h->ca) {
    const bool six = is_betse_six_ions(h);
    if (h->tpb == 192) return six ? launch_persist_t<192, 1>(h, parity, s) : launch_persist_t<192, 0>(h, parity, s);
    return six ? launch_persist_t<256, 1>(h, parity, s) : launch_persist_t<256, 0>(h, parity, s);
  }
  const int code = (h->tpb == 192 ? 4 : 0) | (out ? 2 : 0) | (h->phib_nonzero ? 1 : 0);
  switch (code) {
    case 0: return launch_split_e<256, false, false>(h, parity, s);
    case 1: return launch_split_e<256, false, true>(h, parity, s);
    case 2: return launch_split_e<256, true, false>(h, parity, s);
    case 3: return launch_split_e<256, true, true>(h, parity, s);
    case 4: return launch_split_e<192, false, false>(h, parity, s);
    case 5: return launch_split_e<192, false, true>(h, parity, s);
    case 6: return launch_split_e<192, true, false>(h, parity, s);
    default: return launch_split_e<192, true, true>(h, parity, s);
  }
}

cudaError_t launch_split_env(bx_cluster* h, cudaStream_t s) {
  return launch_pdl(bx::k_split_env<512>, (unsigned)h->ncl, 512, s, (const float*)h->s_part,
                    (const int*)h->d_cl_blk, h->I, h->d_cenv, h->s_cenv_f, (const double*)h->d_env_scale);
}

cudaError_t launch_cell(bx_cluster* h, int parity, bool out, cudaStream_t s) {
  bx::DevGeom g = dev_geom(h);
  bx::StepConst k = make_step_const(h);
  bx::StepPtrs p = step_ptrs(h, parity);
  if (h->kind == KIND_ION && ion_eligible(h, out)) {
    const bx::EnvMix em{h->d_cenv, h->d_cl_blk, h->d_env_scale, h->d_env_ticket};
    switch (h->tpb) {
      case 8: return bx::launch_cell_step_ion<8>(h->nblk, s, g, p, k, em);
      case 16: return bx::launch_cell_step_ion<16>(h->nblk, s, g, p, k, em);
      case 32: return bx::launch_cell_step_ion<32>(h->nblk, s, g, p, k, em);
      default: return bx::launch_cell_step_ion<64>(h->nblk, s, g, p, k, em);
    }
  }
  // partitions of 8 or 16 membrane slots run on 32-thread CTAs
  switch (h->tpb) {
    case 8:
    case 16:
    case 32: return bx::launch_cell_step<double, 32>(h->ecm, out, h->phib_nonzero, h->nblk, s, g, p, k);
    case 64: return bx::launch_cell_step<double, 64>(h->ecm, out, h->phib_nonzero, h->nblk, s, g, p, k);
    case 128: return bx::launch_cell_step<double, 128>(h->ecm, out, h->phib_nonzero, h->nblk, s, g, p, k);
    default: return bx::launch_cell_step<double, 256>(h->ecm, out, h->phib_nonzero, h->nblk, s, g, p, k);
  }
}

// The extracellular grid of one step (update_ecm, update_Co's ECM term, get_current's E_env).
// ECM with the Ca-ATPase, before the step kernel: BETSE's update_ecm runs per
// ion inside the ion loop and ca_handler reads the result, so the
// Nernst-Planck update (and smoothing) of every ion goes first, into d_tmp2 /
// d_cnew, and enqueue_env adds the membrane scatter afterwards.  The
// arithmetic of each grid value is that of the fused path.
cudaError_t enqueue_env_pre(bx_cluster* h, cudaStream_t s) {
  bx::EnvConst ec = make_env_const(h);
  const int gi = env_grid(h->G * h->I);
  bx::k_env_np_flux<double><<<gi, kEnvTPB, 0, s>>>(h->d_cenv, h->d_Denv, h->d_Ex, h->d_Ey, h->d_fx, h->d_fy, ec);
  bx::k_env_update<false><<<gi, kEnvTPB, 0, s>>>(h->d_cenv, h->d_tmp2, h->d_fx, h->d_fy, h->d_env_ptr,
                                                h->d_env_mem, h->d_mem_flux_sa, h->M, ec);
  h->launches += 2;
  if (h->par.sharpness < 1.0) {
    bx::k_env_integrate_scatter<false><<<gi, kEnvTPB, 0, s>>>(h->d_cnew, h->d_tmp2, h->d_env_ptr, h->d_env_mem,
                                                             h->d_mem_flux_sa, h->M, ec);
    h->launches += 1;
  }
  return cudaGetLastError();
}

cudaError_t enqueue_env(bx_cluster* h, bool out, cudaStream_t s) {
  bx::EnvConst ec = make_env_const(h);
  const int gg = env_grid(h->G);
  const int gi = env_grid(h->G * h->I);   // one thread per (ion, grid cell)
  if (h->ca) {
    const double* src = (h->par.sharpness < 1.0) ? h->d_cnew : h->d_tmp2;
    bx::k_env_scatter_add<<<gi, kEnvTPB, 0, s>>>(h->d_cenv, src, h->d_env_ptr, h->d_env_mem,
                                                h->d_mem_flux_sa, h->M, ec);
    h->launches += 1;
  } else if (h->par.sharpness < 1.0) {
    bx::k_env_np_flux<double><<<gi, kEnvTPB, 0, s>>>(h->d_cenv, h->d_Denv, h->d_Ex, h->d_Ey, h->d_fx, h->d_fy, ec);
    bx::k_env_update<false><<<gi, kEnvTPB, 0, s>>>(h->d_cenv, h->d_tmp2, h->d_fx, h->d_fy, h->d_env_ptr,
                                                  h->d_env_mem, h->d_mem_flux_sa, h->M, ec);
    bx::k_env_integrate_scatter<true><<<gi, kEnvTPB, 0, s>>>(h->d_cenv, h->d_tmp2, h->d_env_ptr,
                                                            h->d_env_mem, h->d_mem_flux_sa, h->M, ec);
    h->launches += 3;
  } else {
    // the common configuration: flux, then update + charge fused, then the
    // fields in one tiled launch (4 launches per step with the cell kernel);
    // the split form runs these stencils in FP32 around FP64 state
    const unsigned gc = (unsigned)(((size_t)h->G * 8 + 255) / 256);
    const dim3 gt((unsigned)((h->nx + bx::kEnvTX - 1) / bx::kEnvTX), (unsigned)((h->ny + bx::kEnvTY - 1) / bx::kEnvTY));
    const double* phib = h->phib_nonzero ? h->d_phib : nullptr;
    double* rho = out ? h->d_rho_env : nullptr;
    if (h->mode == MODE_SPLIT) {
      bx::k_env_np_flux<float><<<gi, kEnvTPB, 0, s>>>(h->d_cenv, h->d_Denv, h->d_Ex, h->d_Ey, h->d_fx, h->d_fy, ec);
      bx::k_env_update_charge<float><<<gc, 256, 0, s>>>(h->d_cenv, h->d_fx, h->d_fy, h->d_env_ptr, h->d_env_mem,
                                                        h->d_mem_flux_sa, h->M, h->d_touched, h->d_vsrc, rho, ec);
      bx::k_env_fields_tile<float><<<gt, bx::kEnvTX * bx::kEnvTY, 0, s>>>(h->d_vsrc, phib, h->d_venv, ec.screen,
                                                                         h->d_Ex, h->d_Ey, ec);
    } else {
      bx::k_env_np_flux<double><<<gi, kEnvTPB, 0, s>>>(h->d_cenv, h->d_Denv, h->d_Ex, h->d_Ey, h->d_fx, h->d_fy, ec);
      bx::k_env_update_charge<double><<<gc, 256, 0, s>>>(h->d_cenv, h->d_fx, h->d_fy, h->d_env_ptr, h->d_env_mem,
                                                         h->d_mem_flux_sa, h->M, h->d_touched, h->d_vsrc, rho, ec);
      bx::k_env_fields_tile<double><<<gt, bx::kEnvTX * bx::kEnvTY, 0, s>>>(h->d_vsrc, phib, h->d_venv, ec.screen,
                                                                          h->d_Ex, h->d_Ey, ec);
    }
    h->launches += 3;
    return cudaGetLastError();
  }
  bx::k_env_charge<<<gg, kEnvTPB, 0, s>>>(h->d_cenv, h->d_touched, h->d_vsrc, out ? h->d_rho_env : nullptr, ec);
  h->launches += 1;
  bx::k_env_gauss_y<<<gg, kEnvTPB, 0, s>>>(h->d_vsrc, h->d_tmp, ec);
  bx::k_env_gauss_x<<<gg, kEnvTPB, 0, s>>>(h->d_tmp, h->phib_nonzero ? h->d_phib : nullptr, h->d_venv, ec);
  bx::k_env_neg_grad<<<gg, kEnvTPB, 0, s>>>(h->d_venv, ec.screen, h->d_Ex, h->d_Ey, ec);
  h->launches += 3;
  return cudaGetLastError();
}

// Enqueue one time step (reads parity, writes parity^1).
cudaError_t enqueue_step(bx_cluster* h, int parity, bool out, cudaStream_t s) {
  cudaError_t e;
  if (h->ca && h->ecm) {
    e = enqueue_env_pre(h, s);
    if (e != cudaSuccess) return e;
  }
  if (h->mode == MODE_SPLIT) {
    e = launch_split(h, parity, out, s);
    if (e != cudaSuccess) return e;
    h->launches += 1;
    if (h->ecm) {
      e = enqueue_env(h, out, s);
    } else {
      e = launch_split_env(h, s);
      h->launches += 1;
    }
    if (e != cudaSuccess) return e;
    if (out) {
      bx::SplitOutGeom og{h->C, h->M, h->I, h->d_cell_ptr, h->d_blk, h->d_nn, h->d_map_env,
                          h->d_mem_sa, h->d_nx, h->d_ny, h->d_swm, h->d_swo, h->d_cell_sa,
                          h->d_gj_w, h->d_bflag, h->d_diviterm, h->o_drho};
      bx::SplitOutPtrs op{h->o_fmem, h->o_fgj, h->s_rec[parity ^ 1], h->s_rec[parity], kRec, h->s_cc2,
                          h->S, h->t_slot_of_cell,
                          h->phib_nonzero ? h->s_phib : nullptr, h->o_Jn, h->o_Imem, h->o_Jcx,
                          h->o_Jcy, h->o_Jc, h->o_vmave, h->o_dvm, h->o_Ecx, h->o_Ecy, h->o_Emc,
                          h->o_Egjx, h->o_Egjy, h->o_gjopen, h->o_sigma, h->o_vm_mem};
      bx::SplitOutConst oc{};
      const bx::StepConst d = make_step_const(h);
      oc.I = h->I;
      for (int i = 0; i < h->I; ++i) { oc.zF[i] = d.zF[i]; oc.sig_coef[i] = d.sig_coef[i]; }
      oc.dt = d.dt; oc.gj_len = h->gj_len; oc.gj_block = d.gj_block; oc.cm = h->par.cm;
      oc.vgj = h->vgj ? 1 : 0;
      if (h->tpb == 192) bx::k_split_outputs<192><<<h->nblk, 192, 0, s>>>(og, op, oc);
      else bx::k_split_outputs<256><<<h->nblk, 256, 0, s>>>(og, op, oc);
      bx::k_split_egj<<<(h->M + 255) / 256, 256, 0, s>>>(h->M, h->d_nn, h->o_vm_mem, h->d_nx, h->d_ny,
                                                         h->gj_len, h->o_Egjx, h->o_Egjy);
      h->launches += 2;
    }
    return cudaGetLastError();
  }
  e = launch_cell(h, parity, out, s);
  if (e != cudaSuccess) return e;
  h->launches++;
  if (h->kind == KIND_ION && ion_eligible(h, out)) return cudaSuccess;   // it mixed the environment
  if (!h->ecm) {
    bx::k_env_mix<<<h->ncl, 256, 0, s>>>(h->d_env_part, h->d_cl_blk, h->I, h->d_cenv, h->d_env_scale);
    h->launches++;
    return cudaGetLastError();
  }
  return enqueue_env(h, out, s);
}

int launches_per_step(const bx_cluster* h) {
  if (h->kind == KIND_ION && ion_eligible(h, false)) return 1;
  if (!h->ecm) return 2;
  if (h->ca) return h->par.sharpness < 1.0 ? 9 : 8;
  return h->par.sharpness < 1.0 ? 8 : 4;
}

int upload_fact_cst(bx_cluster* h);

// per-cluster constants that depend on the parameters (dt, cm, alpha_NaK, vol_env)
int upload_param_arrays(bx_cluster* h) {
  std::vector<double> pump(h->ncl), escale(h->ncl);
  std::vector<float> pump_f(h->ncl);
  for (int c = 0; c < h->ncl; ++c) {
    const bx_params& p = h->cl_par[c];
    pump[c] = -3.0 * p.nakatp_block * p.alpha_NaK;
    pump_f[c] = (float)pump[c];
    const int Mc = h->cl_mem[c + 1] - h->cl_mem[c];
    escale[c] = p.dt / (p.vol_env * (double)Mc);
  }
  BX_CU(h2d(h->d_pump, pump.data(), h->ncl));
  BX_CU(h2d(h->d_env_scale, escale.data(), h->ncl));
  if (h->mode == MODE_SPLIT) {
    BX_CU(h2d(h->s_pump, pump_f.data(), h->ncl));
    if (h->t_dtv) {
      std::vector<float> dtv(h->S, 0.f), dvc(h->S, 0.f);
      for (int c = 0; c < h->C; ++c) {
        const int s = h->h_slot_of_cell[c];
        dtv[s] = (float)(h->par.dt / h->h_vol[c]);
        dvc[s] = (float)(h->h_div[c] / h->par.cm);
      }
      BX_CU(h2d(h->t_dtv, dtv.data(), h->S));
      BX_CU(h2d(h->t_dvc, dvc.data(), h->S));
    }
    int rc = upload_fact_cst(h);
    if (rc != BX_OK) return rc;
  }
  return BX_OK;
}

bool same_shared_params(const bx_params& a, const bx_params& b) {
  if (a.n_ions != b.n_ions || a.iNa != b.iNa || a.iK != b.iK || a.is_ecm != b.is_ecm) return false;
  if (a.v_sensitive_gj != b.v_sensitive_gj || a.gj_vthresh != b.gj_vthresh || a.gj_min != b.gj_min) return false;
  if (a.iCa != b.iCa || a.alpha_Ca != b.alpha_Ca || a.KmCa_Ca != b.KmCa_Ca || a.KmCa_ATP != b.KmCa_ATP) return false;
  if (a.cell_polarizability != b.cell_polarizability) return false;
  const double sa[] = {a.F, a.R, a.T, a.dt, a.cm, a.tm, a.gj_surface, a.gj_block, a.KmNK_Na, a.KmNK_K,
                       a.KmNK_ATP, a.cATP, a.cADP, a.cPi, a.deltaGATP};
  const double sb[] = {b.F, b.R, b.T, b.dt, b.cm, b.tm, b.gj_surface, b.gj_block, b.KmNK_Na, b.KmNK_K,
                       b.KmNK_ATP, b.cATP, b.cADP, b.cPi, b.deltaGATP};
  for (size_t q = 0; q < sizeof(sa) / sizeof(sa[0]); ++q)
    if (sa[q] != sb[q]) return false;
  for (int i = 0; i < a.n_ions; ++i)
    if (a.zs[i] != b.zs[i] || a.D_gj[i] != b.D_gj[i] || a.D_free[i] != b.D_free[i]) return false;
  return true;
}

int check_geom(const bx_geom* g, const bx_params* p) {
  const int C = g->n_cells, M = g->n_mems;
  if (C <= 0 || M <= 0) return fail(BX_EINVAL, "empty cluster (n_cells and n_mems must be > 0)");
  if (g->grid_ny < 3 || g->grid_nx < 3) return fail(BX_EINVAL, "environment grid must be at least 3x3");
  if (!g->cell_mem_ptr || !g->nn_i || !g->bflag || !g->map_mem2ecm || !g->mem_sa || !g->gj_weight ||
      !g->cell_vol || !g->cell_sa || !g->diviterm || !g->mem_nx || !g->mem_ny || !g->smooth_weight_mem ||
      !g->smooth_weight_o)
    return fail(BX_EINVAL, "missing geometry array");
  if (!(g->gj_len > 0.0) || !(g->delta > 0.0)) return fail(BX_EINVAL, "gj_len and delta must be > 0");
  const int G = g->grid_ny * g->grid_nx;
  // the CSR map (the bit-exact form of mem_to_cells / cell_to_mems)
  if (g->cell_mem_ptr[0] != 0 || g->cell_mem_ptr[C] != M)
    return fail(BX_EINVAL, "cell_mem_ptr must start at 0 and end at n_mems");
  for (int c = 0; c < C; ++c) {
    const int a = g->cell_mem_ptr[c], b = g->cell_mem_ptr[c + 1];
    if (b <= a) return fail(BX_EINVAL, "cell_mem_ptr must be increasing (every cell needs a membrane)");
    if (b - a > BX_MAX_MEMS_PER_CELL) return fail(BX_EINVAL, "a cell has more than 256 membranes");
    if (!(g->cell_vol[c] > 0.0) || !(g->cell_sa[c] > 0.0))
      return fail(BX_EINVAL, "cell_vol and cell_sa must be > 0");
  }
  for (int m = 0; m < M; ++m) {
    if (g->nn_i[m] < 0 || g->nn_i[m] >= M) return fail(BX_EINVAL, "nn_i out of range");
    if (g->map_mem2ecm[m] < 0 || g->map_mem2ecm[m] >= G) return fail(BX_EINVAL, "map_mem2ecm out of range");
  }
  if (p->is_ecm && !g->mem_sa_per_env) return fail(BX_EINVAL, "ECM needs mem_sa_per_env");
  return BX_OK;
}

// bit casts on the host
inline float bits_to_float(int v) { float f; std::memcpy(&f, &v, sizeof f); return f; }
inline int float_to_bits(float f) { int v; std::memcpy(&v, &f, sizeof v); return v; }

// DSA_i of every cell slot (sum over the cell's membranes of Dm_i * mem_sa,
// accumulated in FP64), for the factored kernels; zero until Dm is set.
int upload_fact_dsa(bx_cluster* h) {
  if (!h->f_dsa) return BX_OK;
  const int I = h->I, S = h->S;
  std::vector<double> acc((size_t)I * S, 0.0);
  if (!h->h_Dm.empty())
    for (int m = 0; m < h->M; ++m) {
      const int sl = h->h_slot_of_cell[h->h_m2c[m]];
      for (int i = 0; i < I; ++i) acc[(size_t)i * S + sl] += h->h_Dm[(size_t)i * h->M + m] * h->h_msa[m];
    }
  std::vector<float> f(acc.size());
  for (size_t q = 0; q < acc.size(); ++q) f[q] = (float)acc[q];
  BX_CU(h2d(h->f_dsa, f.data(), f.size()));
  return BX_OK;
}

// {sum mem_sa, dt/cell_vol, diviterm/cm, gap-junction count} of every cell slot
// (the parameters dt and cm enter here)
int upload_fact_cst(bx_cluster* h) {
  if (!h->f_cst) return BX_OK;
  std::vector<float4> cst(h->S);
  for (int sl = 0; sl < h->S; ++sl) cst[sl] = make_float4(0.f, 0.f, 0.f, bits_to_float(-1));
  for (int c = 0; c < h->C; ++c) {
    const int sl = h->h_slot_of_cell[c];
    cst[sl] = make_float4(h->h_fsa[sl], (float)(h->par.dt / h->h_vol[c]), (float)(h->h_div[c] / h->par.cm),
                          bits_to_float(h->h_gcnt[sl]));
  }
  BX_CU(h2d(h->f_cst, cst.data(), cst.size()));
  return BX_OK;
}

// The factored form's gap-junction lists: per cell slot, the cell's
// membranes that have a partner and a nonzero weight (BETSE zeroes the flux
// of boundary membranes, sim.py:2203), in membrane order, each as the
// partner's cell slot and gj_weight * mem_sa.
int build_fact_layout(bx_cluster* h) {
  const int S = h->S;
  const std::vector<int>& ptr = h->h_cell_ptr;
  h->h_fsa.assign(S, 0.f);
  h->h_gbeg.assign(S, 0);
  h->h_gcnt.assign(S, -1);
  h->h_gj.clear();
  std::vector<int> cell_of_slot(S, -1);
  for (int c = 0; c < h->C; ++c) cell_of_slot[h->h_slot_of_cell[c]] = c;
  for (int sl = 0; sl < S; ++sl) {
    h->h_gbeg[sl] = (int)h->h_gj.size();
    const int c = cell_of_slot[sl];
    if (c < 0) continue;
    double sa = 0.0;
    for (int m = ptr[c]; m < ptr[c + 1]; ++m) {
      sa += h->h_msa[m];
      if (h->h_bflag[m] || h->h_gjw[m] == 0.0) continue;
      const int ps = h->h_slot_of_cell[h->h_m2c[h->h_nn[m]]];
      h->h_gj.push_back(make_int2(ps, float_to_bits((float)(h->h_gjw[m] * h->h_msa[m]))));
    }
    h->h_fsa[sl] = (float)sa;
    h->h_gcnt[sl] = (int)h->h_gj.size() - h->h_gbeg[sl];
  }
  h->f_P = (int)h->h_gj.size();
  void* old[] = {h->f_dsa, h->f_cst, h->f_gbeg, h->f_gj, h->f_tile_e0};
  for (void* q : old)
    if (q) cudaFree(q);
  h->f_dsa = nullptr; h->f_cst = nullptr; h->f_gbeg = nullptr; h->f_gj = nullptr; h->f_tile_e0 = nullptr;
  drop_resident(h);
  // each tile's entries: contiguous, from the first slot's first entry
  std::vector<int> te(h->nblk + 1);
  h->f_max_ent = 0;
  for (int b = 0; b < h->nblk; ++b) te[b] = h->h_gbeg[32 * b];
  te[h->nblk] = h->f_P;
  for (int b = 0; b < h->nblk; ++b) h->f_max_ent = std::max(h->f_max_ent, te[b + 1] - te[b]);
  BX_CU(dalloc(&h->f_dsa, (size_t)h->I * S));
  BX_CU(dalloc(&h->f_cst, S));
  BX_CU(dalloc(&h->f_gbeg, S)); BX_CU(h2d(h->f_gbeg, h->h_gbeg.data(), S));
  BX_CU(dalloc(&h->f_tile_e0, h->nblk + 1)); BX_CU(h2d(h->f_tile_e0, te.data(), h->nblk + 1));
  BX_CU(dalloc(&h->f_gj, h->f_P + 2));
  BX_CU(cudaMemset(h->f_gj, 0, (size_t)(h->f_P + 2) * sizeof(int2)));
  if (h->f_P) BX_CU(h2d(h->f_gj, h->h_gj.data(), h->f_P));
  int rc = upload_fact_dsa(h);
  if (rc != BX_OK) return rc;
  return upload_fact_cst(h);
}

// Tile-major slot layout of the split form for the partition `blk`: tile b
// owns membrane slots [b*tpb, (b+1)*tpb) and cell slots [32b, 32b+32).
// Geometry and Dm are re-laid out; the state buffers are reallocated and
// must be uploaded again.
int build_split_layout(bx_cluster* h, const std::vector<int>& blk) {
  const int nblk = h->nblk, tpb = h->tpb, C = h->C, M = h->M, I = h->I;
  const int Q = tpb * nblk, S = bx::kCellsPerCta * nblk;
  const std::vector<int>& ptr = h->h_cell_ptr;
  std::vector<uint8_t> lcell(Q, 255);
  std::vector<int> nn_slot(Q), map_env(Q, 0), nn_env(Q, 0), t_c0(nblk), t_m0(nblk);
  std::vector<float> sa(Q, 0.f), gw(Q, 0.f);
  std::vector<short2> rng(S, make_short2(0, 0));
  h->h_slot_of_cell.assign(C, 0);
  h->h_slot_of_mem.assign(M, 0);
  for (int b = 0; b < nblk; ++b) {
    const int c0 = blk[b], c1 = blk[b + 1], m0 = ptr[c0];
    t_c0[b] = c0;
    t_m0[b] = m0;
    for (int qq = tpb * b; qq < tpb * (b + 1); ++qq) nn_slot[qq] = bx::kCellsPerCta * b;
    for (int c = c0; c < c1; ++c) {
      const int s = bx::kCellsPerCta * b + (c - c0);
      h->h_slot_of_cell[c] = s;
      rng[s] = make_short2((short)(ptr[c] - m0), (short)(ptr[c + 1] - m0));
      for (int m = ptr[c]; m < ptr[c + 1]; ++m) {
        const int qq = tpb * b + (m - m0);
        h->h_slot_of_mem[m] = qq;
        lcell[qq] = (uint8_t)(c - c0);
        sa[qq] = (float)h->h_msa[m];
        gw[qq] = h->h_bflag[m] ? 0.f : (float)h->h_gjw[m];
        map_env[qq] = h->h_map_env[m];
      }
    }
  }
  for (int m = 0; m < M; ++m) {
    const int qq = h->h_slot_of_mem[m];
    nn_slot[qq] = h->h_slot_of_cell[h->h_m2c[h->h_nn[m]]];
    nn_env[qq] = h->h_map_env[h->h_nn[m]];
  }
  void* old[] = {h->t_lcell, h->t_nn, h->t_map_env, h->t_nn_env, h->t_c0, h->t_m0, h->t_slot_of_cell,
                 h->t_sa, h->t_gw, h->t_dtv, h->t_dvc, h->t_rng, h->d_Dm_f, h->s_cc2, h->s_rec[0], h->s_rec[1],
                 h->t_gjo, h->t_slot_of_mem};
  for (void* q : old)
    if (q) cudaFree(q);
  h->t_lcell = nullptr; h->t_nn = h->t_map_env = h->t_nn_env = h->t_c0 = h->t_m0 = h->t_slot_of_cell = nullptr;
  h->t_sa = h->t_gw = h->t_dtv = h->t_dvc = nullptr; h->t_rng = nullptr; h->d_Dm_f = nullptr;
  h->s_cc2 = nullptr; h->s_rec[0] = h->s_rec[1] = nullptr;
  h->t_gjo = nullptr;
  h->t_slot_of_mem = nullptr;
  h->Q = Q;
  if (h->vgj) {
    BX_CU(dalloc(&h->t_gjo, Q));
    BX_CU(cudaMemset(h->t_gjo, 0, (size_t)Q * sizeof(float)));
  }
  h->S = S;
  BX_CU(dalloc(&h->t_lcell, Q)); BX_CU(h2d(h->t_lcell, lcell.data(), Q));
  BX_CU(dalloc(&h->t_nn, Q)); BX_CU(h2d(h->t_nn, nn_slot.data(), Q));
  BX_CU(dalloc(&h->t_map_env, Q)); BX_CU(h2d(h->t_map_env, map_env.data(), Q));
  BX_CU(dalloc(&h->t_nn_env, Q)); BX_CU(h2d(h->t_nn_env, nn_env.data(), Q));
  BX_CU(dalloc(&h->t_c0, nblk)); BX_CU(h2d(h->t_c0, t_c0.data(), nblk));
  BX_CU(dalloc(&h->t_m0, nblk)); BX_CU(h2d(h->t_m0, t_m0.data(), nblk));
  BX_CU(dalloc(&h->t_slot_of_cell, C)); BX_CU(h2d(h->t_slot_of_cell, h->h_slot_of_cell.data(), C));
  BX_CU(dalloc(&h->t_slot_of_mem, M)); BX_CU(h2d(h->t_slot_of_mem, h->h_slot_of_mem.data(), M));
  BX_CU(dalloc(&h->t_sa, Q)); BX_CU(h2d(h->t_sa, sa.data(), Q));
  BX_CU(dalloc(&h->t_gw, Q)); BX_CU(h2d(h->t_gw, gw.data(), Q));
  BX_CU(dalloc(&h->t_rng, S)); BX_CU(h2d(h->t_rng, rng.data(), S));
  BX_CU(dalloc(&h->t_dtv, S)); BX_CU(dalloc(&h->t_dvc, S));
  BX_CU(dalloc(&h->d_Dm_f, (size_t)I * Q));
  BX_CU(cudaMemset(h->d_Dm_f, 0, (size_t)I * Q * sizeof(float)));
  if (!h->h_Dm.empty()) {
    std::vector<float> f((size_t)I * Q, 0.f);
    for (int i = 0; i < I; ++i)
      for (int m = 0; m < M; ++m) f[(size_t)i * Q + h->h_slot_of_mem[m]] = (float)h->h_Dm[(size_t)i * M + m];
    BX_CU(h2d(h->d_Dm_f, f.data(), f.size()));
  }
  BX_CU(dalloc(&h->s_cc2, (size_t)I * S));
  BX_CU(cudaMemset(h->s_cc2, 0, (size_t)I * S * sizeof(float2)));
  BX_CU(dalloc(&h->s_rec[0], (size_t)kRec * S));
  BX_CU(dalloc(&h->s_rec[1], (size_t)kRec * S));
  BX_CU(cudaMemset(h->s_rec[0], 0, (size_t)kRec * S * sizeof(float)));
  BX_CU(cudaMemset(h->s_rec[1], 0, (size_t)kRec * S * sizeof(float)));
  BX_CU(build_geo_blob(h));
  BX_CU(cudaStreamSynchronize(h->stream));
  h->have_state = false;
  int rc = build_fact_layout(h);
  if (rc != BX_OK) return rc;
  return upload_param_arrays(h);
}

// CTA partition for `tpb` membrane slots: runs of whole cells of one cluster
// with at most tpb membranes; the split form also caps a tile at 32 cells
// (its (ion, cell) phase maps ion -> warp, cell -> lane).  Rebuilt by the
// autotuner.
int build_partition(bx_cluster* h, int tpb) {
  const std::vector<int>& ptr = h->h_cell_ptr;
  if (h->mode == MODE_SPLIT && h->I > tpb / 32) return fail(BX_EINVAL, "CTA too small for the ion count");
  const int max_cells = (h->mode == MODE_SPLIT) ? bx::kCellsPerCta : tpb;
  std::vector<int> blk{0}, blk_cl;
  std::vector<int> cl_blk(h->ncl + 1, 0);
  for (int cl = 0; cl < h->ncl; ++cl) {
    int acc = 0, nc = 0;
    for (int c = h->cl_cell[cl]; c < h->cl_cell[cl + 1]; ++c) {
      const int n = ptr[c + 1] - ptr[c];
      if (n > tpb) return fail(BX_EINVAL, "a cell has more membranes than a CTA has threads");
      if ((acc + n > tpb || nc + 1 > max_cells) && acc > 0) {
        blk.push_back(c);
        blk_cl.push_back(cl);
        acc = 0;
        nc = 0;
      }
      acc += n;
      ++nc;
    }
    blk.push_back(h->cl_cell[cl + 1]);
    blk_cl.push_back(cl);
    cl_blk[cl + 1] = (int)blk.size() - 1;
  }
  const int nblk = (int)blk.size() - 1;
  BX_CU(cudaStreamSynchronize(h->stream));
  void* old[] = {h->d_blk, h->d_blk_cl, h->d_cl_blk, h->d_lcell, h->s_part, h->d_env_part};
  for (void* q : old)
    if (q) cudaFree(q);
  h->d_blk = h->d_blk_cl = h->d_cl_blk = nullptr;
  h->d_lcell = nullptr;
  h->s_part = nullptr;
  h->d_env_part = nullptr;
  BX_CU(dalloc(&h->d_blk, blk.size()));
  BX_CU(h2d(h->d_blk, blk.data(), blk.size()));
  BX_CU(dalloc(&h->d_blk_cl, blk_cl.size()));
  BX_CU(h2d(h->d_blk_cl, blk_cl.data(), blk_cl.size()));
  BX_CU(dalloc(&h->d_cl_blk, cl_blk.size()));
  BX_CU(h2d(h->d_cl_blk, cl_blk.data(), cl_blk.size()));
  if (h->mode == MODE_SPLIT) {
    BX_CU(dalloc(&h->s_part, (size_t)nblk * h->I));
  } else {
    BX_CU(dalloc(&h->d_env_part, (size_t)nblk * h->I));
  }
  h->cl_blk = cl_blk;
  h->nblk = nblk;
  h->tpb = tpb;
  h->graph_valid = false;
  if (h->mode == MODE_SPLIT) return build_split_layout(h, blk);
  return BX_OK;
}

int create_impl(const bx_geom* gs, const bx_params* ps, int ncl, int precision, bx_handle* out) {
  if (!gs || !ps || !out || ncl <= 0) return fail(BX_EINVAL, "null argument");
  *out = nullptr;
  if (precision != BX_PLAIN_FP64 && precision != BX_SPLIT_FP32)
    return fail(BX_EINVAL, "precision must be BX_PLAIN_FP64 or BX_SPLIT_FP32");
  const bx_params& p0 = ps[0];
  const int I = p0.n_ions;
  if (I <= 0 || I > BX_MAX_IONS) return fail(BX_EINVAL, "n_ions must be in [1, 8]");
  if (p0.iNa < 0 || p0.iNa >= I || p0.iK < 0 || p0.iK >= I || p0.iNa == p0.iK)
    return fail(BX_EINVAL, "iNa/iK out of range");
  if (p0.iCa < -1 || p0.iCa >= I) return fail(BX_EINVAL, "iCa must be -1 or an ion row");
  if (p0.cell_polarizability != 0.0) {
    if (precision != BX_PLAIN_FP64)
      return fail(BX_EINVAL, "cell polarizability makes Vmem per-membrane state: the split form keeps one "
                             "Vmem per cell, use BX_PLAIN_FP64");
    for (int c = 0; c < ncl; ++c) {
      if (!gs[c].R_rads) return fail(BX_EINVAL, "cell polarizability needs bx_geom.R_rads");
      for (int m = 0; m < gs[c].n_mems; ++m)
        if (!(gs[c].R_rads[m] > 0.0)) return fail(BX_EINVAL, "R_rads must be positive");
    }
  }
  if (ncl > 1 && p0.is_ecm) return fail(BX_EINVAL, "batches of clusters need is_ecm == 0");
  long long Ctot = 0, Mtot = 0;
  for (int c = 0; c < ncl; ++c) {
    int rc = check_geom(&gs[c], &ps[c]);
    if (rc != BX_OK) return rc;
    if (!same_shared_params(p0, ps[c]))
      return fail(BX_EINVAL, "clusters of a batch may differ only in alpha_NaK, nakatp_block, vol_env");
    if (gs[c].gj_len != gs[0].gj_len) return fail(BX_EINVAL, "clusters of a batch need one gj_len");
    Ctot += gs[c].n_cells;
    Mtot += gs[c].n_mems;
  }
  if (Mtot > 0x7fffffffLL / 8) return fail(BX_EINVAL, "batch too large for int32 indexing");
  const int C = (int)Ctot, M = (int)Mtot;

  bx_cluster* h = new (std::nothrow) bx_cluster();
  if (!h) return fail(BX_ENOMEM, "host allocation failed");
  auto bail = [&](int code, const std::string& msg) {
    free_all(h);
    delete h;
    return fail(code, msg);
  };
  h->ncl = ncl; h->C = C; h->M = M; h->I = I;
  h->ny = gs[0].grid_ny; h->nx = gs[0].grid_nx; h->G = h->ny * h->nx;
  for (int cl = 0; cl < ncl; ++cl) {
    h->cl_ny.push_back(gs[cl].grid_ny);
    h->cl_nx.push_back(gs[cl].grid_nx);
    h->cl_delta.push_back(gs[cl].delta);
  }
  h->precision = precision; h->par = p0; h->ecm = p0.is_ecm != 0; h->vgj = p0.v_sensitive_gj != 0;
  h->ca = ca_pump_on(p0);
  h->polar = p0.cell_polarizability != 0.0;
  h->cl_par.assign(ps, ps + ncl);
  h->mode = (precision == BX_PLAIN_FP64) ? MODE_PLAIN : MODE_SPLIT;
  if (h->mode == MODE_SPLIT && I > kRec - 1) {
    delete h;
    return fail(BX_EINVAL, "the split form holds at most 7 ions (BETSE's full ion set)");
  }
  h->gj_len = gs[0].gj_len; h->delta = gs[0].delta;
  const int G = h->G;

  // ---- concatenate the clusters
  std::vector<int> ptr(C + 1), nn(M), m2c(M), nn_cell(M), map_env(M);
  std::vector<uint8_t> bflag(M);
  std::vector<double> msa(M), mnx(M), mny(M), gjw(M), swm(M), swo(M), vol(C), csa(C), div(C),
      rr(h->polar ? M : 0);
  h->cl_cell.assign(ncl + 1, 0); h->cl_mem.assign(ncl + 1, 0);
  int coff = 0, moff = 0;
  ptr[0] = 0;
  for (int cl = 0; cl < ncl; ++cl) {
    const bx_geom& g = gs[cl];
    for (int c = 0; c < g.n_cells; ++c) {
      ptr[coff + c + 1] = moff + g.cell_mem_ptr[c + 1];
      vol[coff + c] = g.cell_vol[c]; csa[coff + c] = g.cell_sa[c]; div[coff + c] = g.diviterm[c];
      for (int m = g.cell_mem_ptr[c]; m < g.cell_mem_ptr[c + 1]; ++m) m2c[moff + m] = coff + c;
    }
    for (int m = 0; m < g.n_mems; ++m) {
      nn[moff + m] = moff + g.nn_i[m];
      bflag[moff + m] = g.bflag[m] ? 1 : 0;
      map_env[moff + m] = g.map_mem2ecm[m];
      msa[moff + m] = g.mem_sa[m]; mnx[moff + m] = g.mem_nx[m]; mny[moff + m] = g.mem_ny[m];
      gjw[moff + m] = g.gj_weight[m]; swm[moff + m] = g.smooth_weight_mem[m]; swo[moff + m] = g.smooth_weight_o[m];
      if (h->polar) rr[moff + m] = g.R_rads[m];
    }
    coff += g.n_cells;
    moff += g.n_mems;
    h->cl_cell[cl + 1] = coff;
    h->cl_mem[cl + 1] = moff;
  }
  for (int m = 0; m < M; ++m) nn_cell[m] = m2c[nn[m]];
  h->h_cell_ptr = ptr; h->h_m2c = m2c; h->h_map_env = map_env;
  h->h_phib.assign(G, 0.0);
  h->h_gjw = gjw;

  // environment CSR (grid cell -> its membranes, ascending) for the ECM scatter
  std::vector<int> env_ptr(G + 1, 0), env_mem(M);
  std::vector<uint8_t> touched(G, 0);
  if (h->ecm) {
    for (int m = 0; m < M; ++m) env_ptr[map_env[m] + 1]++;
    for (int k = 0; k < G; ++k) env_ptr[k + 1] += env_ptr[k];
    std::vector<int> fill(env_ptr.begin(), env_ptr.end() - 1);
    for (int m = 0; m < M; ++m) env_mem[fill[map_env[m]]++] = m;
    for (int k = 0; k < G; ++k) touched[k] = env_ptr[k + 1] > env_ptr[k];
    double s = 0.0;
    for (int m = 0; m < M; ++m) s += gs[0].mem_sa_per_env[map_env[m]];
    h->env_surf_scale = (p0.cell_height * h->delta * h->delta) / (s / (double)M);
  }

  if (cudaGetDevice(&h->dev) != cudaSuccess) return bail(BX_ECUDA, "no CUDA device");
  if (cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, h->dev) != cudaSuccess)
    return bail(BX_ECUDA, "cudaDeviceGetAttribute");
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(BX_ECUDA, "cudaStreamCreate failed");

#define ALLOC(ptr, n) \
  if (dalloc(&(ptr), (size_t)(n)) != cudaSuccess) return bail(BX_ENOMEM, "cudaMalloc " #ptr)
#define H2D(dst, src, n) \
  if (h2d((dst), (src), (size_t)(n)) != cudaSuccess) return bail(BX_ECUDA, "copy " #dst)
  ALLOC(h->d_cell_ptr, C + 1); H2D(h->d_cell_ptr, ptr.data(), C + 1);
  ALLOC(h->d_m2c, M); H2D(h->d_m2c, m2c.data(), M);
  ALLOC(h->d_nn, M); H2D(h->d_nn, nn.data(), M);
  ALLOC(h->d_nn_cell, M); H2D(h->d_nn_cell, nn_cell.data(), M);
  ALLOC(h->d_map_env, M); H2D(h->d_map_env, map_env.data(), M);
  ALLOC(h->d_bflag, M); H2D(h->d_bflag, bflag.data(), M);
  ALLOC(h->d_mem_sa, M); H2D(h->d_mem_sa, msa.data(), M);
  ALLOC(h->d_gj_w, M); H2D(h->d_gj_w, gjw.data(), M);
  ALLOC(h->d_nx, M); H2D(h->d_nx, mnx.data(), M);
  ALLOC(h->d_ny, M); H2D(h->d_ny, mny.data(), M);
  ALLOC(h->d_swm, M); H2D(h->d_swm, swm.data(), M);
  ALLOC(h->d_swo, M); H2D(h->d_swo, swo.data(), M);
  ALLOC(h->d_cell_vol, C); H2D(h->d_cell_vol, vol.data(), C);
  ALLOC(h->d_cell_sa, C); H2D(h->d_cell_sa, csa.data(), C);
  ALLOC(h->d_diviterm, C); H2D(h->d_diviterm, div.data(), C);
  if (h->polar) { ALLOC(h->d_Rrads, M); H2D(h->d_Rrads, rr.data(), M); }
  ALLOC(h->d_pump, ncl); ALLOC(h->d_env_scale, ncl);
  ALLOC(h->d_phib, G);
  ALLOC(h->d_status, 4);
  ALLOC(h->d_env_ticket, ncl);
  if (cudaMemset(h->d_status, 0, 4 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMemset(h->d_env_ticket, 0, (size_t)ncl * sizeof(unsigned)) != cudaSuccess ||
      cudaMemset(h->d_phib, 0, (size_t)G * sizeof(double)) != cudaSuccess)
    return bail(BX_ECUDA, "cudaMemset");
  if (h->mode == MODE_SPLIT) {
    // host copies for the tile-major relayout (build_split_layout)
    h->h_msa = msa; h->h_bflag = bflag; h->h_nn = nn; h->h_vol = vol; h->h_div = div;
    ALLOC(h->s_cenv_f, (size_t)ncl * I); ALLOC(h->d_cenv, h->ecm ? (size_t)I * G : (size_t)ncl * I);
    ALLOC(h->s_pump, ncl);
    ALLOC(h->s_phib, G);
    if (cudaMemset(h->s_phib, 0, (size_t)G * sizeof(float)) != cudaSuccess) return bail(BX_ECUDA, "cudaMemset");
    ALLOC(h->o_vmc, C); ALLOC(h->o_vm_mem, M); ALLOC(h->o_drho, C);
  } else {
    ALLOC(h->d_Dm, (size_t)I * M);
    ALLOC(h->d_vm[0], M); ALLOC(h->d_vm[1], M);
    ALLOC(h->d_ccm[0], (size_t)I * C); ALLOC(h->d_ccm[1], (size_t)I * C);
    ALLOC(h->d_cc, (size_t)I * C);
    ALLOC(h->d_cenv, h->ecm ? (size_t)I * G : (size_t)ncl * I);
    if (h->vgj) ALLOC(h->d_gjo, M);
  }
  if (h->ecm) {
    ALLOC(h->d_env_ptr, G + 1); H2D(h->d_env_ptr, env_ptr.data(), G + 1);
    ALLOC(h->d_env_mem, M); H2D(h->d_env_mem, env_mem.data(), M);
    ALLOC(h->d_touched, G); H2D(h->d_touched, touched.data(), G);
    ALLOC(h->d_mem_flux_sa, (size_t)I * M);
    ALLOC(h->d_Denv, (size_t)I * G);
    ALLOC(h->d_Ex, G); ALLOC(h->d_Ey, G);
    ALLOC(h->d_fx, (size_t)I * G); ALLOC(h->d_fy, (size_t)I * G);
    ALLOC(h->d_tmp, G); ALLOC(h->d_tmp2, (size_t)I * G);
    ALLOC(h->d_venv, G); ALLOC(h->d_rho_env, G); ALLOC(h->d_vsrc, G);
    if (h->ca) ALLOC(h->d_cnew, (size_t)I * G);
  }
  ALLOC(h->o_fmem, (size_t)I * M); ALLOC(h->o_fgj, (size_t)I * M);
  ALLOC(h->o_rate, M); ALLOC(h->o_rho, C); ALLOC(h->o_Jn, M); ALLOC(h->o_Imem, M);
  ALLOC(h->o_Jcx, C); ALLOC(h->o_Jcy, C); ALLOC(h->o_Jc, M); ALLOC(h->o_vmave, C);
  ALLOC(h->o_dvm, M); ALLOC(h->o_Ecx, C); ALLOC(h->o_Ecy, C); ALLOC(h->o_Emc, M);
  ALLOC(h->o_Egjx, M); ALLOC(h->o_Egjy, M); ALLOC(h->o_gjopen, M); ALLOC(h->o_sigma, C);
#undef ALLOC
#undef H2D
  if (upload_param_arrays(h) != BX_OK || build_partition(h, kTPB) != BX_OK) {
    std::string msg = g_err;
    return bail(BX_ECUDA, msg);
  }
  *out = h;
  return BX_OK;
}

}  // namespace

// shared with the other translation units of the library
void bx_record_error(const char* msg) { g_err = msg; }

extern "C" {

int bx_abi_version(void) { return BX_ABI_VERSION; }
const char* bx_last_error(void) { return g_err.c_str(); }

int bx_cluster_create(const bx_geom* g, const bx_params* p, int precision, bx_handle* out) {
  return create_impl(g, p, 1, precision, out);
}

int bx_batch_create(const bx_geom* g, const bx_params* p, int n_clusters, int precision, bx_handle* out) {
  return create_impl(g, p, n_clusters, precision, out);
}

int bx_batch_layout(bx_handle h, int32_t* cell_offsets, int32_t* mem_offsets) {
  if (!h || !cell_offsets || !mem_offsets) return fail(BX_EINVAL, "null argument");
  for (int c = 0; c <= h->ncl; ++c) {
    cell_offsets[c] = h->cl_cell[c];
    mem_offsets[c] = h->cl_mem[c];
  }
  return BX_OK;
}

void bx_destroy(bx_handle h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_all(h);
  delete h;
}

int bx_set_params(bx_handle h, const bx_params* p) {
  if (!h || !p) return fail(BX_EINVAL, "null argument");
  if (p->n_ions != h->I || (p->is_ecm != 0) != h->ecm || (p->v_sensitive_gj != 0) != h->vgj)
    return fail(BX_EINVAL, "n_ions / is_ecm / v_sensitive_gj cannot change after create");
  if (p->iCa < -1 || p->iCa >= p->n_ions) return fail(BX_EINVAL, "iCa must be -1 or an ion row");
  if (ca_pump_on(*p) != h->ca || (h->ca && p->iCa != h->par.iCa))
    return fail(BX_EINVAL, "the Ca-ATPase cannot be switched on or off, or move row, after create");
  if ((p->cell_polarizability != 0.0) != h->polar)
    return fail(BX_EINVAL, "cell polarizability cannot be switched on or off after create");
  if (h->ncl > 1) return fail(BX_EINVAL, "use bx_batch_set_params for a batch");
  h->par = *p;
  h->cl_par[0] = *p;
  h->graph_valid = false;
  return upload_param_arrays(h);
}

int bx_batch_set_params(bx_handle h, const bx_params* p) {
  if (!h || !p) return fail(BX_EINVAL, "null argument");
  for (int c = 0; c < h->ncl; ++c)
    if (!same_shared_params(p[0], p[c]) || p[c].n_ions != h->I || (p[c].is_ecm != 0) != h->ecm)
      return fail(BX_EINVAL, "clusters of a batch may differ only in alpha_NaK, nakatp_block, vol_env");
  if ((p[0].v_sensitive_gj != 0) != h->vgj || ca_pump_on(p[0]) != h->ca || (h->ca && p[0].iCa != h->par.iCa) ||
      (p[0].cell_polarizability != 0.0) != h->polar)
    return fail(BX_EINVAL, "v_sensitive_gj, the Ca-ATPase and cell polarizability cannot change after create");
  h->par = p[0];
  h->cl_par.assign(p, p + h->ncl);
  h->graph_valid = false;
  return upload_param_arrays(h);
}

int bx_set_membrane_diffusivity(bx_handle h, const double* Dm) {
  if (!h || !Dm) return fail(BX_EINVAL, "null argument");
  const size_t n = (size_t)h->I * h->M;
  for (size_t q = 0; q < n; ++q)
    if (!(Dm[q] >= 0.0) || Dm[q] == INFINITY) return fail(BX_EINVAL, "Dm must be finite and >= 0");
  BX_CU(cudaStreamSynchronize(h->stream));
  if (h->mode == MODE_SPLIT) {
    h->h_Dm.assign(Dm, Dm + n);
    std::vector<float> f((size_t)h->I * h->Q, 0.f);
    for (int i = 0; i < h->I; ++i)
      for (int m = 0; m < h->M; ++m) f[(size_t)i * h->Q + h->h_slot_of_mem[m]] = (float)Dm[(size_t)i * h->M + m];
    BX_CU(cudaMemcpy(h->d_Dm_f, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice));
    BX_CU(build_geo_blob(h));
    BX_CU(cudaStreamSynchronize(h->stream));
    const int rc = upload_fact_dsa(h);
    if (rc != BX_OK) return rc;
  } else if (h->d_Dm_f) {
    std::vector<float> f(n);
    for (size_t q = 0; q < n; ++q) f[q] = (float)Dm[q];
    BX_CU(cudaMemcpy(h->d_Dm_f, f.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  } else {
    BX_CU(cudaMemcpy(h->d_Dm, Dm, n * sizeof(double), cudaMemcpyHostToDevice));
  }
  h->have_dm = true;
  return BX_OK;
}

int bx_set_env_diffusivity(bx_handle h, const double* D_env) {
  if (!h || !D_env) return fail(BX_EINVAL, "null argument");
  if (!h->ecm) return fail(BX_EINVAL, "environment diffusivity needs is_ecm");
  BX_CU(cudaStreamSynchronize(h->stream));
  BX_CU(cudaMemcpy(h->d_Denv, D_env, (size_t)h->I * h->G * sizeof(double), cudaMemcpyHostToDevice));
  h->have_denv = true;
  return BX_OK;
}

// FP32 copy of the well-mixed environment, rounded to nearest on the device
__global__ void k_round_to_float(const double* __restrict__ a, float* __restrict__ b, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = __double2float_rn(a[i]);
}

// Device staging for state transfers: the caller's arrays in BETSE's layouts
// (allocated at the first transfer).
int ensure_state_staging(bx_cluster* h) {
  if (h->st_cam) return BX_OK;
  const size_t M = h->M, C = h->C, I = h->I;
  if (dalloc(&h->st_vm, M) != cudaSuccess || dalloc(&h->st_cc, I * C) != cudaSuccess ||
      dalloc(&h->st_go, M) != cudaSuccess || dalloc(&h->d_flag, 2) != cudaSuccess ||
      dalloc(&h->st_cam, I * M) != cudaSuccess) {
    cudaGetLastError();
    return fail(BX_ENOMEM, "cudaMalloc state staging");
  }
  return BX_OK;
}

bx::StateIO state_io(const bx_cluster* h) {
  bx::StateIO io{};
  io.C = h->C; io.M = h->M; io.I = h->I; io.S = h->S; io.rec = kRec;
  io.cell_ptr = h->d_cell_ptr; io.m2c = h->d_m2c; io.map_env = h->d_map_env;
  io.phib = h->d_phib; io.phib_on = h->phib_nonzero ? 1 : 0;
  io.slot_of_cell = h->t_slot_of_cell; io.slot_of_mem = h->t_slot_of_mem;
  return io;
}

// Phi_b at membrane m's grid cell.  A boundary potential needs a single
// cluster (bx_set_boundary_potential), and a batch's membranes index their own
// clusters' grids, which h_phib (sized by the first cluster's grid) does not
// cover: without a potential the value is zero and h_phib is not read.
double phib_at(const bx_cluster* h, int m) {
  return h->phib_nonzero ? h->h_phib[h->h_map_env[m]] : 0.0;
}

int bx_set_boundary_potential(bx_handle h, const double* Phi_b) {
  if (!h) return fail(BX_EINVAL, "null handle");
  bool nz = false;
  if (Phi_b)
    for (int k = 0; k < h->G; ++k) nz |= (Phi_b[k] != 0.0);
  if (nz && h->ncl > 1) return fail(BX_EINVAL, "a boundary potential needs a single cluster");
  BX_CU(cudaStreamSynchronize(h->stream));
  for (int k = 0; k < h->G; ++k) h->h_phib[k] = nz ? Phi_b[k] : 0.0;
  BX_CU(cudaMemcpy(h->d_phib, h->h_phib.data(), (size_t)h->G * sizeof(double), cudaMemcpyHostToDevice));
  if (h->s_phib) {
    std::vector<float> f(h->G);
    for (int k = 0; k < h->G; ++k) f[k] = (float)h->h_phib[k];
    BX_CU(cudaMemcpy(h->s_phib, f.data(), (size_t)h->G * sizeof(float), cudaMemcpyHostToDevice));
  }
  if (nz != h->phib_nonzero) h->graph_valid = false;
  h->phib_nonzero = nz;
  return BX_OK;
}

int bx_state_upload(bx_handle h, const bx_state* s) {
  if (!h || !s || !s->vm || !s->cc_cells || !s->cc_at_mem || !s->cc_env)
    return fail(BX_EINVAL, "null argument");
  const int C = h->C, M = h->M, I = h->I;
  if (h->ecm && (!s->E_env_x || !s->E_env_y)) return fail(BX_EINVAL, "ECM state needs E_env_x/E_env_y");
  BX_CU(cudaStreamSynchronize(h->stream));
  int rc = ensure_state_staging(h);
  if (rc != BX_OK) return rc;
  cudaStream_t st = h->stream;
  const bx::StateIO io = state_io(h);
  const bool split = h->mode == MODE_SPLIT;
  const size_t nenv = h->ecm ? (size_t)I * h->G : (size_t)h->ncl * I;
  // the caller's arrays cross as they are; the checks and the re-layout run
  // on the device.  A failed check leaves the handle without a state.
  h->have_state = false;
  double* vm_dst = split ? h->st_vm : h->d_vm[0];
  double* cc_dst = split ? h->st_cc : h->d_cc;
  BX_CU(cudaMemcpyAsync(vm_dst, s->vm, (size_t)M * sizeof(double), cudaMemcpyDefault, st));
  BX_CU(cudaMemcpyAsync(cc_dst, s->cc_cells, (size_t)I * C * sizeof(double), cudaMemcpyDefault, st));
  BX_CU(cudaMemcpyAsync(h->st_cam, s->cc_at_mem, (size_t)I * M * sizeof(double), cudaMemcpyDefault, st));
  BX_CU(cudaMemsetAsync(h->d_flag, 0, 2 * sizeof(int), st));
  const int tb = 256;
  bx::k_state_check<<<(M + tb - 1) / tb, tb, 0, st>>>(io, vm_dst, h->st_cam, split ? 1 : 0, h->d_flag);
  BX_CU(cudaGetLastError());
  int flag[2] = {0, 0};
  BX_CU(cudaMemcpyAsync(flag, h->d_flag, sizeof(flag), cudaMemcpyDeviceToHost, st));
  BX_CU(cudaStreamSynchronize(st));
  if (flag[0]) return fail(BX_EINVAL, "cc_at_mem must be constant over each cell's membranes");
  // Vmem is constant per cell (minus Phi_b per membrane) in BETSE's full
  // solver with cell_polarizability == 0 (sim.py:2027-2029)
  if (flag[1]) return fail(BX_EINVAL, "split form: vm must be uniform over each cell's membranes");
  h->parity = 0;
  if (split) {
    BX_CU(cudaMemsetAsync(h->s_rec[0], 0, (size_t)kRec * h->S * sizeof(float), st));
    BX_CU(cudaMemsetAsync(h->s_cc2, 0, (size_t)I * h->S * sizeof(float2), st));
    bx::k_state_pack_split<<<(C + tb - 1) / tb, tb, 0, st>>>(io, h->st_vm, h->st_cc, h->st_cam, h->s_rec[0],
                                                            h->s_cc2);
    BX_CU(cudaGetLastError());
    if (h->vgj) {
      if (s->gjopen)
        BX_CU(cudaMemcpyAsync(h->st_go, s->gjopen, (size_t)M * sizeof(double), cudaMemcpyDefault, st));
      else
        BX_CU(cudaMemcpyAsync(h->st_go, h->d_gj_w, (size_t)M * sizeof(double), cudaMemcpyDeviceToDevice, st));
      BX_CU(cudaMemsetAsync(h->t_gjo, 0, (size_t)h->Q * sizeof(float), st));
      bx::k_state_pack_gjo<<<(M + tb - 1) / tb, tb, 0, st>>>(io, h->st_go, h->t_gjo);
      BX_CU(cudaGetLastError());
    }
    BX_CU(cudaMemcpyAsync(h->d_cenv, s->cc_env, nenv * sizeof(double), cudaMemcpyDefault, st));
    if (h->ecm) {
      BX_CU(cudaMemcpyAsync(h->d_Ex, s->E_env_x, (size_t)h->G * sizeof(double), cudaMemcpyDefault, st));
      BX_CU(cudaMemcpyAsync(h->d_Ey, s->E_env_y, (size_t)h->G * sizeof(double), cudaMemcpyDefault, st));
    } else {
      k_round_to_float<<<(unsigned)((nenv + 255) / 256), 256, 0, st>>>(h->d_cenv, h->s_cenv_f, (int)nenv);
      BX_CU(cudaGetLastError());
    }
  } else {
    bx::k_state_pack_ccm<<<(C + tb - 1) / tb, tb, 0, st>>>(io, h->st_cam, h->d_ccm[0]);
    BX_CU(cudaGetLastError());
    BX_CU(cudaMemcpyAsync(h->d_cenv, s->cc_env, nenv * sizeof(double), cudaMemcpyDefault, st));
    if (h->vgj) {
      if (s->gjopen)
        BX_CU(cudaMemcpyAsync(h->d_gjo, s->gjopen, (size_t)M * sizeof(double), cudaMemcpyDefault, st));
      else
        BX_CU(cudaMemcpyAsync(h->d_gjo, h->d_gj_w, (size_t)M * sizeof(double), cudaMemcpyDeviceToDevice, st));
    }
    if (h->ecm) {
      BX_CU(cudaMemcpyAsync(h->d_Ex, s->E_env_x, (size_t)h->G * sizeof(double), cudaMemcpyDefault, st));
      BX_CU(cudaMemcpyAsync(h->d_Ey, s->E_env_y, (size_t)h->G * sizeof(double), cudaMemcpyDefault, st));
    }
  }
  if (h->r_ctl) BX_CU(cudaMemsetAsync(h->r_ctl, 0, 2 * sizeof(unsigned), st));   // a fresh state: no timeout
  BX_CU(cudaStreamSynchronize(st));
  h->have_state = true;
  h->have_outputs = false;
  h->last_step_outputs = false;
  return BX_OK;
}

int bx_state_download(bx_handle h, bx_state* s) {
  if (!h || !s) return fail(BX_EINVAL, "null argument");
  if (!h->have_state) return fail(BX_ESTATE, "no state uploaded");
  const int C = h->C, M = h->M, I = h->I;
  BX_CU(cudaStreamSynchronize(h->stream));
  int rc = ensure_state_staging(h);
  if (rc != BX_OK) return rc;
  cudaStream_t st = h->stream;
  const bx::StateIO io = state_io(h);
  const size_t nenv = h->ecm ? (size_t)I * h->G : (size_t)h->ncl * I;
  const int tb = 256;
  auto d2h = [&](double* dst, const double* src, size_t n) {
    return dst ? cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDefault, st) : cudaSuccess;
  };
  if (h->mode == MODE_SPLIT) {
    const int n = std::max(M, C);
    const bool go = h->vgj && s->gjopen;
    bx::k_state_unpack_split<<<(n + tb - 1) / tb, tb, 0, st>>>(io, h->s_rec[h->parity], h->s_cc2,
                                                              go ? h->t_gjo : nullptr, h->st_vm, h->st_cam,
                                                              h->st_cc, h->st_go);
    BX_CU(cudaGetLastError());
    BX_CU(d2h(s->vm, h->st_vm, M));
    BX_CU(d2h(s->cc_cells, h->st_cc, (size_t)I * C));
    if (go) BX_CU(d2h(s->gjopen, h->st_go, M));
  } else {
    bx::k_state_unpack_cam<<<(M + tb - 1) / tb, tb, 0, st>>>(io, h->d_ccm[h->parity], h->st_cam);
    BX_CU(cudaGetLastError());
    BX_CU(d2h(s->vm, h->d_vm[h->parity], M));
    BX_CU(d2h(s->cc_cells, h->d_cc, (size_t)I * C));
    if (h->vgj) BX_CU(d2h(s->gjopen, h->d_gjo, M));
  }
  BX_CU(d2h(s->cc_at_mem, h->st_cam, (size_t)I * M));
  if (h->ecm) {
    BX_CU(d2h(s->E_env_x, h->d_Ex, h->G));
    BX_CU(d2h(s->E_env_y, h->d_Ey, h->G));
  }
  BX_CU(d2h(s->cc_env, h->d_cenv, nenv));
  BX_CU(cudaStreamSynchronize(st));
  return BX_OK;
}

int bx_step(bx_handle h, int n_steps, int want_outputs, void* stream) {
  if (!h) return fail(BX_EINVAL, "null handle");
  if (n_steps < 0) return fail(BX_EINVAL, "n_steps must be >= 0");
  if (!h->have_state) return fail(BX_ESTATE, "bx_step before bx_state_upload");
  if (!h->have_dm) return fail(BX_ESTATE, "bx_step before bx_set_membrane_diffusivity");
  if (h->ecm && !h->have_denv) return fail(BX_ESTATE, "ECM step before bx_set_env_diffusivity");
  if (n_steps == 0) return BX_OK;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : h->stream;
  // the cross-stream event, destroyed on every return path
  struct EventGuard {
    cudaEvent_t ev = nullptr;
    ~EventGuard() { if (ev) cudaEventDestroy(ev); }
  } guard;
  if (s != h->stream) {
    // the caller's stream runs after the handle's pending work
    BX_CU(cudaEventCreateWithFlags(&guard.ev, cudaEventDisableTiming));
    BX_CU(cudaEventRecord(guard.ev, h->stream));
    BX_CU(cudaStreamWaitEvent(s, guard.ev, 0));
  }
  int left = n_steps;
  const int tail_out = want_outputs ? 1 : 0;
  if (h->kind == KIND_RESIDENT && fact_eligible(h, false) && left - tail_out >= 2) {
    if (h->r_state == 0) {
      const int rc = build_resident(h);
      if (rc != BX_OK) return rc;
    }
    if (h->r_state == 1) {
      // one cooperative launch per at most 2^20 steps (the barrier counter is 32-bit)
      while (left - tail_out > 0) {
        const int n = std::min(left - tail_out, 1 << 20);
        cudaError_t e = launch_resident(h, h->parity, n, s);
        if (e != cudaSuccess) return fail(BX_ECUDA, std::string("resident step launch: ") + cudaGetErrorString(e));
        h->launches += 1;
        h->parity ^= (n & 1);
        left -= n;
      }
    }
  }
  if (left - tail_out >= kGraphChunk) {
    if (h->parity != 0) {
      cudaError_t e = enqueue_step(h, h->parity, false, s);
      if (e != cudaSuccess) return fail(BX_ECUDA, std::string("step launch: ") + cudaGetErrorString(e));
      h->parity ^= 1;
      --left;
    }
    if (!h->graph_valid) {
      if (h->graph) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
      }
      cudaStream_t cs;
      BX_CU(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      cudaGraph_t graph;
      const int64_t l0 = h->launches;
      BX_CU(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      int par = 0;
      for (int q = 0; q < kGraphChunk; ++q) {
        enqueue_step(h, par, false, cs);
        par ^= 1;
      }
      cudaError_t ce = cudaStreamEndCapture(cs, &graph);
      cudaStreamDestroy(cs);
      h->launches = l0;  // captured launches are counted when the graph replays
      if (ce != cudaSuccess) return fail(BX_ECUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
      ce = cudaGraphInstantiate(&h->graph, graph, 0);
      cudaGraphDestroy(graph);
      if (ce != cudaSuccess) return fail(BX_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
      h->graph_valid = true;
    }
    while (left - tail_out >= kGraphChunk) {
      BX_CU(cudaGraphLaunch(h->graph, s));
      h->launches += (int64_t)kGraphChunk * launches_per_step(h);
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
  h->last_step_outputs = want_outputs != 0;
  if (s != h->stream) {
    BX_CU(cudaEventRecord(guard.ev, s));
    BX_CU(cudaStreamWaitEvent(h->stream, guard.ev, 0));
  }
  return BX_OK;
}

int bx_status(bx_handle h, bx_step_status* st) {
  if (!h || !st) return fail(BX_EINVAL, "null argument");
  unsigned long long v[4];
  BX_CU(cudaStreamSynchronize(h->stream));
  BX_CU(cudaMemcpy(v, h->d_status, sizeof(v), cudaMemcpyDeviceToHost));
  st->steps_done = h->steps_done;
  st->nan_vm = (int32_t)std::min<unsigned long long>(v[0], 0x7fffffff);
  st->nan_conc = (int32_t)std::min<unsigned long long>(v[1], 0x7fffffff);
  st->neg_clamped = (int64_t)v[2];
  st->unstable = (v[0] || v[1]) ? 1 : 0;
  st->precision = h->precision;
  if (h->r_ctl) {
    // the resident kernel's grid barrier gave up (its wait is bounded): the
    // state of that run is incomplete
    unsigned ctl[2] = {0u, 0u};
    BX_CU(cudaMemcpy(ctl, h->r_ctl, sizeof(ctl), cudaMemcpyDeviceToHost));
    if (ctl[1]) {
      h->have_state = false;
      BX_CU(cudaMemset(h->r_ctl, 0, sizeof(ctl)));
      return fail(BX_ECUDA, "the resident kernel's grid barrier timed out; upload the state again");
    }
  }
  return BX_OK;
}

int bx_outputs_download(bx_handle h, bx_outputs* o) {
  if (!h || !o) return fail(BX_EINVAL, "null argument");
  if (!h->have_outputs) return fail(BX_ESTATE, "no step with want_outputs has run");
  BX_CU(cudaStreamSynchronize(h->stream));
  const size_t M = h->M, C = h->C, I = h->I, G = h->G;
  struct Pair {
    double* dst;
    const double* src;
    size_t n;
  };
  Pair pairs[] = {
      {o->fluxes_mem, h->o_fmem, I * M}, {o->fluxes_gj, h->o_fgj, I * M}, {o->rate_NaKATP, h->o_rate, M},
      {o->rho_cells, h->o_rho, C}, {o->Jn, h->o_Jn, M}, {o->I_mem, h->o_Imem, M},
      {o->J_cell_x, h->o_Jcx, C}, {o->J_cell_y, h->o_Jcy, C}, {o->Jc, h->o_Jc, M},
      {o->vm_ave, h->o_vmave, C}, {o->dvm, h->o_dvm, M}, {o->E_cell_x, h->o_Ecx, C},
      {o->E_cell_y, h->o_Ecy, C}, {o->Emc, h->o_Emc, M}, {o->E_gj_x, h->o_Egjx, M},
      {o->E_gj_y, h->o_Egjy, M}, {o->gjopen, h->o_gjopen, M}, {o->sigma_cell, h->o_sigma, C},
      {o->fluxes_env_x, h->ecm ? h->d_fx : nullptr, I * G},
      {o->fluxes_env_y, h->ecm ? h->d_fy : nullptr, I * G},
      {o->rho_env, h->ecm ? h->d_rho_env : nullptr, G},
      {o->v_env, h->ecm ? h->d_venv : nullptr, G},
  };
  for (const Pair& p : pairs)
    if (p.dst && p.src) BX_CU(cudaMemcpy(p.dst, p.src, p.n * sizeof(double), cudaMemcpyDefault));
  return BX_OK;
}

int bx_time_cell_kernel(bx_handle h, int n, double* ms_per_launch) {
  if (!h || !ms_per_launch || n <= 0) return fail(BX_EINVAL, "bad arguments");
  if (!h->have_state || !h->have_dm) return fail(BX_ESTATE, "upload state and Dm first");
  cudaEvent_t e0, e1;
  BX_CU(cudaEventCreate(&e0));
  BX_CU(cudaEventCreate(&e1));
  if (h->kind == KIND_RESIDENT && fact_eligible(h, false)) {
    // one cooperative launch of n steps (the kernel's unit of work), per step
    if (h->r_state == 0) {
      const int rc = build_resident(h);
      if (rc != BX_OK) return rc;
    }
    if (h->r_state == 1 && n >= 2) {
      BX_CU(cudaEventRecord(e0, h->stream));
      cudaError_t e = launch_resident(h, h->parity, n, h->stream);
      if (e != cudaSuccess) return fail(BX_ECUDA, cudaGetErrorString(e));
      BX_CU(cudaEventRecord(e1, h->stream));
      BX_CU(cudaEventSynchronize(e1));
      float ms = 0.f;
      BX_CU(cudaEventElapsedTime(&ms, e0, e1));
      h->parity ^= (n & 1);
      h->launches++;
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      *ms_per_launch = ms / n;
      return BX_OK;
    }
  }
  double tot = 0.0;
  for (int q = 0; q < n; ++q) {
    BX_CU(cudaEventRecord(e0, h->stream));
    cudaError_t e = (h->mode == MODE_SPLIT) ? launch_split(h, h->parity, false, h->stream)
                                            : launch_cell(h, h->parity, false, h->stream);
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

int64_t bx_cell_kernel_bytes(bx_handle h) {
  if (!h) return -1;
  const int64_t M = h->M, C = h->C, I = h->I, B = h->nblk;
  if (h->mode == MODE_SPLIT && (h->kind == KIND_FACT || h->kind == KIND_RESIDENT || h->kind == KIND_FACT_PIPE) &&
      fact_eligible(h, false)) {
    // factored form, per cell slot: cc2 in+out 16I, record in+out 2*4*kRec,
    // DSA 4I, {SA, dt/vol, diviterm/cm, count} 16, first entry 4; per
    // gap-junction entry 8; per tile the partial sums 4I and the cluster id 4
    const int64_t S = h->S, P = h->f_P;
    return S * (16 * I + 8 * kRec + 4 * I + 16 + 4) + P * 8 + B * (4 * I + 4);
  }
  if (h->mode == MODE_SPLIT) {
    // membrane: Dm (4I), nn_slot 4, lcell 1, mem_sa 4, gjw 4
    // cell: cc2 in+out 16I, record in+out 2*4*kRec, dt/vol 4, diviterm/cm 4, range 4
    // tile: partial sums 4I, cluster id 4; ECM: map_env 4, grid concentration
    // 8I and the f*sa export 8I per membrane instead of the partial sums
    // voltage-gated gap junctions: the open fraction in+out, 8 per membrane
    // Ca-ATPase with ECM: the grid's Ca2+ after the Nernst-Planck update, 8 per membrane
    const int64_t gv = (h->vgj ? 8 : 0) + (h->ca && h->ecm ? 8 : 0);
    if (h->ecm) return M * (4 * I + 13 + 4 + 16 * I + gv) + C * (16 * I + 8 * kRec + 12) + B * 4;
    return M * (4 * I + 13 + gv) + C * (16 * I + 8 * kRec + 12) + B * (4 * I + 4);
  }
  const int64_t w = 8;  // Dm, mem_sa, gj_w width
  // membrane: Dm, vm in+out, m2c, nn, nn_cell, bflag, mem_sa, gj_w (+ map_env and the f*sa
  // export with ECM); cell: cc in+out, cc_mem in+out, cell_vol, diviterm, ptr
  // polarizability: R_rads and the two smoothing weights, 24 per membrane
  const int64_t mem = I * w + 16 + 12 + 1 + 2 * w + (h->ecm ? 4 + I * 8 : 0) + (h->vgj ? 16 : 0) +
                      (h->ca && h->ecm ? 8 : 0) + (h->polar ? 24 : 0);
  const int64_t cell = 4 * I * 8 + 16 + 4;
  return M * mem + C * cell + (h->ecm ? 0 : B * I * 8);
}

int64_t bx_launch_count(bx_handle h) { return h ? h->launches : -1; }

int bx_cluster_info(bx_handle h, int32_t* info) {
  if (!h || !info) return fail(BX_EINVAL, "null argument");
  const int32_t v[8] = {h->ncl, h->C, h->M, h->I, h->ny, h->nx, h->ecm ? 1 : 0, h->precision};
  for (int q = 0; q < 8; ++q) info[q] = v[q];
  return BX_OK;
}

int bx_get_launch_config(bx_handle h, int* tpb, int* kernel) {
  if (!h || !tpb || !kernel) return fail(BX_EINVAL, "null argument");
  *tpb = h->tpb;
  *kernel = h->kind;
  return BX_OK;
}

int bx_set_launch_config(bx_handle h, int tpb, int kernel) {
  if (!h) return fail(BX_EINVAL, "null handle");
  const bool ok = (h->mode == MODE_SPLIT) ? (tpb == 192 || tpb == 256)
                                           : (tpb == 8 || tpb == 16 || tpb == 32 || tpb == 64 || tpb == 128 ||
                                              tpb == 256);
  if (!ok) return fail(BX_EINVAL, "unsupported CTA size for this form");
  const int variant = (kernel >> 8) & 0xff;
  kernel &= 0xff;
  if (kernel < KIND_TILE || kernel > KIND_ION) return fail(BX_EINVAL, "kernel must be 0 to 5");
  if (variant && !(variant == 2 || variant == 4 || variant == 12 || variant == 13 || variant == 14 || variant == 16))
    return fail(BX_EINVAL, "factored-kernel variant must be 2, 4, 12, 13, 14 or 16");
  if (kernel == KIND_ION && h->mode == MODE_SPLIT)
    return fail(BX_EINVAL, "the one-lane-per-ion kernel is the plain form's");
  if (kernel == KIND_ION && (h->polar))
    return fail(BX_EINVAL, "the one-lane-per-ion kernel has no polarizability variant");
  if (kernel != KIND_TILE && kernel != KIND_ION && h->mode != MODE_SPLIT)
    return fail(BX_EINVAL, "the persistent, factored and resident kernels are the split form's");
  if (kernel != KIND_TILE && h->ecm) return fail(BX_EINVAL, "only the tile kernel has an extracellular-space variant");
  if (kernel != KIND_TILE && h->vgj)
    return fail(BX_EINVAL, "only the tile kernel has a voltage-gated gap-junction variant");
  if (kernel != KIND_TILE && h->ca) return fail(BX_EINVAL, "only the tile kernel has a Ca-ATPase variant");
  const size_t C = h->C, I = h->I, M = h->M;
  const size_t nenv = h->ecm ? I * h->G : (size_t)h->ncl * I;
  std::vector<double> vm(M), cc(I * C), cam(I * M), cenv(nenv), ex(h->ecm ? h->G : 1), ey(h->ecm ? h->G : 1),
      gjo(h->vgj ? M : 1);
  bx_state sv{vm.data(), cc.data(), cam.data(), cenv.data(), h->ecm ? ex.data() : nullptr,
              h->ecm ? ey.data() : nullptr, h->vgj ? gjo.data() : nullptr};
  const bool had_state = h->have_state;
  int rc;
  if (had_state && (rc = bx_state_download(h, &sv)) != BX_OK) return rc;
  if ((rc = build_partition(h, tpb)) != BX_OK) return rc;
  h->kind = kernel;
  if (variant) h->fact_unroll = variant;
  h->graph_valid = false;
  if (had_state && (rc = bx_state_upload(h, &sv)) != BX_OK) return rc;
  return BX_OK;
}

// Failure detection of the resident kernel without a fault: one launch whose
// grid barrier waits for one CTA more than the grid has, so every CTA's wait
// runs out after timeout_ns; the kernel then raises its timeout flag and
// returns, leaving the state as it was (the run never writes it back).
int bx_resident_barrier_check(bx_handle h, int64_t timeout_ns, int* timed_out) {
  if (!h || !timed_out || timeout_ns <= 0 || timeout_ns > kResTimeoutNs)
    return fail(BX_EINVAL, "timeout_ns must be in (0, 2e9]");
  if (!h->have_state || !h->have_dm) return fail(BX_ESTATE, "upload state and Dm first");
  if (!fact_eligible(h, false)) return fail(BX_EINVAL, "the resident kernel does not cover this handle");
  if (h->r_state == 0) {
    const int rc = build_resident(h);
    if (rc != BX_OK) return rc;
  }
  if (h->r_state != 1) return fail(BX_EINVAL, h->r_why);
  cudaError_t e = launch_resident(h, h->parity, 2, h->stream, (long long)timeout_ns, 1u);
  if (e != cudaSuccess) return fail(BX_ECUDA, cudaGetErrorString(e));
  h->launches++;
  BX_CU(cudaStreamSynchronize(h->stream));
  unsigned ctl[2] = {0u, 0u};
  BX_CU(cudaMemcpy(ctl, h->r_ctl, sizeof(ctl), cudaMemcpyDeviceToHost));
  *timed_out = ctl[1] ? 1 : 0;
  BX_CU(cudaMemset(h->r_ctl, 0, sizeof(ctl)));
  return BX_OK;
}

int bx_resident_info(bx_handle h, int* fits, int* grid, int* threads, int64_t* smem_bytes) {
  if (!h || !fits) return fail(BX_EINVAL, "null argument");
  if (h->mode != MODE_SPLIT || !fact_eligible(h, false)) {
    *fits = 0;
    return fail(BX_EINVAL, "the resident kernel needs the split form without ECM, Phi_b, gating or Ca-ATPase");
  }
  if (h->r_state == 0) {
    const int rc = build_resident(h);
    if (rc != BX_OK) return rc;
  }
  *fits = h->r_state == 1 ? 1 : 0;
  if (grid) *grid = h->r_grid;
  if (threads) *threads = h->r_threads;
  if (smem_bytes) *smem_bytes = (int64_t)h->r_smem;
  if (h->r_state != 1) return fail(BX_EINVAL, h->r_why);
  return BX_OK;
}

// Autotuner: time `n_steps` steps (as bx_step runs them: graph chunks, or
// one cooperative launch for the resident kernel) for each candidate
// partition and kernel, after one untimed run of the same length, and keep
// the fastest.  The state is downloaded before the trials and uploaded
// again after each one (the split form's tile-major layout changes with the
// CTA size), so tuning does not advance the simulation.
int bx_autotune_table(bx_handle h, int n_steps, int max_rows, int* n_rows, int* tpb, int* kernel, int* unroll,
                      double* ms_per_step) {
  if (!h || n_steps <= 0 || max_rows < 0) return fail(BX_EINVAL, "bad arguments");
  if (n_rows) *n_rows = 0;
  if (!h->have_state || !h->have_dm) return fail(BX_ESTATE, "upload state and Dm first");
  const size_t C = h->C, I = h->I, M = h->M;
  const size_t nenv = h->ecm ? I * h->G : (size_t)h->ncl * I;
  std::vector<double> vm(M), cc(I * C), cam(I * M), cenv(nenv), ex(h->ecm ? h->G : 1), ey(h->ecm ? h->G : 1),
      gjo(h->vgj ? M : 1);
  bx_state sv{vm.data(), cc.data(), cam.data(), cenv.data(), h->ecm ? ex.data() : nullptr,
              h->ecm ? ey.data() : nullptr, h->vgj ? gjo.data() : nullptr};
  int rc = bx_state_download(h, &sv);
  if (rc != BX_OK) return rc;
  unsigned long long status[4];
  BX_CU(cudaMemcpy(status, h->d_status, sizeof(status), cudaMemcpyDeviceToHost));
  const int64_t launches0 = h->launches, steps0 = h->steps_done;
  struct Cand { int tpb; int kind; int unroll; };
  std::vector<Cand> cands;
  if (h->mode == MODE_SPLIT && !fact_eligible(h, false)) cands = {{256, KIND_TILE, 4}, {192, KIND_TILE, 4}};
  else if (h->mode == MODE_SPLIT)
    cands = {{256, KIND_TILE, 4},     {192, KIND_TILE, 4},     {256, KIND_PERSIST, 4}, {192, KIND_PERSIST, 4},
             {256, KIND_FACT, 4},     {192, KIND_FACT, 4},     {256, KIND_FACT, 2},    {192, KIND_FACT, 2},
             {256, KIND_FACT, 12},    {192, KIND_FACT, 12},    {256, KIND_FACT, 13},   {192, KIND_FACT, 13},
             {256, KIND_FACT, 14},    {192, KIND_FACT, 14},    {256, KIND_FACT, 16},   {192, KIND_FACT, 16},
             {256, KIND_FACT_PIPE, 4}, {192, KIND_FACT_PIPE, 4},
             {256, KIND_RESIDENT, 4}, {192, KIND_RESIDENT, 4}};
  // plain form: small CTAs spread a small cluster's FP64 work over more SMs
  else {
    cands = {{256, KIND_TILE, 4}, {128, KIND_TILE, 4}, {64, KIND_TILE, 4}, {32, KIND_TILE, 4},
             {16, KIND_TILE, 4},  {8, KIND_TILE, 4}};
    if (!h->phib_nonzero && !h->ecm && !h->vgj && !h->ca && !h->polar)
      for (int mb : {64, 32, 16, 8}) cands.push_back({mb, KIND_ION, 4});
  }
  double best = 1e300;
  int best_tpb = h->tpb, best_kind = h->kind, best_unroll = h->fact_unroll;
  cudaEvent_t e0, e1;
  BX_CU(cudaEventCreate(&e0));
  BX_CU(cudaEventCreate(&e1));
  for (const Cand& cd : cands) {
    if (build_partition(h, cd.tpb) != BX_OK) continue;
    h->kind = cd.kind;
    h->fact_unroll = cd.unroll;
    h->graph_valid = false;
    if (cd.kind == KIND_RESIDENT) {
      if ((rc = build_resident(h)) != BX_OK) return rc;
      if (h->r_state != 1) continue;            // does not fit: not a candidate
    }
    if ((rc = bx_state_upload(h, &sv)) != BX_OK) return rc;
    if ((rc = bx_step(h, n_steps, 0, h->stream)) != BX_OK) return rc;
    BX_CU(cudaEventRecord(e0, h->stream));
    if ((rc = bx_step(h, n_steps, 0, h->stream)) != BX_OK) return rc;
    BX_CU(cudaEventRecord(e1, h->stream));
    BX_CU(cudaEventSynchronize(e1));
    float ms = 0.f;
    BX_CU(cudaEventElapsedTime(&ms, e0, e1));
    const double per = ms / n_steps;
    if (per < best) { best = per; best_tpb = cd.tpb; best_kind = cd.kind; best_unroll = cd.unroll; }
    if (n_rows && *n_rows < max_rows) {
      const int r = (*n_rows)++;
      if (tpb) tpb[r] = cd.tpb;
      if (kernel) kernel[r] = cd.kind;
      if (unroll) unroll[r] = cd.unroll;
      if (ms_per_step) ms_per_step[r] = per;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if ((rc = build_partition(h, best_tpb)) != BX_OK) return rc;
  h->kind = best_kind;
  h->fact_unroll = best_unroll;
  h->tune_ms = best;
  h->graph_valid = false;
  if ((rc = bx_state_upload(h, &sv)) != BX_OK) return rc;
  BX_CU(cudaMemcpy(h->d_status, status, sizeof(status), cudaMemcpyHostToDevice));
  h->launches = launches0;
  h->steps_done = steps0;
  return BX_OK;
}

int bx_autotune(bx_handle h, int n_steps, int* tpb_out, double* ms_per_step_out) {
  const int rc = bx_autotune_table(h, n_steps, 0, nullptr, nullptr, nullptr, nullptr, nullptr);
  if (rc != BX_OK) return rc;
  if (tpb_out) *tpb_out = h->tpb;
  if (ms_per_step_out) *ms_per_step_out = h->tune_ms;
  return BX_OK;
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

}  // extern "C"

namespace {
__device__ __forceinline__ double nan_value() { return __longlong_as_double(0x7ff8000000000000LL); }
// out[c] = max |dvm| over cluster c's membranes (one CTA per cluster)
__global__ void k_max_abs_dvm(const int* __restrict__ cl_mem, const double* __restrict__ dvm, double* out) {
  __shared__ double red[8];
  const int c = blockIdx.x;
  double m = 0.0;
  bool nan = false;
  for (int i = cl_mem[c] + threadIdx.x; i < cl_mem[c + 1]; i += blockDim.x) {
    const double v = fabs(dvm[i]);
    if (v != v) nan = true;
    m = fmax(m, v);
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  nan = __syncthreads_or(nan);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, red[w]);
    out[c] = nan ? nan_value() : r;
  }
}
}  // namespace

extern "C" {

int bx_max_abs_dvm(bx_handle h, double* per_cluster) {
  if (!h || !per_cluster) return fail(BX_EINVAL, "null argument");
  if (!h->last_step_outputs) return fail(BX_ESTATE, "bx_max_abs_dvm needs a last bx_step with want_outputs");
  if (!h->d_cl_mem) {
    if (cudaMalloc(&h->d_cl_mem, (size_t)(h->ncl + 1) * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&h->d_resid, (size_t)h->ncl * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      return fail(BX_ENOMEM, "cudaMalloc residual");
    }
    BX_CU(cudaMemcpy(h->d_cl_mem, h->cl_mem.data(), (size_t)(h->ncl + 1) * sizeof(int), cudaMemcpyHostToDevice));
  }
  k_max_abs_dvm<<<h->ncl, 256, 0, h->stream>>>(h->d_cl_mem, h->o_dvm, h->d_resid);
  BX_CU(cudaGetLastError());
  BX_CU(cudaMemcpyAsync(per_cluster, h->d_resid, (size_t)h->ncl * sizeof(double), cudaMemcpyDeviceToHost,
                        h->stream));
  BX_CU(cudaStreamSynchronize(h->stream));
  return BX_OK;
}

namespace {

bx::FieldGrid field_grid(const bx_cluster* h);
constexpr int kBfPlanes = 17;

// group the clusters by grid shape: each shape's operand has two columns per cluster
void ensure_fshapes(bx_cluster* h) {
  if (!h->fshapes.empty()) return;
  h->cl_goff.assign(h->ncl + 1, 0);
  for (int c = 0; c < h->ncl; ++c) {
    h->cl_goff[c + 1] = h->cl_goff[c] + h->cl_ny[c] * h->cl_nx[c];
    int s = -1;
    for (size_t q = 0; q < h->fshapes.size(); ++q)
      if (h->fshapes[q].ny == h->cl_ny[c] && h->fshapes[q].nx == h->cl_nx[c]) s = (int)q;
    if (s < 0) {
      bx_cluster::FieldShape fs;
      fs.ny = h->cl_ny[c];
      fs.nx = h->cl_nx[c];
      h->fshapes.push_back(fs);
      s = (int)h->fshapes.size() - 1;
    }
    h->fshapes[s].clusters.push_back(c);
  }
  h->Gtot = h->cl_goff[h->ncl];
  int xo = 0, so = 0;
  for (auto& fs : h->fshapes) {
    fs.ncols = 2 * (int)fs.clusters.size();
    fs.xoff = xo;
    fs.soff = so;
    xo += fs.ny * fs.nx * fs.ncols;
    so += fs.ncols;
  }
  h->Xtot = xo;
}

int prepare_batch_fields(bx_cluster* h) {
  if (h->bf_buf) return BX_OK;
  const int ncl = h->ncl;
  std::vector<int> ci((size_t)ncl * bx::kCi), last(h->Gtot, -1);
  std::vector<double> cd((size_t)ncl * 2), scale(2 * ncl);
  for (const auto& fs : h->fshapes) {
    for (size_t j = 0; j < fs.clusters.size(); ++j) {
      const int c = fs.clusters[j];
      int* e = &ci[(size_t)c * bx::kCi];
      e[0] = h->cl_goff[c]; e[1] = fs.ny; e[2] = fs.nx; e[3] = fs.xoff; e[4] = 2 * (int)j; e[5] = fs.ncols;
      e[6] = h->cl_mem[c]; e[7] = h->cl_cell[c];
      const double d2 = h->cl_delta[c] * h->cl_delta[c];   // lapENVinv = delta^2 K(shape)
      scale[fs.soff + 2 * j] = d2;
      scale[fs.soff + 2 * j + 1] = d2;
    }
  }
  for (int c = 0; c < ncl; ++c) {
    cd[2 * c] = h->cl_delta[c];
    cd[2 * c + 1] = h->cl_par[c].sigma;
    for (int m = h->cl_mem[c]; m < h->cl_mem[c + 1]; ++m) last[h->cl_goff[c] + h->h_map_env[m]] = m;
  }
  if (cudaMalloc(&h->bf_ci, ci.size() * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&h->bf_last, (size_t)h->Gtot * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&h->bf_cd, cd.size() * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&h->bf_scale, scale.size() * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&h->bf_X, (size_t)h->Xtot * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&h->bf_Y, (size_t)h->Xtot * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&h->bf_buf, (size_t)kBfPlanes * h->Gtot * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return fail(BX_ENOMEM, "cudaMalloc batched field scratch");
  }
  BX_CU(cudaMemcpy(h->bf_ci, ci.data(), ci.size() * sizeof(int), cudaMemcpyHostToDevice));
  BX_CU(cudaMemcpy(h->bf_last, last.data(), last.size() * sizeof(int), cudaMemcpyHostToDevice));
  BX_CU(cudaMemcpy(h->bf_cd, cd.data(), cd.size() * sizeof(double), cudaMemcpyHostToDevice));
  BX_CU(cudaMemcpy(h->bf_scale, scale.data(), scale.size() * sizeof(double), cudaMemcpyHostToDevice));
  return BX_OK;
}

}  // namespace

int bx_batch_set_lap_env_inv(bx_handle h, int ny, int nx, double delta, const double* lap_env_inv) {
  if (!h || !lap_env_inv || ny < 3 || nx < 3 || !(delta > 0.0)) return fail(BX_EINVAL, "bad arguments");
  if (h->ecm) return fail(BX_EINVAL, "bx_batch_set_lap_env_inv: batches without extracellular spaces only");
  ensure_fshapes(h);
  bx_cluster::FieldShape* fs = nullptr;
  for (auto& q : h->fshapes)
    if (q.ny == ny && q.nx == nx) fs = &q;
  if (!fs) return fail(BX_EINVAL, "bx_batch_set_lap_env_inv: no cluster of the batch has this grid shape");
  const int G = ny * nx;
  // the operator of unit spacing, K(shape) = lapENVinv / delta^2 (finitediff.py:426-429)
  std::vector<double> A((size_t)G * G);
  const double inv_d2 = 1.0 / (delta * delta);
  for (size_t e = 0; e < A.size(); ++e) A[e] = lap_env_inv[e] * inv_d2;
  if (fs->op) {
    bx_dense_op_destroy(fs->op);
    fs->op = nullptr;
  }
  int rc = bx_dense_op_create(A.data(), G, &fs->op);
  if (rc != BX_OK) return rc;
  // forward operator: makeLaplacian at unit spacing (finitediff.py:252-431):
  // 5-point stencil inside, identity rows on the edges
  std::vector<int> ptr(G + 1, 0), col;
  std::vector<double> val;
  for (int k = 0; k < G; ++k) {
    const int i = k / nx, j = k % nx;
    if (i == 0 || j == 0 || i == ny - 1 || j == nx - 1) {
      col.push_back(k); val.push_back(1.0);
    } else {
      const int nb[5] = {k - nx, k - 1, k, k + 1, k + nx};
      const double w[5] = {1.0, 1.0, -4.0, 1.0, 1.0};
      for (int q = 0; q < 5; ++q) { col.push_back(nb[q]); val.push_back(w[q]); }
    }
    ptr[k + 1] = (int)col.size();
  }
  return bx_dense_op_set_forward(fs->op, ptr.data(), col.data(), val.data());
}

int bx_batch_env_fields(bx_handle h, const double* D_env_weight, double* v_env, double* E_env_x, double* E_env_y,
                        double* J_env_x, double* J_env_y, double* B_field) {
  if (!h) return fail(BX_EINVAL, "null handle");
  if (h->ecm) return fail(BX_EINVAL, "bx_batch_env_fields: batches without extracellular spaces only");
  if (!h->last_step_outputs) return fail(BX_ESTATE, "bx_batch_env_fields needs a last bx_step with want_outputs");
  ensure_fshapes(h);
  for (const auto& fs : h->fshapes)
    if (!fs.op) return fail(BX_ESTATE, "bx_batch_env_fields: bx_batch_set_lap_env_inv missing for a grid shape");
  int rc = prepare_batch_fields(h);
  if (rc != BX_OK) return rc;
  const int Gt = h->Gtot, ncl = h->ncl;
  double* b[kBfPlanes];
  for (int q = 0; q < kBfPlanes; ++q) b[q] = h->bf_buf + (size_t)q * Gt;
  double *t0 = b[0], *t1 = b[1], *venv = b[2], *gx = b[3], *gy = b[4], *Frx = b[5], *Fry = b[6], *Fdx = b[7],
         *Fdy = b[8], *Ex = b[9], *Ey = b[10], *jx = b[11], *jy = b[12], *Bf = b[13], *Jex = b[14], *Jey = b[15],
         *w = b[16];
  cudaStream_t s = h->stream;
  if (D_env_weight) BX_CU(cudaMemcpyAsync(w, D_env_weight, (size_t)Gt * sizeof(double), cudaMemcpyDefault, s));
  bx::FieldGrid base = field_grid(h);
  const double* vm = (h->mode == MODE_SPLIT) ? h->o_vm_mem : h->d_vm[h->parity ^ 1];
  const int* ci = h->bf_ci;
  const double* cd = h->bf_cd;
  bx::kb_vce<<<ncl, 256, 0, s>>>(ci, cd, base, h->bf_last, h->d_m2c, vm, t0);
  bx::kb_gauss<true><<<ncl, 256, 0, s>>>(ci, cd, base, t0, t1, 0);
  bx::kb_gauss<true><<<ncl, 256, 0, s>>>(ci, cd, base, t1, venv, 1);
  bx::kb_grad_delta<<<ncl, 256, 0, s>>>(ci, cd, base, venv, gx, gy);
  auto products = [&]() -> int {
    for (const auto& fs : h->fshapes) {
      const int r = bx_dense_op_apply(fs.op, h->bf_X + fs.xoff, h->bf_Y + fs.xoff, fs.ncols, h->bf_scale + fs.soff,
                                      1, s);
      if (r != BX_OK) return r;
    }
    return BX_OK;
  };
  // smooth_flux(gradient(delta Phi)), then the current's Helmholtz-Hodge split
  bx::kb_hh_rhs<<<ncl, 256, 0, s>>>(ci, cd, base, gx, gy, h->bf_X);
  if ((rc = products()) != BX_OK) return rc;
  bx::kb_hh_out<<<ncl, 256, 0, s>>>(ci, cd, base, h->bf_Y, 1.0, nullptr, Frx, Fry, Fdx, Fdy);
  bx::kb_e_and_j<<<ncl, 256, 0, s>>>(ci, cd, base, Frx, Fry, Fdx, Fdy, D_env_weight ? w : nullptr, Ex, Ey, jx, jy);
  bx::kb_hh_rhs<<<ncl, 256, 0, s>>>(ci, cd, base, jx, jy, h->bf_X);
  if ((rc = products()) != BX_OK) return rc;
  bx::kb_hh_out<<<ncl, 256, 0, s>>>(ci, cd, base, h->bf_Y, h->par.mu, Bf, Jex, Jey, nullptr, nullptr);
  BX_CU(cudaGetLastError());
  double* dst[6] = {v_env, E_env_x, E_env_y, J_env_x, J_env_y, B_field};
  const double* src[6] = {venv, Ex, Ey, Jex, Jey, Bf};
  for (int q = 0; q < 6; ++q)
    if (dst[q]) BX_CU(cudaMemcpyAsync(dst[q], src[q], (size_t)Gt * sizeof(double), cudaMemcpyDefault, s));
  BX_CU(cudaStreamSynchronize(s));
  for (const auto& fs : h->fshapes) {
    int timed_out = 0;
    if ((rc = bx_dense_op_status(fs.op, &timed_out)) != BX_OK) return rc;
    if (timed_out) return fail(BX_ECUDA, "bx_batch_env_fields: tensor-core pipeline wait timed out");
  }
  return BX_OK;
}

int bx_lap_env_inv_build(int ny, int nx, double delta, double* A, int64_t lda, void* stream) {
  if (!A || ny < 3 || nx < 3 || !(delta > 0.0) || lda < (int64_t)ny * nx)
    return fail(BX_EINVAL, "bx_lap_env_inv_build: need ny, nx >= 3, delta > 0, lda >= ny*nx");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  BX_CU(cudaMemsetAsync(A, 0, (size_t)ny * nx * (size_t)lda * sizeof(double), s));
  BX_CU(bx::build_lap_env_inv<double>(ny, nx, delta, A, (size_t)lda, s));
  return BX_OK;
}

int bx_build_lap_env_inv(bx_handle h) {
  if (!h) return fail(BX_EINVAL, "null handle");
  if (h->ncl != 1) return fail(BX_EINVAL, "bx_build_lap_env_inv: single-cluster handles only");
  const size_t G = (size_t)h->G;
  const size_t ld = G + (G & 1);
  h->f_ld = (int)ld;
  if (!h->f_lap && cudaMalloc(&h->f_lap, G * ld * sizeof(float2)) != cudaSuccess) {
    h->f_lap = nullptr;
    cudaGetLastError();
    return fail(BX_ENOMEM, "cudaMalloc lapENVinv");
  }
  BX_CU(cudaStreamSynchronize(h->stream));
  BX_CU(cudaMemsetAsync(h->f_lap, 0, G * ld * sizeof(float2), h->stream));
  BX_CU(bx::build_lap_env_inv<float2>(h->ny, h->nx, h->delta, h->f_lap, ld, h->stream));
  return BX_OK;
}

int bx_set_lap_env_inv(bx_handle h, const double* lap_env_inv) {
  if (!h || !lap_env_inv) return fail(BX_EINVAL, "null argument");
  if (h->ncl != 1) return fail(BX_EINVAL, "bx_set_lap_env_inv: single-cluster handles only");
  const size_t G = (size_t)h->G;
  const size_t ld = G + (G & 1);
  h->f_ld = (int)ld;
  if (!h->f_lap && cudaMalloc(&h->f_lap, G * ld * sizeof(float2)) != cudaSuccess) {
    h->f_lap = nullptr;
    cudaGetLastError();
    return fail(BX_ENOMEM, "cudaMalloc lapENVinv");
  }
  // stream the FP64 rows through a bounded staging buffer, splitting on device
  const size_t rows_per = std::max<size_t>(1, std::min<size_t>(G, ((size_t)64 << 20) / (G * sizeof(double))));
  double* stage = nullptr;
  if (cudaMalloc(&stage, rows_per * G * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return fail(BX_ENOMEM, "cudaMalloc staging");
  }
  int rc = BX_OK;
  for (size_t r0 = 0; r0 < G && rc == BX_OK; r0 += rows_per) {
    const size_t nr = std::min(rows_per, G - r0);
    cudaError_t e = cudaMemcpyAsync(stage, lap_env_inv + r0 * G, nr * G * sizeof(double), cudaMemcpyHostToDevice,
                                    h->stream);
    if (e == cudaSuccess) {
      const size_t n = nr * ld;
      const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)h->sm_count * 16);
      bx::k_to_df_rows<<<blocks, 256, 0, h->stream>>>(stage, (int)nr, (int)G, h->f_lap + r0 * ld, (int)ld);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) rc = fail(BX_ECUDA, std::string("lapENVinv upload: ") + cudaGetErrorString(e));
  }
  cudaFree(stage);
  return rc;
}

namespace {

constexpr int kFieldBufs = 14;

bx::FieldGrid field_grid(const bx_cluster* h) {
  bx::FieldGrid g{};
  g.ny = h->ny;
  g.nx = h->nx;
  g.G = h->G;
  g.delta = h->delta;
  const bx::EnvConst e = make_env_const(h);
  for (int q = 0; q < 9; ++q) g.gw[q] = e.gw[q];
  return g;
}

// Enqueue the environment fields of the last step on the handle's stream;
// results in f_buf slots 0..5 = v_env, E_env_x, E_env_y, J_env_x, J_env_y, B_field.
int enqueue_env_fields(bx_cluster* h, const double* d_w) {
  const int G = h->G;
  const bx::FieldGrid fg = field_grid(h);
  cudaStream_t s = h->stream;
  double* b[kFieldBufs];
  for (int q = 0; q < kFieldBufs; ++q) b[q] = h->f_buf + (size_t)q * G;
  double *venv = b[0], *Ex = b[1], *Ey = b[2], *Jex = b[3], *Jey = b[4], *Bf = b[5];
  double *t0 = b[6], *t1 = b[7], *t2 = b[8], *t3 = b[9], *Y = b[10];  // Y spans b[10], b[11]
  double *jx = b[12], *jy = b[13];
  const unsigned gg = (unsigned)((G + 255) / 256);
  const unsigned rows = (unsigned)((((size_t)G + bx::kDenseRows - 1) / bx::kDenseRows * 32 + 255) / 256);
  if (!h->ecm) {
    const double* vm = (h->mode == MODE_SPLIT) ? h->o_vm_mem : h->d_vm[h->parity ^ 1];
    bx::k_fields_vce<<<gg, 256, 0, s>>>(G, h->f_last, h->d_m2c, vm, t0);
    bx::k_fields_gauss<true><<<gg, 256, 0, s>>>(t0, t1, 0, fg);
    bx::k_fields_gauss<true><<<gg, 256, 0, s>>>(t1, venv, 1, fg);
    // smooth_flux(gradient(delta * Phi)) (ion_current.py:133-136)
    bx::k_fields_grad<<<gg, 256, 0, s>>>(venv, h->delta, t0, t1, fg);
    bx::k_fields_hh_rhs<<<gg, 256, 0, s>>>(t0, t1, h->f_X, fg);
    bx::k_dense_rows2_df<bx::kDenseRows><<<rows, 256, 0, s>>>(h->f_lap, h->f_ld, h->f_X, Y, G);
    bx::k_fields_hh_out<<<gg, 256, 0, s>>>(Y, 1.0, nullptr, t0, t1, t2, t3, fg);
    bx::k_fields_e_and_j<<<gg, 256, 0, s>>>(G, t0, t1, t2, t3, d_w, h->par.sigma, Ex, Ey, jx, jy);
  } else {
    BX_CU(cudaMemcpyAsync(venv, h->d_venv, (size_t)G * sizeof(double), cudaMemcpyDeviceToDevice, s));
    BX_CU(cudaMemcpyAsync(Ex, h->d_Ex, (size_t)G * sizeof(double), cudaMemcpyDeviceToDevice, s));
    BX_CU(cudaMemcpyAsync(Ey, h->d_Ey, (size_t)G * sizeof(double), cudaMemcpyDeviceToDevice, s));
    bx::ZF zf{};
    for (int i = 0; i < h->I; ++i) zf.v[i] = h->par.zs[i] * h->par.F;
    bx::k_fields_zf_sum<<<gg, 256, 0, s>>>(G, h->I, h->d_fx, h->d_fy, zf, jx, jy);
  }
  // J_env, B_field: Helmholtz-Hodge split of the current (ion_current.py:70, 147)
  bx::k_fields_hh_rhs<<<gg, 256, 0, s>>>(jx, jy, h->f_X, fg);
  bx::k_dense_rows2_df<bx::kDenseRows><<<rows, 256, 0, s>>>(h->f_lap, h->f_ld, h->f_X, Y, G);
  bx::k_fields_hh_out<<<gg, 256, 0, s>>>(Y, h->par.mu, Bf, Jex, Jey, nullptr, nullptr, fg);
  BX_CU(cudaGetLastError());
  return BX_OK;
}

int prepare_env_fields(bx_cluster* h, const double* D_env_weight, double** d_w) {
  if (h->ncl != 1) return fail(BX_EINVAL, "bx_env_fields: single-cluster handles only");
  if (!h->f_lap) return fail(BX_ESTATE, "bx_env_fields before bx_set_lap_env_inv");
  if (!h->last_step_outputs) return fail(BX_ESTATE, "bx_env_fields needs a last bx_step with want_outputs");
  const size_t G = (size_t)h->G;
  if (!h->f_buf) {
    if (cudaMalloc(&h->f_buf, (kFieldBufs + 1) * G * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&h->f_X, 2 * (G + 1) * sizeof(float2)) != cudaSuccess ||
        cudaMalloc(&h->f_last, G * sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      return fail(BX_ENOMEM, "cudaMalloc field scratch");
    }
    BX_CU(cudaMemset(h->f_X, 0, 2 * (G + 1) * sizeof(float2)));   // the padding row stays zero
    std::vector<int> last(G, -1);
    for (int m = 0; m < h->M; ++m) last[h->h_map_env[m]] = m;  // numpy keeps the last repeat
    BX_CU(cudaMemcpy(h->f_last, last.data(), G * sizeof(int), cudaMemcpyHostToDevice));
  }
  *d_w = nullptr;
  if (D_env_weight) {
    double* w = h->f_buf + (size_t)kFieldBufs * G;  // the spare slot
    BX_CU(cudaMemcpyAsync(w, D_env_weight, G * sizeof(double), cudaMemcpyDefault, h->stream));
    *d_w = w;
  }
  return BX_OK;
}

}  // namespace

int bx_env_fields(bx_handle h, const double* D_env_weight, double* v_env, double* E_env_x, double* E_env_y,
                  double* J_env_x, double* J_env_y, double* B_field) {
  if (!h) return fail(BX_EINVAL, "null handle");
  double* d_w = nullptr;
  int rc = prepare_env_fields(h, D_env_weight, &d_w);
  if (rc != BX_OK) return rc;
  rc = enqueue_env_fields(h, d_w);
  if (rc != BX_OK) return rc;
  const size_t G = (size_t)h->G;
  double* dst[6] = {v_env, E_env_x, E_env_y, J_env_x, J_env_y, B_field};
  for (int q = 0; q < 6; ++q)
    if (dst[q])
      BX_CU(cudaMemcpyAsync(dst[q], h->f_buf + (size_t)q * G, G * sizeof(double), cudaMemcpyDefault,
                            h->stream));
  BX_CU(cudaStreamSynchronize(h->stream));
  return BX_OK;
}

int bx_time_env_fields(bx_handle h, int n, double* ms_fields, double* ms_product) {
  if (!h || n <= 0 || !ms_fields || !ms_product) return fail(BX_EINVAL, "bad arguments");
  double* d_w = nullptr;
  int rc = prepare_env_fields(h, nullptr, &d_w);
  if (rc != BX_OK) return rc;
  cudaEvent_t e0, e1, e2;
  BX_CU(cudaEventCreate(&e0));
  BX_CU(cudaEventCreate(&e1));
  BX_CU(cudaEventCreate(&e2));
  const int G = h->G;
  const unsigned rows = (unsigned)((((size_t)G + bx::kDenseRows - 1) / bx::kDenseRows * 32 + 255) / 256);
  double tf = 0.0, tp = 0.0;
  for (int q = 0; q < n; ++q) {
    BX_CU(cudaEventRecord(e0, h->stream));
    rc = enqueue_env_fields(h, d_w);
    if (rc != BX_OK) break;
    BX_CU(cudaEventRecord(e1, h->stream));
    bx::k_dense_rows2_df<bx::kDenseRows><<<rows, 256, 0, h->stream>>>(h->f_lap, h->f_ld, h->f_X, h->f_buf + (size_t)10 * G, G);
    BX_CU(cudaEventRecord(e2, h->stream));
    BX_CU(cudaEventSynchronize(e2));
    float a = 0.f, b = 0.f;
    BX_CU(cudaEventElapsedTime(&a, e0, e1));
    BX_CU(cudaEventElapsedTime(&b, e1, e2));
    tf += a;
    tp += b;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  if (rc != BX_OK) return rc;
  *ms_fields = tf / n;
  *ms_product = tp / n;
  return BX_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Molecule and gene regulatory networks (bx_network.cuh)
// ---------------------------------------------------------------------------
struct bx_network {
  bx_cluster* h = nullptr;
  int S = 0, R = 0, nblk = 0;
  bool any_ui = false, have_state = false, have_fluxes = false;
  bx::NetTables* d_tab = nullptr;
  double *d_gamma = nullptr, *d_Rr = nullptr /* gamma / R_rads */, *d_gmod = nullptr, *d_cc = nullptr, *d_cm = nullptr,
         *d_cmid = nullptr, *d_cmmid = nullptr, *d_env = nullptr, *d_part = nullptr, *d_fmem = nullptr,
         *d_fgj = nullptr, *d_rates = nullptr;
  uint8_t* d_gmask = nullptr;
  unsigned long long* d_neg = nullptr;
  cudaGraphExec_t graph = nullptr;   // kGraphChunk coupled steps from ion parity 0
  cudaGraphExec_t graph_net = nullptr;   // kGraphChunk network-only steps
  int graph_net_parity = -1;
};

namespace {

void net_free(bx_network* n) {
  void* ptrs[] = {n->d_tab, n->d_gamma, n->d_Rr, n->d_gmod, n->d_cc, n->d_cm, n->d_cmid, n->d_cmmid,
                  n->d_env, n->d_part, n->d_fmem, n->d_fgj, n->d_rates, n->d_gmask, n->d_neg};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (n->graph) cudaGraphExecDestroy(n->graph);
  if (n->graph_net) cudaGraphExecDestroy(n->graph_net);
}

// Checks one influencer range and its order (multiplicative, independent,
// inhibitors, direct), which is how the kernel evaluates it.
bool net_range_ok(const bx_net_spec* sp, int t0, int nt, std::string* why) {
  if (nt == 0) return true;
  if (t0 < 0 || nt < 0 || t0 + nt > sp->n_terms) { *why = "influencer range outside the term table"; return false; }
  int last = 0;
  for (int q = t0; q < t0 + nt; ++q) {
    const bx_net_term& t = sp->terms[q];
    if (t.kind < 0 || t.kind > BX_TERM_DIRECT_NEG) { *why = "unknown influencer kind"; return false; }
    const int rank = t.kind >= BX_TERM_DIRECT_POS ? 3 : t.kind;
    if (rank < last) { *why = "influencer terms out of order (act, independent, inhibitor, direct)"; return false; }
    last = rank;
    if (t.substance < 0 || t.substance >= sp->n_substances) { *why = "influencer names no substance"; return false; }
    if (t.kind != BX_TERM_DIRECT_POS && t.kind != BX_TERM_DIRECT_NEG && !(t.Km > 0.0)) {
      *why = "influencer Km must be > 0";
      return false;
    }
  }
  return true;
}

bx::NetArgs net_args(bx_network* n, int vm_parity) {
  bx_cluster* h = n->h;
  bx::NetArgs a{};
  a.C = h->C; a.M = h->M;
  a.dt = h->par.dt; a.inv_tm = 1.0 / h->par.tm; a.F_RT = h->par.F / (h->par.R * h->par.T);
  a.inv_gj_len = 1.0 / h->gj_len; a.gj_block = h->par.gj_block;
  a.inv_vol_env_M = 1.0 / (h->par.vol_env * (double)h->M);
  a.cell_ptr = h->d_cell_ptr; a.nn = h->d_nn; a.nn_cell = h->d_nn_cell; a.bflag = h->d_bflag;
  a.mem_sa = h->d_mem_sa; a.cell_vol = h->d_cell_vol; a.gj_w = h->d_gj_w;
  a.gjo = h->vgj ? h->d_gjo : nullptr;
  a.vm = h->d_vm[vm_parity];
  a.tab = n->d_tab; a.gamma = n->d_gamma; a.g_over_r = n->d_Rr; a.gmod = n->d_gmod; a.gmask = n->d_gmask;
  a.c_cells = n->d_cc; a.cmem = n->d_cm; a.c_mid = n->d_cmid; a.cmem_mid = n->d_cmmid; a.env = n->d_env;
  a.env_part = n->d_part; a.f_mem = n->d_fmem; a.f_gj = n->d_fgj; a.rates = n->d_rates; a.neg = n->d_neg;
  a.nblk = n->nblk;
  return a;
}

cudaError_t net_enqueue(bx_network* n, int vm_parity, bool out, cudaStream_t s) {
  const bx::NetArgs a = net_args(n, vm_parity);
  if (out) {
    bx::k_net_cell<true><<<n->nblk, bx::kNetTPB, 0, s>>>(a);
    bx::k_net_gj<true><<<n->nblk, bx::kNetTPB, 0, s>>>(a);
  } else {
    bx::k_net_cell<false><<<n->nblk, bx::kNetTPB, 0, s>>>(a);
    bx::k_net_gj<false><<<n->nblk, bx::kNetTPB, 0, s>>>(a);
  }
  n->h->launches += 2;
  return cudaGetLastError();
}

// One time step: the ion step at the cluster's parity (reading Vmem from
// d_vm[parity], writing d_vm[parity ^ 1]) then the network on d_vm[parity].
cudaError_t net_enqueue_coupled(bx_network* n, int parity, bool out, cudaStream_t s) {
  cudaError_t e = enqueue_step(n->h, parity, out, s);
  if (e != cudaSuccess) return e;
  return net_enqueue(n, parity, out, s);
}

int net_capture(bx_network* n, bool coupled, int parity, cudaGraphExec_t* exec) {
  bx_cluster* h = n->h;
  cudaStream_t cs;
  BX_CU(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaGraph_t graph;
  const int64_t l0 = h->launches;
  BX_CU(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
  int par = parity;
  for (int q = 0; q < kGraphChunk; ++q) {
    if (coupled) {
      net_enqueue_coupled(n, par, false, cs);
      par ^= 1;
    } else {
      net_enqueue(n, par, false, cs);
    }
  }
  cudaError_t ce = cudaStreamEndCapture(cs, &graph);
  cudaStreamDestroy(cs);
  h->launches = l0;
  if (ce != cudaSuccess) return fail(BX_ECUDA, std::string("network graph capture: ") + cudaGetErrorString(ce));
  ce = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ce != cudaSuccess) return fail(BX_ECUDA, std::string("network graph instantiate: ") + cudaGetErrorString(ce));
  return BX_OK;
}

}  // namespace

extern "C" {

int bx_network_create(bx_handle h, const bx_net_spec* sp, bx_network_handle* out) {
  if (!h || !sp || !out) return fail(BX_EINVAL, "null argument");
  *out = nullptr;
  if (h->mode != MODE_PLAIN) return fail(BX_EINVAL, "networks step with the plain FP64 form");
  if (h->ncl != 1) return fail(BX_EINVAL, "networks step on a single-cluster handle");
  if (h->ecm) return fail(BX_EINVAL, "networks with extracellular spaces are not built");
  if (sp->n_substances < 1 || sp->n_substances > bx::kNetMaxSub)
    return fail(BX_EINVAL, "n_substances must be 1.." + std::to_string(bx::kNetMaxSub));
  if (sp->n_reactions < 0 || sp->n_reactions > bx::kNetMaxReact)
    return fail(BX_EINVAL, "n_reactions must be 0.." + std::to_string(bx::kNetMaxReact));
  if (sp->n_terms < 0 || sp->n_terms > bx::kNetMaxTerms)
    return fail(BX_EINVAL, "n_terms must be 0.." + std::to_string(bx::kNetMaxTerms));
  if (!sp->substances || (sp->n_reactions && !sp->reactions) || (sp->n_terms && !sp->terms))
    return fail(BX_EINVAL, "null table");
  const int S = sp->n_substances, R = sp->n_reactions, C = h->C, M = h->M;
  std::unique_ptr<bx::NetTables> tb(new bx::NetTables());
  std::memset(tb.get(), 0, sizeof(bx::NetTables));
  tb->S = S; tb->R = R; tb->T = sp->n_terms;
  std::string why;
  bool any_ui = false;
  int mod_rows = 0, mask_rows = 0;
  for (int k = 0; k < S; ++k) {
    const bx_net_substance& u = sp->substances[k];
    bx::NetSubD& d = tb->sub[k];
    d.z = u.z; d.Dm = u.Dm; d.Do = u.Do; d.Dgj = u.Dgj; d.tdf = u.time_factor;
    d.r_prod = u.r_production; d.r_decay = u.r_decay; d.decay_max = u.decay_max;
    d.inv_gsf = u.gad_scale_factor != 0.0 ? 1.0 / u.gad_scale_factor : 0.0;
    d.growth = u.growth ? 1 : 0; d.ui = u.update_intra ? 1 : 0; d.gj_imp = u.gj_impermeable ? 1 : 0;
    d.gt0 = u.growth_term0; d.gnt = u.growth_nterm; d.dt0 = u.decay_term0; d.dnt = u.decay_nterm;
    d.mod_row = (u.growth && u.growth_mod) ? mod_rows++ : -1;
    d.mask_row = (u.growth && u.growth_target) ? mask_rows++ : -1;
    if (u.growth && !(u.gad_scale_factor != 0.0)) return fail(BX_EINVAL, "gad_scale_factor must be nonzero");
    if (u.update_intra) {
      if (u.z != 0.0)
        return fail(BX_EINVAL, "intracellular transport of a charged substance reads the intracellular field "
                               "E_cell; not built ('update intracellular' with z != 0)");
      any_ui = true;
    }
    if (u.growth && (!net_range_ok(sp, u.growth_term0, u.growth_nterm, &why) ||
                     !net_range_ok(sp, u.decay_term0, u.decay_nterm, &why)))
      return fail(BX_EINVAL, "substance " + std::to_string(k) + ": " + why);
  }
  if (any_ui && (!sp->mem_vol || !sp->R_rads))
    return fail(BX_EINVAL, "'update intracellular' needs mem_vol and R_rads");
  for (int j = 0; j < R; ++j) {
    const bx_net_reaction& r = sp->reactions[j];
    bx::NetReactD& d = tb->react[j];
    if (r.n_reactants < 1 || r.n_reactants > BX_NET_MAX_STOICH || r.n_products < 0 ||
        r.n_products > BX_NET_MAX_STOICH)
      return fail(BX_EINVAL, "reaction " + std::to_string(j) + ": 1..4 reactants and 0..4 products");
    if (r.keq != 0.0 && r.n_products < 1)
      return fail(BX_EINVAL, "reaction " + std::to_string(j) + ": a standard free energy needs products");
    if (r.keq < 0.0 || !std::isfinite(r.keq)) return fail(BX_EINVAL, "reaction keq must be >= 0 and finite");
    d.nr = r.n_reactants; d.np = r.n_products; d.vmax = r.vmax; d.inv_keq = r.keq > 0.0 ? 1.0 / r.keq : 0.0;
    d.t0 = r.term0; d.nt = r.nterm;
    for (int q = 0; q < r.n_reactants; ++q) {
      if (r.reactant[q] < 0 || r.reactant[q] >= S) return fail(BX_EINVAL, "reactant names no substance");
      if (!(r.reactant_Km[q] > 0.0)) return fail(BX_EINVAL, "reactant Km must be > 0");
      d.r[q] = r.reactant[q]; d.rc[q] = r.reactant_coeff[q]; d.inv_rkm[q] = 1.0 / r.reactant_Km[q];
      tb->rm[r.reactant[q]][j] += -r.reactant_coeff[q];
    }
    for (int q = 0; q < r.n_products; ++q) {
      if (r.product[q] < 0 || r.product[q] >= S) return fail(BX_EINVAL, "product names no substance");
      d.p[q] = r.product[q]; d.pc[q] = r.product_coeff[q];
      tb->rm[r.product[q]][j] += r.product_coeff[q];
    }
    if (!net_range_ok(sp, r.term0, r.nterm, &why)) return fail(BX_EINVAL, "reaction " + std::to_string(j) + ": " + why);
  }
  for (int q = 0; q < sp->n_terms; ++q) {
    const bx_net_term& t = sp->terms[q];
    tb->term[q] = bx::NetTermD{t.kind, t.substance, t.env_zone ? 1 : 0, 0,
                               (t.kind == BX_TERM_DIRECT_POS || t.kind == BX_TERM_DIRECT_NEG) ? 0.0 : 1.0 / t.Km, t.n};
  }
  std::unique_ptr<bx_network> n(new bx_network());
  struct Guard {
    std::unique_ptr<bx_network>* p;
    ~Guard() { if (*p) net_free(p->get()); }
  } guard{&n};
  n->h = h; n->S = S; n->R = R; n->any_ui = any_ui;
  n->nblk = (C + bx::kNetTPB - 1) / bx::kNetTPB;
  if (dalloc(&n->d_tab, 1) != cudaSuccess || dalloc(&n->d_cc, (size_t)S * C) != cudaSuccess ||
      dalloc(&n->d_cm, (size_t)S * M) != cudaSuccess || dalloc(&n->d_cmid, (size_t)S * C) != cudaSuccess ||
      dalloc(&n->d_cmmid, (size_t)S * M) != cudaSuccess || dalloc(&n->d_env, (size_t)S) != cudaSuccess ||
      dalloc(&n->d_part, (size_t)n->nblk * S) != cudaSuccess || dalloc(&n->d_fmem, (size_t)S * M) != cudaSuccess ||
      dalloc(&n->d_fgj, (size_t)S * M) != cudaSuccess || dalloc(&n->d_neg, 1) != cudaSuccess ||
      dalloc(&n->d_rates, (size_t)std::max(R, 1) * C) != cudaSuccess)
    return fail(BX_ENOMEM, "network allocation");
  BX_CU(cudaMemcpy(n->d_tab, tb.get(), sizeof(bx::NetTables), cudaMemcpyHostToDevice));
  BX_CU(cudaMemset(n->d_neg, 0, sizeof(unsigned long long)));
  BX_CU(cudaMemset(n->d_fmem, 0, (size_t)S * M * sizeof(double)));
  BX_CU(cudaMemset(n->d_fgj, 0, (size_t)S * M * sizeof(double)));
  BX_CU(cudaMemset(n->d_rates, 0, (size_t)std::max(R, 1) * C * sizeof(double)));
  if (any_ui) {
    std::vector<double> msa(M);
    BX_CU(cudaMemcpy(msa.data(), h->d_mem_sa, (size_t)M * sizeof(double), cudaMemcpyDeviceToHost));
    std::vector<double> gam(M), rr(M);
    for (int m = 0; m < M; ++m) {
      const double mv = sp->mem_vol[m];
      if (!(mv > 0.0) || !(sp->R_rads[m] > 0.0)) return fail(BX_EINVAL, "mem_vol and R_rads must be > 0");
      gam[m] = msa[m] / ((3.0 / 4.0) * mv);
      rr[m] = gam[m] / sp->R_rads[m];
    }
    if (dalloc(&n->d_gamma, M) != cudaSuccess || dalloc(&n->d_Rr, M) != cudaSuccess)
      return fail(BX_ENOMEM, "network allocation");
    BX_CU(cudaMemcpy(n->d_gamma, gam.data(), (size_t)M * sizeof(double), cudaMemcpyHostToDevice));
    BX_CU(cudaMemcpy(n->d_Rr, rr.data(), (size_t)M * sizeof(double), cudaMemcpyHostToDevice));
  }
  if (mod_rows) {
    if (dalloc(&n->d_gmod, (size_t)mod_rows * C) != cudaSuccess) return fail(BX_ENOMEM, "network allocation");
    for (int k = 0; k < S; ++k)
      if (tb->sub[k].mod_row >= 0)
        BX_CU(cudaMemcpy(n->d_gmod + (size_t)tb->sub[k].mod_row * C, sp->substances[k].growth_mod,
                         (size_t)C * sizeof(double), cudaMemcpyDefault));
  }
  if (mask_rows) {
    if (dalloc(&n->d_gmask, (size_t)mask_rows * C) != cudaSuccess) return fail(BX_ENOMEM, "network allocation");
    for (int k = 0; k < S; ++k)
      if (tb->sub[k].mask_row >= 0)
        BX_CU(cudaMemcpy(n->d_gmask + (size_t)tb->sub[k].mask_row * C, sp->substances[k].growth_target,
                         (size_t)C, cudaMemcpyDefault));
  }
  *out = n.release();
  return BX_OK;
}

int bx_network_upload(bx_network_handle n, const double* c_cells, const double* cc_at_mem, const double* c_env) {
  if (!n || !c_cells || !cc_at_mem || !c_env) return fail(BX_EINVAL, "null argument");
  const size_t S = n->S, C = n->h->C, M = n->h->M;
  cudaStream_t s = n->h->stream;
  BX_CU(cudaMemcpyAsync(n->d_cc, c_cells, S * C * sizeof(double), cudaMemcpyDefault, s));
  BX_CU(cudaMemcpyAsync(n->d_cm, cc_at_mem, S * M * sizeof(double), cudaMemcpyDefault, s));
  BX_CU(cudaMemcpyAsync(n->d_env, c_env, S * sizeof(double), cudaMemcpyDefault, s));
  BX_CU(cudaMemsetAsync(n->d_neg, 0, sizeof(unsigned long long), s));
  BX_CU(cudaStreamSynchronize(s));
  n->have_state = true;
  n->have_fluxes = false;
  return BX_OK;
}

int bx_network_download(bx_network_handle n, double* c_cells, double* cc_at_mem, double* c_env) {
  if (!n) return fail(BX_EINVAL, "null handle");
  if (!n->have_state) return fail(BX_ESTATE, "bx_network_download before bx_network_upload");
  const size_t S = n->S, C = n->h->C, M = n->h->M;
  cudaStream_t s = n->h->stream;
  if (c_cells) BX_CU(cudaMemcpyAsync(c_cells, n->d_cc, S * C * sizeof(double), cudaMemcpyDefault, s));
  if (cc_at_mem) BX_CU(cudaMemcpyAsync(cc_at_mem, n->d_cm, S * M * sizeof(double), cudaMemcpyDefault, s));
  if (c_env) BX_CU(cudaMemcpyAsync(c_env, n->d_env, S * sizeof(double), cudaMemcpyDefault, s));
  BX_CU(cudaStreamSynchronize(s));
  return BX_OK;
}

int bx_network_fluxes(bx_network_handle n, double* f_mem, double* f_gj, double* rates) {
  if (!n) return fail(BX_EINVAL, "null handle");
  if (!n->have_fluxes) return fail(BX_ESTATE, "no network step with want_outputs yet");
  const size_t bytes = (size_t)n->S * n->h->M * sizeof(double);
  cudaStream_t s = n->h->stream;
  if (f_mem) BX_CU(cudaMemcpyAsync(f_mem, n->d_fmem, bytes, cudaMemcpyDefault, s));
  if (f_gj) BX_CU(cudaMemcpyAsync(f_gj, n->d_fgj, bytes, cudaMemcpyDefault, s));
  if (rates && n->R)
    BX_CU(cudaMemcpyAsync(rates, n->d_rates, (size_t)n->R * n->h->C * sizeof(double), cudaMemcpyDefault, s));
  BX_CU(cudaStreamSynchronize(s));
  return BX_OK;
}

int bx_network_step(bx_network_handle n, int n_steps, int with_ions, int want_outputs) {
  if (!n) return fail(BX_EINVAL, "null handle");
  if (n_steps < 0) return fail(BX_EINVAL, "n_steps must be >= 0");
  if (!n->have_state) return fail(BX_ESTATE, "bx_network_step before bx_network_upload");
  bx_cluster* h = n->h;
  if (!h->have_state) return fail(BX_ESTATE, "bx_network_step before the cluster's bx_state_upload");
  if (with_ions && !h->have_dm) return fail(BX_ESTATE, "bx_network_step before bx_set_membrane_diffusivity");
  if (n_steps == 0) return BX_OK;
  cudaStream_t s = h->stream;
  int left = n_steps;
  const int tail = want_outputs ? 1 : 0;
  if (with_ions) {
    if (left - tail >= kGraphChunk) {
      if (h->parity != 0) {
        cudaError_t e = net_enqueue_coupled(n, h->parity, false, s);
        if (e != cudaSuccess) return fail(BX_ECUDA, std::string("network step launch: ") + cudaGetErrorString(e));
        h->parity ^= 1;
        --left;
      }
      if (!n->graph) {
        const int rc = net_capture(n, true, 0, &n->graph);
        if (rc != BX_OK) return rc;
      }
      while (left - tail >= kGraphChunk) {
        BX_CU(cudaGraphLaunch(n->graph, s));
        h->launches += (int64_t)kGraphChunk * (launches_per_step(h) + 2);
        left -= kGraphChunk;
      }
    }
    while (left > 0) {
      const bool out = want_outputs && left == 1;
      cudaError_t e = net_enqueue_coupled(n, h->parity, out, s);
      if (e != cudaSuccess) return fail(BX_ECUDA, std::string("network step launch: ") + cudaGetErrorString(e));
      h->parity ^= 1;
      --left;
    }
    h->steps_done += n_steps;
    if (want_outputs) h->have_outputs = true;
    h->last_step_outputs = want_outputs != 0;
  } else {
    if (left - tail >= kGraphChunk) {
      if (!n->graph_net || n->graph_net_parity != h->parity) {
        if (n->graph_net) cudaGraphExecDestroy(n->graph_net);
        n->graph_net = nullptr;
        const int rc = net_capture(n, false, h->parity, &n->graph_net);
        if (rc != BX_OK) return rc;
        n->graph_net_parity = h->parity;
      }
      while (left - tail >= kGraphChunk) {
        BX_CU(cudaGraphLaunch(n->graph_net, s));
        h->launches += (int64_t)kGraphChunk * 2;
        left -= kGraphChunk;
      }
    }
    while (left > 0) {
      const bool out = want_outputs && left == 1;
      cudaError_t e = net_enqueue(n, h->parity, out, s);
      if (e != cudaSuccess) return fail(BX_ECUDA, std::string("network step launch: ") + cudaGetErrorString(e));
      --left;
    }
  }
  if (want_outputs) n->have_fluxes = true;
  return BX_OK;
}

int bx_network_time_step(bx_network_handle n, int n_steps, int with_ions, double* ms_per_step) {
  if (!n || !ms_per_step || n_steps <= 0) return fail(BX_EINVAL, "bad argument");
  cudaStream_t s = n->h->stream;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  BX_CU(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return fail(BX_ECUDA, "cudaEventCreate");
  }
  cudaEventRecord(e0, s);
  const int rc = bx_network_step(n, n_steps, with_ions, 0);
  cudaEventRecord(e1, s);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != BX_OK) return rc;
  if (e != cudaSuccess) return fail(BX_ECUDA, cudaGetErrorString(e));
  *ms_per_step = (double)ms / n_steps;
  return BX_OK;
}

int bx_network_status(bx_network_handle n, int64_t* negative) {
  if (!n || !negative) return fail(BX_EINVAL, "null argument");
  unsigned long long v = 0;
  BX_CU(cudaStreamSynchronize(n->h->stream));
  BX_CU(cudaMemcpy(&v, n->d_neg, sizeof(v), cudaMemcpyDeviceToHost));
  *negative = (int64_t)v;
  return BX_OK;
}

int bx_network_info(bx_network_handle n, int32_t* info) {
  if (!n || !info) return fail(BX_EINVAL, "null argument");
  info[0] = n->S; info[1] = n->R; info[2] = n->h->C; info[3] = n->h->M;
  return BX_OK;
}

int bx_network_destroy(bx_network_handle n) {
  if (!n) return BX_OK;
  if (n->h && n->h->stream) cudaStreamSynchronize(n->h->stream);
  net_free(n);
  delete n;
  return BX_OK;
}

}  // extern "C"
