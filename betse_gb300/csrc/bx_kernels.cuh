// bx_kernels.cuh -- sm_103a kernels of the cell-network electrodiffusion step.
//
// Data layout in HBM (structure of arrays, row = ion):
//   per membrane : Dm[I][M] (FP64 or FP32), vm[2][M] FP64 ping-pong,
//                  m2c, nn, nn_cell, map_env (int32), bflag (u8),
//                  mem_sa, gj_w (FP64 or FP32)
//   per cell     : cc_cells[I][C] FP64 (post-GJ, clamped; owned by one CTA),
//                  cc_mem[2][I][C] FP64 ping-pong (the value BETSE broadcasts
//                  to cc_at_mem: cells + membrane term, before the GJ term),
//                  cell_vol, diviterm (FP64), cell_mem_ptr (int32)
//   per CTA      : blk_cell[nblk+1] (host-built partition of whole cells with
//                  at most TPB membranes), env partial sums [nblk][I]
//
// One CTA owns a contiguous run of whole cells, so every segment sum over a
// cell's membranes (BETSE's dense M_sum_mems products) is a fixed-order sum in
// shared memory: deterministic, no atomics.  Gap-junction partners are read
// from the previous step's ping-pong buffers, so CTAs never wait on each other.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace bx {

constexpr int kMaxIons = 8;
constexpr double kNonce = 1.0e-25;   // sim_toolbox.py:52

struct DevGeom {
  int C, M, I, G, ny, nx;
  const int* cell_ptr;    // [C+1]
  const int* m2c;         // [M]
  const int* nn;          // [M]
  const int* nn_cell;     // [M] = m2c[nn]
  const uint8_t* bflag;   // [M]
  const int* map_env;     // [M]
  const double* mem_sa;   // [M] FP64 copy
  const float* mem_sa_f;  // [M] FP32 copy (split form)
  const double* gj_w;     // [M]
  const float* gj_w_f;    // [M]
  const double* mem_nx;   // [M]
  const double* mem_ny;   // [M]
  const double* sw_mem;   // [M]
  const double* sw_o;     // [M]
  const double* cell_vol; // [C]
  const double* cell_sa;  // [C]
  const double* diviterm; // [C]
  const int* blk_cell;    // [nblk+1]
  const int* blk_cluster; // [nblk] cluster of each CTA (batched sweeps)
  const double* R_rads;   // [M] membrane distance from the cell centre (cell polarizability)
};

// Per-step constants (kernel parameter, passed by value).
struct StepConst {
  int I, iNa, iK;
  int zcode[kMaxIons];     // +1,-1,+2,-2 fast paths; 0 = generic z
  double z[kMaxIons];
  double zF[kMaxIons];     // z*F
  double sig_coef[kMaxIons]; // z^2 F^2 D_free 0.1 / (R T)
  double dgj_gs[kMaxIons]; // D_gj * gj_surface
  double F_RT;             // F / (R T)
  double dt, inv_cm, tm, gj_len;
  double inv_tm, inv_gj_len;  // 1/tm, 1/gj_len (IEEE divisions on the host: the bits a device division gives)
  double gj_block;
  double inv_KmNa, inv_KmK, atp_term; // 1/Km, (cATP/KmATP)
  double atp_den;          // 1 + cATP/KmATP
  double qnum_c;           // (cADP*1e-3)*(cPi*1e-3)
  double qden_c;           // cATP*1e-3
  double K0;               // exp(-deltaGATP / (R T))
  int vgj;                 // voltage-gated gap junctions: gjopen is state (p.gjo)
  double gj_vth, gj_min, gj_dt_ms;   // threshold (mV), closed fraction, dt in ms
  int iCa;                 // Ca-ATPase ion row, -1 = pump off
  double ca_alpha;         // alpha_Ca
  double ca_inv_Km;        // 1/KmCa_Ca
  double ca_atp_term;      // cATP/KmCa_ATP
  double ca_atp_den;       // 1 + cATP/KmCa_ATP
  double ca_qnum_c;        // cADP*cPi
  double ca_qden_c;        // cATP
  int polar;               // cell polarizability != 0: the implicit Vmem update of update_V
  double cm;               // membrane capacitance
  double true_ratio;       // true_cell_size / cell_radius
};

// Harris et al. (1983) gap-junction gating constants (channels/gap_junction.py:26-31)
constexpr double kGjLambda = 0.0013, kGjA1 = 0.077, kGjA2 = 0.14;

struct StepPtrs {
  const double* vm_in;  double* vm_out;
  const double* ccm_in; double* ccm_out;   // [I][C] membrane-side concentrations
  double* cc;                              // [I][C] cell concentrations (in place)
  const double* Dm;                        // [I][M] FP64 (plain form)
  const float* Dm_f;                       // [I][M] FP32 (split form)
  const double* cenv;                      // [ncl][I] (no ECM) or [I][G] (ECM)
  const double* pump_coef;                 // [ncl] -3 block alpha_NaK (0 = pump off)
  const double* phib;                      // [G] or nullptr
  double* env_part;                        // [nblk][I] partial sums (no ECM)
  double* mem_flux_sa;                     // [I][M] f_mem*sa (ECM scatter input)
  unsigned long long* status;              // [4]: nan_vm, nan_conc, neg clamps, spare
  double* gjo;                             // [M] gap-junction open fraction (vgj), in place
  const double* ca_env;                    // [G] Ca2+ of the environment after this step's
                                           // Nernst-Planck update (ECM with the Ca-ATPase)
  // outputs (OUT variant)
  double* o_fmem; double* o_fgj; double* o_rate; double* o_rho; double* o_Jn;
  double* o_Imem; double* o_Jcx; double* o_Jcy; double* o_Jc; double* o_vmave;
  double* o_dvm; double* o_Ecx; double* o_Ecy; double* o_Emc; double* o_Egjx;
  double* o_Egjy; double* o_gjopen; double* o_sigma;
};

// ---------------------------------------------------------------------------
// math helpers
// ---------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ T bx_expm1(T x);
template <> __device__ __forceinline__ double bx_expm1<double>(double x) { return expm1(x); }
template <> __device__ __forceinline__ float bx_expm1<float>(float x) { return expm1f(x); }
template <typename T> __device__ __forceinline__ T bx_exp(T x);
template <> __device__ __forceinline__ double bx_exp<double>(double x) { return exp(x); }
template <> __device__ __forceinline__ float bx_exp<float>(float x) { return expf(x); }

// Shared exponentials of one GHK voltage: alpha1 = (v + nonce) F/(RT) for a
// unit charge; every |z| in {1,2} flux is derived from expm1(-alpha1).
template <typename T>
struct GhkShared {
  T a1, em1, e1, r, q2;
  __device__ __forceinline__ void init(double v_nonce, double F_RT) {
    a1 = (T)(v_nonce * F_RT);
    em1 = bx_expm1<T>(-a1);         // expm1(-alpha1)
    e1 = (T)1 + em1;                // exp(-alpha1)
    r = (T)1 / em1;
    q2 = (T)1 / ((T)2 + em1);
  }
};

// GHK flux of sim_toolbox.electroflux (sim_toolbox.py:18-69) for charge z,
// written in terms of the shared exponentials:
//   f = -(Dc*alpha/d) * (cB - cA*exp(-alpha)) / (-expm1(-alpha)),
//   alpha = z*alpha1.  Exact identities give, with e1 = exp(-alpha1),
//   em1 = expm1(-alpha1):
//   z=+1: (Dc a1/d)(cB - cA e1)/em1          z=-1: (Dc a1/d)(cB e1 - cA)/em1
//   z=+2: 2(Dc a1/d)(cB - cA e1^2)/(em1(2+em1))
//   z=-2: 2(Dc a1/d)(cB e1^2 - cA)/(em1(2+em1))
template <typename T>
__device__ __forceinline__ T ghk_flux(const GhkShared<T>& s, int zcode, double zval,
                                      double v_nonce, double F_RT, T cA, T cB, T Dc, T inv_d) {
  const T k = Dc * s.a1 * inv_d;
  switch (zcode) {
    case 1:  return k * (cB - cA * s.e1) * s.r;
    case -1: return k * (cB * s.e1 - cA) * s.r;
    case 2:  { T e2 = s.e1 * s.e1; return (T)2 * k * (cB - cA * e2) * s.r * s.q2; }
    case -2: { T e2 = s.e1 * s.e1; return (T)2 * k * (cB * e2 - cA) * s.r * s.q2; }
    default: {
      // generic charge: ((z + nonce) * vBA * F) / (R T), then the formula as is
      T a = (T)(((zval + kNonce) * v_nonce) * F_RT);
      T ea = bx_exp<T>(-a);
      T den = -bx_expm1<T>(-a);
      return -((Dc * a) * inv_d) * ((cB - cA * ea) / den);
    }
  }
}

// Na/K-ATPase (sim_toolbox.pumpNaKATP, sim_toolbox.py:71-122), rearranged to
// one division: f_Na = -3 block alpha fwd (1 - Q/Keq) with Keq = K0/e1,
// e1 = exp(-F V/(R T)) shared with the GHK fluxes.
template <typename T>
__device__ __forceinline__ T pump_fna(const StepConst& k, T pcoef, T e1, T cNai, T cNao, T cKi, T cKo) {
  const T nai = cNai * (T)1e-3, nao = cNao * (T)1e-3, ki = cKi * (T)1e-3, ko = cKo * (T)1e-3;
  const T qnum = (T)k.qnum_c * (nao * nao * nao) * (ki * ki);
  T qden = (T)k.qden_c * (nai * nai * nai) * (ko * ko);
  if (qden == (T)0) qden = (T)1.0e-15;
  const T xna = cNai * (T)k.inv_KmNa, xk = cKo * (T)k.inv_KmK;
  const T na3 = xna * xna * xna, k2 = xk * xk;
  const T num_e = na3 * k2 * (T)k.atp_term;
  const T den_e = ((T)1 + na3) * ((T)1 + k2) * (T)k.atp_den;
  // fwd * (1 - Q/Keq) = num_e (qden K0 - qnum e1) / (den_e qden K0)
  const T K0 = (T)k.K0;
  return pcoef * num_e * (qden * K0 - qnum * e1) / (den_e * qden * K0);
}

// pumpCaATP (sim_toolbox.py:124-180), into the cell positive:
// -alpha_Ca fwd (1 - Q/Keq) with Q = cADP cPi cCao / (cATP cCai) (1e-16 for a
// zero denominator) and Keq = exp(-(dG/RT - 2 F Vm/RT)) = K0 / e1^2.
// The reference clamps both concentrations at zero first (no_negs).
template <typename T>
__device__ __forceinline__ T pump_fca(const StepConst& k, T e1, T cCai, T cCao) {
  cCai = cCai > (T)0 ? cCai : (T)0;
  cCao = cCao > (T)0 ? cCao : (T)0;
  const T qnum = (T)k.ca_qnum_c * cCao;
  T qden = (T)k.ca_qden_c * cCai;
  if (qden == (T)0) qden = (T)1.0e-16;
  const T x = cCai * (T)k.ca_inv_Km;
  const T num_e = x * (T)k.ca_atp_term;
  const T den_e = ((T)1 + x) * (T)k.ca_atp_den;
  const T K0 = (T)k.K0;
  return -(T)k.ca_alpha * num_e * (qden * K0 - qnum * (e1 * e1)) / (den_e * qden * K0);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// The fused cell step.  TPB threads = TPB membrane slots of one CTA.
//   T   : arithmetic type of fluxes and pumps (double: plain, float: split)
//   ECM : extracellular grid on (env gathered per membrane, f*sa exported)
//   OUT : also compute the step outputs BETSE stores
//   PHIB: subtract the boundary potential Phi_b[map_mem2ecm]
// ---------------------------------------------------------------------------
template <typename T, int TPB, bool ECM, bool OUT, bool PHIB>
__global__ void __launch_bounds__(TPB)
k_cell_step(DevGeom g, StepPtrs p, StepConst k) {
  extern __shared__ double smem[];
  const int I = k.I;
  double* sA = smem;                    // [I][TPB] f_mem*sa
  double* sB = sA + I * TPB;            // [I][TPB] -f_gj*sa
  double* sV = sB + I * TPB;            // [TPB]   per-cell Vmem (by local cell)
  double* sX = sV + TPB;                // [4][TPB] output scratch; [7][TPB] with polarizability

  const int b = blockIdx.x;
  const int c0 = g.blk_cell[b], c1 = g.blk_cell[b + 1];
  const int cl = g.blk_cluster[b];
  const double* cenv_cl = ECM ? p.cenv : p.cenv + (size_t)cl * I;
  const int m0 = g.cell_ptr[c0], m1 = g.cell_ptr[c1];
  const int t = threadIdx.x;
  const int m = m0 + t;
  const bool active = m < m1;
  const T inv_tm = (T)k.inv_tm;
  const T inv_gjl = (T)k.inv_gj_len;

  double env_acc[kMaxIons];
#pragma unroll
  for (int i = 0; i < kMaxIons; ++i) env_acc[i] = 0.0;

  double v = 0.0, vgj = 0.0;
  double Jraw_p = 0.0;                    // polarizability: -sum z F f_mem + sum z F f_gj
  int c = 0, lc = 0;
  T fmem_o[kMaxIons], fgj_o[kMaxIons];
  T rate_o = (T)0;
  if (active) {
    v = p.vm_in[m];
    c = g.m2c[m];
    lc = c - c0;
    const int nn = g.nn[m];
    const int cn = g.nn_cell[m];
    const double vn = p.vm_in[nn];
    const bool bnd = g.bflag[m] != 0;
    // BETSE adds 1e-25 to vm in place in each electroflux call (sim_toolbox.py:54);
    // for |vm| > 1e-8 V the addition is below one ulp, so every ion sees v1.
    const double v1 = v + kNonce;
    vgj = (vn + kNonce) - v1;                   // update_gj, sim.py:2166
    const double vgj1 = vgj + kNonce;
    GhkShared<T> sm, sg;
    sm.init(v1, k.F_RT);
    sg.init(vgj1, k.F_RT);
    double msa;
    T msa_t, gjw_t;
    if constexpr (sizeof(T) == 8) { msa = g.mem_sa[m]; msa_t = (T)msa; gjw_t = (T)g.gj_w[m]; }
    else { msa_t = (T)g.mem_sa_f[m]; msa = (double)msa_t; gjw_t = (T)g.gj_w_f[m]; }
    const int ge = ECM ? g.map_env[m] : 0;

    // Na/K-ATPase first, on the start-of-step concentrations (sim.py:1196-1234)
    T fNa = (T)0;
    const double pcoef = p.pump_coef[cl];
    if (pcoef != 0.0) {
      const T cNai = (T)p.ccm_in[k.iNa * g.C + c];
      const T cKi = (T)p.ccm_in[k.iK * g.C + c];
      const T cNao = (T)(ECM ? cenv_cl[k.iNa * g.G + ge] : cenv_cl[k.iNa]);
      const T cKo = (T)(ECM ? cenv_cl[k.iK * g.G + ge] : cenv_cl[k.iK]);
      // the pump sees vm before any nonce (it runs before the ion loop);
      // e1 of v1 equals exp(-F vm/(R T)) for |vm| > 1e-8 V
      fNa = pump_fna<T>(k, (T)pcoef, sm.e1, cNai, cNao, cKi, cKo);
    }
    rate_o = -fNa;
    // Gap_Junction.run (channels/gap_junction.py:52-81): alpha, beta from
    // |vgj| in mV; one implicit-Euler update per ion, as update_gj calls it
    // once per ion (sim.py:2181-2183), each before that ion's flux
    double gg = 0.0, ga = 0.0, gr = 0.0;
    double jm = 0.0, jg = 0.0;
    if (k.vgj) {
      const double V1 = 1.0e3 * fabs(vgj);
      const double al = kGjLambda * exp(-kGjA1 * (V1 - k.gj_vth));
      double be = kGjLambda * exp(kGjA2 * (V1 - k.gj_vth));
      be = be / (1.0 + 50.0 * be);
      ga = k.gj_dt_ms * (al + be * k.gj_min);
      gr = 1.0 / (1.0 + al * k.gj_dt_ms + be * k.gj_dt_ms);
      gg = p.gjo[m];
    }
    for (int i = 0; i < I; ++i) {
      const T cin = (T)p.ccm_in[i * g.C + c];
      const T cout = (T)(ECM ? cenv_cl[i * g.G + ge] : cenv_cl[i]);
      T dm;
      if constexpr (sizeof(T) == 8) dm = (T)p.Dm[(size_t)i * g.M + m];
      else dm = p.Dm_f[(size_t)i * g.M + m];
      T f = ghk_flux<T>(sm, k.zcode[i], k.z[i], v1, k.F_RT, cout, cin, dm, inv_tm);
      if (i == k.iNa) f = fNa + f;
      else if (i == k.iK) f = (T)(-(2.0 / 3.0)) * fNa + f;
      if (i == k.iCa) {
        // ca_handler after the ion loop (sim.py:2126-2155): cell side is
        // cc_cells at the start of the step (update_intra), environment side
        // after this step's Nernst-Planck update with extracellular spaces
        const T cCao = (T)(ECM ? p.ca_env[ge] : cenv_cl[i]);
        f = f + pump_fca<T>(k, sm.e1, (T)p.cc[i * g.C + c], cCao);
      }
      // gap junction (sim.py:2189-2206): from this membrane's cell into the partner's
      const T cn_i = (T)p.ccm_in[i * g.C + cn];
      T dgj;
      if (k.vgj) {
        gg = k.gj_block * ((gg + ga) * gr);
        dgj = (T)(k.dgj_gs[i] * gg);
      } else {
        dgj = (T)k.dgj_gs[i] * (gjw_t * (T)k.gj_block);
      }
      T fg = ghk_flux<T>(sg, k.zcode[i], k.z[i], vgj1, k.F_RT, cin, cn_i, dgj, inv_gjl);
      if (bnd) fg = (T)0;
      const double a = (double)(f * msa_t);
      sA[i * TPB + t] = a;
      sB[i * TPB + t] = (double)(-fg * msa_t);
      if (ECM) p.mem_flux_sa[(size_t)i * g.M + m] = a;
      else env_acc[i] = a;
      if (OUT) { fmem_o[i] = f; fgj_o[i] = fg; }
      if (k.polar) { jm += k.zF[i] * (double)f; jg += k.zF[i] * (double)fg; }
    }
    if (k.vgj) p.gjo[m] = gg;
    if (k.polar) {
      Jraw_p = -jm + jg;                       // Jmem + Jgj (ion_current.py:22-28)
      sX[t] = Jraw_p * g.mem_sa[m];
    }
    (void)msa;
  } else {
    for (int i = 0; i < I; ++i) { sA[i * TPB + t] = 0.0; sB[i * TPB + t] = 0.0; }
    if (k.polar) sX[t] = 0.0;
  }

  // no-ECM well-mixed environment: per-CTA partial sums of f_mem*sa per ion
  if (!ECM) {
    __shared__ double red[kMaxIons][TPB / 32];
    for (int i = 0; i < I; ++i) {
      double s = warp_sum(env_acc[i]);
      if ((t & 31) == 0) red[i][t >> 5] = s;
    }
    __syncthreads();
    if (t < I) {
      double s = 0.0;
      for (int w = 0; w < TPB / 32; ++w) s += red[t][w];
      p.env_part[(size_t)b * I + t] = s;
    }
  }
  __syncthreads();

  // ---- cell phase: one thread per cell of this CTA (update_all_concs, update_V)
  const int ncell = c1 - c0;
  int bad_conc = 0, neg = 0;
  if (t < ncell) {
    const int cc = c0 + t;
    const int a0 = g.cell_ptr[cc] - m0, a1 = g.cell_ptr[cc + 1] - m0;
    // one FP64 division per cell: update_Co and the gap-junction term divide by
    // cell_vol per ion; multiplying by 1/vol differs by at most one rounding
    const double inv_vol = 1.0 / g.cell_vol[cc];
    double rho = 0.0, sig = 0.0;
    for (int i = 0; i < I; ++i) {
      double s1 = 0.0, s2 = 0.0;
      for (int j = a0; j < a1; ++j) { s1 += sA[i * TPB + j]; s2 += sB[i * TPB + j]; }
      double x = p.cc[i * g.C + cc] + (s1 * inv_vol) * k.dt;  // update_Co, sim_toolbox.py:1182-1183
      p.ccm_out[i * g.C + cc] = x;                            // cc_at_mem = cX_cell[mem_to_cells]
      x = x + k.dt * (s2 * inv_vol);                          // gap-junction term, sim.py:2105-2108
      if (x != x) bad_conc++;
      if (x < 0.0) { x = 0.0; neg++; }                        // no_negs
      p.cc[i * g.C + cc] = x;
      rho += k.zF[i] * x;                                     // rho_cells, ion_current.py:19
      if (OUT || k.polar) sig += k.sig_coef[i] * x;
    }
    const double vcell = k.inv_cm * (rho * g.diviterm[cc]);   // sim.py:2027-2029
    sV[t] = vcell;
    if (OUT) { p.o_rho[cc] = rho; p.o_sigma[cc] = sig / (double)I; }
    if (k.polar) {
      // Jn averaged over the cell (ion_current.py:31), sigma_cell (sim.py:2016-2017)
      double sj = 0.0;
      for (int j = a0; j < a1; ++j) sj += sX[j];
      sX[TPB + t] = sj / g.cell_sa[cc];
      sX[2 * TPB + t] = sig / (double)I;
    }
  }
  if (bad_conc) atomicAdd(&p.status[1], (unsigned long long)bad_conc);
  if (neg) atomicAdd(&p.status[2], (unsigned long long)neg);
  __syncthreads();

  // ---- membrane phase 2: new Vmem
  double vnew = 0.0;
  if (active) {
    if (k.polar) {
      // implicit polarizable form (sim.py:2048-2058): the smoothed Jn
      // (ion_current.py:33) charges the membrane while the cytoplasm relaxes
      // it towards the cell's charge potential; self.vm carries the I
      // in-place nonces of the ion loop
      const double Jn = g.sw_mem[m] * Jraw_p + sX[TPB + lc] * g.sw_o[m];
      const double sg = sX[2 * TPB + lc];
      double vold = v;
      for (int i = 0; i < I; ++i) vold += kNonce;
      const double R = g.R_rads[m];
      vnew = (vold - (k.dt / k.cm) * Jn + ((k.dt * sg * sV[lc]) / (k.cm * R))) /
             (1 + ((k.dt * sg) / (k.cm * R)));
    } else {
      vnew = sV[lc];
      if (PHIB) vnew -= p.phib[g.map_env[m]];
    }
    p.vm_out[m] = vnew;
    if (vnew != vnew) atomicAdd(&p.status[0], 1ull);
  }

  if constexpr (OUT) {
    if (k.polar) __syncthreads();      // phase 2 read the scratch rows the outputs reuse
    // fluxes, rate, Jn smoothing and cell currents (ion_current.py:19-47, sim.py:2031-2083)
    double Jraw = 0.0;
    if (active) {
      for (int i = 0; i < I; ++i) {
        p.o_fmem[(size_t)i * g.M + m] = (double)fmem_o[i];
        p.o_fgj[(size_t)i * g.M + m] = (double)fgj_o[i];
      }
      double Jmem = 0.0, Jgj = 0.0;
      for (int i = 0; i < I; ++i) { Jmem += k.zF[i] * (double)fmem_o[i]; Jgj += k.zF[i] * (double)fgj_o[i]; }
      Jraw = -Jmem + Jgj;
      p.o_rate[m] = (double)rate_o;
      const double Egj = -vgj / k.gj_len;
      p.o_Egjx[m] = Egj * g.mem_nx[m];
      p.o_Egjy[m] = Egj * g.mem_ny[m];
      p.o_gjopen[m] = k.vgj ? p.gjo[m] : k.gj_block * g.gj_w[m];
      sX[t] = Jraw * g.mem_sa[m];
      sX[TPB + t] = vnew;
    } else { sX[t] = 0.0; sX[TPB + t] = 0.0; }
    __syncthreads();
    if (t < ncell) {
      const int cc = c0 + t;
      const int a0 = g.cell_ptr[cc] - m0, a1 = g.cell_ptr[cc + 1] - m0;
      double s = 0.0, sv = 0.0;
      for (int j = a0; j < a1; ++j) { s += sX[j]; sv += sX[TPB + j]; }
      sV[t] = s / g.cell_sa[cc];              // Jn_ave
      p.o_vmave[cc] = sv / (double)(a1 - a0);
      if (k.polar) sX[4 * TPB + t] = sv / (double)(a1 - a0);
    }
    __syncthreads();
    double Jn = 0.0;
    if (active) {
      Jn = g.sw_mem[m] * Jraw + sV[lc] * g.sw_o[m];
      p.o_Jn[m] = Jn;
      p.o_Imem[m] = -Jn * g.mem_sa[m];
      sX[2 * TPB + t] = Jn * g.mem_nx[m] * g.mem_sa[m];
      sX[3 * TPB + t] = Jn * g.mem_ny[m] * g.mem_sa[m];
      double vmo = v;
      for (int i = 0; i < I; ++i) vmo += kNonce;
      p.o_dvm[m] = (vnew - vmo) / k.dt;
      if (k.polar) {
        // cell field from the membrane voltage profile (sim.py:2063-2074)
        const double gE = (vnew - sX[4 * TPB + lc]) / (g.R_rads[m] * k.true_ratio);
        sX[5 * TPB + t] = (-gE * g.mem_nx[m]) * g.mem_sa[m];
        sX[6 * TPB + t] = (-gE * g.mem_ny[m]) * g.mem_sa[m];
      }
    } else {
      sX[2 * TPB + t] = 0.0; sX[3 * TPB + t] = 0.0;
      if (k.polar) { sX[5 * TPB + t] = 0.0; sX[6 * TPB + t] = 0.0; }
    }
    __syncthreads();
    if (t < ncell) {
      const int cc = c0 + t;
      const int a0 = g.cell_ptr[cc] - m0, a1 = g.cell_ptr[cc + 1] - m0;
      double sx = 0.0, sy = 0.0;
      for (int j = a0; j < a1; ++j) { sx += sX[2 * TPB + j]; sy += sX[3 * TPB + j]; }
      const double jx = sx / g.cell_sa[cc], jy = sy / g.cell_sa[cc];
      p.o_Jcx[cc] = jx; p.o_Jcy[cc] = jy;
      const double sg = p.o_sigma[cc];
      double ex = jx / sg, ey = jy / sg;
      if (k.polar) {
        double gx = 0.0, gy = 0.0;
        for (int j = a0; j < a1; ++j) { gx += sX[5 * TPB + j]; gy += sX[6 * TPB + j]; }
        ex = gx / g.cell_sa[cc];
        ey = gy / g.cell_sa[cc];
      }
      p.o_Ecx[cc] = ex; p.o_Ecy[cc] = ey;
      sA[t] = jx; sA[TPB + t] = jy; sB[t] = ex; sB[TPB + t] = ey;
    }
    __syncthreads();
    if (active) {
      const double nx = g.mem_nx[m], ny = g.mem_ny[m];
      p.o_Jc[m] = sA[lc] * nx + sA[TPB + lc] * ny;
      p.o_Emc[m] = sB[lc] * nx + sB[TPB + lc] * ny;
    }
  }
}

// The well-mixed environment folded into the step: the last CTA of a
// cluster to finish (a ticket counter, reset by that CTA) adds the cluster's
// CTA partials in CTA order and updates its environment, as k_env_mix does.
struct EnvMix {
  double* cenv;               // [ncl][I]
  const int* cl_blk;          // [ncl + 1] first CTA of each cluster
  const double* env_scale;    // [ncl] dt / (vol_env M)
  unsigned* ticket;           // [ncl] zero between steps
};

// The plain FP64 step for small clusters.  On a 1.4k-membrane cluster
// k_cell_step spends ~3200 FP64-heavy instructions per thread on a few
// dozen SMs, and an FP64 warp instruction costs the same whatever the
// number of lanes it uses; here the work is spread and no lane idles:
//   A. four jobs per membrane, each in its own warp where the CTA has
//      four: the shared exponentials of the membrane voltage; those of the
//      gap-junction voltage; the Na/K-ATPase rate (with its own copy of
//      exp(-alpha1), the same bits); the geometry loads and 1/cell_vol of
//      the CTA's cells;
//   B. eight lanes per membrane slot, lane i = ion i: the transmembrane and
//      gap-junction GHK fluxes of that ion;
//   C. eight lanes per cell, lane i = ion i: the concentration update, and
//      the charge sum gathered in ion order by shuffles; then Vmem.
// The arithmetic of every flux and every (cell, ion) update is
// k_cell_step<double>'s in the same order; the environment partials add in
// slot order.  The configuration without extracellular spaces, outputs,
// Phi_b, gating, Ca-ATPase and polarizability; MB membrane slots per CTA,
// MB * 8 threads.
template <int MB>
__global__ void __launch_bounds__(MB * 8)
k_cell_step_ion(DevGeom g, StepPtrs p, StepConst k, EnvMix em) {
  __shared__ double sA[kMaxIons][MB];   // f_mem*sa
  __shared__ double sB[kMaxIons][MB];   // -f_gj*sa
  __shared__ double sV[MB];             // per-cell Vmem (by local cell)
  __shared__ double sh_m[5][MB], sh_g[5][MB];   // GhkShared {a1, em1, e1, r, q2} of vm and vgj
  __shared__ double sh_v1[MB], sh_vg1[MB], sh_na[MB], sh_sa[MB], sh_gw[MB];
  __shared__ double sh_ivol[MB];        // 1/cell_vol by local cell
  __shared__ int sh_c[MB], sh_cn[MB], sh_bnd[MB];
  __shared__ int s_last;
  const int I = k.I;
  const int b = blockIdx.x;
  const int c0 = g.blk_cell[b], c1 = g.blk_cell[b + 1];
  const int cl = g.blk_cluster[b];
  const double* cenv_cl = p.cenv + (size_t)cl * I;
  const int m0 = g.cell_ptr[c0], m1 = g.cell_ptr[c1];
  const int nmem = m1 - m0;
  const int t = threadIdx.x;

  // ---- A: job q of membrane slot e, q = entry / MP (one warp per job when MB <= 32)
  constexpr int MP = (MB + 31) / 32 * 32;
  const int ncell = c1 - c0;
  for (int entry = t; entry < 4 * MP; entry += MB * 8) {
    const int q = entry / MP, e = entry - q * MP;
    const int m = m0 + e;
    if (q < 3 && e >= nmem) continue;
    if (q == 0) {
      const double v1 = p.vm_in[m] + kNonce;
      GhkShared<double> sm;
      sm.init(v1, k.F_RT);
      sh_m[0][e] = sm.a1; sh_m[1][e] = sm.em1; sh_m[2][e] = sm.e1; sh_m[3][e] = sm.r; sh_m[4][e] = sm.q2;
      sh_v1[e] = v1;
    } else if (q == 1) {
      const double v1 = p.vm_in[m] + kNonce;
      const double vn = p.vm_in[g.nn[m]];
      const double vgj = (vn + kNonce) - v1;     // update_gj, sim.py:2166
      const double vgj1 = vgj + kNonce;
      GhkShared<double> sg;
      sg.init(vgj1, k.F_RT);
      sh_g[0][e] = sg.a1; sh_g[1][e] = sg.em1; sh_g[2][e] = sg.e1; sh_g[3][e] = sg.r; sh_g[4][e] = sg.q2;
      sh_vg1[e] = vgj1;
    } else if (q == 2) {
      double fNa = 0.0;
      const double pcoef = p.pump_coef[cl];
      if (pcoef != 0.0) {                        // Na/K-ATPase (sim.py:1196-1234)
        const int c = g.m2c[m];
        const double a1 = (p.vm_in[m] + kNonce) * k.F_RT;   // GhkShared::init's e1
        const double e1 = 1.0 + bx_expm1<double>(-a1);
        fNa = pump_fna<double>(k, pcoef, e1, p.ccm_in[k.iNa * g.C + c], cenv_cl[k.iNa],
                               p.ccm_in[k.iK * g.C + c], cenv_cl[k.iK]);
      }
      sh_na[e] = fNa;
    } else {
      if (e < nmem) {
        sh_sa[e] = g.mem_sa[m];
        sh_gw[e] = g.gj_w[m];
        sh_c[e] = g.m2c[m];
        sh_cn[e] = g.nn_cell[m];
        sh_bnd[e] = g.bflag[m] != 0;
      }
      if (e < ncell) sh_ivol[e] = 1.0 / g.cell_vol[c0 + e];
    }
  }
  __syncthreads();

  // ---- B: lane i of slot s, ion i of membrane m0 + s
  const int slot = t >> 3, i = t & 7;
  if (slot < nmem && i < I) {
    const int m = m0 + slot;
    GhkShared<double> sm, sg;
    sm.a1 = sh_m[0][slot]; sm.em1 = sh_m[1][slot]; sm.e1 = sh_m[2][slot]; sm.r = sh_m[3][slot];
    sm.q2 = sh_m[4][slot];
    sg.a1 = sh_g[0][slot]; sg.em1 = sh_g[1][slot]; sg.e1 = sh_g[2][slot]; sg.r = sh_g[3][slot];
    sg.q2 = sh_g[4][slot];
    const int c = sh_c[slot], cn = sh_cn[slot];
    const double msa = sh_sa[slot];
    const double fNa = sh_na[slot];
    const double cin = p.ccm_in[i * g.C + c];
    const double cout = cenv_cl[i];
    const double dm = p.Dm[(size_t)i * g.M + m];
    double f = ghk_flux<double>(sm, k.zcode[i], k.z[i], sh_v1[slot], k.F_RT, cout, cin, dm, k.inv_tm);
    if (i == k.iNa) f = fNa + f;
    else if (i == k.iK) f = -(2.0 / 3.0) * fNa + f;
    const double cn_i = p.ccm_in[i * g.C + cn];
    const double dgj = k.dgj_gs[i] * (sh_gw[slot] * k.gj_block);
    double fg = ghk_flux<double>(sg, k.zcode[i], k.z[i], sh_vg1[slot], k.F_RT, cin, cn_i, dgj, k.inv_gj_len);
    if (sh_bnd[slot]) fg = 0.0;
    sA[i][slot] = f * msa;
    sB[i][slot] = -fg * msa;
  }
  __syncthreads();

  // ---- the CTA's environment partial of ion t, in slot order
  if (t < I) {
    double sum = 0.0;
    for (int j = 0; j < nmem; ++j) sum += sA[t][j];
    p.env_part[(size_t)b * I + t] = sum;
  }

  // ---- C: lane i of group c, ion i of cell c0 + c
  const int lc = t >> 3;
  double x = 0.0;
  if (lc < ncell && i < I) {
    const int cc = c0 + lc;
    const int a0 = g.cell_ptr[cc] - m0, a1 = g.cell_ptr[cc + 1] - m0;
    const double inv_vol = sh_ivol[lc];
    double s1 = 0.0, s2 = 0.0;
    for (int j = a0; j < a1; ++j) { s1 += sA[i][j]; s2 += sB[i][j]; }
    x = p.cc[i * g.C + cc] + (s1 * inv_vol) * k.dt;   // update_Co, sim_toolbox.py:1182-1183
    p.ccm_out[i * g.C + cc] = x;
    x = x + k.dt * (s2 * inv_vol);                    // gap-junction term, sim.py:2105-2108
    const bool bad = x != x;
    const bool neg = x < 0.0;
    if (neg) x = 0.0;                                 // no_negs
    p.cc[i * g.C + cc] = x;
    if (bad) atomicAdd(&p.status[1], 1ull);
    if (neg) atomicAdd(&p.status[2], 1ull);
  }
  // rho_cells (ion_current.py:19): the group's ions in ion order
  const int base = (t & 31) & ~7;
  double rho = 0.0;
  for (int j = 0; j < I; ++j) rho += k.zF[j] * __shfl_sync(0xffffffffu, x, base + j);
  if (lc < ncell && i == 0) sV[lc] = k.inv_cm * (rho * g.diviterm[c0 + lc]);   // sim.py:2027-2029
  __syncthreads();

  // ---- new Vmem, one lane per membrane
  if (t < nmem) {
    const double vnew = sV[sh_c[t] - c0];
    p.vm_out[m0 + t] = vnew;
    if (vnew != vnew) atomicAdd(&p.status[0], 1ull);
  }

  // ---- the last CTA of the cluster mixes the environment (sim_toolbox.py:1196-1205)
  if (t == 0) {
    __threadfence();
    const unsigned n_cl = (unsigned)(em.cl_blk[cl + 1] - em.cl_blk[cl]);
    s_last = atomicAdd(&em.ticket[cl], 1u) == n_cl - 1u;
  }
  __syncthreads();
  if (s_last) {
    // every thread adds a stride of CTA rows (all ions at once), then warps
    // reduce by shuffles and thread i adds the warps' sums of ion i in order
    __shared__ double s_w[kMaxIons][MB * 8 / 32];
    __threadfence();
    double acc[kMaxIons];
#pragma unroll
    for (int q = 0; q < kMaxIons; ++q) acc[q] = 0.0;
    for (int bb = em.cl_blk[cl] + t; bb < em.cl_blk[cl + 1]; bb += MB * 8)
#pragma unroll
      for (int q = 0; q < kMaxIons; ++q)
        if (q < I) acc[q] += __ldcg(p.env_part + (size_t)bb * I + q);
#pragma unroll
    for (int q = 0; q < kMaxIons; ++q) {
      const double w = warp_sum(acc[q]);
      if ((t & 31) == 0) s_w[q][t >> 5] = w;
    }
    __syncthreads();
    if (t < I) {
      double tot = 0.0;
      for (int w = 0; w < MB * 8 / 32; ++w) tot += s_w[t][w];
      em.cenv[(size_t)cl * I + t] = em.cenv[(size_t)cl * I + t] - tot * em.env_scale[cl];
    }
    if (t == 0) em.ticket[cl] = 0u;
  }
}

// No-ECM environment: the well-mixed value per cluster and ion
// (sim_toolbox.py:1196-1205) c_env <- mean_m(c_env - f_m sa_m / vol_env * dt);
// one CTA per cluster reduces its CTAs' partial sums in a fixed order.
static __global__ void k_env_mix(const double* __restrict__ part, const int* __restrict__ cl_blk, int I,
                                 double* cenv, const double* __restrict__ env_scale) {
  __shared__ double red[32];
  const int cl = blockIdx.x;
  const int b0 = cl_blk[cl], b1 = cl_blk[cl + 1];
  for (int i = 0; i < I; ++i) {
    double s = 0.0;
    for (int b = b0 + (int)threadIdx.x; b < b1; b += blockDim.x) s += part[(size_t)b * I + i];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
      cenv[(size_t)cl * I + i] = cenv[(size_t)cl * I + i] - tot * env_scale[cl];
    }
    __syncthreads();
  }
}

}  // namespace bx
