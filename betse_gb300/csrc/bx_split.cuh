// bx_split.cuh -- the FP32/FP64-split step without any FP64 arithmetic.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so this form keeps
// FP64 accuracy only where BETSE's physics needs it -- the cell
// concentrations and the charge sum behind Vmem -- and carries those as
// compensated FP32 pairs (hi + lo, about 48 significant bits) updated with
// error-free transformations (Knuth's TwoSum, Dekker/FMA TwoProd).  Fluxes and
// pumps are plain FP32.
//
// State in HBM (structure of arrays, row = ion):
//   cc2[I][C]      float2  cell concentrations (hi, lo), owned by one CTA
//   ccm[2][I][C]   float   membrane-side concentration (BETSE's cc_at_mem,
//                          cell value + membrane term before the GJ term)
//   vcell[2][C]    float   Vmem of each cell (BETSE's vm is constant over a
//                          cell's membranes when cell_polarizability == 0;
//                          Phi_b, if any, is subtracted per membrane)
//   Dm[I][M]       float   channel diffusivities
//   per membrane   nn_cell (int32), lcell (u8: cell index within the CTA),
//                  mem_sa, gjw (float; gjw = 0 on boundary membranes)
//   per cell       dt/cell_vol, diviterm/cm (float), cell_mem_ptr (int32)
//   per CTA        cluster id; per cluster the well-mixed environment and the
//                  pump constant (batched parameter sweeps share one launch)
#pragma once
#include "bx_kernels.cuh"

namespace bx {

struct df { float hi, lo; };

// TwoSum-based add of a float to a double-float, renormalised.
__device__ __forceinline__ df df_add_f(df a, float b) {
  const float s = __fadd_rn(a.hi, b);
  const float bb = __fsub_rn(s, a.hi);
  const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  const float lo = __fadd_rn(a.lo, err);
  const float hi = __fadd_rn(s, lo);
  return df{hi, __fsub_rn(lo, __fsub_rn(hi, s))};
}

// double-float + double-float (accurate to a few ulp of 2^-48)
__device__ __forceinline__ df df_add(df a, df b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  const float lo = __fadd_rn(__fadd_rn(a.lo, b.lo), err);
  const float hi = __fadd_rn(s, lo);
  return df{hi, __fsub_rn(lo, __fsub_rn(hi, s))};
}

// double-float k times double-float x; k.hi*x.hi split exactly by FMA
__device__ __forceinline__ df df_mul(df x, float khi, float klo) {
  const float p = __fmul_rn(khi, x.hi);
  const float e = __fmaf_rn(khi, x.hi, -p);
  const float lo = __fmaf_rn(khi, x.lo, __fmaf_rn(klo, x.hi, e));
  const float hi = __fadd_rn(p, lo);
  return df{hi, __fsub_rn(lo, __fsub_rn(hi, p))};
}

// FP32 GHK flux (same identities as ghk_flux); the generic-charge branch
// evaluates BETSE's formula directly in FP32.
__device__ __forceinline__ float ghk_flux_f(const GhkShared<float>& s, int zcode, float zval,
                                            float v_nonce, float F_RT, float cA, float cB,
                                            float Dc, float inv_d) {
  const float kk = Dc * s.a1 * inv_d;
  switch (zcode) {
    case 1:  return kk * (cB - cA * s.e1) * s.r;
    case -1: return kk * (cB * s.e1 - cA) * s.r;
    case 2:  { const float e2 = s.e1 * s.e1; return 2.f * kk * (cB - cA * e2) * s.r * s.q2; }
    case -2: { const float e2 = s.e1 * s.e1; return 2.f * kk * (cB * e2 - cA) * s.r * s.q2; }
    default: {
      const float a = ((zval + 1.0e-25f) * v_nonce) * F_RT;
      return -((Dc * a) * inv_d) * ((cB - cA * expf(-a)) / (-expm1f(-a)));
    }
  }
}

struct SplitGeom {
  int C, M, I, G;
  const int* cell_ptr;      // [C+1]
  const int* nn_cell;       // [M]
  const uint8_t* lcell;     // [M]
  const float* mem_sa;      // [M]
  const float* gjw;         // [M]  (0 on boundary membranes)
  const float* dtv;         // [C]  dt / cell_vol
  const float* dvc;         // [C]  diviterm / cm
  const int* blk_cell;      // [nblk+1]
  const int* blk_cluster;   // [nblk]
  const int* map_env;       // [M]  (PHIB only)
  const int* nn;            // [M]  (PHIB only)
};

struct SplitConst {
  int I, iNa, iK;
  int zcode[kMaxIons];
  float z[kMaxIons];
  float zF_hi[kMaxIons];    // z F as a double-float (hi + lo)
  float zF_lo[kMaxIons];
  float dgj_gs[kMaxIons];
  float F_RT;
  float inv_tm, inv_gjl, gj_block;
  float inv_KmNa, inv_KmK, atp_term, atp_den, qnum_c, qden_c, K0;
};

struct SplitPtrs {
  const float* vc_in; float* vc_out;    // [C]
  const float* ccm_in; float* ccm_out;  // [I][C]
  float2* cc2;                          // [I][C]
  const float* Dm;                      // [I][M]
  const float* cenv_f;                  // [ncl][I] FP32 copy of the environment
  const float* pump_coef;               // [ncl] -3 block alpha_NaK (0 = pump off)
  const float* phib;                    // [G] (PHIB)
  float* env_part;                      // [nblk][I]
  unsigned long long* status;           // nan_vm, nan_conc, neg clamps
  // outputs (OUT)
  double* o_fmem; double* o_fgj; double* o_rate; double* o_rho; double* o_vmem;
};

template <int TPB, bool OUT, bool PHIB>
__global__ void __launch_bounds__(TPB)
k_split_step(SplitGeom g, SplitPtrs p, SplitConst k) {
  __shared__ float sA[kMaxIons][TPB];
  __shared__ float sB[kMaxIons][TPB];
  __shared__ float red[kMaxIons][TPB / 32];
  const int I = k.I;
  const int b = blockIdx.x;
  const int c0 = g.blk_cell[b], c1 = g.blk_cell[b + 1];
  const int cl = g.blk_cluster[b];
  const int m0 = g.cell_ptr[c0], m1 = g.cell_ptr[c1];
  const int t = threadIdx.x;
  const int m = m0 + t;
  const bool active = m < m1;
  float env_acc[kMaxIons];
#pragma unroll
  for (int i = 0; i < kMaxIons; ++i) env_acc[i] = 0.f;

  if (active) {
    const int c = c0 + g.lcell[m];
    const int cn = g.nn_cell[m];
    float v = p.vc_in[c];
    float vn = p.vc_in[cn];
    if (PHIB) { v -= p.phib[g.map_env[m]]; vn -= p.phib[g.map_env[g.nn[m]]]; }
    // BETSE's 1e-25 nonces (sim_toolbox.py:52-56) keep alpha != 0 at zero volts
    const float v1 = v + 1.0e-25f;
    const float vgj1 = ((vn + 1.0e-25f) - v1) + 1.0e-25f;
    GhkShared<float> sm, sg;
    sm.a1 = v1 * k.F_RT;
    sm.em1 = expm1f(-sm.a1); sm.e1 = 1.f + sm.em1; sm.r = 1.f / sm.em1; sm.q2 = 1.f / (2.f + sm.em1);
    sg.a1 = vgj1 * k.F_RT;
    sg.em1 = expm1f(-sg.a1); sg.e1 = 1.f + sg.em1; sg.r = 1.f / sg.em1; sg.q2 = 1.f / (2.f + sg.em1);
    const float sa = g.mem_sa[m];
    const float gw = g.gjw[m] * k.gj_block;
    const float* ce = p.cenv_f + (size_t)cl * I;
    float fNa = 0.f;
    const float pc = p.pump_coef[cl];
    if (pc != 0.f) {
      // pumpNaKATP (sim_toolbox.py:71-122), one division
      const float cNai = p.ccm_in[k.iNa * g.C + c], cKi = p.ccm_in[k.iK * g.C + c];
      const float cNao = ce[k.iNa], cKo = ce[k.iK];
      const float nai = cNai * 1e-3f, nao = cNao * 1e-3f, ki = cKi * 1e-3f, ko = cKo * 1e-3f;
      const float qnum = k.qnum_c * (nao * nao * nao) * (ki * ki);
      float qden = k.qden_c * (nai * nai * nai) * (ko * ko);
      if (qden == 0.f) qden = 1.0e-15f;
      const float xna = cNai * k.inv_KmNa, xk = cKo * k.inv_KmK;
      const float na3 = xna * xna * xna, k2 = xk * xk;
      const float num_e = na3 * k2 * k.atp_term;
      const float den_e = (1.f + na3) * (1.f + k2) * k.atp_den;
      fNa = pc * num_e * (qden * k.K0 - qnum * sm.e1) / (den_e * qden * k.K0);
    }
#pragma unroll
    for (int i = 0; i < kMaxIons; ++i) {
      if (i >= I) break;
      const float cin = p.ccm_in[i * g.C + c];
      const float dm = p.Dm[(size_t)i * g.M + m];
      float f = ghk_flux_f(sm, k.zcode[i], k.z[i], v1, k.F_RT, ce[i], cin, dm, k.inv_tm);
      if (i == k.iNa) f = fNa + f;
      else if (i == k.iK) f = (-(2.f / 3.f)) * fNa + f;
      const float cn_i = p.ccm_in[i * g.C + cn];
      const float fg = ghk_flux_f(sg, k.zcode[i], k.z[i], vgj1, k.F_RT, cin, cn_i,
                                  k.dgj_gs[i] * gw, k.inv_gjl);
      const float a = f * sa;
      sA[i][t] = a;
      sB[i][t] = -fg * sa;
      env_acc[i] = a;
      if (OUT) {
        p.o_fmem[(size_t)i * g.M + m] = (double)f;
        p.o_fgj[(size_t)i * g.M + m] = (double)fg;
      }
    }
    if (OUT) p.o_rate[m] = (double)(-fNa);
  } else {
    for (int i = 0; i < I; ++i) { sA[i][t] = 0.f; sB[i][t] = 0.f; }
  }
  // per-CTA partial sums of f_mem*sa per ion for the well-mixed environment
#pragma unroll
  for (int i = 0; i < kMaxIons; ++i) {
    if (i >= I) break;
    float s = env_acc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((t & 31) == 0) red[i][t >> 5] = s;
  }
  __syncthreads();
  if (t < I) {
    float s = 0.f;
    for (int w = 0; w < TPB / 32; ++w) s += red[t][w];
    p.env_part[(size_t)b * I + t] = s;
  }

  // cell phase: update_all_concs + update_V for the CTA's cells
  const int ncell = c1 - c0;
  if (t < ncell) {
    const int c = c0 + t;
    const int a0 = g.cell_ptr[c] - m0, a1 = g.cell_ptr[c + 1] - m0;
    const float dtv = g.dtv[c];
    df rho{0.f, 0.f};
    int bad = 0, neg = 0;
    for (int i = 0; i < I; ++i) {
      float s1 = 0.f, s2 = 0.f;
      for (int j = a0; j < a1; ++j) { s1 += sA[i][j]; s2 += sB[i][j]; }
      const float2 x2 = p.cc2[i * g.C + c];
      df x{x2.x, x2.y};
      x = df_add_f(x, s1 * dtv);                         // update_Co
      p.ccm_out[i * g.C + c] = x.hi + x.lo;              // cc_at_mem (pre-GJ)
      x = df_add_f(x, s2 * dtv);                         // gap-junction term
      if (x.hi != x.hi) bad++;
      if (x.hi < 0.f || (x.hi == 0.f && x.lo < 0.f)) { x = df{0.f, 0.f}; neg++; }   // no_negs
      p.cc2[i * g.C + c] = make_float2(x.hi, x.lo);
      rho = df_add(rho, df_mul(x, k.zF_hi[i], k.zF_lo[i]));   // rho_cells = sum z F c
    }
    const float vc = (rho.hi + rho.lo) * g.dvc[c];      // vm = rho diviterm / cm
    p.vc_out[c] = vc;
    if (vc != vc) atomicAdd(&p.status[0], 1ull);
    if (bad) atomicAdd(&p.status[1], (unsigned long long)bad);
    if (neg) atomicAdd(&p.status[2], (unsigned long long)neg);
    if (OUT) { p.o_rho[c] = (double)rho.hi + (double)rho.lo; p.o_vmem[c] = (double)vc; }
  }
}

// Well-mixed environment per cluster (sim_toolbox.py:1196-1205): one CTA per
// cluster reduces its CTAs' partial sums in a fixed order; FP64 master copy,
// FP32 copy for the flux kernel.
static __global__ void k_split_env_mix(const float* __restrict__ part, const int* __restrict__ cl_blk,
                                       int I, double* cenv64, float* cenv_f,
                                       const double* __restrict__ env_scale) {
  __shared__ double red[32];
  const int cl = blockIdx.x;
  const int b0 = cl_blk[cl], b1 = cl_blk[cl + 1];
  for (int i = 0; i < I; ++i) {
    double s = 0.0;
    for (int b = b0 + threadIdx.x; b < b1; b += blockDim.x) s += (double)part[(size_t)b * I + i];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
      const double v = cenv64[(size_t)cl * I + i] - tot * env_scale[cl];
      cenv64[(size_t)cl * I + i] = v;
      cenv_f[(size_t)cl * I + i] = (float)v;
    }
    __syncthreads();
  }
}

// Step outputs of the split form that BETSE stores at sampled steps
// (ion_current.py:19-47, sim.py:2031-2083, 2166-2174), derived on the GPU
// from the output step's fluxes and the new state.  Runs only on output
// steps, so it computes in FP64.
struct SplitOutGeom {
  int C, M, I;
  const int* cell_ptr; const int* blk_cell; const int* nn; const int* map_env;
  const double* mem_sa; const double* nx; const double* ny; const double* sw_mem;
  const double* sw_o; const double* cell_sa; const double* gj_w; const uint8_t* bflag;
};
struct SplitOutPtrs {
  const double* fmem; const double* fgj; const float* vc_new; const float* vc_old;
  const float2* cc2; const float* phib;
  double* Jn; double* Imem; double* Jcx; double* Jcy; double* Jc; double* vmave; double* dvm;
  double* Ecx; double* Ecy; double* Emc; double* Egjx; double* Egjy; double* gjopen; double* sigma;
  double* vm_mem;
};
struct SplitOutConst {
  int I; double zF[kMaxIons]; double sig_coef[kMaxIons]; double dt; double gj_len; double gj_block;
};

template <int TPB>
__global__ void __launch_bounds__(TPB)
k_split_outputs(SplitOutGeom g, SplitOutPtrs p, SplitOutConst k) {
  __shared__ double sX[4][TPB];
  __shared__ double sC[4][TPB];
  const int b = blockIdx.x;
  const int c0 = g.blk_cell[b], c1 = g.blk_cell[b + 1];
  const int m0 = g.cell_ptr[c0], m1 = g.cell_ptr[c1];
  const int t = threadIdx.x, m = m0 + t, ncell = c1 - c0;
  const bool active = m < m1;
  int lc = 0;
  double Jraw = 0.0, vm = 0.0;
  if (active) {
    int lo = 0, hi = ncell - 1;                       // cell of m within the CTA
    while (lo < hi) { const int mid = (lo + hi + 1) >> 1; if (g.cell_ptr[c0 + mid] <= m) lo = mid; else hi = mid - 1; }
    lc = lo;
    const int c = c0 + lc;
    double Jm = 0.0, Jg = 0.0;
    for (int i = 0; i < k.I; ++i) { Jm += k.zF[i] * p.fmem[(size_t)i * g.M + m]; Jg += k.zF[i] * p.fgj[(size_t)i * g.M + m]; }
    Jraw = -Jm + Jg;
    const double ph = p.phib ? (double)p.phib[g.map_env[m]] : 0.0;
    vm = (double)p.vc_new[c] - ph;
    p.vm_mem[m] = vm;
    sX[0][t] = Jraw * g.mem_sa[m];
    sX[1][t] = vm;
  } else { sX[0][t] = 0.0; sX[1][t] = 0.0; }
  __syncthreads();
  if (t < ncell) {
    const int c = c0 + t;
    const int a0 = g.cell_ptr[c] - m0, a1 = g.cell_ptr[c + 1] - m0;
    double s = 0.0, sv = 0.0;
    for (int j = a0; j < a1; ++j) { s += sX[0][j]; sv += sX[1][j]; }
    sC[0][t] = s / g.cell_sa[c];
    p.vmave[c] = sv / (double)(a1 - a0);
    double sig = 0.0;
    for (int i = 0; i < k.I; ++i) { const float2 x = p.cc2[i * g.C + c]; sig += k.sig_coef[i] * ((double)x.x + (double)x.y); }
    sig /= (double)k.I;
    p.sigma[c] = sig;
    sC[3][t] = sig;
  }
  __syncthreads();
  if (active) {
    const double Jn = g.sw_mem[m] * Jraw + sC[0][lc] * g.sw_o[m];
    p.Jn[m] = Jn;
    p.Imem[m] = -Jn * g.mem_sa[m];
    sX[2][t] = Jn * g.nx[m] * g.mem_sa[m];
    sX[3][t] = Jn * g.ny[m] * g.mem_sa[m];
    const int c = c0 + lc;
    double vmo = (double)p.vc_old[c] - (p.phib ? (double)p.phib[g.map_env[m]] : 0.0);
    for (int i = 0; i < k.I; ++i) vmo += kNonce;
    p.dvm[m] = (vm - vmo) / k.dt;
  } else { sX[2][t] = 0.0; sX[3][t] = 0.0; }
  __syncthreads();
  if (t < ncell) {
    const int c = c0 + t;
    const int a0 = g.cell_ptr[c] - m0, a1 = g.cell_ptr[c + 1] - m0;
    double sx = 0.0, sy = 0.0;
    for (int j = a0; j < a1; ++j) { sx += sX[2][j]; sy += sX[3][j]; }
    const double jx = sx / g.cell_sa[c], jy = sy / g.cell_sa[c];
    p.Jcx[c] = jx; p.Jcy[c] = jy;
    p.Ecx[c] = jx / sC[3][t]; p.Ecy[c] = jy / sC[3][t];
    sC[1][t] = jx; sC[2][t] = jy;
  }
  __syncthreads();
  if (active) {
    const int c = c0 + lc;
    const double nxm = g.nx[m], nym = g.ny[m];
    p.Jc[m] = sC[1][lc] * nxm + sC[2][lc] * nym;
    p.Emc[m] = (sC[1][lc] / sC[3][lc]) * nxm + (sC[2][lc] / sC[3][lc]) * nym;
    (void)c;
    p.gjopen[m] = k.gj_block * g.gj_w[m];
  }
}

// E_gj needs the partner's Vmem: a separate pass over membranes.
__global__ void k_split_egj(int M, const int* __restrict__ nn, const double* __restrict__ vm_mem,
                            const double* __restrict__ nx, const double* __restrict__ ny,
                            double gj_len, double* Egjx, double* Egjy) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  const double v1 = vm_mem[m] + kNonce;
  const double vgj = (vm_mem[nn[m]] + kNonce) - v1;
  const double E = -vgj / gj_len;
  Egjx[m] = E * nx[m];
  Egjy[m] = E * ny[m];
}

}  // namespace bx
