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

// expm1 in FP32 from its Taylor series: x + x^2/2! + ... + x^7/7! for
// |x| < 0.5 (truncation below 2e-8 relative), exp(x) - 1 with the MUFU
// exponential above, where the cancellation factor e^x/(e^x - 1) is at most
// 2.6.  Accurate to a few 1e-7 relative -- the FP32 flux budget of the split
// form -- at a fraction of the instructions of the libm expm1f.
__device__ __forceinline__ float expm1_split(float x) {
  if (fabsf(x) < 0.5f) {
    float p = 1.0f / 5040.0f;
    p = fmaf(p, x, 1.0f / 720.0f);
    p = fmaf(p, x, 1.0f / 120.0f);
    p = fmaf(p, x, 1.0f / 24.0f);
    p = fmaf(p, x, 1.0f / 6.0f);
    p = fmaf(p, x, 0.5f);
    return fmaf(p * x, x, x);
  }
  return __expf(x) - 1.0f;
}

// Shared exponentials of one voltage for the split form; ka1 = alpha1 / d.
__device__ __forceinline__ void ghk_init_f(GhkShared<float>& s, float v_nonce, float F_RT) {
  s.a1 = v_nonce * F_RT;
  s.em1 = expm1_split(-s.a1);
  s.e1 = 1.f + s.em1;
  s.r = __fdividef(1.f, s.em1);
  s.q2 = __fdividef(1.f, 2.f + s.em1);
}

// FP32 GHK flux (same identities as ghk_flux) with ka1 = alpha1/d hoisted;
// the generic-charge branch evaluates BETSE's formula directly in FP32.
__device__ __forceinline__ float ghk_flux_fk(const GhkShared<float>& s, float ka1, int zcode, float zval,
                                             float v_nonce, float F_RT, float cA, float cB, float Dc,
                                             float inv_d) {
  const float kk = Dc * ka1;
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

// Tile-major layout of the split form.  Tile b (a run of at most 32 whole
// cells of one cluster holding at most TPB membranes) owns membrane slots
// [b*TPB, (b+1)*TPB) and cell slots [32b, 32b+32); unused slots are padding.
// Every address a CTA needs follows from blockIdx, so the loads of a step
// form two independent waves: geometry before the grid dependency wait, and
// all state (own record, partner record, concentrations) right after it.
struct SplitGeom {
  int C, M, I, G;
  int Q, S;                                // membrane slots (TPB*nblk), cell slots (32*nblk)
  const uint8_t* __restrict__ lcell;       // [Q] cell of the slot within its tile, 255 = padding
  const int* __restrict__ nn_slot;         // [Q] cell slot of the gap-junction partner
  const float* __restrict__ mem_sa;        // [Q]
  const float* __restrict__ gjw;           // [Q] (0 on boundary membranes and padding)
  const short2* __restrict__ cell_rng;     // [S] local membrane range [x, y) of the cell slot
  const float* __restrict__ dtv;           // [S] dt / cell_vol
  const float* __restrict__ dvc;           // [S] diviterm / cm
  const int* __restrict__ blk_cluster;     // [nblk]
  const int* __restrict__ tile_c0;         // [nblk] first cell (natural order) of the tile
  const int* __restrict__ tile_m0;         // [nblk] first membrane (natural order) of the tile
  const int* __restrict__ map_env;         // [Q]  (PHIB only)
  const int* __restrict__ nn_env;          // [Q]  map_mem2ecm of the partner membrane (PHIB only)
  const void* __restrict__ geo_blob;       // [nblk] PersistGeo: each tile's static data, contiguous
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
  int vgj;                                  // voltage-gated gap junctions (gjo is state)
  float gj_vth, gj_min, gj_dt_ms;
  int iCa;                                  // Ca-ATPase ion row, -1 = pump off
  float ca_alpha, ca_inv_Km, ca_atp_term, ca_atp_den, ca_qnum_c, ca_qden_c;
};

// Per-cell record, REC floats, 16-byte aligned: slots [0, I) hold the
// membrane-side concentration of each ion (BETSE's cc_at_mem), slot REC-1
// the cell's Vmem.
struct SplitPtrs {
  const float* __restrict__ rec_in; float* __restrict__ rec_out;   // [S][REC]
  float2* __restrict__ cc2;                // [I][S]
  const float* __restrict__ Dm;            // [I][Q]
  const float* __restrict__ cenv_f;        // [ncl][I] FP32 copy of the environment
  const float* __restrict__ pump_coef;     // [ncl] -3 block alpha_NaK (0 = pump off)
  const float* __restrict__ phib;          // [G] (PHIB)
  float* __restrict__ env_part;            // [nblk][I] per-tile partial sums
  const double* __restrict__ cenv_grid;    // [I][G] environment grid concentrations (ECM)
  double* __restrict__ mfs;                // [I][M] f_mem*sa per membrane, natural order (ECM scatter)
  float* __restrict__ gjo;                 // [Q] gap-junction open fraction per slot (vgj), in place
  double* __restrict__ o_gjopen;           // [M] output steps with vgj: the open fraction
  const double* __restrict__ ca_env;       // [G] Ca2+ of the grid after this step's Nernst-Planck
                                           // update (ECM with the Ca-ATPase)
  unsigned long long* status;              // nan_vm, nan_conc, neg clamps
  // outputs (OUT), natural order
  double* o_fmem; double* o_fgj; double* o_rate; double* o_rho; double* o_vmem;
  double* o_drho;      // [C] output steps: new minus old charge density (FP64 from double-float)
};

template <int REC>
__device__ __forceinline__ void load_rec(const float* __restrict__ rec, int c, float (&v)[REC]) {
  const float4* r4 = reinterpret_cast<const float4*>(rec + (size_t)c * REC);
#pragma unroll
  for (int q = 0; q < REC / 4; ++q) {
    const float4 x = r4[q];
    v[4 * q] = x.x; v[4 * q + 1] = x.y; v[4 * q + 2] = x.z; v[4 * q + 3] = x.w;
  }
}

// 2-ulp FP32 reciprocal (MUFU-based); operands here are far from the
// denormal range except at exactly zero volts, where BETSE's 1e-25 nonce keeps
// them above 1e-24.
__device__ __forceinline__ float rcp_fast(float x) { return __fdividef(1.f, x); }

constexpr int kCellsPerCta = 32;

// The two segmented sums of one cell (update_all_concs' M_sum_mems products):
// membranes [rng.x, rng.y) of the tile, added in order.  The first eight terms
// are predicated straight-line code (a Voronoi cell has ~6 membranes), so a
// warp whose cells differ in size runs no loop for them.
__device__ __forceinline__ void seg_sums(const float* __restrict__ a, const float* __restrict__ b, short2 rng,
                                         float& s1, float& s2) {
  float x = 0.f, y = 0.f;
  const int j0 = rng.x, n = rng.y - rng.x;
#pragma unroll
  for (int u = 0; u < 8; ++u)
    if (u < n) { x += a[j0 + u]; y += b[j0 + u]; }
  for (int j = j0 + 8; j < rng.y; ++j) { x += a[j]; y += b[j]; }
  s1 = x;
  s2 = y;
}   // cells per tile: the (ion, cell) phase maps ion -> warp, cell -> lane

// Charge patterns compiled as constants.  ZP = 0: any ion set, charges read
// at run time.  ZP = 1: BETSE's six-ion set (ion profiles 'mammal' and
// 'amphibian': Na, K, Cl, Ca, P, M with z = +1, +1, -1, +2, -1, -1; Na row 0,
// K row 1).
template <int ZP> struct IonSet {
  static constexpr int NI = kMaxIons;
  __device__ static int zc(const SplitConst& k, int i) { return k.zcode[i]; }
  __device__ static int n(const SplitConst& k) { return k.I; }
  __device__ static int iNa(const SplitConst& k) { return k.iNa; }
  __device__ static int iK(const SplitConst& k) { return k.iK; }
};
template <> struct IonSet<1> {
  static constexpr int NI = 6;
  __device__ static constexpr int zc(const SplitConst&, int i) {
    return i == 0 ? 1 : i == 1 ? 1 : i == 2 ? -1 : i == 3 ? 2 : -1;
  }
  __device__ static constexpr int n(const SplitConst&) { return 6; }
  __device__ static constexpr int iNa(const SplitConst&) { return 0; }
  __device__ static constexpr int iK(const SplitConst&) { return 1; }
};

// One time step of the split form for one tile.
//   prologue  geometry and Dm of the tile's slots (overlaps the previous kernel)
//   wait      cudaGridDependencySynchronize
//   loads     own record, partner record, cc2, environment -- one wave
//   membranes GHK + pump + gap-junction fluxes (FP32), per-ion f*sa into smem
//   cells     warp i = ion i, lane = cell: update_all_concs in double-float
//   charge    warp 0: rho = sum_i z_i F c_i (double-float) -> Vmem record
// ECM: the environment concentration of each membrane is its grid cell's
// (cc_env[i][map_mem2ecm], sim.py:1256-1259) and f_mem*sa is exported for the
// grid scatter (update_Co's ECM term) instead of the well-mixed partials.
template <int TPB, int REC, int ZP, bool OUT, bool PHIB, bool ECM = false>
__global__ void __launch_bounds__(TPB, 2048 / TPB / 2)
k_split_step(SplitGeom g, SplitPtrs p, SplitConst k) {
  using IS = IonSet<ZP>;
  constexpr int NI = IS::NI;
  __shared__ float sA[NI][TPB];
  __shared__ float sB[NI][TPB];
  __shared__ float sRec[kCellsPerCta][REC];
  __shared__ float2 sQ[NI][kCellsPerCta];
  __shared__ float2 sQo[OUT ? NI : 1][kCellsPerCta];   // output steps: charge of the old state
  const int I = IS::n(k);
  const int b = blockIdx.x;
  const int t = threadIdx.x;
  const int lane = t & 31, wid = t >> 5;
  const int q = b * TPB + t;                 // membrane slot
  const int s0 = b * kCellsPerCta;           // first cell slot of the tile

#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 900)
  cudaTriggerProgrammaticLaunchCompletion();
#endif
  // ---- prologue: geometry and channel data (read-only during stepping)
  const int lc = g.lcell[q];
  const bool active = lc != 255;                // padding slots load nothing more
  int cn = s0;
  float sa = 0.f, gw = 0.f;
  float dmv[NI];
#pragma unroll
  for (int i = 0; i < NI; ++i) dmv[i] = 0.f;
  if (active) {
    cn = g.nn_slot[q];
    sa = g.mem_sa[q];
    gw = g.gjw[q] * k.gj_block;
#pragma unroll
    for (int i = 0; i < NI; ++i)
      if (i < I) dmv[i] = p.Dm[(size_t)i * g.Q + q];
  }
  const int cl = g.blk_cluster[b];
  const bool cell_thr = (wid < I);
  const short2 rng = g.cell_rng[s0 + lane];
  const float dtv = g.dtv[s0 + lane];
  const float dvc = (t < kCellsPerCta) ? g.dvc[s0 + t] : 0.f;

  // ---- wait for the previous step's state
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 900)
  cudaGridDependencySynchronize();
#endif
  float2 x2 = make_float2(0.f, 0.f);
  if (cell_thr) x2 = p.cc2[(size_t)wid * g.S + s0 + lane];
  float own[REC], nbr[REC];
  load_rec<REC>(p.rec_in, s0 + (active ? lc : 0), own);
  load_rec<REC>(p.rec_in, cn, nbr);
  float cenv[NI];
  if (ECM) {
    const int ge = active ? g.map_env[q] : 0;
#pragma unroll
    for (int i = 0; i < NI; ++i) cenv[i] = (i < I && active) ? (float)p.cenv_grid[(size_t)i * g.G + ge] : 0.f;
  } else {
    const float* ce = p.cenv_f + (size_t)cl * I;
#pragma unroll
    for (int i = 0; i < NI; ++i) cenv[i] = (i < I) ? ce[i] : 0.f;
  }
  const float pc = p.pump_coef[cl];

  if (active) {
    float v = own[REC - 1];
    float vn = nbr[REC - 1];
    if (PHIB) { v -= p.phib[g.map_env[q]]; vn -= p.phib[g.nn_env[q]]; }
    // BETSE's 1e-25 nonces (sim_toolbox.py:52-56) keep alpha != 0 at zero volts
    const float v1 = v + 1.0e-25f;
    const float vgj1 = ((vn + 1.0e-25f) - v1) + 1.0e-25f;
    GhkShared<float> sm, sg;
    ghk_init_f(sm, v1, k.F_RT);
    ghk_init_f(sg, vgj1, k.F_RT);
    const float ka_m = sm.a1 * k.inv_tm, ka_g = sg.a1 * k.inv_gjl;
    // Gap_Junction.run (channels/gap_junction.py:52-81), once per ion
    float gg = 0.f, ga = 0.f, gr = 0.f;
    if (k.vgj) {
      const float V1 = 1.0e3f * fabsf(vn - v);
      const float al = 0.0013f * __expf(-0.077f * (V1 - k.gj_vth));
      float be = 0.0013f * __expf(0.14f * (V1 - k.gj_vth));
      be = be * rcp_fast(1.f + 50.f * be);
      ga = k.gj_dt_ms * (al + be * k.gj_min);
      gr = rcp_fast(1.f + al * k.gj_dt_ms + be * k.gj_dt_ms);
      gg = p.gjo[q];
    }
    float fNa = 0.f;
    if (pc != 0.f) {
      // pumpNaKATP (sim_toolbox.py:71-122), one reciprocal
      float cNai = 0.f, cKi = 0.f, cNao = 0.f, cKo = 0.f;
#pragma unroll
      for (int i = 0; i < NI; ++i) {
        if (i == IS::iNa(k)) { cNai = own[i]; cNao = cenv[i]; }
        if (i == IS::iK(k)) { cKi = own[i]; cKo = cenv[i]; }
      }
      const float nai = cNai * 1e-3f, nao = cNao * 1e-3f, ki = cKi * 1e-3f, ko = cKo * 1e-3f;
      const float qnum = k.qnum_c * (nao * nao * nao) * (ki * ki);
      float qden = k.qden_c * (nai * nai * nai) * (ko * ko);
      if (qden == 0.f) qden = 1.0e-15f;
      const float xna = cNai * k.inv_KmNa, xk = cKo * k.inv_KmK;
      const float na3 = xna * xna * xna, k2 = xk * xk;
      const float num_e = na3 * k2 * k.atp_term;
      const float den_e = (1.f + na3) * (1.f + k2) * k.atp_den;
      fNa = pc * num_e * (qden * k.K0 - qnum * sm.e1) * rcp_fast(den_e * qden * k.K0);
    }
#pragma unroll
    for (int i = 0; i < NI; ++i) {
      if (i >= I) break;
      const int z = IS::zc(k, i);
      const float cin = own[i];
      float f = ghk_flux_fk(sm, ka_m, z, k.z[i], v1, k.F_RT, cenv[i], cin, dmv[i], k.inv_tm);
      if (i == IS::iNa(k)) f = fNa + f;
      else if (i == IS::iK(k)) f = (-(2.f / 3.f)) * fNa + f;
      if (i == k.iCa) {
        // ca_handler (sim.py:2126-2155) on the start-of-step cell
        // concentration (update_intra) and, with ECM, the environment after
        // this step's Nernst-Planck update; pumpCaATP in FP32, one reciprocal
        float cCai = p.cc2[(size_t)i * g.S + s0 + lc].x;
        float cCao = ECM ? (float)p.ca_env[g.map_env[q]] : cenv[i];
        cCai = cCai > 0.f ? cCai : 0.f;
        cCao = cCao > 0.f ? cCao : 0.f;
        const float qn = k.ca_qnum_c * cCao;
        float qd = k.ca_qden_c * cCai;
        if (qd == 0.f) qd = 1.0e-16f;
        const float x = cCai * k.ca_inv_Km;
        const float num_e = x * k.ca_atp_term;
        const float den_e = (1.f + x) * k.ca_atp_den;
        f = f - k.ca_alpha * num_e * (qd * k.K0 - qn * (sm.e1 * sm.e1)) * rcp_fast(den_e * qd * k.K0);
      }
      float dgjv = k.dgj_gs[i] * gw;
      if (k.vgj) {
        gg = k.gj_block * ((gg + ga) * gr);
        dgjv = k.dgj_gs[i] * gg;
      }
      const float fg = ghk_flux_fk(sg, ka_g, z, k.z[i], vgj1, k.F_RT, cin, nbr[i], dgjv, k.inv_gjl);
      sA[i][t] = f * sa;
      sB[i][t] = -fg * sa;
      if (ECM) p.mfs[(size_t)i * g.M + g.tile_m0[b] + t] = (double)(f * sa);
      if (OUT) {
        const int mn = g.tile_m0[b] + t;
        p.o_fmem[(size_t)i * g.M + mn] = (double)f;
        p.o_fgj[(size_t)i * g.M + mn] = (double)fg;
      }
    }
    if (OUT) p.o_rate[g.tile_m0[b] + t] = (double)(-fNa);
    if (k.vgj) {
      p.gjo[q] = gg;
      if (OUT) p.o_gjopen[g.tile_m0[b] + t] = (double)gg;
    }
  } else {
#pragma unroll
    for (int i = 0; i < NI; ++i) if (i < I) { sA[i][t] = 0.f; sB[i][t] = 0.f; }
  }
  __syncthreads();

  // ---- cells: warp = ion, lane = cell -- update_all_concs (sim.py:2086-2111)
  int bad = 0, neg = 0;
  const bool cell_live = cell_thr && rng.y > rng.x;
  float s1 = 0.f, s2 = 0.f;
  if (cell_thr) {
    seg_sums(sA[wid], sB[wid], rng, s1, s2);
    // per-tile partial sum of f_mem*sa of this ion (k_split_env reduces them)
    float e = s1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
    if (!ECM && lane == 0) p.env_part[(size_t)b * I + wid] = e;
  }
  if (cell_live) {
    const int i = wid;
    df x{x2.x, x2.y};
    if (OUT) {
      const df qo = df_mul(x, k.zF_hi[i], k.zF_lo[i]);
      sQo[i][lane] = make_float2(qo.hi, qo.lo);
    }
    x = df_add_f(x, s1 * dtv);                         // update_Co
    sRec[lane][i] = x.hi + x.lo;                       // cc_at_mem (before the GJ term)
    x = df_add_f(x, s2 * dtv);                         // gap-junction term
    if (x.hi != x.hi) bad = 1;
    if (x.hi < 0.f || (x.hi == 0.f && x.lo < 0.f)) { x = df{0.f, 0.f}; neg = 1; }   // no_negs
    p.cc2[(size_t)i * g.S + s0 + lane] = make_float2(x.hi, x.lo);
    const df qz = df_mul(x, k.zF_hi[i], k.zF_lo[i]);
    sQ[i][lane] = make_float2(qz.hi, qz.lo);
  }
  // NaN and no_negs counts: rare, one atomic per affected (ion, cell)
  if (bad) atomicAdd(&p.status[1], 1ull);
  if (neg) atomicAdd(&p.status[2], 1ull);
  __syncthreads();
  // ---- charge -> Vmem (update_V, sim.py:2027-2029), one lane per cell
  if (t < kCellsPerCta) {
    const short2 r0 = g.cell_rng[s0 + t];
    if (r0.y > r0.x) {
      df rho{0.f, 0.f};
#pragma unroll
      for (int i = 0; i < NI; ++i)
        if (i < I) rho = df_add(rho, df{sQ[i][t].x, sQ[i][t].y});
      const float vc = (rho.hi + rho.lo) * dvc;
      float o[REC];
#pragma unroll
      for (int i = 0; i < REC - 1; ++i) o[i] = (i < I) ? sRec[t][i] : 0.f;
      o[REC - 1] = vc;
      float4* out4 = reinterpret_cast<float4*>(p.rec_out + (size_t)(s0 + t) * REC);
#pragma unroll
      for (int w = 0; w < REC / 4; ++w) out4[w] = make_float4(o[4 * w], o[4 * w + 1], o[4 * w + 2], o[4 * w + 3]);
      if (vc != vc) atomicAdd(&p.status[0], 1ull);
      if (OUT) {
        const int cc = g.tile_c0[b] + t;
        p.o_rho[cc] = (double)rho.hi + (double)rho.lo;
        p.o_vmem[cc] = (double)vc;
        df rho_o{0.f, 0.f};
#pragma unroll
        for (int i = 0; i < NI; ++i)
          if (i < I) rho_o = df_add(rho_o, df{sQo[i][t].x, sQo[i][t].y});
        // dVm/dt from the FP64 charge change: the FP32 record's Vmem resolves
        // only ~4e-9 V, too coarse for a residual test on dVm/dt
        p.o_drho[cc] = ((double)rho.hi + (double)rho.lo) - ((double)rho_o.hi + (double)rho_o.lo);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Persistent, software-pipelined form of k_split_step (no outputs, no Phi_b).
// Each CTA walks tiles b = blockIdx.x + j*gridDim.x.  Tiles are staged in
// shared memory with cp.async (16-byte asynchronous copies that complete at
// cp.async.wait_group -- no waits of ours): the geometry of tile j+2 and the
// state of tile j+1 (own and partner records, concentrations) are in flight
// while tile j computes.  Same arithmetic, same order as k_split_step, so the
// results are bit-identical.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp4(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

template <int TPB>
__device__ __forceinline__ void cp_block(void* smem, const void* gmem, int bytes) {
  char* s = static_cast<char*>(smem);
  const char* gp = static_cast<const char*>(gmem);
  for (int off = (int)threadIdx.x * 16; off < bytes; off += TPB * 16) cp16(s + off, gp + off);
}

// One tile's static data for the persistent kernel, laid out in global memory
// exactly as it is staged in shared memory, so one contiguous copy moves it:
// Dm per ion, membrane area, gap-junction weight, partner cell slot, cell of
// the slot, and the tile's cluster.  k_split_blob builds it from the
// tile-major arrays whenever the layout or Dm changes.
template <int TPB, int NI>
struct PersistGeo {
  float Dm[NI][TPB];
  float sa[TPB];
  float gw[TPB];
  int nn[TPB];
  uint8_t lcell[TPB];
  int cl;                            // the tile's cluster
  int pad[3];
};

template <int TPB, int NI>
__global__ void __launch_bounds__(TPB)
k_split_blob(PersistGeo<TPB, NI>* blob, const float* __restrict__ Dm, const float* __restrict__ sa,
             const float* __restrict__ gw, const int* __restrict__ nn, const uint8_t* __restrict__ lcell,
             const int* __restrict__ blk_cluster, int I, int Q) {
  const int b = blockIdx.x, t = threadIdx.x;
  const size_t q = (size_t)b * TPB + t;
  PersistGeo<TPB, NI>& g = blob[b];
#pragma unroll
  for (int i = 0; i < NI; ++i) g.Dm[i][t] = (i < I) ? Dm[(size_t)i * Q + q] : 0.f;
  g.sa[t] = sa[q];
  g.gw[t] = gw[q];
  g.nn[t] = nn[q];
  g.lcell[t] = lcell[q];
  if (t == 0) { g.cl = blk_cluster[b]; g.pad[0] = g.pad[1] = g.pad[2] = 0; }
}

template <int TPB, int NI>
struct PersistSmem {
  using Geo = PersistGeo<TPB, NI>;
  struct State {                     // one tile's state
    float own[kCellsPerCta][8];
    float nbr[TPB][8];
    float2 cc2[NI][kCellsPerCta];
    short2 rng[kCellsPerCta];
    float dtv[kCellsPerCta];
    float dvc[kCellsPerCta];
    float cenv[kMaxIons];            // the cluster's environment (written by the previous step)
    float pump;                      // and its pump coefficient
    int pad[3];
  };
  // 16-byte copies land at 16-byte multiples of the (16-byte aligned) base
  static_assert(sizeof(Geo) % 16 == 0 && sizeof(State) % 16 == 0, "16-byte staging blocks");
  static_assert(NI <= kMaxIons, "ion rows");
  Geo geo[3];
  State st[2];
  float sA[NI][TPB];
  float sB[NI][TPB];
  float sRec[kCellsPerCta][8];
  float2 sQ[NI][kCellsPerCta];
};

template <int TPB, int ZP>
__global__ void __launch_bounds__(TPB)
k_split_persist(SplitGeom g, SplitPtrs p, SplitConst k, int ntile) {
  using IS = IonSet<ZP>;
  constexpr int NI = IS::NI;
  constexpr int REC = 8;
  using SM = PersistSmem<TPB, NI>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SM& sm = *reinterpret_cast<SM*>(smem_raw);
  const int I = IS::n(k);
  const int t = threadIdx.x;
  const int lane = t & 31, wid = t >> 5;
  const int G = gridDim.x;

#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 900)
  cudaTriggerProgrammaticLaunchCompletion();
#endif
  // the tile's static data: one contiguous block (PersistGeo), 16 bytes a copy
  auto issue_geo = [&](int tile, int buf) {
    if (tile >= ntile) return;
    cp_block<TPB>(&sm.geo[buf], static_cast<const typename SM::Geo*>(g.geo_blob) + tile,
                  (int)sizeof(typename SM::Geo));
  };
  // the tile's state as one flat range of 16-byte copies: the own records
  // (64 copies), then 16 per ion of (hi, lo) pairs, then 8 each of the
  // membrane ranges, dt/vol and diviterm/cm
  auto issue_state = [&](int tile, int sbuf, int gbuf) {
    if (tile >= ntile) return;
    typename SM::State& st = sm.st[sbuf];
    const typename SM::Geo& ge = sm.geo[gbuf];
    const int s0 = tile * kCellsPerCta;
    constexpr int kOwn = kCellsPerCta * REC * 4 / 16, kPair = kCellsPerCta * 8 / 16, kSmall = kCellsPerCta * 4 / 16;
    const int n_copy = kOwn + kPair * I + 3 * kSmall;
    for (int c = t; c < n_copy; c += TPB) {
      const char* src;
      char* dst;
      if (c < kOwn) {
        src = reinterpret_cast<const char*>(p.rec_in + (size_t)s0 * REC) + 16 * c;
        dst = reinterpret_cast<char*>(&st.own[0][0]) + 16 * c;
      } else if (c < kOwn + kPair * I) {
        const int i = (c - kOwn) / kPair, o = 16 * ((c - kOwn) % kPair);
        src = reinterpret_cast<const char*>(p.cc2 + (size_t)i * g.S + s0) + o;
        dst = reinterpret_cast<char*>(st.cc2[i]) + o;
      } else {
        const int r = c - kOwn - kPair * I, which = r / kSmall, o = 16 * (r % kSmall);
        src = which == 0 ? reinterpret_cast<const char*>(g.cell_rng + s0) + o
            : which == 1 ? reinterpret_cast<const char*>(g.dtv + s0) + o
                         : reinterpret_cast<const char*>(g.dvc + s0) + o;
        dst = which == 0 ? reinterpret_cast<char*>(st.rng) + o
            : which == 1 ? reinterpret_cast<char*>(st.dtv) + o
                         : reinterpret_cast<char*>(st.dvc) + o;
      }
      cp16(dst, src);
    }
    // the cluster's environment and pump rate: the cluster index came with the
    // geometry, so these loads do not wait on another load in the tile's compute
    if (t < I) cp4(&st.cenv[t], p.cenv_f + (size_t)ge.cl * I + t);
    else if (t == I) cp4(&st.pump, p.pump_coef + ge.cl);
    if (ge.lcell[t] != 255) {         // partner record of this slot
      const float* src = p.rec_in + (size_t)ge.nn[t] * REC;
      cp16(&st.nbr[t][0], src);
      cp16(&st.nbr[t][4], src + 4);
    }
  };

  // geometry is read-only while stepping: fetch it before the dependency wait
  const int T0 = blockIdx.x;
  issue_geo(T0, 0);
  issue_geo(T0 + G, 1);
  cp_commit();
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 900)
  cudaGridDependencySynchronize();
#endif
  cp_wait_all();
  __syncthreads();
  issue_state(T0, 0, 0);
  cp_commit();

  unsigned long long n_bad = 0, n_neg = 0, n_nan = 0;
  int j = 0;
  for (int tile = T0; tile < ntile; tile += G, ++j) {
    const int gb = j % 3, sb = j & 1;
    cp_wait_all();                   // state(tile) and geometry(tile + G) have landed
    __syncthreads();
    issue_state(tile + G, sb ^ 1, (j + 1) % 3);
    issue_geo(tile + 2 * G, (j + 2) % 3);
    cp_commit();

    const typename SM::Geo& ge = sm.geo[gb];
    const typename SM::State& st = sm.st[sb];
    const int s0 = tile * kCellsPerCta;
    const int lc = ge.lcell[t];
    const bool active = lc != 255;
    if (active) {
      float own[REC], nbr[REC];
#pragma unroll
      for (int r = 0; r < REC; ++r) { own[r] = st.own[lc][r]; nbr[r] = st.nbr[t][r]; }
      float cenv[NI];
#pragma unroll
      for (int i = 0; i < NI; ++i) cenv[i] = (i < I) ? st.cenv[i] : 0.f;
      const float pc = st.pump;
      const float v = own[REC - 1];
      const float vn = nbr[REC - 1];
      const float v1 = v + 1.0e-25f;
      const float vgj1 = ((vn + 1.0e-25f) - v1) + 1.0e-25f;
      GhkShared<float> gm, gg;
      ghk_init_f(gm, v1, k.F_RT);
      ghk_init_f(gg, vgj1, k.F_RT);
      const float ka_m = gm.a1 * k.inv_tm, ka_g = gg.a1 * k.inv_gjl;
      float fNa = 0.f;
      if (pc != 0.f) {
        float cNai = 0.f, cKi = 0.f, cNao = 0.f, cKo = 0.f;
#pragma unroll
        for (int i = 0; i < NI; ++i) {
          if (i == IS::iNa(k)) { cNai = own[i]; cNao = cenv[i]; }
          if (i == IS::iK(k)) { cKi = own[i]; cKo = cenv[i]; }
        }
        const float nai = cNai * 1e-3f, nao = cNao * 1e-3f, ki = cKi * 1e-3f, ko = cKo * 1e-3f;
        const float qnum = k.qnum_c * (nao * nao * nao) * (ki * ki);
        float qden = k.qden_c * (nai * nai * nai) * (ko * ko);
        if (qden == 0.f) qden = 1.0e-15f;
        const float xna = cNai * k.inv_KmNa, xk = cKo * k.inv_KmK;
        const float na3 = xna * xna * xna, k2 = xk * xk;
        const float num_e = na3 * k2 * k.atp_term;
        const float den_e = (1.f + na3) * (1.f + k2) * k.atp_den;
        fNa = pc * num_e * (qden * k.K0 - qnum * gm.e1) * rcp_fast(den_e * qden * k.K0);
      }
      const float sa = ge.sa[t];
      const float gw = ge.gw[t] * k.gj_block;
#pragma unroll
      for (int i = 0; i < NI; ++i) {
        if (i >= I) break;
        const int z = IS::zc(k, i);
        const float cin = own[i];
        float f = ghk_flux_fk(gm, ka_m, z, k.z[i], v1, k.F_RT, cenv[i], cin, ge.Dm[i][t], k.inv_tm);
        if (i == IS::iNa(k)) f = fNa + f;
        else if (i == IS::iK(k)) f = (-(2.f / 3.f)) * fNa + f;
        const float fgv = ghk_flux_fk(gg, ka_g, z, k.z[i], vgj1, k.F_RT, cin, nbr[i], k.dgj_gs[i] * gw, k.inv_gjl);
        sm.sA[i][t] = f * sa;
        sm.sB[i][t] = -fgv * sa;
      }
    } else {
#pragma unroll
      for (int i = 0; i < NI; ++i) if (i < I) { sm.sA[i][t] = 0.f; sm.sB[i][t] = 0.f; }
    }
    __syncthreads();
    // cells: warp = ion, lane = cell (update_all_concs)
    // one pass over the cell's membranes for both sums, each in the order of k_split_step
    const short2 rng = st.rng[lane];
    float s1 = 0.f, s2 = 0.f;
    if (wid < I) {
      seg_sums(sm.sA[wid], sm.sB[wid], rng, s1, s2);
      float e = s1;                  // per-tile partial sum of f_mem*sa of this ion
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
      if (lane == 0) p.env_part[(size_t)tile * I + wid] = e;
    }
    if (wid < I && rng.y > rng.x) {
      const int i = wid;
      const float dtv = st.dtv[lane];
      const float2 x2 = st.cc2[i][lane];
      df x{x2.x, x2.y};
      x = df_add_f(x, s1 * dtv);
      sm.sRec[lane][i] = x.hi + x.lo;
      x = df_add_f(x, s2 * dtv);
      if (x.hi != x.hi) ++n_bad;
      if (x.hi < 0.f || (x.hi == 0.f && x.lo < 0.f)) { x = df{0.f, 0.f}; ++n_neg; }
      p.cc2[(size_t)i * g.S + s0 + lane] = make_float2(x.hi, x.lo);
      const df qz = df_mul(x, k.zF_hi[i], k.zF_lo[i]);
      sm.sQ[i][lane] = make_float2(qz.hi, qz.lo);
    }
    __syncthreads();
    if (t < kCellsPerCta) {
      const short2 r0 = st.rng[t];
      if (r0.y > r0.x) {
        df rho{0.f, 0.f};
#pragma unroll
        for (int i = 0; i < NI; ++i)
          if (i < I) rho = df_add(rho, df{sm.sQ[i][t].x, sm.sQ[i][t].y});
        const float vc = (rho.hi + rho.lo) * st.dvc[t];
        float o[REC];
#pragma unroll
        for (int i = 0; i < REC - 1; ++i) o[i] = (i < I) ? sm.sRec[t][i] : 0.f;
        o[REC - 1] = vc;
        float4* out4 = reinterpret_cast<float4*>(p.rec_out + (size_t)(s0 + t) * REC);
        out4[0] = make_float4(o[0], o[1], o[2], o[3]);
        out4[1] = make_float4(o[4], o[5], o[6], o[7]);
        if (vc != vc) ++n_nan;
      }
    }
    // no barrier here: the buffers of this tile are refilled only after the
    // next tile's first barrier, which every thread reaches after this tile
  }
  cp_wait_all();
  if (n_bad) atomicAdd(&p.status[1], n_bad);
  if (n_neg) atomicAdd(&p.status[2], n_neg);
  if (n_nan) atomicAdd(&p.status[0], n_nan);
}

// Well-mixed environment per cluster (sim_toolbox.py:1196-1205):
// c_env <- mean_m(c_env - f_m sa_m / vol_env * dt).  One CTA per cluster sums
// the cluster's per-CTA partials in a fixed order (double-float), so the
// result is deterministic.  Launched after the step kernel with programmatic
// dependent launch.
template <int NT>
__global__ void __launch_bounds__(NT)
k_split_env(const float* __restrict__ part, const int* __restrict__ cl_blk, int I,
            double* cenv64, float* cenv_f, const double* __restrict__ env_scale) {
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 900)
  cudaTriggerProgrammaticLaunchCompletion();
  cudaGridDependencySynchronize();
#endif
  __shared__ float2 fin[kMaxIons][NT / 32];
  const int cl = blockIdx.x, t = threadIdx.x;
  const int b0 = cl_blk[cl], b1 = cl_blk[cl + 1];
  df acc[kMaxIons];
#pragma unroll
  for (int i = 0; i < kMaxIons; ++i) acc[i] = df{0.f, 0.f};
  for (int b = b0 + t; b < b1; b += NT) {
    const float* pp = part + (size_t)b * I;
#pragma unroll
    for (int i = 0; i < kMaxIons; ++i)
      if (i < I) acc[i] = df_add_f(acc[i], pp[i]);
  }
#pragma unroll
  for (int i = 0; i < kMaxIons; ++i) {
    if (i >= I) break;
    df a = acc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      df other{__shfl_down_sync(0xffffffffu, a.hi, o), __shfl_down_sync(0xffffffffu, a.lo, o)};
      a = df_add(a, other);
    }
    if ((t & 31) == 0) fin[i][t >> 5] = make_float2(a.hi, a.lo);
  }
  __syncthreads();
  if (t < I) {
    df a{0.f, 0.f};
    for (int w = 0; w < NT / 32; ++w) a = df_add(a, df{fin[t][w].x, fin[t][w].y});
    const double tot = (double)a.hi + (double)a.lo;
    const double v = cenv64[(size_t)cl * I + t] - tot * env_scale[cl];
    cenv64[(size_t)cl * I + t] = v;
    cenv_f[(size_t)cl * I + t] = (float)v;
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
  const double* diviterm; const double* drho;
};
struct SplitOutPtrs {
  const double* fmem; const double* fgj; const float* rec_new; const float* rec_old; int rec;
  const float2* cc2; int S; const int* slot_of_cell; const float* phib;
  double* Jn; double* Imem; double* Jcx; double* Jcy; double* Jc; double* vmave; double* dvm;
  double* Ecx; double* Ecy; double* Emc; double* Egjx; double* Egjy; double* gjopen; double* sigma;
  double* vm_mem;      // [M] start-of-step Vmem per membrane (update_gj reads it)
};
struct SplitOutConst {
  int I; double zF[kMaxIons]; double sig_coef[kMaxIons]; double dt; double gj_len; double gj_block;
  double cm;
  int vgj;   // the open fraction was written by the step kernel
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
    const int sc = p.slot_of_cell[c];
    vm = (double)p.rec_new[(size_t)sc * p.rec + p.rec - 1] - ph;
    p.vm_mem[m] = (double)p.rec_old[(size_t)sc * p.rec + p.rec - 1] - ph;
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
    const int sc = p.slot_of_cell[c];
    for (int i = 0; i < k.I; ++i) { const float2 x = p.cc2[(size_t)i * p.S + sc]; sig += k.sig_coef[i] * ((double)x.x + (double)x.y); }
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
    p.dvm[m] = g.drho[c] * g.diviterm[c] / k.cm / k.dt;   // update_V's (vm - vmo)/dt, sim.py:2083
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
    if (!k.vgj) p.gjopen[m] = k.gj_block * g.gj_w[m];
  }
}

// E_gj needs the partner's start-of-step Vmem (update_gj runs before
// update_V, sim.py:2166-2174): a separate pass over membranes.
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
