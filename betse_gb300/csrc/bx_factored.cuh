// bx_factored.cuh -- the split form of the step, factored by cell.
//
// Without cell polarizability, without an applied boundary potential and with
// the well-mixed environment, every membrane of a cell sees the same Vmem,
// the same membrane-side concentrations (BETSE's cc_at_mem is the cell value
// broadcast to its membranes, sim.py:2310) and the same environment.  The
// GHK transmembrane flux of membrane m is then Dm_i(m) times a per-cell
// factor h_i, and the Na/K-ATPase rate is one per cell, so the first
// M_sum_mems product of update_all_concs (sim.py:2086-2111) collapses:
//
//   sum_m (f_pump,i + Dm_i(m) h_i) mem_sa(m) = f_pump,i SA + h_i DSA_i,
//   SA = sum_m mem_sa(m),  DSA_i = sum_m Dm_i(m) mem_sa(m)   (static)
//
// Only the gap-junction flux (update_gj, sim.py:2162-2206) stays per
// membrane, and only for membranes with a partner (BETSE zeroes the flux of
// boundary membranes, sim.py:2203).  The arithmetic of each term is the split
// form's (bx_split.cuh: FP32 fluxes, double-float concentrations and charge);
// the results differ from the per-membrane evaluation only by FP32 rounding.
//
// One thread advances one cell: it walks the cell's gap-junction list (the
// partner's record: membrane-side concentrations and Vmem, 32 bytes), then
// computes the per-cell terms and updates the cell.  A warp holds one tile
// (32 cell slots), so the per-tile environment partials of k_split_env come
// from one warp reduction.
//
// Two kernels use it:
//   k_split_fact      one time step per launch, streaming every array (batched
//                     sweeps, and clusters too large for the resident kernel);
//   k_split_resident  one cooperative launch for many time steps: each CTA
//                     keeps its cells' static data, concentrations and the
//                     records it reads in shared memory for the whole run, and
//                     the CTAs meet once per step at a bounded grid barrier.
#pragma once
#include "bx_split.cuh"

namespace bx {

// Static per-cell data of the factored form, in the cell slots of the
// tile-major layout (tile b owns slots [32b, 32b+32)).
struct FactGeom {
  int S;                                   // cell slots
  int ntile;
  const float* __restrict__ dsa;           // [I][S] sum over the cell's membranes of Dm_i * mem_sa
  const float4* __restrict__ cst;          // [S] {sum mem_sa, dt/cell_vol, diviterm/cm,
                                           //      int: gap-junction count, -1 = padding slot}
  const int* __restrict__ gbeg;            // [S] first gap-junction entry of the cell
  const int2* __restrict__ gj;             // [P] {partner cell slot, float bits of gj_weight*mem_sa}
  const int* __restrict__ blk_cluster;     // [ntile]
};

// GHK flux (electroflux, sim_toolbox.py:18-69) times Dc for the factored
// sums, where Dc may be as small as ~1e-28 (a cell's sum of Dm * mem_sa).
// The bounded factor kr = (alpha/d) / expm1(-alpha) (about -1/d near zero
// volts) is formed first and Dc applied last, so no intermediate falls into
// FP32's denormal range even at BETSE's 1e-25 V nonce.
template <int ZC>
__device__ __forceinline__ float ghk_scaled(float kr, float kr2, float e1, float e2, float cA, float cB, float Dc) {
  if (ZC == 1) return Dc * (kr * fmaf(-cA, e1, cB));
  if (ZC == -1) return Dc * (kr * fmaf(cB, e1, -cA));
  if (ZC == 2) return Dc * (kr2 * fmaf(-cA, e2, cB));
  return Dc * (kr2 * fmaf(cB, e2, -cA));     // ZC == -2
}

// any charge: BETSE's formula with the same ordering of the small factors
__device__ __forceinline__ float ghk_scaled_generic(float zval, float v_nonce, float F_RT, float inv_d, float cA,
                                                   float cB, float Dc) {
  const float a = ((zval + 1.0e-25f) * v_nonce) * F_RT;
  return -(Dc * (((a * inv_d) / (-expm1f(-a))) * (cB - cA * expf(-a))));
}

template <int ZP>
__device__ __forceinline__ float ghk_by_charge(const SplitConst& k, int i, float kr, float kr2, float e1, float e2,
                                               float v_nonce, float inv_d, float cA, float cB, float Dc) {
  switch (IonSet<ZP>::zc(k, i)) {
    case 1: return ghk_scaled<1>(kr, kr2, e1, e2, cA, cB, Dc);
    case -1: return ghk_scaled<-1>(kr, kr2, e1, e2, cA, cB, Dc);
    case 2: return ghk_scaled<2>(kr, kr2, e1, e2, cA, cB, Dc);
    case -2: return ghk_scaled<-2>(kr, kr2, e1, e2, cA, cB, Dc);
    default: return ghk_scaled_generic(k.z[i], v_nonce, k.F_RT, inv_d, cA, cB, Dc);
  }
}

// -fgj * mem_sa of one gap junction, added to s2 (update_gj: the flux from the
// partner into this cell, with cA = this cell's and cB = the partner's
// membrane-side concentration, vgj = V_partner - V_cell, sim.py:2166-2199).
// gws = gj_weight * mem_sa of the membrane; the junction's diffusivity is
// D_gj,i * gj_surface * gj_block * gj_weight.
template <int ZP, int NI>
__device__ __forceinline__ void fact_gj_add(const SplitConst& k, int I, float v1, const float (&cin)[NI],
                                            const float4 n0, const float4 n1, float gws, float (&s2)[NI]) {
  const float nbr[8] = {n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, n1.z, n1.w};
  const float vgj1 = ((n1.w + 1.0e-25f) - v1) + 1.0e-25f;     // BETSE's nonces, sim_toolbox.py:52-56
  GhkShared<float> sg;
  ghk_init_f(sg, vgj1, k.F_RT);
  const float kr = gws * ((sg.a1 * k.inv_gjl) * sg.r);
  const float kr2 = 2.f * kr * sg.q2;
  const float e2 = sg.e1 * sg.e1;
#pragma unroll
  for (int i = 0; i < NI; ++i) {
    if (i >= I) break;
    const float dg = k.dgj_gs[i] * k.gj_block;
    if (IonSet<ZP>::zc(k, i) == 0)
      s2[i] -= gws * ghk_scaled_generic(k.z[i], vgj1, k.F_RT, k.inv_gjl, cin[i], nbr[i], dg);
    else
      s2[i] -= ghk_by_charge<ZP>(k, i, kr, kr2, sg.e1, e2, vgj1, k.inv_gjl, cin[i], nbr[i], dg);
  }
}

// The cell's transmembrane sums s1_i = sum_m f_i(m) mem_sa(m): GHK with the
// cell's DSA_i as diffusivity, plus the Na/K-ATPase (pumpNaKATP,
// sim_toolbox.py:71-122) times SA.
template <int ZP, int NI>
__device__ __forceinline__ void fact_trans(const SplitConst& k, int I, float v1, const float (&cin)[NI],
                                           const float (&cenv)[NI], float pc, const float (&dsa)[NI],
                                           float SA, float (&s1)[NI]) {
  using IS = IonSet<ZP>;
  GhkShared<float> sm;
  ghk_init_f(sm, v1, k.F_RT);
  const float kr = (sm.a1 * k.inv_tm) * sm.r;
  const float kr2 = 2.f * kr * sm.q2;
  const float e2 = sm.e1 * sm.e1;
  float fNa = 0.f;
  if (pc != 0.f) {
    float cNai = 0.f, cKi = 0.f, cNao = 0.f, cKo = 0.f;
#pragma unroll
    for (int i = 0; i < NI; ++i) {
      if (i == IS::iNa(k)) { cNai = cin[i]; cNao = cenv[i]; }
      if (i == IS::iK(k)) { cKi = cin[i]; cKo = cenv[i]; }
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
    float f = ghk_by_charge<ZP>(k, i, kr, kr2, sm.e1, e2, v1, k.inv_tm, cenv[i], cin[i], dsa[i]);
    if (i == IS::iNa(k)) f = fmaf(fNa, SA, f);
    else if (i == IS::iK(k)) f = fmaf((-(2.f / 3.f)) * fNa, SA, f);
    s1[i] = f;
  }
}

// update_all_concs (sim.py:2086-2111) and update_V (sim.py:2027-2029) of one
// cell in double-float, in the order of k_split_step: concentration plus the
// transmembrane term (that value is cc_at_mem, the record), plus the
// gap-junction term, no_negs, then the charge sum and Vmem.  cc points at the
// cell's first ion; ion i is cc[i * stride].
template <int NI>
__device__ __forceinline__ void fact_update(const SplitConst& k, int I, const float (&s1)[NI],
                                            const float (&s2)[NI], float dtv, float dvc, float2* cc,
                                            size_t stride, float (&rec)[8], unsigned& bad, unsigned& neg,
                                            unsigned& nanv) {
  df rho{0.f, 0.f};
#pragma unroll
  for (int i = 0; i < 7; ++i) rec[i] = 0.f;
#pragma unroll
  for (int i = 0; i < NI; ++i) {
    if (i >= I) break;
    const float2 x2 = cc[(size_t)i * stride];
    df x{x2.x, x2.y};
    x = df_add_f(x, s1[i] * dtv);
    if (i < 7) rec[i] = x.hi + x.lo;
    x = df_add_f(x, s2[i] * dtv);
    if (x.hi != x.hi) ++bad;
    if (x.hi < 0.f || (x.hi == 0.f && x.lo < 0.f)) { x = df{0.f, 0.f}; ++neg; }
    cc[(size_t)i * stride] = make_float2(x.hi, x.lo);
    rho = df_add(rho, df_mul(x, k.zF_hi[i], k.zF_lo[i]));
  }
  const float vc = (rho.hi + rho.lo) * dvc;
  rec[7] = vc;
  if (vc != vc) ++nanv;
}

// Sum of v over the warp's lanes (the order of k_split_step's tile partials).
__device__ __forceinline__ float warp_sum_down(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// One time step, streaming: NW warps per CTA, warp = tile, lane = cell slot.
// Each lane walks its cell's gap-junction entries U at a time (U = 2 or 4,
// chosen by the autotuner): the U entries, then the U partner records, are
// loaded before any of them is used, so a cell waits on two latency rounds
// per U junctions rather than two per junction.  Launched with programmatic dependent launch after
// k_split_env of the previous step; the static data is read before the
// dependency wait.
// ---------------------------------------------------------------------------
// PF > 0: the first PF gap-junction entries of each cell (static data) are
// loaded before the grid dependency wait, so after it each round of U
// junctions waits for the partner records only, not for the entry first.
template <int NW, int ZP, int U, int PF>
__global__ void __launch_bounds__(NW * 32)
k_split_fact(FactGeom fg, SplitPtrs p, SplitConst k) {
  static_assert(PF % U == 0, "prefetched entries come in whole rounds");
  using IS = IonSet<ZP>;
  constexpr int NI = IS::NI;
  const int I = IS::n(k);
  const int lane = threadIdx.x & 31;
  const int tile = blockIdx.x * NW + (threadIdx.x >> 5);
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 900)
  cudaTriggerProgrammaticLaunchCompletion();
#endif
  const bool tile_ok = tile < fg.ntile;            // warp-uniform
  const int s = tile * 32 + lane;
  float4 cs = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
  int gb = 0, cl = 0;
  float dsa[NI];
#pragma unroll
  for (int i = 0; i < NI; ++i) dsa[i] = 0.f;
  if (tile_ok) {
    cs = fg.cst[s];
    gb = fg.gbeg[s];
    cl = fg.blk_cluster[tile];
#pragma unroll
    for (int i = 0; i < NI; ++i)
      if (i < I) dsa[i] = fg.dsa[(size_t)i * fg.S + s];
  }
  const int gcnt = __float_as_int(cs.w);
  const bool live = tile_ok && gcnt >= 0;
  int2 pf[PF > 0 ? PF : 1];
#pragma unroll
  for (int u = 0; u < PF; ++u) pf[u] = (live && u < gcnt) ? fg.gj[gb + u] : make_int2(s, 0);

#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 900)
  cudaGridDependencySynchronize();
#endif
  float s1[NI];
#pragma unroll
  for (int i = 0; i < NI; ++i) s1[i] = 0.f;
  unsigned bad = 0, neg = 0, nanv = 0;
  if (live) {
    float own[8];
    load_rec<8>(p.rec_in, s, own);
    float cin[NI], cenv[NI], s2[NI];
#pragma unroll
    for (int i = 0; i < NI; ++i) {
      cin[i] = (i < I && i < 7) ? own[i] : 0.f;
      cenv[i] = (i < I) ? p.cenv_f[(size_t)cl * I + i] : 0.f;
      s2[i] = 0.f;
    }
    const float pc = p.pump_coef[cl];
    const float v1 = own[7] + 1.0e-25f;
    const int2* e = fg.gj + gb;
#pragma unroll
    for (int j = 0; j < PF; j += U) {
      if (j >= gcnt) break;
      float4 r0[U], r1[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const float4* r4 = reinterpret_cast<const float4*>(p.rec_in + (size_t)pf[j + u].x * 8);
        r0[u] = r4[0];
        r1[u] = r4[1];
      }
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (j + u < gcnt) fact_gj_add<ZP, NI>(k, I, v1, cin, r0[u], r1[u], __int_as_float(pf[j + u].y), s2);
    }
    for (int j = PF; j < gcnt; j += U) {
      int2 en[U];
#pragma unroll
      for (int u = 0; u < U; ++u) en[u] = (j + u < gcnt) ? e[j + u] : make_int2(s, 0);
      float4 r0[U], r1[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const float4* r4 = reinterpret_cast<const float4*>(p.rec_in + (size_t)en[u].x * 8);
        r0[u] = r4[0];
        r1[u] = r4[1];
      }
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (j + u < gcnt) fact_gj_add<ZP, NI>(k, I, v1, cin, r0[u], r1[u], __int_as_float(en[u].y), s2);
    }
    fact_trans<ZP, NI>(k, I, v1, cin, cenv, pc, dsa, cs.x, s1);
    float rec[8];
    fact_update<NI>(k, I, s1, s2, cs.y, cs.z, p.cc2 + s, (size_t)fg.S, rec, bad, neg, nanv);
    float4* o4 = reinterpret_cast<float4*>(p.rec_out + (size_t)s * 8);
    o4[0] = make_float4(rec[0], rec[1], rec[2], rec[3]);
    o4[1] = make_float4(rec[4], rec[5], rec[6], rec[7]);
  }
  if (tile_ok) {
#pragma unroll
    for (int i = 0; i < NI; ++i) {
      if (i >= I) break;
      const float e = warp_sum_down(s1[i]);
      if (lane == 0) p.env_part[(size_t)tile * I + i] = e;
    }
  }
  if (nanv) atomicAdd(&p.status[0], (unsigned long long)nanv);
  if (bad) atomicAdd(&p.status[1], (unsigned long long)bad);
  if (neg) atomicAdd(&p.status[2], (unsigned long long)neg);
}

// ---------------------------------------------------------------------------
// Many time steps in one cooperative launch (one cluster, no outputs).
//
// CTA j owns the tiles [tile0, tile0 + ntile) (ResCta).  For the whole run
// its shared memory holds the cells' static data, their concentrations
// (double-float) and a table of 32-byte cell records: its own cells first,
// then the "halo", the cells outside the CTA that its gap junctions name.
// Each cell's gap-junction entries carry the partner's index in that table,
// the partners the CTA owns first.  One thread advances one cell.  Step t:
//   a. the gap junctions to halo partners (table of parity t);
//   b. the per-cell terms and the update; the new record goes to the other
//      table and to the global record buffer, s1 to shared memory;
//   c. warp i sums ion i's s1 over the CTA's cells in a fixed order
//      (double-float), stores the CTA's partial in global memory
//      (double-buffered by parity) and arrives at the grid barrier (release);
//   d. meanwhile, and until the barrier completes, every thread sums the gap
//      junctions of step t+1 to partners the CTA owns: their records are in
//      the new table already;
//   e. thread 0 waits for the barrier (acquire, bounded);
//   f. every CTA sums all CTAs' partials in the same fixed order (so the
//      environment is identical everywhere), updates the well-mixed
//      environment in FP64 as k_split_env does, and copies its halo records
//      from global memory into the new table.
// So the barrier's latency overlaps most of the gap-junction work.  The wait
// gives up after `timeout_ns` (it then raises ctl[1] = 1 and returns), so a
// lost CTA cannot hang the GPU.
// ---------------------------------------------------------------------------
struct ResCta {
  int tile0, ntile;        // tiles (cell slots [32*tile0, 32*(tile0+ntile)))
  int ent0, nent;          // gap-junction entries in ResArrays::gj
  int halo0, nhalo;        // halo cell slots in ResArrays::halo
  int pad[2];
};

struct ResArrays {
  const ResCta* __restrict__ cta;          // [grid]
  const int2* __restrict__ gj;             // {index in the CTA's record table, bits of gj_weight*mem_sa}
  const int2* __restrict__ gbeg;           // [S] {first entry relative to the CTA's ent0, entries to owned cells}
  const int* __restrict__ halo;            // global cell slots of each CTA's halo
  float2* __restrict__ cpart;              // [2][grid][I] per-CTA environment partials (hi, lo)
  unsigned* __restrict__ ctl;              // [0] barrier counter (zeroed before the launch), [1] timeout flag
  double* __restrict__ cenv64;             // [I] well-mixed environment (FP64)
  float* __restrict__ cenv_f;              // [I] its FP32 copy (the tile kernels read it)
  const double* __restrict__ env_scale;    // [1] dt / (vol_env * M)
  float* __restrict__ rec_glob[2];         // the global record buffers (rec_in = [0] at step 0)
  int ntile_max, nent_max, nhalo_max;
  long long timeout_ns;
  unsigned barrier_bias;                   // 0; > 0 only in the barrier self-check (a target never reached)
};

// Shared-memory layout of k_split_resident, in bytes from the (16-byte
// aligned) base; the host sizes the launch with the same function.
struct ResSmem {
  int n_own, n_tab;
  size_t tab, cc2, dsa, s1, cst, gbeg, gj, halo, cenv, flag, total;
  __host__ __device__ static size_t up16(size_t x) { return (x + 15) & ~size_t(15); }
  __host__ __device__ ResSmem(int ntile_max, int nent_max, int nhalo_max, int NI) {
    n_own = 32 * ntile_max;
    n_tab = n_own + nhalo_max;
    size_t o = 0;
    tab = o;   o = up16(o + (size_t)2 * n_tab * 8 * sizeof(float));
    cc2 = o;   o = up16(o + (size_t)NI * n_own * sizeof(float2));
    dsa = o;   o = up16(o + (size_t)NI * n_own * sizeof(float));
    s1 = o;    o = up16(o + (size_t)NI * n_own * sizeof(float));
    cst = o;   o = up16(o + (size_t)n_own * sizeof(float4));
    gbeg = o;  o = up16(o + (size_t)n_own * sizeof(int2));
    gj = o;    o = up16(o + (size_t)(nent_max > 0 ? nent_max : 1) * sizeof(int2));
    halo = o;  o = up16(o + (size_t)(nhalo_max > 0 ? nhalo_max : 1) * sizeof(int));
    cenv = o;  o = up16(o + (size_t)NI * (sizeof(double) + sizeof(float)));
    flag = o;  o = up16(o + 16);
    total = o;
  }
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Arrival at the grid barrier: release, so this thread's writes (and those
// it observed, e.g. through the preceding bar.sync) are visible first.
__device__ __forceinline__ void res_arrive(unsigned* ctl) {
  asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(ctl) : "memory");
}

// Thread 0 waits until ctl[0] reaches `target` (acquire), or until another
// CTA raised ctl[1], or until timeout_ns passed (then it raises ctl[1]
// itself); the result is broadcast through *sflag after a bar.sync.
__device__ __forceinline__ bool res_wait(unsigned* ctl, unsigned target, long long timeout_ns, int* sflag) {
  if (threadIdx.x == 0) {
    const unsigned long long t0 = global_ns();
    int ok = 1;
    unsigned n = 0;
    while (true) {
      unsigned v, f;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctl) : "memory");
      if ((int)(v - target) >= 0) break;
      if ((++n & 31u) == 0) {
        asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(f) : "l"(ctl + 1) : "memory");
        if (f) { ok = 0; break; }
        if ((long long)(global_ns() - t0) > timeout_ns) {
          atomicExch(ctl + 1, 1u);
          ok = 0;
          break;
        }
      }
    }
    *sflag = ok;
  }
  __syncthreads();
  return *sflag != 0;
}

// Gap-junction entries [j0, j1) of one cell from table T into s2.
template <int ZP, int NI>
__device__ __forceinline__ void res_gj_range(const SplitConst& k, int I, const float* __restrict__ T,
                                             const int2* __restrict__ e, int j0, int j1, const float* own,
                                             float (&s2)[NI]) {
  const float4 o1 = reinterpret_cast<const float4*>(own)[1];
  const float4 o0 = reinterpret_cast<const float4*>(own)[0];
  const float ov[8] = {o0.x, o0.y, o0.z, o0.w, o1.x, o1.y, o1.z, o1.w};
  float cin[NI];
#pragma unroll
  for (int i = 0; i < NI; ++i) cin[i] = (i < I && i < 7) ? ov[i] : 0.f;
  const float v1 = o1.w + 1.0e-25f;
  for (int j = j0; j < j1; ++j) {
    const int2 en = e[j];
    const float4* r4 = reinterpret_cast<const float4*>(T + (size_t)en.x * 8);
    fact_gj_add<ZP, NI>(k, I, v1, cin, r4[0], r4[1], __int_as_float(en.y), s2);
  }
}

template <int ZP>
__global__ void __launch_bounds__(1024, 1)
k_split_resident(FactGeom fg, SplitPtrs p, SplitConst k, ResArrays ra, int n_steps) {
  using IS = IonSet<ZP>;
  constexpr int NI = IS::NI;
  constexpr int CPT = 2;                                         // cells per thread kept in registers (max)
  const int I = IS::n(k);
  extern __shared__ __align__(16) unsigned char res_smem[];
  const ResSmem L(ra.ntile_max, ra.nent_max, ra.nhalo_max, NI);
  float* tab = reinterpret_cast<float*>(res_smem + L.tab);      // [2][n_tab][8]
  float2* scc = reinterpret_cast<float2*>(res_smem + L.cc2);    // [NI][n_own]
  float* sdsa = reinterpret_cast<float*>(res_smem + L.dsa);     // [NI][n_own]
  float* ss1 = reinterpret_cast<float*>(res_smem + L.s1);       // [NI][n_own]
  float4* scst = reinterpret_cast<float4*>(res_smem + L.cst);   // [n_own]
  int2* sgb = reinterpret_cast<int2*>(res_smem + L.gbeg);       // [n_own]
  int2* sgj = reinterpret_cast<int2*>(res_smem + L.gj);         // [nent]
  int* shalo = reinterpret_cast<int*>(res_smem + L.halo);       // [nhalo]
  double* cenv64 = reinterpret_cast<double*>(res_smem + L.cenv);  // [NI]
  float* cenvf = reinterpret_cast<float*>(cenv64 + NI);         // [NI]
  int* sflag = reinterpret_cast<int*>(res_smem + L.flag);

  const ResCta me = ra.cta[blockIdx.x];
  const int t = threadIdx.x, NT = blockDim.x;
  const int lane = t & 31, w = t >> 5, NW = NT >> 5;
  const int n_own = 32 * me.ntile, n_tab = L.n_tab;
  const int slot0 = 32 * me.tile0;

  // ---- stage the CTA's data (once per launch)
  for (int ls = t; ls < n_own; ls += NT) {
    const int s = slot0 + ls;
    scst[ls] = fg.cst[s];
    sgb[ls] = ra.gbeg[s];
#pragma unroll
    for (int i = 0; i < NI; ++i)
      if (i < I) {
        sdsa[(size_t)i * n_own + ls] = fg.dsa[(size_t)i * fg.S + s];
        scc[(size_t)i * n_own + ls] = p.cc2[(size_t)i * fg.S + s];
        ss1[(size_t)i * n_own + ls] = 0.f;
      }
    const float4* r4 = reinterpret_cast<const float4*>(ra.rec_glob[0] + (size_t)s * 8);
    float4* t4 = reinterpret_cast<float4*>(tab + (size_t)ls * 8);
    t4[0] = r4[0];
    t4[1] = r4[1];
  }
  for (int j = t; j < me.nent; j += NT) sgj[j] = ra.gj[me.ent0 + j];
  for (int h = t; h < me.nhalo; h += NT) {
    const int s = ra.halo[me.halo0 + h];
    shalo[h] = s;
    const float4* r4 = reinterpret_cast<const float4*>(ra.rec_glob[0] + (size_t)s * 8);
    float4* t4 = reinterpret_cast<float4*>(tab + (size_t)(n_own + h) * 8);
    t4[0] = r4[0];
    t4[1] = r4[1];
  }
  if (t < I) {
    cenv64[t] = ra.cenv64[t];
    cenvf[t] = (float)cenv64[t];
  }
  const float pc = p.pump_coef[0];
  const double escale = ra.env_scale[0];
  __syncthreads();

  // cells of this thread: ls = t + q * NT (q < CPT); their gap-junction sums
  // to owned partners are carried across the barrier in registers
  float s2c[CPT][NI];
#pragma unroll
  for (int q = 0; q < CPT; ++q) {
    const int ls = t + q * NT;
#pragma unroll
    for (int i = 0; i < NI; ++i) s2c[q][i] = 0.f;
    if (ls < n_own && __float_as_int(scst[ls].w) >= 0) {
      const int2 gb = sgb[ls];
      res_gj_range<ZP, NI>(k, I, tab, sgj, gb.x, gb.x + gb.y, tab + (size_t)ls * 8, s2c[q]);
    }
  }

  unsigned bad = 0, neg = 0, nanv = 0;
  int step = 0;
  for (; step < n_steps; ++step) {
    const int par = step & 1;
    const float* T = tab + (size_t)par * n_tab * 8;
    float* Tn = tab + (size_t)(par ^ 1) * n_tab * 8;
    float* rg = ra.rec_glob[par ^ 1];
    // ---- a, b: halo gap junctions, per-cell terms, update
#pragma unroll
    for (int q = 0; q < CPT; ++q) {
      const int ls = t + q * NT;
      if (ls >= n_own) continue;
      const float4 cs = scst[ls];
      const int gcnt = __float_as_int(cs.w);
      if (gcnt < 0) continue;
      const float* own = T + (size_t)ls * 8;
      const int2 gb = sgb[ls];
      res_gj_range<ZP, NI>(k, I, T, sgj, gb.x + gb.y, gb.x + gcnt, own, s2c[q]);
      const float4 o0 = reinterpret_cast<const float4*>(own)[0];
      const float4 o1 = reinterpret_cast<const float4*>(own)[1];
      const float ov[8] = {o0.x, o0.y, o0.z, o0.w, o1.x, o1.y, o1.z, o1.w};
      float cin[NI], cenv[NI], dsa[NI], s1[NI];
#pragma unroll
      for (int i = 0; i < NI; ++i) {
        cin[i] = (i < I && i < 7) ? ov[i] : 0.f;
        cenv[i] = (i < I) ? cenvf[i] : 0.f;
        dsa[i] = (i < I) ? sdsa[(size_t)i * n_own + ls] : 0.f;
      }
      fact_trans<ZP, NI>(k, I, o1.w + 1.0e-25f, cin, cenv, pc, dsa, cs.x, s1);
      float rec[8];
      fact_update<NI>(k, I, s1, s2c[q], cs.y, cs.z, scc + ls, (size_t)n_own, rec, bad, neg, nanv);
#pragma unroll
      for (int i = 0; i < NI; ++i)
        if (i < I) ss1[(size_t)i * n_own + ls] = s1[i];
      const float4 r0 = make_float4(rec[0], rec[1], rec[2], rec[3]);
      const float4 r1 = make_float4(rec[4], rec[5], rec[6], rec[7]);
      reinterpret_cast<float4*>(Tn + (size_t)ls * 8)[0] = r0;
      reinterpret_cast<float4*>(Tn + (size_t)ls * 8)[1] = r1;
      reinterpret_cast<float4*>(rg + (size_t)(slot0 + ls) * 8)[0] = r0;
      reinterpret_cast<float4*>(rg + (size_t)(slot0 + ls) * 8)[1] = r1;
    }
    __syncthreads();
    // ---- c: the CTA's partial of ion i (warp w takes ions w, w + NW, ...),
    // lane l sums cells l, l + 32, ... in order, then a fixed shuffle tree
    float2* cp = ra.cpart + (size_t)par * gridDim.x * I;
    for (int i = w; i < I; i += NW) {
      const float* v = ss1 + (size_t)i * n_own;
      float f = 0.f;
      for (int ls = lane; ls < n_own; ls += 32) f += v[ls];
      df a{f, 0.f};
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const df b{__shfl_down_sync(0xffffffffu, a.hi, o), __shfl_down_sync(0xffffffffu, a.lo, o)};
        a = df_add(a, b);
      }
      if (lane == 0) {
        cp[(size_t)blockIdx.x * I + i] = make_float2(a.hi, a.lo);
        res_arrive(ra.ctl);
      }
    }
    const bool last = step + 1 == n_steps;
    // ---- d: gap junctions of step t+1 to owned partners, from the new table
    if (!last) {
#pragma unroll
      for (int q = 0; q < CPT; ++q) {
        const int ls = t + q * NT;
#pragma unroll
        for (int i = 0; i < NI; ++i) s2c[q][i] = 0.f;
        if (ls < n_own && __float_as_int(scst[ls].w) >= 0) {
          const int2 gb = sgb[ls];
          res_gj_range<ZP, NI>(k, I, Tn, sgj, gb.x, gb.x + gb.y, Tn + (size_t)ls * 8, s2c[q]);
        }
      }
    }
    // ---- e: the barrier
    const unsigned target = (unsigned)(step + 1) * gridDim.x * (unsigned)I + ra.barrier_bias;
    if (!res_wait(ra.ctl, target, ra.timeout_ns, sflag)) break;
    // ---- f: the environment (identical in every CTA) and the halo records
    for (int i = w; i < I; i += NW) {
      df a{0.f, 0.f};
      for (int c = lane; c < (int)gridDim.x; c += 32) {
        const float2 v = __ldcg(cp + (size_t)c * I + i);
        a = df_add(a, df{v.x, v.y});
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const df b{__shfl_down_sync(0xffffffffu, a.hi, o), __shfl_down_sync(0xffffffffu, a.lo, o)};
        a = df_add(a, b);
      }
      if (lane == 0) {
        const double v = cenv64[i] - ((double)a.hi + (double)a.lo) * escale;
        cenv64[i] = v;
        cenvf[i] = (float)v;
      }
    }
    if (!last)
      for (int h = t; h < me.nhalo; h += NT) {
        const float4* r4 = reinterpret_cast<const float4*>(rg + (size_t)shalo[h] * 8);
        float4* t4 = reinterpret_cast<float4*>(Tn + (size_t)(n_own + h) * 8);
        t4[0] = __ldcg(r4);
        t4[1] = __ldcg(r4 + 1);
      }
    __syncthreads();
  }
  // ---- write back: concentrations; CTA 0 the environment
  if (step == n_steps) {
    for (int ls = t; ls < n_own; ls += NT) {
      const int s = slot0 + ls;
#pragma unroll
      for (int i = 0; i < NI; ++i)
        if (i < I) p.cc2[(size_t)i * fg.S + s] = scc[(size_t)i * n_own + ls];
    }
    if (blockIdx.x == 0 && t < I) {
      ra.cenv64[t] = cenv64[t];
      ra.cenv_f[t] = cenvf[t];
    }
  }
  if (nanv) atomicAdd(&p.status[0], (unsigned long long)nanv);
  if (bad) atomicAdd(&p.status[1], (unsigned long long)bad);
  if (neg) atomicAdd(&p.status[2], (unsigned long long)neg);
}

// ---------------------------------------------------------------------------
// The streaming factored step, persistent and software-pipelined.  Each warp
// walks its own tiles t_j = warp + j * (warps of the grid) and stages them in
// shared memory with cp.async (16-byte asynchronous copies that complete at
// cp.async.wait_group -- no waits of ours): while it computes tile t_j, the
// cell data of t_{j+1}, the gap-junction entries of t_{j+2} and the partner
// records of t_{j+1} (gathered by the entries, which landed one iteration
// earlier) are in flight.  The arithmetic is k_split_fact's, term by term, so
// the results are bit-identical.  Per warp: two cell-data buffers, three
// entry buffers and two record buffers (FactPipeSmem).
// ---------------------------------------------------------------------------
template <int NI>
struct FactCellBuf {                   // one tile's cell data, in the order of its copy
  float4 cst[32];
  int gbeg[32];
  float dsa[NI][32];
  float2 cc2[NI][32];
  float rec[32][8];
};

struct FactPipeSmem {
  int emax;                            // entries per tile buffer (the largest tile's, + 2 for alignment)
  size_t cell_bytes, ent_bytes, rec_bytes, warp_bytes;
  __host__ __device__ FactPipeSmem(int max_entries, int NI) {
    emax = max_entries + 2;
    cell_bytes = (size_t)32 * 16 + 32 * 4 + (size_t)NI * 32 * 4 + (size_t)NI * 32 * 8 + 32 * 32;
    ent_bytes = (size_t)emax * 8;
    ent_bytes = (ent_bytes + 15) & ~(size_t)15;
    rec_bytes = (size_t)emax * 32;
    warp_bytes = 2 * cell_bytes + 3 * ent_bytes + 2 * rec_bytes;
  }
};

template <int NW, int ZP>
__global__ void __launch_bounds__(NW * 32)
k_split_fact_pipe(FactGeom fg, SplitPtrs p, SplitConst k, const int* __restrict__ tile_e0, int max_entries) {
  using IS = IonSet<ZP>;
  constexpr int NI = IS::NI;
  using CB = FactCellBuf<NI>;
  const int I = IS::n(k);
  extern __shared__ __align__(16) unsigned char fp_smem[];
  const FactPipeSmem L(max_entries, NI);
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  unsigned char* base = fp_smem + (size_t)wl * L.warp_bytes;
  const unsigned cell_b = (unsigned)L.cell_bytes, ent_b = (unsigned)L.ent_bytes, rec_b = (unsigned)L.rec_bytes;
  auto cb = [&](int q) { return reinterpret_cast<CB*>(base + q * cell_b); };
  auto eb = [&](int q) { return reinterpret_cast<int2*>(base + 2 * cell_b + q * ent_b); };
  auto rb = [&](int q) { return reinterpret_cast<float*>(base + 2 * cell_b + 3 * ent_b + q * rec_b); };
  const int stride = gridDim.x * NW;
  const int t0 = blockIdx.x * NW + wl;
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 900)
  cudaTriggerProgrammaticLaunchCompletion();
  cudaGridDependencySynchronize();
#endif
  // the copies of one tile's cell data (contiguous ranges of the per-slot arrays)
  auto issue_cells = [&](int t, CB* d) {
    if (t >= fg.ntile) return;
    const int s0 = t * 32;
    char* dst = reinterpret_cast<char*>(d);
    const int n_cst = 32, n_gb = 8, n_dsa = NI * 8, n_cc = NI * 16, n_rec = 64;
    const int total = n_cst + n_gb + n_dsa + n_cc + n_rec;
    for (int c = lane; c < total; c += 32) {
      const char* src;
      char* to;
      int r = c;
      if (r < n_cst) { src = reinterpret_cast<const char*>(fg.cst + s0) + 16 * r; to = reinterpret_cast<char*>(d->cst) + 16 * r; }
      else if ((r -= n_cst) < n_gb) { src = reinterpret_cast<const char*>(fg.gbeg + s0) + 16 * r; to = reinterpret_cast<char*>(d->gbeg) + 16 * r; }
      else if ((r -= n_gb) < n_dsa) {
        const int i = r / 8, o = 16 * (r % 8);
        if (i >= I) continue;
        src = reinterpret_cast<const char*>(fg.dsa + (size_t)i * fg.S + s0) + o; to = reinterpret_cast<char*>(d->dsa[i]) + o;
      } else if ((r -= n_dsa) < n_cc) {
        const int i = r / 16, o = 16 * (r % 16);
        if (i >= I) continue;
        src = reinterpret_cast<const char*>(p.cc2 + (size_t)i * fg.S + s0) + o; to = reinterpret_cast<char*>(d->cc2[i]) + o;
      } else {
        r -= n_cc;
        src = reinterpret_cast<const char*>(p.rec_in + (size_t)s0 * 8) + 16 * r; to = reinterpret_cast<char*>(d->rec) + 16 * r;
      }
      (void)dst;
      cp16(to, src);
    }
  };
  // the tile's entries, from the 16-byte boundary at or below its first
  auto issue_entries = [&](int t, int2* d) {
    if (t >= fg.ntile) return;
    const int e0 = tile_e0[t] & ~1, e1 = tile_e0[t + 1];
    const int n16 = (e1 - e0 + 1) >> 1;
    for (int c = lane; c < n16; c += 32) cp16(d + 2 * c, fg.gj + e0 + 2 * c);
  };
  // the partner records of the tile's entries, in entry order
  auto issue_records = [&](int t, const int2* e, float* d) {
    if (t >= fg.ntile) return;
    const int ea = tile_e0[t], off = ea - (ea & ~1), n = tile_e0[t + 1] - ea;
    for (int j = lane; j < n; j += 32) {
      const float* src = p.rec_in + (size_t)e[off + j].x * 8;
      cp16(d + 8 * j, src);
      cp16(d + 8 * j + 4, src + 4);
    }
  };

  // prologue: cells and entries of t0, entries of t1; then records of t0
  issue_cells(t0, cb(0));
  issue_entries(t0, eb(0));
  cp_commit();
  issue_entries(t0 + stride, eb(1));
  cp_commit();
  asm volatile("cp.async.wait_group 1;\n" ::: "memory");
  __syncwarp();
  issue_records(t0, eb(0), rb(0));
  cp_commit();

  unsigned bad = 0, neg = 0, nanv = 0;
  int j = 0;
  for (int t = t0; t < fg.ntile; t += stride, ++j) {
    const int ca = j & 1, ea = j % 3;
    issue_cells(t + stride, cb(ca ^ 1));
    issue_entries(t + 2 * stride, eb((j + 2) % 3));
    cp_commit();
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");   // cells, entries and records of t; entries of t+1
    __syncwarp();
    issue_records(t + stride, eb((j + 1) % 3), rb(ca ^ 1));
    cp_commit();

    const CB& c = *cb(ca);
    const int2* e = eb(ea);
    const float* rr = rb(ca);
    const float4 cs = c.cst[lane];
    const int gcnt = __float_as_int(cs.w);
    const int cl = fg.blk_cluster[t];
    const int tfirst = tile_e0[t];
    const int eoff = tfirst - (tfirst & ~1);
    float s1[NI];
#pragma unroll
    for (int i = 0; i < NI; ++i) s1[i] = 0.f;
    if (gcnt >= 0) {
      const float* own = c.rec[lane];
      const float4 o0 = reinterpret_cast<const float4*>(own)[0];
      const float4 o1 = reinterpret_cast<const float4*>(own)[1];
      const float ov[8] = {o0.x, o0.y, o0.z, o0.w, o1.x, o1.y, o1.z, o1.w};
      float cin[NI], cenv[NI], s2[NI], dsa[NI];
#pragma unroll
      for (int i = 0; i < NI; ++i) {
        cin[i] = (i < I && i < 7) ? ov[i] : 0.f;
        cenv[i] = (i < I) ? p.cenv_f[(size_t)cl * I + i] : 0.f;
        dsa[i] = (i < I) ? c.dsa[i][lane] : 0.f;
        s2[i] = 0.f;
      }
      const float pc = p.pump_coef[cl];
      const float v1 = o1.w + 1.0e-25f;
      const int j0 = c.gbeg[lane] - tfirst;
      for (int q = j0; q < j0 + gcnt; ++q) {
        const float4* r4 = reinterpret_cast<const float4*>(rr + 8 * q);
        fact_gj_add<ZP, NI>(k, I, v1, cin, r4[0], r4[1], __int_as_float(e[eoff + q].y), s2);
      }
      fact_trans<ZP, NI>(k, I, v1, cin, cenv, pc, dsa, cs.x, s1);
      // the update reads the staged concentrations and writes the new ones to global memory
      float2 x2[NI];
#pragma unroll
      for (int i = 0; i < NI; ++i) x2[i] = (i < I) ? c.cc2[i][lane] : make_float2(0.f, 0.f);
      float rec[8];
      fact_update<NI>(k, I, s1, s2, cs.y, cs.z, x2, (size_t)1, rec, bad, neg, nanv);
      const int s = t * 32 + lane;
#pragma unroll
      for (int i = 0; i < NI; ++i)
        if (i < I) p.cc2[(size_t)i * fg.S + s] = x2[i];
      float4* o4 = reinterpret_cast<float4*>(p.rec_out + (size_t)s * 8);
      o4[0] = make_float4(rec[0], rec[1], rec[2], rec[3]);
      o4[1] = make_float4(rec[4], rec[5], rec[6], rec[7]);
    }
#pragma unroll
    for (int i = 0; i < NI; ++i) {
      if (i >= I) break;
      const float v = warp_sum_down(s1[i]);
      if (lane == 0) p.env_part[(size_t)t * I + i] = v;
    }
    __syncwarp();     // every lane is done with the buffers of t before they are refilled
  }
  cp_wait_all();
  if (nanv) atomicAdd(&p.status[0], (unsigned long long)nanv);
  if (bad) atomicAdd(&p.status[1], (unsigned long long)bad);
  if (neg) atomicAdd(&p.status[2], (unsigned long long)neg);
}

}  // namespace bx
