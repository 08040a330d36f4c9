// bx_network.cuh -- the molecule / gene-regulatory-network step on the GPU.
//
// MasterOfNetworks.run_loop (chemistry/networks.py:2805-2983) for the
// substances of one network on a plain FP64 cluster without extracellular
// spaces, as two kernels per time step, one thread per cell:
//
//   k_net_cell  per cell: Molecule.update_intra of every substance
//               (networks.py:5714-5807); growth/decay and cell-zone reaction
//               rates from the influencer tables (write_growth_and_decay,
//               write_reactions, get_influencers); c += (RM @ rates) dt; then
//               molecule_mover's membrane GHK flux and update_Co
//               (sim_toolbox.py:939-964, 1155-1207).  Writes the cell and
//               membrane values after the membrane step ("mid") and one
//               partial sum of flux * mem_sa per substance per CTA (the
//               auto-mixed environment, sim_toolbox.py:1196-1205).
//   k_net_gj    per cell: the gap-junction GHK flux (sim_toolbox.py:967-1000)
//               between the mid values of the membrane and its partner, the
//               final cell and membrane values and the negative-concentration
//               checks (sim_toolbox.py:1125-1151).  CTA 0 also reduces the
//               environment partials in a fixed order.
//
// The split into two launches is the one place the step needs every cell:
// the gap-junction flux reads the partner cell after its membrane step.
//
// Data layout in HBM (row = substance): c_cells [S][C], cc_at_mem [S][M] and
// their "mid" copies, the last step's fluxes f_mem/f_gj [S][M] and reaction
// rates [R][C], growth
// modulation [S][C] and target masks [S][C] only for the substances that have
// them, env [S], env partials [nblk][S]; the tables (substances, terms,
// reactions, stoichiometry) are one small block in global memory that every
// warp reads uniformly.  Geometry and Vmem are the cluster handle's own arrays.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "bx_kernels.cuh"

namespace bx {

constexpr int kNetMaxSub = 16;
constexpr int kNetMaxReact = 32;
constexpr int kNetMaxTerms = 256;
constexpr int kNetStoich = 4;
constexpr int kNetTPB = 128;

enum NetTermKind { NT_ACT = 0, NT_ACT_INDEP = 1, NT_INH = 2, NT_DIRECT_POS = 3, NT_DIRECT_NEG = 4 };

struct NetTermD {
  int kind, sub, env, pad;
  double inv_km, n;        // 1 / Km (the host divides once)
};

struct NetSubD {
  double z, Dm, Do, Dgj, tdf, r_prod, r_decay, decay_max, inv_gsf;
  int growth, ui, gj_imp, gt0, gnt, dt0, dnt, mod_row, mask_row, pad;
};

struct NetReactD {
  int nr, np, r[kNetStoich], p[kNetStoich];
  double rc[kNetStoich], inv_rkm[kNetStoich], pc[kNetStoich];
  double vmax, inv_keq;    // inv_keq 0: no standard free energy
  int t0, nt;
};

// The tables, one block of plain data.
struct NetTables {
  int S, R, T, pad;
  NetSubD sub[kNetMaxSub];
  NetReactD react[kNetMaxReact];
  double rm[kNetMaxSub][kNetMaxReact];   // stoichiometry of the reactions (create_reaction_matrix)
  NetTermD term[kNetMaxTerms];
};

struct NetArgs {
  int C, M;
  double dt, inv_tm, F_RT, inv_gj_len, gj_block, inv_vol_env_M;
  // cluster geometry and state (the handle's arrays)
  const int* cell_ptr;
  const int* nn;
  const int* nn_cell;
  const uint8_t* bflag;
  const double* mem_sa;
  const double* cell_vol;
  const double* gj_w;        // static weights (times gj_block: sim.gjopen)
  const double* gjo;         // gated open fraction, or nullptr
  const double* vm;          // Vmem the network reads (the start of the ion step)
  // network
  const NetTables* tab;
  const double* gamma;       // [M] mem_sa / ((3/4) mem_vol)
  const double* g_over_r;    // [M] gamma / R_rads
  const double* gmod;        // [rows][C]
  const uint8_t* gmask;      // [rows][C]
  double* c_cells;           // [S][C]
  double* cmem;              // [S][M]
  double* c_mid;             // [S][C]
  double* cmem_mid;          // [S][M]
  double* env;               // [S]
  double* env_part;          // [nblk][S]
  double* f_mem;             // [S][M] (OUT)
  double* f_gj;              // [S][M] (OUT)
  double* rates;             // [R][C] (OUT) cell-zone reaction rates (MasterOfNetworks.reaction_rates)
  unsigned long long* neg;   // negative concentrations seen
  int nblk;
};

// sim_toolbox.electroflux (sim_toolbox.py:18-69) for a general charge, FP64,
// with Dk = Dc / d and zF = (z + 1e-25) F / (R T) hoisted out of the
// membrane loops, and the FP64 transcendentals only where they carry
// information (the GPU's FP64 pipe bounds these kernels):
//   |a| < 1e-17 (every neutral substance: a = 1e-25 v F/RT): exp(-a) rounds
//     to 1 and expm1(-a) to -a, in FP64 as in NumPy, so the flux is
//     -Dk (cB - cA) (a few ulp from BETSE's order of operations);
//   |a| > 1e-3: -expm1(-a) = 1 - exp(-a) to within 1e-13 relative;
//   otherwise (small gap-junction voltages) the Taylor series of expm1(-a)
//   to the fifth power, whose remainder a^6/720 is below 2e-21 |a|.
__device__ __forceinline__ bool net_neutral(double zF) { return fabs(zF) < 1.0e-20; }

__device__ __forceinline__ double net_ghk(double cA, double cB, double Dk, double zF, bool neutral, double v) {
  if (neutral) return -Dk * (cB - cA);
  const double a = zF * (v + kNonce);
  const double aa = fabs(a);
  if (aa < 1.0e-17) return -Dk * (cB - cA);
  double ea, den;
  if (aa > 1.0e-3) {
    ea = exp(-a);
    den = 1.0 - ea;
  } else {
    const double x = -a;
    const double em1 = x * (1.0 + x * (0.5 + x * (1.0 / 6.0 + x * (1.0 / 24.0 + x * (1.0 / 120.0)))));
    ea = 1.0 + em1;
    den = -em1;
  }
  return -(Dk * a) * ((cB - cA * ea) / den);
}

// (c/Km)^n: BETSE's '**' (C pow); exponents 1 and 2 by multiplication (the
// same value as a correctly rounded pow), others by pow.
__device__ __forceinline__ double net_pow(double x, double n) {
  if (n == 1.0) return x;
  if (n == 2.0) return x * x;
  return pow(x, n);
}

__device__ __forceinline__ double net_conc(const NetTermD& t, const double* cs, const double* env) {
  return t.env ? env[t.sub] : cs[t.sub];
}

// One influencer factor (get_influencers, networks.py:5084-5600).  The host
// orders a factor's terms as BETSE composes its string: multiplicative
// activators, independent activators, inhibitors, then the direct terms
// (activators' before inhibitors'), so one pass evaluates it in BETSE's
// operation order: ((a1*a2) + i1 + i2) * (h1*h2) * (d1 + d2 ...).
__device__ double net_factor(const NetTables& tb, int t0, int nt, const double* cs, const double* env) {
  double act = 1.0, inh = 1.0, dsum = 0.0;
  bool any_mult = false, any_inh = false, any_direct = false;
  for (int q = t0; q < t0 + nt; ++q) {
    const NetTermD& t = tb.term[q];
    const double c = net_conc(t, cs, env);
    switch (t.kind) {
      case NT_ACT: {
        const double x = net_pow(c * t.inv_km, t.n);
        const double h = x / (1.0 + x);
        act = any_mult ? act * h : h;
        any_mult = true;
        break;
      }
      case NT_ACT_INDEP: {
        const double x = net_pow(c * t.inv_km, t.n);
        act = act + x / (1.0 + x);
        break;
      }
      case NT_INH: {
        const double h = 1.0 / (1.0 + net_pow(c * t.inv_km, t.n));
        inh = any_inh ? inh * h : h;
        any_inh = true;
        break;
      }
      case NT_DIRECT_POS:
        dsum = any_direct ? dsum + c : c;
        any_direct = true;
        break;
      default:
        dsum = any_direct ? dsum - c : -c;
        any_direct = true;
        break;
    }
  }
  const double a = act * inh;
  return any_direct ? a * dsum : a;
}

// Sums v over the CTA in a fixed order (warp tree, then warps in order) and
// writes the total from thread 0.
__device__ __forceinline__ double net_block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
  __syncthreads();
  return s;
}

template <bool OUT>
__global__ void __launch_bounds__(kNetTPB) k_net_cell(NetArgs a) {
  // the tables are read in place: every lane of a warp reads the same entry,
  // one broadcast load from L1
  const NetTables& tb = *a.tab;
  __shared__ double red[kNetTPB / 32];
  const int S = tb.S, R = tb.R;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = c < a.C;
  double cs[kNetMaxSub], env[kNetMaxSub], fsum[kNetMaxSub];
  for (int k = 0; k < S; ++k) {
    cs[k] = live ? a.c_cells[(size_t)k * a.C + c] : 0.0;
    env[k] = a.env[k];
    fsum[k] = 0.0;
  }
  int neg = 0;
  if (live) {
    const int m0 = a.cell_ptr[c], m1 = a.cell_ptr[c + 1];
    // rates (write_growth_and_decay / write_reactions) on the concentrations
    // at the start of the step
    double delta[kNetMaxSub];
    for (int k = 0; k < S; ++k) {
      const NetSubD& sb = tb.sub[k];
      double r = 0.0;
      const bool target = sb.mask_row < 0 || a.gmask[(size_t)sb.mask_row * a.C + c];
      if (sb.growth && target) {
        const double mod = sb.mod_row < 0 ? 1.0 : a.gmod[(size_t)sb.mod_row * a.C + c];
        const double cc = cs[k] * sb.inv_gsf;
        const double ga = net_factor(tb, sb.gt0, sb.gnt, cs, env);
        const double da = net_factor(tb, sb.dt0, sb.dnt, cs, env);
        r = mod * (sb.r_prod * sb.tdf) * ga - (sb.r_decay * sb.tdf) * cc - (sb.decay_max * sb.tdf) * da * cc;
      }
      delta[k] = r;
    }
    for (int j = 0; j < R; ++j) {
      const NetReactD& rx = tb.react[j];
      const double al = net_factor(tb, rx.t0, rx.nt, cs, env);
      double rate;
      if (rx.inv_keq == 0.0) {
        double fwd = 1.0;
        for (int q = 0; q < rx.nr; ++q) {
          const double x = net_pow(cs[rx.r[q]] * rx.inv_rkm[q], rx.rc[q]);
          fwd = q == 0 ? x / (1.0 + x) : fwd * (x / (1.0 + x));
        }
        rate = rx.vmax * al * fwd;
      } else {
        // BETSE's quotient applies the power before the 1e-3 (networks.py:1364-1396)
        double num = 1.0, den = 1.0;
        for (int q = 0; q < rx.np; ++q) {
          const double t = 1.0e-3 * net_pow(cs[rx.p[q]], rx.pc[q]);
          num = q == 0 ? t : num * t;
        }
        for (int q = 0; q < rx.nr; ++q) {
          const double t = 1.0e-3 * net_pow(cs[rx.r[q]], rx.rc[q]);
          den = q == 0 ? t : den * t;
        }
        rate = rx.vmax * al * (1.0 - (num / den) * rx.inv_keq);
      }
      if (OUT) a.rates[(size_t)j * a.C + c] = rate;
      for (int k = 0; k < S; ++k) delta[k] += tb.rm[k][j] * rate;
    }
    const double inv_vol = 1.0 / a.cell_vol[c];
    for (int k = 0; k < S; ++k) {
      const NetSubD& sb = tb.sub[k];
      const double c1 = cs[k] + delta[k] * a.dt;
      const double zF = (sb.z + kNonce) * a.F_RT, Dk = sb.Dm * a.inv_tm;
      const bool neutral = net_neutral(zF);
      double s = 0.0;
      for (int m = m0; m < m1; ++m) {
        double cm;
        if (sb.ui) {
          // Molecule.update_intra, implicit Euler toward the cell centre
          // (neutral substance: no field term); kq = gamma Do dt' / R_rads
          const double kq = a.g_over_r[m] * (sb.Do * (a.dt * sb.tdf));
          cm = (kq * cs[k] + a.cmem[(size_t)k * a.M + m]) / (1.0 + kq);
          neg += cm < 0.0;
        } else {
          cm = cs[k];
        }
        const double f = sb.Dm != 0.0 ? net_ghk(env[k], cm, Dk, zF, neutral, a.vm[m]) : 0.0;
        const double fa = f * a.mem_sa[m];
        s += fa;
        if (sb.ui) a.cmem_mid[(size_t)k * a.M + m] = cm + f * a.gamma[m] * a.dt;
        if (OUT) a.f_mem[(size_t)k * a.M + m] = f;
      }
      fsum[k] = s;
      a.c_mid[(size_t)k * a.C + c] = c1 + (s * inv_vol) * a.dt;
    }
  }
  for (int k = 0; k < S; ++k) {
    const double t = net_block_sum(fsum[k], red);
    if (threadIdx.x == 0) a.env_part[(size_t)blockIdx.x * S + k] = t;
  }
  if (neg) atomicAdd(a.neg, (unsigned long long)neg);
}

template <bool OUT>
__global__ void __launch_bounds__(kNetTPB) k_net_gj(NetArgs a) {
  const NetTables& tb = *a.tab;
  const int S = tb.S;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  int neg = 0;
  if (c < a.C) {
    const int m0 = a.cell_ptr[c], m1 = a.cell_ptr[c + 1];
    const double inv_vol = 1.0 / a.cell_vol[c];
    for (int k = 0; k < S; ++k) {
      const NetSubD& sb = tb.sub[k];
      const double c2 = a.c_mid[(size_t)k * a.C + c];
      double c3 = c2;
      if (!sb.gj_imp) {
        const double zF = (sb.z + kNonce) * a.F_RT, Dk = sb.Dgj * a.gj_block * a.inv_gj_len;
        const bool neutral = net_neutral(zF);
        double s = 0.0;
        for (int m = m0; m < m1; ++m) {
          const int n = a.nn[m];
          const double cA = sb.ui ? a.cmem_mid[(size_t)k * a.M + m] : c2;
          const double cB = sb.ui ? a.cmem_mid[(size_t)k * a.M + n] : a.c_mid[(size_t)k * a.C + a.nn_cell[m]];
          const double go = a.gjo ? a.gjo[m] : a.gj_block * a.gj_w[m];
          double f = 0.0;
          if (!a.bflag[m]) f = net_ghk(cA, cB, Dk * go, zF, neutral, a.vm[n] - a.vm[m]);
          s += -f * a.mem_sa[m];
          if (sb.ui) {
            const double cm = cA + (-f) * a.gamma[m] * sb.tdf * a.dt;
            a.cmem[(size_t)k * a.M + m] = cm;
            neg += cm < 0.0;
          }
          if (OUT) a.f_gj[(size_t)k * a.M + m] = f;
        }
        c3 = c2 + a.dt * (s * inv_vol) * sb.tdf;
      } else {
        for (int m = m0; m < m1; ++m) {
          if (sb.ui) {
            const double cm = a.cmem_mid[(size_t)k * a.M + m];
            a.cmem[(size_t)k * a.M + m] = cm;
            neg += cm < 0.0;
          }
          if (OUT) a.f_gj[(size_t)k * a.M + m] = 0.0;
        }
      }
      if (!sb.ui)
        for (int m = m0; m < m1; ++m) a.cmem[(size_t)k * a.M + m] = c3;
      a.c_cells[(size_t)k * a.C + c] = c3;
      neg += c3 < 0.0;
    }
  }
  if (blockIdx.x == 0) {
    // the auto-mixed environment: mean over membranes of env - f sa dt / vol_env
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = w; k < S; k += (int)(blockDim.x >> 5)) {
      double s = 0.0;
      for (int b = lane; b < a.nblk; b += 32) s += a.env_part[(size_t)b * S + k];
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (lane == 0) {
        const double e = a.env[k] - (s * a.dt) * a.inv_vol_env_M;
        a.env[k] = e;
        if (e < 0.0) atomicAdd(a.neg, 1ull);
      }
    }
  }
  if (neg) atomicAdd(a.neg, (unsigned long long)neg);
}

}  // namespace bx
