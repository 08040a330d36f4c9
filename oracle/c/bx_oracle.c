/* bx_oracle.c -- TEST INFRASTRUCTURE AND CPU BASELINE ONLY.
 *
 * A C restatement of BETSE's per-timestep electrodiffusion step
 * (Simulator._run_sim_core_loop, betse/science/sim.py:1169-1363), with or
 * without extracellular spaces, following the NumPy oracle (oracle/step.py)
 * operator by operator, with OpenMP over membranes, grid cells and cells.
 * Only tests/ and the CPU legs of bench.py load it; the CUDA library never
 * does.
 *
 * Order within one step (sim.py:1196-1363):
 *   Na/K-ATPase on the start-of-step state (sim_toolbox.py:71-122);
 *   per ion: GHK transmembrane flux (sim_toolbox.py:18-69, sim.py:1256-1269),
 *     then vm += 1e-25 in place (sim_toolbox.py:54), then the gap-junction
 *     flux from this membrane's cell into its partner's (update_gj,
 *     sim.py:2162-2206; boundary membranes carry none);
 *   with extracellular spaces, per ion: update_ecm (sim.py:2209-2254): the
 *     grid edges set to c_env_bound, the Nernst-Planck flux from fd.gradient
 *     and the previous step's E_env, fd.divergence with the reference's
 *     flipped one-sided edges, fd.integrator when sharpness < 1;
 *   update_all_concs (sim.py:2086-2111, sim_toolbox.py:1155-1207): the
 *     membrane-flux segment sum per cell, the environment (the well-mixed
 *     mean, or the membrane scatter onto the grid), the gap-junction segment
 *     sum, no_negs;
 *   update_V (sim.py:2007-2029): rho = sum_i z_i F c_i, vm = rho diviterm / cm;
 *     with extracellular spaces get_current's E_env (ion_current.py:79-110):
 *     the environment charge on the touched grid cells, a sigma-1 Gaussian
 *     with zero padding, the screened gradient.
 * Voltage-gated gap junctions (Gap_Junction.run, channels/gap_junction.py:
 * 52-75, once per ion before that ion's gap-junction flux), the Ca-ATPase of
 * ca_handler (sim.py:2126-2155, after the ion loop) and the polarizable Vmem
 * form of update_V (sim.py:2048-2058, from get_current's smoothed Jn,
 * ion_current.py:19-33) are restated as well.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define BXO_MAX_IONS 8
#define BXO_NONCE 1.0e-25

typedef struct bxo_cluster {
  int32_t C, M, I, iNa, iK;
  int32_t pad0;
  const int64_t* cell_ptr;   /* [C+1] membranes of cell c: [cell_ptr[c], cell_ptr[c+1]) */
  const int64_t* m2c;        /* [M] mem_to_cells */
  const int64_t* nn;         /* [M] nn_i: the gap-junction partner membrane */
  const uint8_t* bflag;      /* [M] boundary membrane */
  const double* mem_sa;      /* [M] */
  const double* gj_w;        /* [M] gj_default_weights */
  const double* cell_vol;    /* [C] */
  const double* diviterm;    /* [C] */
  const double* Dm;          /* [I][M] Dm_cells */
  double zs[BXO_MAX_IONS];
  double D_gj[BXO_MAX_IONS];
  double F, R, T, dt, cm, tm, gj_surface, gj_block, gj_len, nakatp_block;
  double alpha_NaK, KmNK_Na, KmNK_K, KmNK_ATP, cATP, cADP, cPi, deltaGATP, vol_env;
  int32_t vgj;               /* voltage-gated gap junctions: gjopen is state */
  int32_t iCa;               /* Ca2+ row; the Ca-ATPase runs when iCa >= 0 and alpha_Ca > 0 */
  double gj_vthresh, gj_min, alpha_Ca, KmCa_Ca, KmCa_ATP;
  /* extracellular spaces (is_ecm): the environment grid, row-major (ny, nx) */
  int32_t is_ecm, ny, nx, pad1;
  const int64_t* map_env;    /* [M] map_mem2ecm */
  const double* D_env;       /* [I][G] environment diffusivity (D_env * TJ_modulator) */
  const double* msa_env;     /* [G] memSa_per_envSquare */
  double c_bound[BXO_MAX_IONS];  /* c_env_bound: the grid-edge concentration */
  double delta, cell_height, q, kb, eo, er, ko_env, cell_radius, true_cell_size, sharpness;
  /* cell polarizability (polar): Vmem is per-membrane state */
  int32_t polar, pad2;
  const double* R_rads;      /* [M] */
  const double* sw_mem;      /* [M] smooth_weight_mem */
  const double* sw_o;        /* [M] smooth_weight_o */
  const double* cell_sa;     /* [C] */
  double D_free[BXO_MAX_IONS];
  /* boundary potential Phi_b [G] (NULL: zero), read through map_env */
  const double* phib;
} bxo_cluster;

/* GHK flux from A (outside) into B (inside), sim_toolbox.py:18-69 */
static inline double electroflux(double cA, double cB, double Dc, double d, double z, double vBA,
                                 double F, double R, double T) {
  const double v = vBA + BXO_NONCE;
  const double zc = z + BXO_NONCE;
  const double alpha = (zc * v * F) / (R * T);
  const double exp_alpha = exp(-alpha);
  const double deno = -expm1(-alpha);
  return -((Dc * alpha) / d) * ((cB - cA * exp_alpha) / deno);
}

/* f_Na of the Na/K-ATPase, sim_toolbox.py:71-122 */
static inline double pump_fna(const bxo_cluster* k, double cNai, double cNao, double cKi, double cKo, double Vm) {
  const double nao = cNao * 1e-3, ki = cKi * 1e-3, nai = cNai * 1e-3, ko = cKo * 1e-3;
  const double Qnumo = (k->cADP * 1e-3) * (k->cPi * 1e-3) * (nao * nao * nao) * (ki * ki);
  double Qdenomo = (k->cATP * 1e-3) * (nai * nai * nai) * (ko * ko);
  if (Qdenomo == 0.0) Qdenomo = 1.0e-15;
  const double Q = Qnumo / Qdenomo;
  const double Keq = exp(-(k->deltaGATP / (k->R * k->T) - ((k->F * Vm) / (k->R * k->T))));
  const double xna = cNai / k->KmNK_Na, xk = cKo / k->KmNK_K;
  const double numo_E = (xna * xna * xna) * (xk * xk) * (k->cATP / k->KmNK_ATP);
  const double denomo_E = (1 + xna * xna * xna) * (1 + xk * xk) * (1 + (k->cATP / k->KmNK_ATP));
  const double fwd_co = numo_E / denomo_E;
  return -3 * k->nakatp_block * k->alpha_NaK * fwd_co * (1 - (Q / Keq));
}

/* Gap_Junction.run: implicit Euler step of the open fraction (ms units), then
 * the block factor; Harris et al. (1983) rates */
static inline double gj_run(const bxo_cluster* k, double g, double vgj) {
  const double V1 = 1.0e3 * fabs(vgj);
  const double alpha = 0.0013 * exp(-0.077 * (V1 - k->gj_vthresh));
  double beta = 0.0013 * exp(0.14 * (V1 - k->gj_vthresh));
  beta = beta / (1 + 50 * beta);
  const double dt = k->dt * 1e3;
  return k->gj_block * ((g + dt * (alpha + beta * k->gj_min)) / (1 + alpha * dt + beta * dt));
}

/* pumpCaATP (sim_toolbox.py:124-180), into the cell positive; both
 * concentrations clamped at zero first (no_negs) */
static inline double pump_fca(const bxo_cluster* k, double cCai, double cCao, double Vm) {
  cCai = cCai > 0.0 ? cCai : 0.0;
  cCao = cCao > 0.0 ? cCao : 0.0;
  const double Qnumo = k->cADP * k->cPi * cCao;
  double Qdenomo = k->cATP * cCai;
  if (Qdenomo == 0.0) Qdenomo = 1.0e-16;
  const double Q = Qnumo / Qdenomo;
  const double Keq = exp(-(k->deltaGATP / (k->R * k->T) - 2 * ((k->F * Vm) / (k->R * k->T))));
  const double numo_E = (cCai / k->KmCa_Ca) * (k->cATP / k->KmCa_ATP);
  const double denomo_E = (1 + (cCai / k->KmCa_Ca)) * (1 + (k->cATP / k->KmCa_ATP));
  return -k->alpha_Ca * (numo_E / denomo_E) * (1 - (Q / Keq));
}

/* fd.gradient (finitediff.py:1236-1266) of a row-major (ny, nx) grid at
 * (i, j): central differences inside, one-sided on the edges */
static inline void grid_gradient(const double* F, int ny, int nx, int i, int j, double d, double* gx,
                                 double* gy) {
  const int k = i * nx + j;
  if (j == 0) *gx = (F[k + 1] - F[k]) / d;
  else if (j == nx - 1) *gx = (F[k] - F[k - 1]) / d;
  else *gx = -(F[k - 1] - F[k + 1]) / (2 * d);
  if (i == 0) *gy = (F[k + nx] - F[k]) / d;
  else if (i == ny - 1) *gy = (F[k] - F[k - nx]) / d;
  else *gy = -(F[k - nx] - F[k + nx]) / (2 * d);
}

/* fd.divergence (finitediff.py:1305-1311) = fd.diff along x + along y, whose
 * one-sided edge terms carry the reference's flipped signs (:1276-1277,
 * :1292-1293) */
static inline double grid_divergence(const double* Fx, const double* Fy, int ny, int nx, int i, int j,
                                     double d) {
  const int k = i * nx + j;
  double dx, dy;
  if (j == 0) dx = (Fx[k] - Fx[k + 1]) / d;
  else if (j == nx - 1) dx = (Fx[k - 1] - Fx[k]) / d;
  else dx = -(Fx[k - 1] - Fx[k + 1]) / (2 * d);
  if (i == 0) dy = -(Fy[k + nx] - Fy[k]) / d;
  else if (i == ny - 1) dy = -(Fy[k] - Fy[k - nx]) / d;
  else dy = -(Fy[k - nx] - Fy[k + nx]) / (2 * d);
  return dx + dy;
}

int bxo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Advance n_steps.  State: vm [M], cc_cells [I][C], cc_mem [I][C] (BETSE's
 * cc_at_mem, constant over each cell's membranes), cc_env [I] (the well-mixed
 * environment), gjopen [M] (with vgj).  threads <= 0 uses every thread OpenMP
 * offers.  Returns 0, or 1 when a concentration or Vmem became NaN (check_v /
 * no_negs). */
int bxo_step(const bxo_cluster* k, double* vm, double* cc_cells, double* cc_mem, double* cc_env,
             double* gjopen, double* E_env_x, double* E_env_y, int n_steps, int threads) {
  const int C = k->C, M = k->M, I = k->I;
  const int ecm = k->is_ecm != 0, ny = k->ny, nx = k->nx, G = ecm ? ny * nx : 1;
  if (I <= 0 || I > BXO_MAX_IONS || C <= 0 || M <= 0 || (k->vgj && !gjopen)) return 2;
  if (ecm && (ny < 3 || nx < 3 || !k->map_env || !k->D_env || !k->msa_env || !E_env_x || !E_env_y)) return 2;
  if (k->polar && (!k->R_rads || !k->sw_mem || !k->sw_o || !k->cell_sa)) return 2;
  if (k->phib && !k->map_env) return 2;
  const int ca_on = k->iCa >= 0 && k->iCa < I && k->alpha_Ca > 0.0;
  /* the thread count applies to this call's parallel regions only */
#ifdef _OPENMP
  const int nt = threads > 0 ? threads : omp_get_max_threads();
#else
  const int nt = 1;
  (void)threads;
#endif
  double* fmem = (double*)malloc(sizeof(double) * (size_t)I * M);
  double* fgj = (double*)malloc(sizeof(double) * (size_t)I * M);
  /* fixed-size blocks of membranes for the environment mean: the partial sums
   * and their order do not depend on the thread count */
  const int kBlk = 4096;
  const int nblk = (M + kBlk - 1) / kBlk;
  double* part = (double*)malloc(sizeof(double) * (size_t)I * nblk);
  /* extracellular grid work arrays: edges set, fluxes, updated grid */
  double* cb = ecm ? (double*)malloc(sizeof(double) * (size_t)I * G) : NULL;
  double* fx = ecm ? (double*)malloc(sizeof(double) * (size_t)I * G) : NULL;
  double* fy = ecm ? (double*)malloc(sizeof(double) * (size_t)I * G) : NULL;
  double* cn = ecm ? (double*)malloc(sizeof(double) * (size_t)I * G) : NULL;
  double* ve = ecm ? (double*)malloc(sizeof(double) * (size_t)G * 2) : NULL;
  if (!fmem || !fgj || !part || (ecm && (!cb || !fx || !fy || !cn || !ve))) {
    free(fmem); free(fgj); free(part); free(cb); free(fx); free(fy); free(cn); free(ve);
    return 3;
  }
  /* get_current's mean membrane area per grid square over the membranes, and
   * the sigma-1 Gaussian of scipy.ndimage (radius 4, normalised) */
  double msa = 0.0, gw[9], gsum = 0.0;
  if (ecm) {
    for (int m = 0; m < M; ++m) msa += k->msa_env[k->map_env[m]];
    msa /= (double)M;
    for (int q = 0; q < 9; ++q) {
      const double x = (double)(q - 4);
      gw[q] = exp(-0.5 / (1.0 * 1.0) * x * x);
      gsum += gw[q];
    }
    for (int q = 0; q < 9; ++q) gw[q] /= gsum;
  }
#define ENV_AT(i, m) (ecm ? cc_env[(size_t)(i) * G + k->map_env[m]] : cc_env[i])
  const double inv_cm = 1.0 / k->cm;
  int bad = 0;
  for (int step = 0; step < n_steps && !bad; ++step) {
    /* ---- membranes: pump, GHK and gap-junction fluxes */
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int m = 0; m < M; ++m) {
      const int64_t c = k->m2c[m], n = k->nn[m], cn = k->m2c[n];
      double fNa = 0.0, fK = 0.0;
      if (k->alpha_NaK > 0.0) {
        fNa = pump_fna(k, cc_mem[(size_t)k->iNa * C + c], ENV_AT(k->iNa, m), cc_mem[(size_t)k->iK * C + c],
                       ENV_AT(k->iK, m), vm[m]);
        fK = -(2.0 / 3.0) * fNa;
      }
      double v = vm[m], vn = vm[n];            /* in-place nonces of the reference */
      for (int i = 0; i < I; ++i) {
        const double cin = cc_mem[(size_t)i * C + c];
        const double f_ED = electroflux(ENV_AT(i, m), cin, k->Dm[(size_t)i * M + m], k->tm, k->zs[i], v,
                                        k->F, k->R, k->T);
        double f = 0.0;
        if (i == k->iNa) f = fNa;
        else if (i == k->iK) f = fK;
        fmem[(size_t)i * M + m] = f + f_ED;
        v = v + BXO_NONCE;
        vn = vn + BXO_NONCE;
        const double vgj = vn - v;
        double go;
        if (k->vgj) {
          gjopen[m] = gj_run(k, gjopen[m], vgj);
          go = gjopen[m];
        } else {
          go = k->gj_block * k->gj_w[m];
        }
        double fg = electroflux(cin, cc_mem[(size_t)i * C + cn], k->D_gj[i] * k->gj_surface * go,
                                k->gj_len, k->zs[i], vgj, k->F, k->R, k->T);
        if (k->bflag[m]) fg = 0.0;
        fgj[(size_t)i * M + m] = 0.0 + fg;
      }
    }
    /* ---- update_ecm per ion: edges to c_env_bound, Nernst-Planck flux,
     * divergence, smoothing; the grid before the membrane scatter goes to cn */
    if (ecm) {
#pragma omp parallel for schedule(static) num_threads(nt)
      for (int t = 0; t < I * G; ++t) {
        const int i = t / G, g = t - i * G, gi = g / nx, gj = g - gi * nx;
        const int edge = gi == 0 || gi == ny - 1 || gj == 0 || gj == nx - 1;
        cb[t] = edge ? k->c_bound[i] : cc_env[t];
      }
#pragma omp parallel for schedule(static) num_threads(nt)
      for (int t = 0; t < I * G; ++t) {
        const int i = t / G, g = t - i * G, gi = g / nx, gj = g - gi * nx;
        double gcx, gcy;
        grid_gradient(cb + (size_t)i * G, ny, nx, gi, gj, k->delta, &gcx, &gcy);
        const double denv = k->D_env[t];
        const double alpha = (denv * k->zs[i] * k->q) / (k->kb * k->T);
        const double gvx = -E_env_x[g], gvy = -E_env_y[g];
        /* the divergence takes -f */
        fx[t] = -(-denv * gcx - alpha * gvx * cb[t]);
        fy[t] = -(-denv * gcy - alpha * gvy * cb[t]);
      }
#pragma omp parallel for schedule(static) num_threads(nt)
      for (int t = 0; t < I * G; ++t) {
        const int i = t / G, g = t - i * G, gi = g / nx, gj = g - gi * nx;
        const double div = grid_divergence(fx + (size_t)i * G, fy + (size_t)i * G, ny, nx, gi, gj, k->delta);
        cn[t] = cb[t] + div * k->dt;
      }
      if (k->sharpness < 1.0) {
        /* fd.integrator (finitediff.py:1479-1512): neighbour blend, edges kept */
        const double sides = (1 - k->sharpness) / 4;
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int t = 0; t < I * G; ++t) {
          const int i = t / G, g = t - i * G, gi = g / nx, gj = g - gi * nx;
          const double* P = cn + (size_t)i * G;
          if (gi == 0 || gi == ny - 1 || gj == 0 || gj == nx - 1) {
            fx[t] = P[g];
          } else {
            double F = k->sharpness * P[g];
            F += sides * P[g + nx];
            F += sides * P[g - nx];
            F += sides * P[g + 1];
            F += sides * P[g - 1];
            fx[t] = F;
          }
        }
        memcpy(cn, fx, sizeof(double) * (size_t)I * G);
      }
    }
    /* ---- ca_handler after the ion loop: the cell side is cc_cells at the
     * start of the step (update_intra), the environment side the grid after
     * update_ecm, and vm carries the I in-place nonces */
    if (ca_on) {
      const int i = k->iCa;
#pragma omp parallel for schedule(static) num_threads(nt)
      for (int m = 0; m < M; ++m) {
        double v = vm[m];
        for (int q = 0; q < I; ++q) v = v + BXO_NONCE;
        const double ce = ecm ? cn[(size_t)i * G + k->map_env[m]] : cc_env[i];
        fmem[(size_t)i * M + m] += pump_fca(k, cc_cells[(size_t)i * C + k->m2c[m]], ce, v);
      }
    }
    /* ---- environment: mean over membranes of c_env - f sa / vol_env dt */
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int b = 0; b < (ecm ? 0 : nblk); ++b) {
      const int m0 = b * kBlk, m1 = (m0 + kBlk < M) ? m0 + kBlk : M;
      for (int i = 0; i < I; ++i) {
        double s = 0.0;
        for (int m = m0; m < m1; ++m)
          s += cc_env[i] + (-fmem[(size_t)i * M + m] * (k->mem_sa[m] / k->vol_env)) * k->dt;
        part[(size_t)i * nblk + b] = s;
      }
    }
    /* ---- cells: update_all_concs and update_V */
#pragma omp parallel for schedule(static) num_threads(nt) reduction(|| : bad)
    for (int c = 0; c < C; ++c) {
      const int64_t a0 = k->cell_ptr[c], a1 = k->cell_ptr[c + 1];
      double rho = 0.0;
      for (int i = 0; i < I; ++i) {
        double s1 = 0.0, s2 = 0.0;
        for (int64_t m = a0; m < a1; ++m) {
          s1 += fmem[(size_t)i * M + m] * k->mem_sa[m];
          s2 += -fgj[(size_t)i * M + m] * k->mem_sa[m];
        }
        double x = cc_cells[(size_t)i * C + c] + (s1 / k->cell_vol[c]) * k->dt;
        cc_mem[(size_t)i * C + c] = x;
        x = x + k->dt * (s2 / k->cell_vol[c]);
        if (x != x) bad = 1;
        if (x < 0.0) x = 0.0;
        cc_cells[(size_t)i * C + c] = x;
        rho += (k->zs[i] * k->F) * x;
      }
      const double vc = inv_cm * (rho * k->diviterm[c]);
      if (vc != vc) bad = 1;
      if (!k->polar) {
        /* vm = rho diviterm / cm - Phi_b[map_mem2ecm] (sim.py:2029) */
        for (int64_t m = a0; m < a1; ++m) vm[m] = k->phib ? vc - k->phib[k->map_env[m]] : vc;
      } else {
        /* get_current's smoothed Jn (ion_current.py:22-33) and sigma_cell
         * (sim.py:2016-2017), then the implicit update of each membrane's
         * vm, which carries the I in-place nonces (sim.py:2058-2059) */
        double sj = 0.0, sig = 0.0;
        for (int64_t m = a0; m < a1; ++m) {
          double jm = 0.0, jg = 0.0;
          for (int i = 0; i < I; ++i) {
            jm += (k->zs[i] * k->F) * fmem[(size_t)i * M + m];
            jg += (k->zs[i] * k->F) * fgj[(size_t)i * M + m];
          }
          sj += (-jm + jg) * k->mem_sa[m];
        }
        for (int i = 0; i < I; ++i)
          sig += ((k->zs[i] * k->zs[i]) * (k->F * k->F) * cc_cells[(size_t)i * C + c] * k->D_free[i] * 0.1) /
                 (k->R * k->T);
        sig = sig / (double)I;
        const double jave = sj / k->cell_sa[c];
        for (int64_t m = a0; m < a1; ++m) {
          double jm = 0.0, jg = 0.0;
          for (int i = 0; i < I; ++i) {
            jm += (k->zs[i] * k->F) * fmem[(size_t)i * M + m];
            jg += (k->zs[i] * k->F) * fgj[(size_t)i * M + m];
          }
          const double Jn = k->sw_mem[m] * (-jm + jg) + jave * k->sw_o[m];
          double v = vm[m];
          for (int q = 0; q < I; ++q) v = v + BXO_NONCE;
          const double R = k->R_rads[m];
          const double vn = (v - (k->dt / k->cm) * Jn + ((k->dt * sig * vc) / (k->cm * R))) /
                            (1 + ((k->dt * sig) / (k->cm * R)));
          if (vn != vn) bad = 1;
          vm[m] = vn;
        }
      }
    }
    if (!ecm) {
      for (int i = 0; i < I; ++i) {
        double s = 0.0;
        for (int b = 0; b < nblk; ++b) s += part[(size_t)i * nblk + b];
        cc_env[i] = s / (double)M;
      }
    } else {
      /* the membrane exchange onto the grid (cells.M_divmap_mem2ecm, in
       * membrane order), then get_current's E_env from the new grid */
      const double hd2 = k->cell_height * (k->delta * k->delta);
#pragma omp parallel for schedule(static) num_threads(nt)
      for (int i = 0; i < I; ++i) {
        double* acc = fx + (size_t)i * G;
        for (int g = 0; g < G; ++g) acc[g] = 0.0;
        for (int m = 0; m < M; ++m) acc[k->map_env[m]] += k->mem_sa[m] * (-fmem[(size_t)i * M + m]);
        for (int g = 0; g < G; ++g) cc_env[(size_t)i * G + g] = cn[(size_t)i * G + g] + (acc[g] / hd2) * k->dt;
      }
      double* vsrc = ve;
      double* tmp = ve + G;
      for (int g = 0; g < G; ++g) vsrc[g] = 0.0;
      for (int m = 0; m < M; ++m) {
        const int64_t g = k->map_env[m];
        double rho = 0.0;
        for (int i = 0; i < I; ++i) rho += (k->zs[i] * k->F) * cc_env[(size_t)i * G + g];
        vsrc[g] = (rho * hd2) / msa / (k->ko_env * k->eo * k->er);
      }
      /* separable Gaussian, zero padding: axis 0 (rows), then axis 1 */
#pragma omp parallel for schedule(static) num_threads(nt)
      for (int g = 0; g < G; ++g) {
        const int gi = g / nx, gj = g - gi * nx;
        double a = 0.0;
        for (int q = 0; q < 9; ++q) {
          const int ii = gi + q - 4;
          a += gw[q] * ((ii >= 0 && ii < ny) ? vsrc[ii * nx + gj] : 0.0);
        }
        tmp[g] = a;
      }
      const double screen = (2 / (k->ko_env * k->delta)) * (k->cell_radius / k->true_cell_size);
#pragma omp parallel for schedule(static) num_threads(nt)
      for (int g = 0; g < G; ++g) {
        const int gi = g / nx, gj = g - gi * nx;
        double a = 0.0;
        for (int q = 0; q < 9; ++q) {
          const int jj = gj + q - 4;
          a += gw[q] * ((jj >= 0 && jj < nx) ? tmp[gi * nx + jj] : 0.0);
        }
        vsrc[g] = screen * (k->phib ? a + k->phib[g] : a);   /* v_env = Gaussian + Phi_b */
      }
#pragma omp parallel for schedule(static) num_threads(nt)
      for (int g = 0; g < G; ++g) {
        const int gi = g / nx, gj = g - gi * nx;
        double gx, gy;
        grid_gradient(vsrc, ny, nx, gi, gj, k->delta, &gx, &gy);
        E_env_x[g] = -gx;
        E_env_y[g] = -gy;
      }
    }
  }
#undef ENV_AT
  free(fmem);
  free(fgj);
  free(part);
  free(cb);
  free(fx);
  free(fy);
  free(cn);
  free(ve);
  return bad;
}
