/*
 * bx.h -- C ABI of the GB300-native electrodiffusion step (libbx.so).
 *
 * One handle ("cluster") owns device copies of a cell cluster's index maps and
 * geometry, its per-membrane channel diffusivities and its evolving state, and
 * advances BETSE's full-solver time step on the GPU.  Every entry point
 * returns 0 on success or a negative errno-style code (BX_E*); no C++
 * exception crosses this boundary.  bx_last_error() gives a message for the
 * last failure on the calling thread.  A handle is not thread-safe: drive each
 * handle from one host thread.  All host pointers are plain arrays in the
 * layouts documented below; none is retained after the call returns.
 *
 * Reference interfaces each entry point replaces (BETSE, pure Python):
 *   bx_cluster_create   Cells index maps / geometry consumed by the step:
 *                       cells.py:1126-1146 (mem_to_cells, cell_to_mems),
 *                       cells.py:1498-1533 (nn_i), cells.py:1446 (bflags_mems),
 *                       cells.py:1385-1390 (cell_vol, diviterm),
 *                       cells.py:1150-1155 (cell_sa), cells.py:1758
 *                       (map_mem2ecm), and Simulator.init_core/init_dynamics
 *                       constants, sim.py:452-1012.
 *   bx_set_membrane_diffusivity   sim.Dm_cells written by
 *                       TissueHandler.init_profiles (tishandler.py:363-452).
 *   bx_set_env_diffusivity        sim.D_env from Simulator.initDenv
 *                       (sim.py:2347-2400).
 *   bx_set_boundary_potential     sim.Phi_b = lapENVinv @ (-div_Jb)
 *                       (physics/ion_current.py:100-102,164-169).
 *   bx_state_upload / bx_state_download   the Simulator attributes vm,
 *                       cc_cells, cc_at_mem, cc_env (sim.py:452-755).
 *   bx_step             Simulator._run_sim_core_loop body, sim.py:1169-1363
 *                       (pumpNaKATP, electroflux, update_gj, update_ecm,
 *                       update_all_concs, update_V, check_v).
 *   bx_outputs_download the per-step attributes write2storage reads
 *                       (sim.py:1789-1884): fluxes_mem, fluxes_gj,
 *                       rate_NaKATP, rho_cells, Jn, I_mem, J_cell_x/y, Jc,
 *                       vm_ave, dvm, E_cell_x/y, Emc, E_gj_x/y, gjopen,
 *                       sigma_cell.
 *   bx_status           stb.check_v (sim_toolbox.py:332-344) and stb.no_negs
 *                       (sim_toolbox.py:475-503): NaN and clamp counters.
 *   bx_set_lap_env_inv  cells.lapENVinv (cells.py:503-504), kept on the GPU
 *   bx_dense_op_*       np.dot(cells.lapGJinv | cells.lapENVinv, block of
 *                       right-hand sides) on tcgen05 (pressures.py:59,
 *                       ion_current.py:90,170)
 *   bx_env_fields       get_current's environment branches
 *                       (physics/ion_current.py:50-171): v_env, E_env_x/y,
 *                       J_env_x/y, B_field with dense lapENVinv products.
 *   bx_dense_apply      np.dot(cells.lapENVinv, .) / np.dot(cells.lapGJinv, .)
 *                       (ion_current.py:90,170; sim_toolbox.py:1263,1284;
 *                       physics/pressures.py:59).
 *   bx_network_*        MasterOfNetworks (chemistry/networks.py): tissue_init
 *                       / read_reactions tables (:307-657, 814-922) and
 *                       run_loop (:2805-2983), called from sim.py:1290-1319
 *                       and gene.py:220-308.
 */
#ifndef BX_H
#define BX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BX_ABI_VERSION 1
#define BX_MAX_IONS 8
#define BX_MAX_MEMS_PER_CELL 256

/* error codes */
#define BX_OK 0
#define BX_EINVAL (-22)      /* bad argument or inconsistent geometry */
#define BX_ENOMEM (-12)      /* device or host allocation failed */
#define BX_ECUDA (-5)        /* a CUDA runtime call failed */
#define BX_EUNSTABLE (-1001) /* NaN in Vmem or a concentration (check_v) */
#define BX_ESTATE (-1002)    /* call out of order (e.g. step before upload) */

/* precision forms of the step */
#define BX_PLAIN_FP64 0 /* every flux, pump and sum in FP64 */
#define BX_SPLIT_FP32 1 /* fluxes/pumps in FP32; sums, concentrations, Vmem FP64 */

typedef struct bx_cluster* bx_handle;

/* Cluster geometry and index maps.  Membranes of cell c are the contiguous
 * range [cell_mem_ptr[c], cell_mem_ptr[c+1]) -- the CSR form of BETSE's
 * cell_to_mems / mem_to_cells.  Arrays are host pointers, copied at create. */
typedef struct bx_geom {
    int32_t n_cells;
    int32_t n_mems;
    int32_t grid_ny, grid_nx;   /* environment grid (cells.X.shape); >= 3 each */
    const int32_t* cell_mem_ptr; /* [n_cells+1] */
    const int32_t* nn_i;         /* [n_mems] gap-junction partner (self at boundary) */
    const uint8_t* bflag;        /* [n_mems] 1 = outer-boundary membrane */
    const int32_t* map_mem2ecm;  /* [n_mems] environment grid index of each membrane */
    const double* mem_sa;        /* [n_mems] membrane surface area (m^2) */
    const double* mem_nx;        /* [n_mems] outward normal x (mem_vects_flat[:,2]) */
    const double* mem_ny;        /* [n_mems] outward normal y (mem_vects_flat[:,3]) */
    const double* gj_weight;     /* [n_mems] static gap-junction open fraction */
    const double* smooth_weight_mem; /* [n_mems] Jn smoothing weights (sim.py:783-786) */
    const double* smooth_weight_o;   /* [n_mems] */
    const double* cell_vol;      /* [n_cells] */
    const double* cell_sa;       /* [n_cells] */
    const double* diviterm;      /* [n_cells] cell_vol / cell_sa */
    const double* mem_sa_per_env; /* [grid] cells.memSa_per_envSquare (ECM only; may be NULL) */
    double gj_len;               /* cells.gj_len (= p.cell_space) */
    double delta;                /* environment grid spacing (cells.delta) */
    const double* R_rads;        /* [n_mems] membrane distance from the cell centre (cells.R_rads,
                                    cells.py:1173); read only with cell_polarizability, else may be NULL */
} bx_geom;

/* Scalar parameters and per-ion constants (Parameters + Simulator fields). */
typedef struct bx_params {
    int32_t n_ions;
    int32_t iNa, iK;             /* ion rows of Na+ and K+ */
    int32_t is_ecm;              /* 1 = extracellular spaces on */
    double F, R, T, dt, cm, tm;
    double gj_surface, gj_block, nakatp_block;
    double alpha_NaK, KmNK_Na, KmNK_K, KmNK_ATP, cATP, cADP, cPi, deltaGATP;
    double vol_env;              /* well-mixed environment volume (no ECM) */
    double cell_height, q, kb, eo, er, sharpness, cell_radius, true_cell_size;
    double ko_env;               /* inverse Debye length of the environment (ECM) */
    double sigma;                /* mean environment conductivity (no-ECM fields) */
    double mu;                   /* magnetic permeability (B_field output) */
    double zs[BX_MAX_IONS];
    double D_free[BX_MAX_IONS];
    double D_gj[BX_MAX_IONS];
    double c_env_bound[BX_MAX_IONS]; /* Dirichlet value on the grid edge (ECM) */
    /* voltage-gated gap junctions (p.v_sensitive_gj; channels/gap_junction.py:57-81):
     * the open fraction is state (bx_state.gjopen) and replaces gj_weight */
    int32_t v_sensitive_gj;
    /* Ca-ATPase (Simulator.ca_handler, sim.py:2126-2155; pumpCaATP,
     * sim_toolbox.py:124-180): on when iCa >= 0 and alpha_Ca > 0, so a
     * zero-initialised struct leaves it off */
    int32_t iCa;                 /* ion row of Ca2+ */
    double gj_vthresh;           /* mV at which junctions are half closed */
    double gj_min;               /* open fraction of a closed junction */
    double alpha_Ca, KmCa_Ca, KmCa_ATP;
    /* p.cell_polarizability != 0 selects update_V's implicit membrane-voltage
     * form (sim.py:2048-2080): Vmem becomes per-membrane state (plain FP64
     * form only; needs bx_geom.R_rads) */
    double cell_polarizability;
} bx_params;

/* Host views of the evolving state, BETSE layouts (row = ion).
 * cc_env is [n_ions] without ECM (one well-mixed value per ion; BETSE keeps a
 * uniform vector of length n_mems) and [n_ions * grid] with ECM.
 * cc_at_mem is [n_ions * n_mems]; it is constant over each cell's membranes
 * in BETSE, and upload checks that.  E_env_x/y ([grid], ECM only) are the
 * environment field from the previous update_V. */
typedef struct bx_state {
    double* vm;
    double* cc_cells;
    double* cc_at_mem;
    double* cc_env;
    double* E_env_x;
    double* E_env_y;
    double* gjopen;   /* [n_mems] gap-junction open fraction (v_sensitive_gj only;
                         NULL on upload = gj_weight, BETSE's initial value) */
} bx_state;

/* Host destinations for one step's outputs; any pointer may be NULL. */
typedef struct bx_outputs {
    double* fluxes_mem;   /* [n_ions * n_mems] */
    double* fluxes_gj;    /* [n_ions * n_mems] */
    double* rate_NaKATP;  /* [n_mems] */
    double* rho_cells;    /* [n_cells] */
    double* Jn;           /* [n_mems] */
    double* I_mem;        /* [n_mems] */
    double* J_cell_x;     /* [n_cells] */
    double* J_cell_y;     /* [n_cells] */
    double* Jc;           /* [n_mems] */
    double* vm_ave;       /* [n_cells] */
    double* dvm;          /* [n_mems] */
    double* E_cell_x;     /* [n_cells] */
    double* E_cell_y;     /* [n_cells] */
    double* Emc;          /* [n_mems] */
    double* E_gj_x;       /* [n_mems] */
    double* E_gj_y;       /* [n_mems] */
    double* gjopen;       /* [n_mems] */
    double* sigma_cell;   /* [n_cells] */
    double* fluxes_env_x; /* [n_ions * grid] (ECM) */
    double* fluxes_env_y; /* [n_ions * grid] (ECM) */
    double* rho_env;      /* [grid] (ECM) */
    double* v_env;        /* [grid] (ECM) */
} bx_outputs;

typedef struct bx_step_status {
    int64_t steps_done;
    int32_t nan_vm;        /* membranes whose Vmem became NaN (last failing step) */
    int32_t nan_conc;      /* cell concentrations that became NaN */
    int64_t neg_clamped;   /* negative cell concentrations set to 0 (no_negs), cumulative */
    int32_t unstable;      /* 1 once a NaN was seen; further steps are refused */
    int32_t precision;
} bx_step_status;

/* Create a handle; copies geometry to the device of the current CUDA context.
 * precision is BX_PLAIN_FP64 or BX_SPLIT_FP32. */
int bx_cluster_create(const bx_geom* g, const bx_params* p, int precision,
                      bx_handle* out);
/* A batch of independent clusters stepped together (a parameter sweep; no
 * reference counterpart beyond running Simulator once per cluster).  g[k] and
 * p[k] describe cluster k; the clusters may differ in size, geometry,
 * alpha_NaK, nakatp_block and vol_env, and share every other parameter.  The
 * handle's arrays are the clusters' arrays concatenated in order (state rows
 * still ion-major: cc_cells is [n_ions][sum n_cells]); without ECM cc_env is
 * [n_clusters][n_ions].  Batches need is_ecm == 0. */
int bx_batch_create(const bx_geom* g, const bx_params* p, int n_clusters, int precision,
                    bx_handle* out);
/* Offsets of each cluster's cells and membranes in the concatenation
 * ([n_clusters+1] each). */
int bx_batch_layout(bx_handle h, int32_t* cell_offsets, int32_t* mem_offsets);
/* Replace every cluster's parameters (p[n_clusters]). */
int bx_batch_set_params(bx_handle h, const bx_params* p);
void bx_destroy(bx_handle h);

/* Per-membrane channel diffusivities Dm[n_ions * n_mems] (sim.Dm_cells). */
int bx_set_membrane_diffusivity(bx_handle h, const double* Dm);
/* Environment diffusivities D_env[n_ions * grid] (ECM; sim.D_env). */
int bx_set_env_diffusivity(bx_handle h, const double* D_env);
/* Boundary potential Phi_b[grid]; NULL resets it to zero. */
int bx_set_boundary_potential(bx_handle h, const double* Phi_b);
/* Replace the scalar parameters (e.g. dt between phases). */
int bx_set_params(bx_handle h, const bx_params* p);

/* Copy state in / out (synchronous on the handle's stream).  The arrays
 * cross as they are and are checked and re-laid on the device; each pointer
 * may be host or device memory (copies use unified addressing).  Upload
 * refuses (BX_EINVAL) a cc_at_mem that differs within a cell and, in the
 * split form, a vm that is not uniform within a cell; after a refused upload
 * the handle holds no state until the next successful one.  Download fills
 * every non-NULL pointer (page-locked destinations copy fastest). */
int bx_state_upload(bx_handle h, const bx_state* s);
int bx_state_download(bx_handle h, bx_state* s);

/* Advance n_steps time steps on `stream` (a cudaStream_t; NULL = the handle's
 * own stream).  If want_outputs != 0 the last step also computes the step
 * outputs.  Asynchronous: returns after enqueueing; bx_status synchronises. */
int bx_step(bx_handle h, int n_steps, int want_outputs, void* stream);
int bx_outputs_download(bx_handle h, bx_outputs* o);   /* host or device destinations */
int bx_status(bx_handle h, bx_step_status* st);
/* Steady-state residual of each cluster after a step with want_outputs:
 * per_cluster[c] = max over its membranes of |dVm/dt| (sim.dvm, sim.py:2083),
 * NaN if any is NaN.  n_clusters values (1 for bx_cluster_create).  Synchronous. */
int bx_max_abs_dvm(bx_handle h, double* per_cluster);

/* Dense lapENVinv ([grid x grid] row-major FP64, host) for bx_env_fields:
 * cells.lapENVinv (cells.py:503-504, the pinv of
 * FiniteDiffSolver.makeLaplacian, finitediff.py:252-431).  Stored on the GPU
 * once as double-float (hi, lo) FP32 pairs; single-cluster handles only. */
int bx_set_lap_env_inv(bx_handle h, const double* lap_env_inv);
/* The same operator built on the GPU from the handle's grid shape and
 * spacing, with no host array: makeLaplacian (finitediff.py:252-431) is the
 * identity on the grid edges and the 5-point Laplacian inside, and its
 * interior block is diagonalised by sine transforms, so its inverse is one
 * FP64 GEMM over the eigenvectors (about (ny nx)^2 sqrt(ny nx) multiply-adds
 * instead of BETSE's O((ny nx)^3) pinv).  Synchronous. */
int bx_build_lap_env_inv(bx_handle h);
/* cells.lapENVinv (cells.py:503-504) for an (ny, nx) grid of spacing delta,
 * built as above into the DEVICE array A ([ny*nx] rows of lda >= ny*nx FP64
 * values, row-major), on `stream` (synchronous). */
int bx_lap_env_inv_build(int ny, int nx, double delta, double* A, int64_t lda, void* stream);

/* Environment fields of get_current (physics/ion_current.py:50-171) for the
 * last step, which must have run with want_outputs: v_env, E_env_x/y,
 * J_env_x/y and B_field, each [grid], any pointer NULL to skip.  Without ECM
 * they come from that step's start-of-step Vmem (Gaussian LFP, smooth_flux,
 * sigma*E*D_env_weight, HH_Decomp: sim_toolbox.py:1236-1333); with ECM v_env
 * and E_env are the step's own and J_env/B_field come from the grid fluxes.
 * D_env_weight [grid] (sim.D_env_weight; NULL = 1) weights the no-ECM current.
 * Boundary voltages are zero (sim.bound_V, sim.py:702-706).  Synchronous. */
int bx_env_fields(bx_handle h, const double* D_env_weight, double* v_env,
                  double* E_env_x, double* E_env_y, double* J_env_x,
                  double* J_env_y, double* B_field);
/* Environment fields for a batch of clusters without ECM (a parameter sweep):
 * clusters that share a grid shape share lapENVinv = delta^2 K(shape)
 * (finitediff.py:426-429), so every product of every such cluster runs as one
 * tcgen05 GEMM (bx_dense_op_*) with a per-column delta^2, refined once against
 * the 5-point Laplacian.  bx_batch_set_lap_env_inv gives one cluster's
 * lapENVinv (host, [ny*nx]^2) and its grid spacing for each grid shape in the
 * batch; bx_batch_env_fields then returns the fields of the last step (which
 * ran with want_outputs) for all clusters, concatenated over the clusters'
 * grids in batch order (D_env_weight likewise, NULL = 1).  Synchronous. */
int bx_batch_set_lap_env_inv(bx_handle h, int ny, int nx, double delta, const double* lap_env_inv);
int bx_batch_env_fields(bx_handle h, const double* D_env_weight, double* v_env, double* E_env_x,
                        double* E_env_y, double* J_env_x, double* J_env_y, double* B_field);
/* Diagnostics: mean duration of bx_env_fields' device work and of one
 * two-column lapENVinv product over n runs (CUDA events). */
int bx_time_env_fields(bx_handle h, int n, double* ms_fields, double* ms_product);

/* Dense products y[n x nrhs] = A[n x n] @ x[n x nrhs] (row-major, FP64) on the
 * GPU, device pointers; the kernel BETSE's lapENVinv / lapGJinv matvecs use. */
int bx_dense_apply_f64(const double* A, const double* x, double* y, int n,
                       int nrhs, void* stream);

/* Dense operator products on the tensor cores, for right-hand sides that
 * batch: Y = A X with A [n x n] (np.dot(cells.lapGJinv, .), pressures.py:59;
 * np.dot(cells.lapENVinv, .), ion_current.py:90,170) applied to nrhs columns.
 * A is split once into BF16 hi/lo planes (BF16x3 products, FP32 accumulation
 * in TMEM, tcgen05); bx_dense_op_set_forward gives the operator L that A
 * inverts (CSR, FP64) and enables one refinement step Y += A (X - L Y).
 * X, Y, col_scale are DEVICE pointers: X, Y [n x nrhs] row-major FP64,
 * col_scale [nrhs] (NULL = 1) multiplies column j of the result (e.g. the
 * delta^2 of clusters that share a grid-shape operator).  Asynchronous on
 * `stream`; bx_dense_op_status synchronises and reports a pipeline timeout. */
typedef struct bx_dense_op* bx_dense_op_handle;
int bx_dense_op_create(const double* A, int n, bx_dense_op_handle* out);  /* host A */
int bx_dense_op_set_forward(bx_dense_op_handle op, const int32_t* row_ptr,
                            const int32_t* col, const double* val);      /* host CSR */
int bx_dense_op_apply(bx_dense_op_handle op, const double* X, double* Y, int nrhs,
                      const double* col_scale, int refine, void* stream);
int bx_dense_op_status(bx_dense_op_handle op, int* timed_out);
/* mean ms of one GEMM launch (no refinement) over n_iter, CUDA events */
int bx_dense_op_time(bx_dense_op_handle op, const double* X, double* Y, int nrhs,
                     int n_iter, double* ms);
int bx_dense_op_destroy(bx_dense_op_handle op);
/* An operator built on the device: zero planes, then column blocks (device
 * src [n x ncols] row-major, col0 a multiple of 64, ncols a multiple of 64
 * unless the block ends at n), asynchronous on `stream`. */
int bx_dense_op_create_empty(int n, bx_dense_op_handle* out);
int bx_dense_op_set_columns(bx_dense_op_handle op, int col0, int ncols, const double* src, void* stream);

/* Cells.graphLaplacian at any cluster size (cells.py:1845-1894):
 *   lapGJinv = pinv(D) diag(tri_len/vor_len) (-pinv(D)^T) diag(vor_sa)
 *            = -L+ Lw L+ A
 * with L = D^T D the graph Laplacian of the triangulation's edges D, L+ its
 * pseudo-inverse, Lw = D^T diag(tri_len/vor_len) D and A = diag(vor_sa);
 * np.dot(cells.lapGJinv, .) at physics/pressures.py:59.  L+ is applied by
 * FP64 conjugate gradients per right-hand side, preconditioned by an
 * aggregation multigrid V-cycle.  levels[0] is L (n nodes); level l+1 is
 * the Galerkin operator of level l's aggregates of 4 consecutive nodes
 * (node i -> i / 4), down to the coarsest level, whose pseudo-inverse
 * [nc x nc] row-major is coarse_pinv; host CSR arrays, copied.  `weighted`
 * is Lw, vor_sa [n] the cell areas.  max_rhs bounds nrhs (the workspace is
 * 12 n max_rhs doubles).  Right-hand sides and results are DEVICE arrays
 * [n x nrhs] row-major; a solve stops when every column's residual is below
 * tol relative to its right-hand side (checked every 4 iterations) or after
 * max_iter iterations; iters and rel_res report the worst column. */
typedef struct bx_graph_level {
    int32_t n, nnz;
    const int32_t* row_ptr;
    const int32_t* col;
    const double* val;
} bx_graph_level;
typedef struct bx_graph_solver* bx_graph_handle;
int bx_graph_create(int n_levels, const bx_graph_level* levels, const double* coarse_pinv,
                    const bx_graph_level* weighted, const double* vor_sa, int max_rhs,
                    bx_graph_handle* out);
/* X = L+ B (B's component along the constants is removed first) */
int bx_graph_solve(bx_graph_handle h, const double* B, double* X, int nrhs, double tol, int max_iter,
                   int* iters, double* rel_res, void* stream);
/* Y = lapGJinv X, FP64, two solves */
int bx_lap_gj_apply(bx_graph_handle h, const double* X, double* Y, int nrhs, double tol, int max_iter,
                    int* iters, double* rel_res, void* stream);
/* the dense lapGJinv as a BF16x3 tensor-core operator (bx_dense_op_*), built
 * column block by column block (max_rhs rounded down to 64 columns per
 * block) from bx_lap_gj_apply on scaled identity columns; no n x n FP64
 * matrix is formed */
int bx_lap_gj_dense(bx_graph_handle h, double tol, int max_iter, int* iters, double* rel_res,
                    void* stream, bx_dense_op_handle* out);
int bx_graph_destroy(bx_graph_handle h);

/* Warm-start graph network (no reference counterpart: BETSE's init phase
 * always starts from the uniform profile).  A 3-layer, 64-wide message-passing
 * network on the cell adjacency predicts per-cell steady-state concentrations
 * and Vmem; it is trained here in BF16 with FP32 master weights (Adam).
 * Parameters are a flat FP32 vector of bx_gnn_n_params() values (layout:
 * W0[64x64], b0, then (Ws, Wn, b) for each layer, Wd[64x64], bd).  The graph
 * is host CSR over all nodes; calls act on a node range [lo, hi) that must
 * hold whole clusters.  x [rows x n_in], y / targets [rows x n_out] are FP32
 * DEVICE pointers (n_in, n_out <= 64). */
typedef struct bx_gnn* bx_gnn_handle;
int bx_gnn_create(bx_gnn_handle* out);
int bx_gnn_n_params(void);
int bx_gnn_set_params(bx_gnn_handle h, const float* params);   /* host; resets Adam */
int bx_gnn_get_params(bx_gnn_handle h, float* params);         /* host */
int bx_gnn_set_graph(bx_gnn_handle h, int n_nodes, const int32_t* ptr, const int32_t* nbr);
int bx_gnn_forward(bx_gnn_handle h, int lo, int hi, const float* x, int n_in, float* y, int n_out);
int bx_gnn_gradients(bx_gnn_handle h, int lo, int hi, const float* x, int n_in, const float* y,
                     int n_out, float* grad_host, float* loss_host);
int bx_gnn_train_step(bx_gnn_handle h, int lo, int hi, const float* x, int n_in, const float* y,
                      int n_out, float lr, float* loss_host);
int bx_gnn_destroy(bx_gnn_handle h);

/* Diagnostics: launch the fused cell kernel alone n times on the handle's
 * stream (state ping-pongs as in bx_step) and return the mean duration of one
 * launch in *ms_per_launch, measured with CUDA events around each launch.
 * Intended for roofline measurement; it advances the state by n steps
 * without the environment update, so re-upload the state afterwards. */
int bx_time_cell_kernel(bx_handle h, int n, double* ms_per_launch);
/* Algorithmic bytes one launch of the fused cell kernel moves (each array
 * counted once at its stored width; reads plus writes). */
int64_t bx_cell_kernel_bytes(bx_handle h);

/* FP64 throughput probe (no counterpart in the reference: it measures the
 * FP64 pipe that bounds the plain form's step).  Launches n_blocks CTAs of
 * 256 threads on `stream`; each thread runs 8 independent chains of `iters`
 * FMAs a = fma(a, b, c) from a = thread index + chain index and writes the
 * sum of its chains to out[thread index] (out: n_blocks * 256 doubles on
 * the device).  The launch issues n_blocks * 64 * iters FP64 warp FMAs;
 * the caller times it.  Asynchronous; BX_EINVAL on bad arguments
 * (n_blocks outside [1, 2^22], iters < 1, out NULL). */
int bx_fp64_fma_probe(int n_blocks, int iters, double b, double c, double* out, void* stream);

/* No-allocation step.  No counterpart in the reference (BETSE has no device
 * memory); it serves callers that cannot allocate GPU memory while they step,
 * e.g. a host framework that owns every device buffer through its own pool,
 * or a loop where cudaMalloc is forbidden.  It advances n_steps plain FP64
 * steps of one cluster without ECM on the caller's device buffers and calls
 * no cudaMalloc/cudaFree: its scratch is a fixed file-scope device array of
 * about 1.1 MB, present on every GPU that loads the library until exit.
 *   g      bx_geom whose array pointers are DEVICE pointers (cell_mem_ptr,
 *          nn_i, bflag, map_mem2ecm, mem_sa, gj_weight, cell_vol, diviterm)
 *   Dm     [n_ions * n_mems] device, read only
 *   vm, cc_mem, cc_cells, cc_env   device state in BETSE layouts: vm [n_mems],
 *          cc_mem [n_ions * n_cells] (cc_at_mem, one value per cell),
 *          cc_cells [n_ions * n_cells], cc_env [n_ions] (well mixed); updated
 *   vm_work [n_mems], cc_mem_work [n_ions * n_cells]   device work buffers
 * Limits (BX_EINVAL beyond them): n_cells <= 16384, n_mems <= 131072, and at
 * most 256 membranes in any 16 consecutive cells.  cell_mem_ptr and nn_i are
 * checked on the device before the first step (ptr[0] == 0, ptr[n_cells] ==
 * n_mems, strictly increasing; 0 <= nn_i < n_mems): BX_EINVAL, nothing
 * stepped.  check_v / no_negs (sim_toolbox.py:332-344, 475-503): a NaN in
 * Vmem or a cell concentration during the call returns BX_EUNSTABLE (the
 * buffers then hold the unstable state); negatives are clamped to 0 as BETSE
 * does.  The first call in a CUDA context looks up the array's device address
 * (cudaGetSymbolAddress) and caches it per context; make that first call
 * before any stream capture.  Every call shares the array and leaves the last
 * call's contents in it; calls that overlap on the GPU race on it, so
 * serialise them.  Synchronises `stream` twice per call: after the checks and
 * after the last step, to read the NaN counters. */
int bx_step_fp64_noalloc(const bx_geom* g, const bx_params* p, const double* Dm, double* vm,
                         double* vm_work, double* cc_cells, double* cc_mem, double* cc_mem_work,
                         double* cc_env, int n_steps, void* stream);

/* Launch configuration: CTA size (plain form 8, 16, 32, 64, 128 or 256
 * membrane slots per CTA -- the small ones spread a small cluster over more
 * SMs, 8 and 16 on 32-thread CTAs; split form 192 or
 * 256 membrane slots per tile, which sets how cells are grouped into tiles)
 * and, for the split form, the kernel:
 *   0  tile kernel (one tile per CTA, one launch per step; every variant)
 *   1  persistent pipelined tile kernel
 *   2  factored kernel: one thread per cell; the transmembrane flux and the
 *      pump are computed once per cell from the cell's sum of Dm * mem_sa,
 *      the gap-junction flux once per paired membrane (one launch per step)
 *   3  resident kernel: the factored step for many steps in one cooperative
 *      launch, each SM keeping its cells in shared memory (one cluster that
 *      fits; otherwise kernel 2 runs)
 *   4  factored kernel, persistent and software-pipelined: each warp stages
 *      its next tiles' cell data, gap-junction entries and partner records
 *      in shared memory (cp.async) while it computes (results as kernel 2)
 *   5  (plain form, 8, 16, 32 or 64 slots) the small-cluster FP64 step: one
 *      lane per membrane for the shared exponentials and the pump, one lane
 *      per (membrane, ion) for the fluxes and per (cell, ion) for the update,
 *      the environment mixed by the last CTA (one launch per step); no
 *      outputs, Phi_b, extracellular spaces, gating, Ca-ATPase or
 *      polarizability (else the tile kernel runs)
 * Bits 8-15 of kernel, when nonzero, pick the factored kernel's variant (the
 * third column of bx_autotune_table: 2, 4, 12, 13, 14 or 16).
 * Kernels 1-4 need no extracellular spaces, no voltage-gated gap junctions
 * and no Ca-ATPase; steps with outputs or a nonzero Phi_b always run the
 * tile kernel.  The state is kept.  bx_autotune picks these by timing. */
int bx_set_launch_config(bx_handle h, int tpb, int kernel);
int bx_get_launch_config(bx_handle h, int* tpb, int* kernel);
/* Whether the resident kernel fits this handle (*fits), and its grid, CTA
 * size and shared memory per CTA.  BX_EINVAL (with the reason) if not. */
int bx_resident_info(bx_handle h, int* fits, int* grid, int* threads, int64_t* smem_bytes);
/* Failure detection of the resident kernel, tested without a fault: one
 * launch whose grid barrier can never complete, so every CTA's bounded wait
 * runs out after timeout_ns (at most 2e9).  *timed_out = 1 if the kernel
 * reported the timeout; the state is left as it was. */
int bx_resident_barrier_check(bx_handle h, int64_t timeout_ns, int* timed_out);

/* Autotuner: times n_steps steps (run as bx_step runs them) for each
 * launch configuration -- tile size and, for the split form, the tile,
 * persistent, factored (at two load depths, with and without prefetched
 * junction entries), pipelined factored and resident kernels -- on the
 * uploaded state, keeps the fastest, and restores the state so the
 * simulation does not advance.
 * Reports the choice and its ms per step (either pointer may be NULL). */
int bx_autotune(bx_handle h, int n_steps, int* tpb_out, double* ms_per_step_out);
/* The same search, reporting every candidate it timed: up to max_rows rows of
 * (membrane slots per tile, kernel, factored-kernel variant, ms per step);
 * *n_rows is set to the rows written.  The variant is the number of gap
 * junctions loaded per round (2, 3, 4 or 6), plus 10 when the first entries
 * of each cell (6, or 8 with 4 per round) are loaded before the grid
 * dependency wait: 2, 4, 12, 13, 14, 16.  The fastest candidate is kept, as
 * by bx_autotune. */
int bx_autotune_table(bx_handle h, int n_steps, int max_rows, int* n_rows, int* tpb, int* kernel, int* unroll,
                      double* ms_per_step);

/* Version / diagnostics. */
int bx_abi_version(void);
const char* bx_last_error(void);
/* Number of kernel launches this handle has enqueued (cumulative). */
int64_t bx_launch_count(bx_handle h);
/* Sizes of a handle, for callers that hold only the handle (the PyTorch
 * operators): info[8] = {n_clusters, n_cells, n_mems, n_ions, grid_ny,
 * grid_nx, is_ecm, precision} (cells and membranes summed over a batch). */
int bx_cluster_info(bx_handle h, int32_t* info);

/* ---- Molecule and gene regulatory networks ------------------------------
 * MasterOfNetworks.run_loop (chemistry/networks.py:2805-2983) for the
 * user-defined substances of a general network (sim.molecules, sim.py:
 * 1290-1303) or a gene regulatory network (sim.grn, sim.py:1305-1319;
 * gene.py:220-308 runs it without the ions), on a plain FP64 single-cluster
 * handle without extracellular spaces.  BETSE builds every rate as a Python
 * string and evals it each step; the network here is the same arithmetic as
 * tables: substances, influencer terms and cell-zone reactions.
 *
 * An influencer factor (get_influencers, networks.py:5084-5600) is a range of
 * terms; its value is
 *   (prod of BX_TERM_ACT terms, or 1 if none) + sum of BX_TERM_ACT_INDEP terms
 *   times prod of BX_TERM_INH terms, times the sum of the direct terms if any,
 * with act = (c/Km)^n / (1 + (c/Km)^n), inh = 1 / (1 + (c/Km)^n) and direct
 * terms +c (BX_TERM_DIRECT_POS, an '&' activator) or -c (BX_TERM_DIRECT_NEG,
 * an '&' inhibitor); c is the substance's cell concentration, or its
 * well-mixed environment concentration when env_zone is 1. */
#define BX_NET_MAX_SUBSTANCES 16
#define BX_NET_MAX_REACTIONS 32
#define BX_NET_MAX_TERMS 256
#define BX_NET_MAX_STOICH 4
#define BX_TERM_ACT 0
#define BX_TERM_ACT_INDEP 1
#define BX_TERM_INH 2
#define BX_TERM_DIRECT_POS 3
#define BX_TERM_DIRECT_NEG 4

typedef struct bx_net_term {
    int32_t kind;        /* BX_TERM_* */
    int32_t substance;   /* index into the network's substances */
    int32_t env_zone;    /* 0: cell concentration, 1: environment */
    int32_t pad;
    double Km, n;
} bx_net_term;

typedef struct bx_net_substance {   /* Molecule fields (networks.py:337-600) */
    double z, Dm, Do, Dgj;
    double time_factor;             /* modify_time_factor: the time dilation factor or 1 */
    double r_production, r_decay, decay_max, gad_scale_factor;
    int32_t growth;                 /* 'growth and decay' given (simple_growth) */
    int32_t update_intra;           /* 'update intracellular' */
    int32_t gj_impermeable;         /* 'GJ impermeable' */
    int32_t growth_term0, growth_nterm;   /* growth influencers */
    int32_t decay_term0, decay_nterm;     /* decay influencers */
    int32_t pad;
    const double* growth_mod;       /* [n_cells] growth_mod_function_cells, or NULL (1) */
    const uint8_t* growth_target;   /* [n_cells] 1 on growth_targets_cell, or NULL (all) */
} bx_net_substance;

typedef struct bx_net_reaction {    /* Reaction fields (networks.py:814-922) */
    int32_t n_reactants, n_products;
    int32_t reactant[BX_NET_MAX_STOICH], product[BX_NET_MAX_STOICH];
    double reactant_coeff[BX_NET_MAX_STOICH], reactant_Km[BX_NET_MAX_STOICH];
    double product_coeff[BX_NET_MAX_STOICH];
    double vmax;
    double keq;                     /* exp(-delta_Go / (R T)); 0: no standard free energy */
    int32_t term0, nterm;           /* reaction activators and inhibitors */
} bx_net_reaction;

typedef struct bx_net_spec {
    int32_t n_substances, n_reactions, n_terms, pad;
    const bx_net_substance* substances;
    const bx_net_reaction* reactions;
    const bx_net_term* terms;
    const double* mem_vol;          /* [n_mems] cells.mem_vol (update intracellular) */
    const double* R_rads;           /* [n_mems] cells.R_rads (update intracellular) */
} bx_net_spec;

typedef struct bx_network* bx_network_handle;
/* Build a network on a cluster handle; copies the spec.  The handle must
 * outlive the network.  Refuses (BX_EINVAL) split-form, batched and ECM
 * handles and out-of-range tables. */
int bx_network_create(bx_handle cluster, const bx_net_spec* spec, bx_network_handle* out);
/* The substance state (Molecule.c_cells [S][C], cc_at_mem [S][M], c_env [S]:
 * the well-mixed value), host or device arrays. */
int bx_network_upload(bx_network_handle n, const double* c_cells, const double* cc_at_mem, const double* c_env);
int bx_network_download(bx_network_handle n, double* c_cells, double* cc_at_mem, double* c_env);
/* n_steps time steps.  with_ions = 1: each step is the cluster's ion step
 * (bx_step) followed by the network step in BETSE's order -- the network
 * reads Vmem from the start of the step and the gap-junction state that
 * step leaves; with_ions = 0: the network alone on the cluster's current
 * Vmem and gap-junction state (gene.py:220-308).  want_outputs = 1: the last
 * step also computes the ion step's outputs (bx_outputs_download) and keeps
 * the network's fluxes and reaction rates for bx_network_fluxes. */
int bx_network_step(bx_network_handle n, int n_steps, int with_ions, int want_outputs);
/* The last output step's Molecule.f_mem and f_gj ([S][M] each) and
 * MasterOfNetworks.reaction_rates ([R][C]); any pointer may be NULL. */
int bx_network_fluxes(bx_network_handle n, double* f_mem, double* f_gj, double* rates);
/* Negative substance concentrations seen since the upload (BETSE raises
 * BetseSimUnstableException on them, sim_toolbox.py:1132-1151,
 * networks.py:5802-5807). */
int bx_network_status(bx_network_handle n, int64_t* negative);
/* Runs bx_network_step(n, n_steps, with_ions, 0) between two CUDA events on
 * the cluster's stream; reports ms per time step (the state advances). */
int bx_network_time_step(bx_network_handle n, int n_steps, int with_ions, double* ms_per_step);
/* info[4] = {substances, reactions, n_cells, n_mems}. */
int bx_network_info(bx_network_handle n, int32_t* info);
int bx_network_destroy(bx_network_handle n);

/* ---- synthetic clusters on the GPU (Cells.make_world's seeding,
 * cells.py:414-961; _make_cell_lattice :742-801; DECMesh.clip_and_refine's
 * two passes, math/mesh.py:189,2290-2372; cellVerts :978-1175; cell_vols
 * :1358-1390; near_neigh :1477-1573; makeECM/environment :1576-1843).
 *
 * The lattice is BETSE's bit for bit: numpy.linspace rows (the caller passes
 * each row's start, stop and count, computed as _make_cell_lattice does) and
 * the jitter jitter * (rand - 0.5), x draws then y draws, from MT19937 seeded
 * as numpy.random.RandomState(seed).  Pass one: the centroid-Voronoi cell of
 * each lattice point (with the lattice's bounding-box corners added) and its
 * area centroid; the centroids inside the disc of `radius` about the
 * lattice's mean are the points of pass two, whose closed cells are the
 * cluster, ordered along a Z curve of their area centroids.  Membranes are
 * each cell's polygon edges scaled by scale_cell about its centre, listed as
 * cellVerts lists them; gap-junction partners are the membranes across each
 * shared Delaunay edge (a membrane without one is paired with itself); the
 * grid is the lattice box widened by cell_radius, grid_size cells wide. */
typedef struct bx_gen_spec {
    uint32_t seed;          /* numpy.random.RandomState seed of the jitter */
    int32_t grid_size;      /* p.grid_size */
    int32_t nbx, nby, nrx, nry;                 /* linspace counts of the four rows */
    double bx0, bx1, by0, by1, rx0, rx1, ry0, ry1;   /* their starts and stops */
    double jitter;          /* p.cell_lattice_disorder * d_cell */
    double radius;          /* disc radius (m) */
    double d_cell;          /* lattice spacing (m) */
    double cell_radius;     /* d_cell / 2 */
    double scale_cell;      /* p.scale_cell */
    double cell_height;     /* p.cell_height */
} bx_gen_spec;

typedef struct bx_gen_arrays {      /* destinations, host or device; NULL skips */
    int32_t* cell_mem_ptr;          /* [C+1] */
    int32_t* nn_i;                  /* [M] */
    int32_t* map_mem2ecm;           /* [M] */
    double *mem_sa, *mem_nx, *mem_ny, *R_rads, *mem_mid_x, *mem_mid_y;   /* [M] */
    double *cell_vol, *cell_sa, *diviterm, *cell_centre_x, *cell_centre_y;  /* [C] */
    double* mem_sa_per_env;         /* [grid_ny * grid_nx] */
    int32_t* cell_nn_ptr;           /* [C+1] */
    int32_t* cell_nn;               /* [n_cell_nn]: each cell's neighbours, ascending */
    double *lattice_x, *lattice_y;  /* [n_lattice] the jittered seed lattice */
} bx_gen_arrays;

typedef struct bx_generated* bx_gen_handle;
/* Runs the whole generation on `stream` (allocates; returns when done).
 * BX_EINVAL on a bad specification or a degenerate point set. */
int bx_generate_cluster(const bx_gen_spec* spec, void* stream, bx_gen_handle* out);
/* sizes[6] = {C, M, grid_ny, grid_nx, n_cell_nn, n_lattice};
 * box[5] = {xmin, xmax, ymin, ymax, delta} of the environment grid. */
int bx_generated_info(bx_gen_handle g, int32_t* sizes, double* box);
int bx_generated_download(bx_gen_handle g, const bx_gen_arrays* a);
int bx_generated_destroy(bx_gen_handle g);

#ifdef __cplusplus
}
#endif
#endif /* BX_H */
