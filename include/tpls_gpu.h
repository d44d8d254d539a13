/*
 * tpls_gpu.h -- C ABI of the GB300 implementation of the TPLS per-timestep
 * hot path (level-set advection, redistancing, CSF, momentum operator with
 * Jacobi / red-black SOR Crank-Nicolson sweeps, pressure Poisson solve,
 * projection).
 *
 * Conventions (chosen so a Fortran driver can bind every entry with
 * ISO_C_BINDING without wrappers):
 *   - every array is the reference's explicit-shape, column-major array of a
 *     single rank: p-grid (0:nx+1,0:ny+1,0:nz+1), u/v (0:nx+1,0:ny+1,0:nz-1),
 *     w (0:nx+1,0:ny+1,0:nz), viscosity_aug (-1:nx+2,-1:ny+2,0:nz+1);
 *   - scalars are passed by reference, in the reference's argument order;
 *     index bounds (sx, ex, ...) are checked against the context and must be
 *     the single-rank values; MPI-only arguments (neighbours, communicator,
 *     derived-datatype handles) are accepted and ignored;
 *   - every entry returns an int status: 0 = OK, >0 = error (TPLS_ERR_* or a
 *     CUDA error code + TPLS_ERR_CUDA_BASE), <0 = KSP-style divergence of the
 *     pressure solve (-3 DIVERGED_ITS, -9 DIVERGED_NAN);
 *   - calls on one context are single-threaded and stream-ordered; separate
 *     contexts may be driven from separate host threads.
 * The per-routine entries take HOST arrays (copied in and out around the
 * kernels, or standing for device mirrors once registered with
 * tpls_register_host); tpls_step() runs whole timesteps on device-resident
 * state.
 */
#ifndef TPLS_GPU_H
#define TPLS_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define TPLS_OK 0
#define TPLS_ERR_ARG 1         /* bad argument / bounds mismatch */
#define TPLS_ERR_ALLOC 2       /* device allocation failed */
#define TPLS_ERR_STATE 3       /* call sequence error */
#define TPLS_ERR_NOT_BUILT 4   /* feature not compiled into the library */
#define TPLS_ERR_IO 6          /* a file could not be opened, written or parsed */
#define TPLS_ERR_CUDA_BASE 1000 /* + cudaError_t */
#define TPLS_KSP_CONVERGED_RTOL 2
#define TPLS_KSP_CONVERGED_ATOL 3
#define TPLS_KSP_DIVERGED_ITS (-3)
#define TPLS_KSP_DIVERGED_NAN (-9)

#define TPLS_PREC_FP64 0      /* FP64 everywhere (optionally FP32 multigrid
                                  levels in the CG preconditioner: mg_fp32) */
#define TPLS_PREC_FP32_MIXED 1 /* FP32 stencils/sweeps/smoothing, FP64 state,
                                  dots, residuals, volume integral, coarse solve */

/* Physical and solver parameters.  Names follow the reference's .opt keys
 * (option_names.F90) and main_ns_hybrid.F90 variables. */
typedef struct tpls_params {
  double dx, dy, dz, dt;          /* dx,dy,dz,dt */
  double re, mu_plus, mu_minus;   /* re, mu_plus (upper), mu_minus (lower) */
  double height, scap, smooth_width;
  int mom_u, mom_v, mom_w;        /* max_iteration_mom_{u,v,w} (outer its = /2) */
  int levelset;                   /* max_iteration_levelset */
  double p_rtol;                  /* pressure solve: ||r||_2 <= rtol*||b||_2 */
  int p_maxits;                   /* pressure solve iteration cap */
  int precision;                  /* TPLS_PREC_* */
  int fp64_parts;                 /* FP32-mixed form only: TPLS_PART_* bits of
                                     the parts kept in FP64 (0 = all FP32) */
  int mg_fp32;                    /* FP64 form: 1 = FP32 multigrid levels in the
                                     CG preconditioner (CG itself stays FP64 and
                                     meets p_rtol on its FP64 residual) */
  int idm;                        /* idm: TPLS_IDM_LSM (level set, default) or
                                     TPLS_IDM_DIM (diffuse interface, FP64 form) */
  int max_iteration_dim;          /* max_iteration_dim (DIM SOR iterations) */
  int flags;                      /* TPLS_FLAG_* (0 = defaults) */
  int reserved;
  double epn, pe;                 /* epn, Pe (DIM interface width, Peclet number) */
} tpls_params;

/* tpls_params.flags: TPLS_FLAG_NO_TMA makes the FP32-mixed form's advection
 * read phi through the caches instead of staging its tiles with TMA
 * (bit-identical results). */
#define TPLS_FLAG_NO_TMA 1
/* tpls_params.flags: TPLS_FLAG_ODD_COLUMNS makes the odd half-sweep of the
 * FP64 coefficient records walk each column in one block instead of one
 * block per 64-level segment chained up the column (bit-identical). */
#define TPLS_FLAG_ODD_COLUMNS 2

/* Interface method (main_ns_hybrid.F90:595-612, option_names.F90:35-37). */
#define TPLS_IDM_LSM 0
#define TPLS_IDM_DIM 1

/* Parts of the FP32-mixed form that can be kept in FP64 (tpls_params.fp64_parts). */
#define TPLS_PART_ADVECT 1    /* WENO5 advection */
#define TPLS_PART_LEVELSET 2  /* redistancing iterations */
#define TPLS_PART_MOMENTUM 4  /* momentum stencils, records and sweeps */
#define TPLS_PART_MULTIGRID 8 /* multigrid preconditioner */
#define TPLS_PART_MOM_STENCIL 16 /* momentum stencils in FP64 (the FP32 sweeps'
                                    defect right-hand side stored FP32) */

/* Per-step diagnostics, the quantities the reference logs each timestep
 * (main_ns_hybrid.F90:601-605, 803-808, 840-845, 882-887, 903-911). */
typedef struct tpls_stats {
  double err_phi;   /* last redistancing sum (phi_reinit - updated)^2 */
  double err_u, err_v, err_w; /* get_difference(u3, u3_old) etc. */
  double p_rnorm;   /* final ||r||_2 of the pressure solve */
  double p_bnorm;   /* ||b||_2 of the (projected) pressure right-hand side */
  int p_its;        /* pressure iterations */
  int p_reason;     /* KSP-style converged/diverged reason */
  long steps_done;
  double liquid_volume; /* sum over cells of (1-H(phi)) dV after the step */
  int p_worst;      /* lowest reason of the solves since the previous
                       tpls_get_stats (0 when none diverged) */
  int kernel_timeouts; /* blocks whose bounded wait for staged data ran out
                          (their outputs are NaN); 0 in a healthy run */
  int reserved_i[2];
} tpls_stats;

/* Field identifiers for tpls_set_field / tpls_get_field and the oracle.
 * Kind P = p-grid, UV = u/v grid, W = w grid (see shapes above). */
enum tpls_field {
  TPLS_F_PHI2 = 0,      /* P  */
  TPLS_F_U2, TPLS_F_V2, /* UV */
  TPLS_F_W2,            /* W  */
  TPLS_F_PRES,          /* P  */
  TPLS_F_PRES_OLD,      /* P  */
  TPLS_F_CONV0_U, TPLS_F_CONV1_U, TPLS_F_CONV0_V, TPLS_F_CONV1_V, /* UV */
  TPLS_F_CONV0_W, TPLS_F_CONV1_W,                                 /* W */
  TPLS_F_CSF_U0, TPLS_F_CSF_U1, TPLS_F_CSF_V0, TPLS_F_CSF_V1,     /* UV */
  TPLS_F_CSF_W0, TPLS_F_CSF_W1,                                   /* W */
  TPLS_F_CONV0_PHI, TPLS_F_CONV1_PHI,                             /* P */
  /* intermediates of the last step (read-only) */
  TPLS_F_CONV2_PHI,     /* P  */
  TPLS_F_PHI3,          /* P  (DIM: the reference's phi3 array, the starting
                                  guess of the next step's iteration: 0 at
                                  creation, then the last step's phi) */
  TPLS_F_RHS_P,         /* P  */
  TPLS_F_U3, TPLS_F_V3, /* UV (before projection) */
  TPLS_F_W3,            /* W  */
  /* diffuse-interface state (TPLS_IDM_DIM contexts only) */
  TPLS_F_CONVPREV_PHI,  /* P  ConvPrevPhi (main_ns_hybrid.F90:449, cahn_hilliard_solver.f90:270) */
  TPLS_F_COUNT
};

typedef struct tpls_ctx tpls_ctx;

/* ---- context ---------------------------------------------------------- */
/* Replaces the allocation / set-up of main_ns_hybrid.F90:216-549 and
 * setup_MPI (configure_mpi_petsc.F90:61-212) for one channel on one GPU.
 * u_inlet has nz entries (u_inlet(0:maxn-2)). */
int tpls_gpu_create(int nx, int ny, int nz, const tpls_params *prm,
                    const double *u_inlet, tpls_ctx **out);
int tpls_gpu_destroy(tpls_ctx *ctx);
int tpls_set_field(tpls_ctx *ctx, int field, const double *host);
int tpls_get_field(tpls_ctx *ctx, int field, double *host);
/* Grid of the context. */
int tpls_get_dims(const tpls_ctx *ctx, int *nx, int *ny, int *nz);
/* Several fields per call (no counterpart in the reference, which keeps its
 * arrays on the host): fields[i] to / from host[i], in the layouts of
 * tpls_set_field / tpls_get_field, without a host wait between fields.
 * Downloads are 2-D copies from the device fields on one copy stream;
 * right after a graph-launched step, the fields that step no longer writes
 * after its front half (the level set, the CSF and convection histories)
 * are copied as soon as that half is done, while the rest of the step
 * runs.  Uploads go through staging buffers on another stream (as many as
 * the call's fields, allocated on first use and not counted by
 * tpls_footprint_bytes) and are repacked on the context's stream, so
 * successive fields overlap.  An upload of an array still being downloaded, or into a
 * field still being downloaded, waits for that download on the device: a
 * get of the state followed by a set of the same arrays runs both copy
 * directions at once.  Both calls return once the copies are enqueued:
 * steps enqueued afterwards run after the uploads and do not overwrite a
 * field before its download has read it; the host arrays of a get may be
 * read after tpls_sync (or tpls_xfer_join and a wait on the context's
 * stream).  Pinned host memory gives the link's full speed. */
int tpls_set_fields(tpls_ctx *ctx, int n, const int *fields,
                    const double *const *host);
int tpls_get_fields(tpls_ctx *ctx, int n, const int *fields,
                    double *const *host);
/* Make later work on the context's stream (tpls_stream) wait for every
 * download enqueued so far. */
int tpls_xfer_join(tpls_ctx *ctx);
/* Step counter reported in tpls_stats.steps_done, for a restarted run that
 * continues an earlier one's count (the driver's `iteration`). */
int tpls_set_steps_done(tpls_ctx *ctx, long steps_done);
/* Device-resident fast path: nsteps full timesteps of main_ns_hybrid.F90:
 * 583-918 followed by the history rotation :2480-2509.  Returns TPLS_OK;
 * TPLS_KSP_DIVERGED_ITS if any pressure solve hit p_maxits (the remaining
 * steps still run, as in the reference's loop); TPLS_KSP_DIVERGED_NAN, an
 * argument or a CUDA error at the failing step, which ends the call. */
int tpls_step(tpls_ctx *ctx, int nsteps);
/* The same steps enqueued without waiting: with graphs enabled (the
 * default) each step is one CUDA-graph launch on the context's stream whose
 * pressure iterations run under a device-side WHILE node, so no host round
 * trip happens inside a step.  Returns TPLS_OK or a launch/capture error;
 * the solves' outcome is read by tpls_get_stats (p_worst) or tpls_step.
 * With graphs disabled or timing enabled it runs tpls_step. */
int tpls_step_async(tpls_ctx *ctx, int nsteps);
/* ---- sweep tile autotuner (no counterpart in the reference) ------------
 * Times each candidate block shape of the Jacobi and even half-sweep
 * kernels (reps launches each, on the context's own arrays) and keeps the
 * fastest; results are cached per grid and sweep precision for the process.
 * Clobbers the last step's U3/V3/W3 intermediates; captured step graphs are
 * rebuilt at the next step (batches included).  The state a run produces
 * does not depend on the choice (same arithmetic per point). */
int tpls_autotune(tpls_ctx *ctx, int reps);
/* tiles3 = {Jacobi shape 0..3, even shape 0..3, odd half-sweep shape (0)} */
int tpls_get_tiles(const tpls_ctx *ctx, int *tiles3);

/* ---- job-serving helpers (no counterpart in the reference) ------------ */
/* Device bytes tpls_gpu_create allocates for this grid and precision (each
 * allocation rounded to the allocator's 2 MiB unit), or -1 for bad
 * arguments.  Host-only: used for admission before anything is allocated.
 * For TPLS_PREC_FP32_MIXED it counts the FP64 arrays of TPLS_PART_LEVELSET
 * and TPLS_PART_MOM_STENCIL (an upper bound when those parts are off);
 * keeping TPLS_PART_MOMENTUM in FP64 allocates more. */
long long tpls_footprint_bytes(int nx, int ny, int nz, int precision);
/* 1 when every step enqueued on the context has finished, 0 while work is
 * pending, or an error status.  Does not block. */
int tpls_query(tpls_ctx *ctx);
/* Interface height h(x, y) of the current phi: for each column (i, j),
 * i = 1..nx, j = 1..ny, the lowest z where phi changes sign between
 * consecutive cell centres, by linear interpolation (cell centres at
 * z_k = (k - 1/2) dz); columns without a sign change get -1.  h_host holds
 * nx*ny doubles, i fastest. */
int tpls_interface_height(tpls_ctx *ctx, double *h_host);

/* ---- batches (no counterpart in the reference, which runs one channel
 * per MPI job) ------------------------------------------------------------
 * n independent channels advanced in lockstep: each batch step is ONE
 * CUDA-graph launch holding every member's step as a parallel branch (the
 * members' pressure iterations as device-side WHILE nodes), so the
 * instances' kernels share the GPU concurrently.  Members must be at the
 * same history phase (created together, or stepped the same number of
 * times) and must not be stepped on their own while in a batch.  The
 * members keep their state, fields and stats; the batch only launches. */
typedef struct tpls_batch tpls_batch;
int tpls_batch_create(tpls_ctx *const *ctxs, int n, tpls_batch **out);
int tpls_batch_destroy(tpls_batch *b);
/* Enqueue nsteps batch steps (one graph launch each) without waiting. */
int tpls_batch_step_async(tpls_batch *b, int nsteps);
/* The same, then wait; returns the lowest pressure reason of any member
 * (0 when every solve converged) or an error. */
int tpls_batch_step(tpls_batch *b, int nsteps);
/* on = 1: run the members' FP32 momentum sweeps (every Jacobi sweep and
 * half-sweep of the three components) as multi-instance launches: one
 * persistent launch per sweep for all members, blocks taking the members'
 * tiles in order from an atomic ticket, instead of one launch per member.
 * The rest of each member's step stays a parallel branch of the batch
 * graph.  Results are bit-identical to on = 0.  Requires every member to be
 * in the FP32-mixed form with FP32 sweeps (TPLS_PART_MOMENTUM not kept in
 * FP64), an even ny, and the same mom_u, mom_v, mom_w; TPLS_ERR_ARG
 * otherwise.  on = 0 returns to one branch per member. */
int tpls_batch_multi_sweeps(tpls_batch *b, int on);

/* Graph mode on (1, default) or off (0: every step launched kernel by
 * kernel, the pressure iterations driven by the host).  Both give
 * bit-identical results. */
int tpls_graphs_enable(tpls_ctx *ctx, int on);
int tpls_get_stats(tpls_ctx *ctx, tpls_stats *out);
/* Waits for the context's stream and its copy streams. */
int tpls_sync(tpls_ctx *ctx);
/* Self-test of the bounded wait of the TMA-staged advection (no
 * counterpart in the reference): one block of that kernel is launched
 * with no load issued, so its wait for the staged tile runs out after a
 * short limit; *timeouts returns how many blocks reported it (1) and
 * *nan_out whether the block wrote NaN into its output cells (1), into a
 * scratch array (the context's state is untouched).  TPLS_ERR_STATE for a
 * context without the TMA path (FP64 form, or TPLS_FLAG_NO_TMA). */
int tpls_selftest_wait_limit(tpls_ctx *ctx, int *timeouts, int *nan_out);
const char *tpls_status_string(int status);
/* Number of kernels the library has launched on this context (counted on
 * the host at every launch site). */
long tpls_kernel_launches(tpls_ctx *ctx);

/* Device timing by phase, with CUDA events recorded on the context's stream
 * around every launch of a phase (kernels of the momentum sweeps are timed
 * one launch at a time).  tpls_timing_read accumulates since the last reset
 * (reset=1 clears after reading).  ms and launches have TPLS_T_COUNT
 * entries. */
enum tpls_timer {
  TPLS_T_ADVECT = 0, TPLS_T_LEVELSET, TPLS_T_CSF, TPLS_T_VISC, TPLS_T_MOM_RHS,
  TPLS_T_JACOBI, TPLS_T_SOR, TPLS_T_SOR_ODD, TPLS_T_PRESSURE, TPLS_T_PROJECT,
  TPLS_T_OTHER,
  TPLS_T_COUNT
};
int tpls_timing_enable(tpls_ctx *ctx, int on);
int tpls_timing_read(tpls_ctx *ctx, double *ms, long *launches, int reset);
/* The cudaStream_t every kernel of this context is launched on. */
void *tpls_stream(tpls_ctx *ctx);

/* Reference initial-condition tool restated for the harness:
 * twophase_initialisation_wave.F90:79-122 base profile (Gauss-Seidel,
 * 10000 sweeps) -- writes u_oned(0:nz-1). */
int tpls_base_profile(int nz, double dz, double re, double dpdl,
                      double mu_minus, double mu_plus, double height,
                      double smooth_width, double *u_oned);

/* ---- host-array registry ----------------------------------------------
 * Keeps the driver's arrays (state.F90:21-53: phi2, u2, u3, RHS_u,
 * viscosity2_aug, pres, ...) device-resident while its call sites in
 * main_ns_hybrid.F90 keep passing the same host addresses to the
 * per-routine entries below.  tpls_register_host(ctx, a, n) allocates a
 * device mirror of the n doubles at a and copies them once; from then on
 * every copy the library makes to or from an address inside [a, a+n)
 * (the per-routine entries, tpls_set_field/get_field and the batched
 * transfers) goes to the same place in the mirror, so a routine's inputs
 * and outputs stay on the device and the host array is NOT updated.
 * tpls_download_host(ctx, a) refreshes the host array from its mirror (at
 * the driver's output frequency; a = NULL: every registered array),
 * tpls_upload_host(ctx, a) the mirror from the host array (after host code
 * changed it).  Registered ranges may not overlap (TPLS_ERR_ARG).  Mirrors
 * are freed by tpls_unregister_host or tpls_gpu_destroy (no copy back), and
 * are not counted by tpls_footprint_bytes. */
int tpls_register_host(tpls_ctx *ctx, double *host, long long count);
int tpls_unregister_host(tpls_ctx *ctx, double *host);
int tpls_download_host(tpls_ctx *ctx, double *host);
int tpls_upload_host(tpls_ctx *ctx, const double *host);

/* ---- per-routine drop-in entries (host arrays) ------------------------ */

/* advect_phi.f90:19-27  do_advect_phi (incl. weno.f90:18 WENOAppoxConvection) */
int tpls_do_advect_phi(tpls_ctx *ctx, const double *phi2, double *u2,
                       double *v2, double *w2, double *conv2_phi,
                       const int *sx, const int *ex, const int *sy,
                       const int *ey, const int *sz_p, const int *ez_p,
                       const int *sz_uv, const int *sz_w, const int *ez_uv,
                       const int *ez_w, const int *maxl, const int *maxn,
                       const int *ex_max, const int *neighbours,
                       const int *comm2d_quasiperiodic, const double *dx,
                       const double *dy, const double *dz,
                       const int *stride_p_augaug1_xz,
                       const int *stride_p_augaug1_yz,
                       const int *stride_p_augaug2_xz,
                       const int *stride_p_augaug2_yz,
                       const int *stride_p_augaug3_xz,
                       const int *stride_p_augaug3_yz,
                       const int *stride_uv_xz, const int *stride_uv_yz,
                       const int *stride_w_xz, const int *stride_w_yz);

/* two_phase_levelset.f90:20-25  do_tpls (AB3 update + redistancing) */
int tpls_do_tpls(tpls_ctx *ctx, double *phi2, double *phi3,
                 double *conv0_phi, double *conv1_phi, double *conv2_phi,
                 const int *sx, const int *ex, const int *sy, const int *ey,
                 const int *sz_p, const int *ez_p, const int *maxn,
                 const int *ex_max, const int *stride_p_xz,
                 const int *stride_p_yz, const int *max_iteration_levelset,
                 const int *neighbours, const int *comm2d_quasiperiodic,
                 const double *height, double *err2, const double *dx,
                 const double *dz, const double *dt);

/* cahn_hilliard_solver.f90:41-382  dim (diffuse-interface update): phi and
 * phiOld are the concentration fields C = phi + 0.5 (the driver passes
 * phi2+0.5 and phi_old+0.5, main_ns_hybrid.F90:608), phiNew holds the
 * starting guess on entry and C^{n+1} on return, ConvPrevPhi is updated in
 * place.  p-grid arrays, host memory. */
int tpls_dim(tpls_ctx *ctx, const int *maxl, const int *maxn, const double *dx,
             const double *dy, const double *dz, const double *dt,
             const double *epn, const double *pe, const double *phi,
             const double *phi_old, const double *conv2_phi,
             double *conv_prev_phi, double *phi_new, const int *sx,
             const int *ex, const int *sy, const int *ey, const int *sz_p,
             const int *ez_p, const double *height, const int *stride_p_xz,
             const int *stride_p_yz, const int *neighbours,
             const int *comm2d_quasiperiodic, const int *max_iteration_dim);

/* levelset.f90:241-242  get_csf */
int tpls_get_csf(tpls_ctx *ctx, double *fx_csf, double *fy_csf,
                 double *fz_csf, const double *fi, const int *sx,
                 const int *ex, const int *sy, const int *ey, const int *n,
                 const int *ex_max, const double *dx, const double *dy,
                 const double *dz, const double *scap,
                 const double *smooth_width);

/* momentum_allflux.f90:474  get_viscosity, plus the augmented-viscosity
 * assembly of main_ns_hybrid.F90:646-724 (x ghost planes from phi2 and the
 * 2-row periodic-y wrap).  viscosity_aug is (-1:nx+2,-1:ny+2,0:nz+1). */
int tpls_get_viscosity(tpls_ctx *ctx, double *viscosity_aug,
                       const double *phi, const int *ex, const int *ey,
                       const int *sx, const int *sy, const int *maxn,
                       const double *smooth_width, const double *re,
                       const double *mu_minus, const double *mu_plus);

/* momentum_allflux.f90:224-225  get_conv_all */
int tpls_get_conv_all(tpls_ctx *ctx, double *conv_u2, double *conv_v2,
                      double *conv_w2, const double *viscosity_aug,
                      const double *u2, const double *v2, const double *w2,
                      const int *sx, const int *sy, const int *ex,
                      const int *ey, const int *maxn, const int *ex_max,
                      const double *dx, const double *dy, const double *dz);

/* momentum_allflux.f90:22-23  get_diffusion_all */
int tpls_get_diffusion_all(tpls_ctx *ctx, double *diff_u, double *diff_v,
                           double *diff_w, const double *viscosity,
                           const double *u2, const double *v2,
                           const double *w2, const int *sx, const int *sy,
                           const int *ex, const int *ey, const int *maxn,
                           const int *ex_max, const double *dx,
                           const double *dy, const double *dz);

/* jacobi_iteration_allflux.f90:21-22, 102-103, 195-196  do_jacobi_{u,v,w} */
int tpls_do_jacobi_u(tpls_ctx *ctx, double *u3, const double *u3_old,
                     const double *rhs, const double *viscosity,
                     const double *dx, const double *dy, const double *dz,
                     const double *dt, const int *ex, const int *ey,
                     const int *sx, const int *sy, const int *maxn,
                     const int *ex_max);
int tpls_do_jacobi_v(tpls_ctx *ctx, double *v3, const double *v3_old,
                     const double *rhs, const double *viscosity,
                     const double *dx, const double *dy, const double *dz,
                     const double *dt, const int *ex, const int *ey,
                     const int *sx, const int *sy, const int *maxn,
                     const int *ex_max);
int tpls_do_jacobi_w(tpls_ctx *ctx, double *w3, const double *w3_old,
                     const double *rhs, const double *viscosity,
                     const double *dx, const double *dy, const double *dz,
                     const double *dt, const int *ex, const int *ey,
                     const int *sx, const int *sy, const int *maxn,
                     const int *ex_max);

/* sor_iteration_allflux.f90:19-20, 152-153, 280-281  do_sor_{u,v,w} */
int tpls_do_sor_u(tpls_ctx *ctx, double *u3, const double *rhs,
                  const double *viscosity, const double *dx,
                  const double *dy, const double *dz, const double *dt,
                  const int *ex, const int *ey, const int *sx, const int *sy,
                  const int *maxn, const int *ex_max, const int *flg,
                  const int *iteration_time);
int tpls_do_sor_v(tpls_ctx *ctx, double *v3, const double *rhs,
                  const double *viscosity, const double *dx,
                  const double *dy, const double *dz, const double *dt,
                  const int *ex, const int *ey, const int *sx, const int *sy,
                  const int *maxn, const int *flg, const int *iteration_time);
int tpls_do_sor_w(tpls_ctx *ctx, double *w3, const double *rhs,
                  const double *viscosity, const double *dx,
                  const double *dy, const double *dz, const double *dt,
                  const int *ex, const int *ey, const int *sx, const int *sy,
                  const int *maxn, const int *flg, const int *iteration_time);

/* jacobi_iteration_allflux.f90:285  get_difference (z range sz:ez) */
int tpls_get_difference(tpls_ctx *ctx, const double *ua, const double *ub,
                        const int *ex, const int *ey, const int *ez,
                        const int *sx, const int *sy, const int *sz,
                        double *diff);

/* pressure.f90:16  get_source_pres */
int tpls_get_source_pres(tpls_ctx *ctx, double *rhs, const double *u3,
                         const double *v3, const double *w3, const int *ex,
                         const int *ey, const int *sx, const int *sy,
                         const int *maxn, const double *dx, const double *dy,
                         const double *dz, const double *dt);

/* pressure.f90:59  get_uvw_pres */
int tpls_get_uvw_pres(tpls_ctx *ctx, double *u3, double *v3, double *w3,
                      const double *p, const int *ex, const int *ey,
                      const int *sx, const int *sy, const int *maxn,
                      const int *ex_max, const double *dx, const double *dy,
                      const double *dz, const double *dt,
                      const double *u_inlet);

/* main_ns_hybrid.F90:896-913 `pres=pres_old; KSPSolve(ksp);
 * copy_pressure_out_of_petsc` with the callbacks of pressure_solver.F90:
 * 205-486 (initial guess, RHS incl. inlet rows, 7-point matrix with Neumann
 * ghost rows, constant null space).  Solved by geometric-multigrid
 * preconditioned CG on the symmetric reduced system.  pres is the full
 * p-grid array (ghost planes and periodic-y rows written). rtol<=0 takes
 * the context's p_rtol; maxits<=0 takes p_maxits. */
int tpls_pressure_solve(tpls_ctx *ctx, double *pres, const double *pres_old,
                        const double *rhs_p, const double *u3,
                        const double *u_inlet, const double *dx,
                        const double *dy, const double *dz, const double *dt,
                        const double *rtol, const int *maxits, int *its,
                        double *rnorm, int *reason);

/* ---- no-allocation entry ------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory: a time-step loop that cannot wait for cudaMalloc/cudaFree (they
 * may block until the device is idle), or a program whose device memory is
 * owned by another runtime's pool or by a fixed HBM budget.  Same sum as
 * tpls_get_difference, on DEVICE arrays ua, ub in the reference layout
 * (0:nx+1, 0:ny+1, 0:nzp-1), result written to the device address diff,
 * enqueued on `stream` (a cudaStream_t; NULL = default stream).  It allocates
 * nothing: its scratch is a fixed 512 KB array inside the library (one
 * partial per row), so ny*nzp may not exceed TPLS_NOALLOC_MAX_ROWS (larger
 * calls return TPLS_ERR_NOALLOC_LIMIT and launch nothing).  The first call
 * on a device looks up that array's device address (make it before any
 * stream capture) and keeps it for the life of the process: a
 * cudaDeviceReset of that device destroys the array, and the entry must not
 * be called on that device afterwards.  All calls share the array: calls
 * that overlap on the GPU race and must be serialised by the caller. */
#define TPLS_NOALLOC_MAX_ROWS 65536
#define TPLS_ERR_NOALLOC_LIMIT 5
int tpls_get_difference_noalloc(const double *ua, const double *ub, int nx,
                                int ny, int nzp, double *diff, void *stream);

/* ---- backup / restart files ----------------------------------------------
 * io.F90:647-716 backup_channel: the reference's text backup (one record
 * per point, i fastest: u2, conv0_u, conv1_u over the u grid; the same for
 * v; w2, conv0_w, conv1_w over the w grid; phi, conv0_phi, conv1_phi and
 * pres, pres_old over the p grid), from host arrays with the routine's
 * argument list (l = nx+1, m = ny+1, n = nz+1, by reference).  Values carry
 * 17 significant digits, so a load restores them bit for bit.  Returns
 * TPLS_ERR_IO when the file cannot be written. */
int tpls_write_backup(const double *u2, const double *v2, const double *w2,
                      const double *conv0_u, const double *conv1_u,
                      const double *conv0_v, const double *conv1_v,
                      const double *conv0_w, const double *conv1_w,
                      const double *pres_old, const double *pres,
                      const double *phi, const double *conv0_phi,
                      const double *conv1_phi, const int *l, const int *m,
                      const int *n, const char *filename);
/* io.F90:721-791 dataload_channel: reads that layout (any list-directed
 * number form: E or D exponents, r*value repeats); TPLS_ERR_IO when the file
 * is missing or short. */
int tpls_read_backup(double *u2, double *v2, double *w2, double *conv0_u,
                     double *conv1_u, double *conv0_v, double *conv1_v,
                     double *conv0_w, double *conv1_w, double *pres_old,
                     double *pres, double *phi, double *conv0_phi,
                     double *conv1_phi, const int *l, const int *m,
                     const int *n, const char *filename);
/* No counterpart in the reference, whose backup leaves out the AB3 history
 * of the surface-tension force: csf_u0, csf_u1 over the u grid, csf_v0,
 * csf_v1 over the v grid, csf_w0, csf_w1 over the w grid, in the same text
 * style.  With it a restart continues the run bit for bit. */
int tpls_write_backup_csf(const double *csf_u0, const double *csf_u1,
                          const double *csf_v0, const double *csf_v1,
                          const double *csf_w0, const double *csf_w1,
                          const int *l, const int *m, const int *n,
                          const char *filename);
int tpls_read_backup_csf(double *csf_u0, double *csf_u1, double *csf_v0,
                         double *csf_v1, double *csf_w0, double *csf_w1,
                         const int *l, const int *m, const int *n,
                         const char *filename);
/* The same files written from / read into a context's device state
 * (main_ns_hybrid.F90:2450-2468 writes fieldbackup0.dat / fieldbackup1.dat
 * alternately).  csf_filename may be NULL (the CSF histories are then not
 * written / left as they are).  The load reads both files completely before
 * it changes the device state. */
int tpls_backup_channel(tpls_ctx *ctx, const char *filename,
                        const char *csf_filename);
int tpls_dataload_channel(tpls_ctx *ctx, const char *filename,
                          const char *csf_filename);

/* mpi.f90:110  exchange2d on one rank = periodic-y ghost rows over the full
 * x span, for an array (0:nx+1,0:ny+1,sz:ez). */
int tpls_exchange2d(tpls_ctx *ctx, double *uu, const int *ex, const int *ey,
                    const int *ez, const int *sx, const int *sy,
                    const int *sz);

#ifdef __cplusplus
}
#endif
#endif /* TPLS_GPU_H */
