/*
 * tpls_oracle.h -- CPU restatement of the TPLS per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle: tests, the smoke
 * check and bench.py's CPU-baseline leg may call it; the product library
 * (tpls_gb300) never links or calls it.
 *
 * PARITY UNPINNED: the reference (Fortran 2003 + MPI + PETSc) cannot be
 * compiled here or on the GPU host (no Fortran compiler, MPI or PETSc), and
 * its own tests hold no golden vectors for this path.  Every routine below is
 * a line-by-line restatement of the cited reference source with sequential
 * (OMP_NUM_THREADS=1) loop order, and is pinned only by mathematical
 * known-answer tests (tests/test_oracle_kats.py).
 *
 * Layout: every array is the reference's explicit-shape, column-major array
 * for a single MPI rank (sx=1, ex=nx, sy=1, ey=ny, ex_max=nx, maxl=nx+1,
 * maxm=ny+1, maxn=nz+1):
 *   p-grid  (0:nx+1, 0:ny+1, 0:nz+1)   phi, pres, RHS_p, csf forces, viscosity
 *   u/v     (0:nx+1, 0:ny+1, 0:nz-1)
 *   w       (0:nx+1, 0:ny+1, 0:nz)
 *   viscosity_aug (-1:nx+2, -1:ny+2, 0:nz+1)
 *   phi_augaug    (-2:nx+3, -2:ny+3, 0:nz+1)
 */
#ifndef TPLS_ORACLE_H
#define TPLS_ORACLE_H

#include "../include/tpls_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

/* Sizes (elements) of the reference arrays for an nx*ny*nz channel. */
long orc_size_p(int nx, int ny, int nz);
long orc_size_uv(int nx, int ny, int nz);
long orc_size_w(int nx, int ny, int nz);
long orc_size_visc_aug(int nx, int ny, int nz);

/* ---- single routines (arrays in the reference layout above) ---- */
double orc_weno5(double v1, double v2, double v3, double v4, double v5);
void orc_do_advect_phi(int nx, int ny, int nz, const double *phi2, double *u2,
                       double *v2, double *w2, double *conv2_phi, double dx,
                       double dy, double dz);
void orc_get_levelset_status(int nx, int ny, int nz, const double *phi,
                             double *D, int *istatus, double *sgn, double h);
void orc_do_levelset_iteration(int nx, int ny, int nz, const double *phi,
                               double *phi_reinit, const double *D,
                               const int *istatus, const double *sgn, double h,
                               double height, double *err);
void orc_dim(int nx, int ny, int nz, double dx, double dy, double dz, double dt,
             double epn, double pe, const double *phi, const double *phi_old,
             const double *conv2_phi, double *conv_prev, double *phi_new,
             double height, int max_iteration_dim);
void orc_do_tpls(int nx, int ny, int nz, const double *phi2, double *phi3,
                 const double *c0, const double *c1, const double *c2,
                 int levelset, double height, double dx, double dz, double dt,
                 double *err2);
void orc_get_csf(int nx, int ny, int nz, double *fx, double *fy, double *fz,
                 const double *fi, double dx, double dy, double dz,
                 double scap, double smooth_width);
void orc_csf_faces(int nx, int ny, int nz, const double *fx, const double *fy,
                   const double *fz, double *csf_u, double *csf_v,
                   double *csf_w);
void orc_viscosity_aug(int nx, int ny, int nz, const double *phi2,
                       double *visc_aug, double smooth_width, double re,
                       double mu_minus, double mu_plus);
void orc_get_conv_all(int nx, int ny, int nz, double *cu, double *cv,
                      double *cw, const double *va, const double *u2,
                      const double *v2, const double *w2, double dx,
                      double dy, double dz);
void orc_get_diffusion_all(int nx, int ny, int nz, double *du, double *dv,
                           double *dw, const double *va, const double *u2,
                           const double *v2, const double *w2, double dx,
                           double dy, double dz);
void orc_do_jacobi(int comp, int nx, int ny, int nz, double *x3,
                   const double *x3_old, const double *rhs, const double *va,
                   double dx, double dy, double dz, double dt);
void orc_do_sor(int comp, int nx, int ny, int nz, double *x3,
                const double *rhs, const double *va, double dx, double dy,
                double dz, double dt, int flg, int iteration_time);
void orc_momentum(int comp, int nx, int ny, int nz, double *x3, double *x3_old,
                  const double *rhs, const double *va, const double *pres,
                  int max_iteration, double dx, double dy, double dz,
                  double dt, double *err);
void orc_get_source_pres(int nx, int ny, int nz, double *rhs, const double *u3,
                         const double *v3, const double *w3, double dx,
                         double dy, double dz, double dt);
void orc_get_uvw_pres(int nx, int ny, int nz, double *u3, double *v3,
                      double *w3, const double *p, double dx, double dy,
                      double dz, double dt, const double *u_inlet);
void orc_pressure_solve(int nx, int ny, int nz, double *pres,
                        const double *rhs_p, const double *u3,
                        const double *u_inlet, double dx, double dy,
                        double dz, double dt, double *rnorm);
void orc_exchange2d(int nx, int ny, int zlo, int zhi, double *a);
/* twophase_initialisation_wave.F90:79-122: base velocity u(z), nz values. */
void orc_base_profile(int nz, double dz, double reynolds, double dpdl,
                      double mu_minus, double mu_plus, double height,
                      double smooth_width, double *u_oned);

/* ---- whole-step driver (main_ns_hybrid.F90:583-918, 2480-2509) ---- */
orc_ctx *orc_create(int nx, int ny, int nz, const tpls_params *prm,
                    const double *u_inlet);
void orc_destroy(orc_ctx *c);
int orc_set_field(orc_ctx *c, int field, const double *host);
int orc_get_field(orc_ctx *c, int field, double *host);
void orc_step(orc_ctx *c, int nsteps);
void orc_get_stats(orc_ctx *c, tpls_stats *st);

#ifdef __cplusplus
}
#endif
#endif
