/*
 * tpls_oracle.c -- CPU restatement of the TPLS per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY (parity oracle and CPU baseline).  Not linked into
 * the product library.  PARITY UNPINNED: the Fortran reference cannot be
 * built here (no gfortran / MPI / PETSc) and ships no golden vectors for
 * this path; the oracle is pinned by mathematical known-answer tests.
 *
 * Every routine restates the cited reference routine for one MPI rank
 * (sx=1, ex=ex_max=nx, sy=1, ey=ny, maxl=nx+1, maxn=nz+1) with
 *   - the reference's sequential loop order (k outer, then j, then i), which
 *     is what the reference computes with OMP_NUM_THREADS=1;
 *   - the reference's literal precisions (single-precision epslon and pi);
 *   - the reference's left-to-right evaluation order (build with
 *     -ffp-contract=off so no FMA contraction happens);
 *   - NaN canaries in every scratch element the Fortran leaves undefined,
 *     so an accidental read of one shows up in the outputs.
 * On one rank every halo exchange of mpi.f90 reduces to a periodic copy of
 * y-ghost rows (x has MPI_PROC_NULL neighbours).
 *
 * Built with OpenMP for the CPU-baseline timing; loops marked parallel have
 * no loop-carried dependency in the sequential semantics (the odd SOR sweep
 * is parallel only within a k-plane), so results do not depend on the thread
 * count except for the order of the logged residual sums.
 */
#include "tpls_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#define OMP_FOR _Pragma("omp parallel for schedule(static)")
#else
#define OMP_FOR
#endif

/* Single-precision literals of the reference, widened to double exactly as
 * Fortran does for `double precision, parameter :: x = <real literal>`. */
#define WENO_EPS ((double)1.e-7f)          /* weno.f90:184 */
#define PI_SP ((double)3.1415926535f)      /* levelset.f90:388, momentum_allflux.f90:489 */
#define PI_MAIN ((double)3.14159265359f)   /* main_ns_hybrid.F90:181 */

/* Normal halo'd arrays: x 0..nx+1, y 0..ny+1, z from 0. */
#define IX(i, j, k) ((size_t)(i) + (size_t)NX2 * ((size_t)(j) + (size_t)NY2 * (size_t)(k)))
/* viscosity_aug: x -1..nx+2, y -1..ny+2, z 0..nz+1 */
#define IVA(i, j, k) ((size_t)((i) + 1) + (size_t)(NX2 + 2) * ((size_t)((j) + 1) + (size_t)(NY2 + 2) * (size_t)(k)))
/* phi_augaug: x -2..nx+3, y -2..ny+3, z 0..nz+1 */
#define IAA(i, j, k) ((size_t)((i) + 2) + (size_t)(NX2 + 4) * ((size_t)((j) + 2) + (size_t)(NY2 + 4) * (size_t)(k)))
#define DIMS const int NX2 = nx + 2, NY2 = ny + 2; (void)NX2; (void)NY2

long orc_size_p(int nx, int ny, int nz) { return (long)(nx + 2) * (ny + 2) * (nz + 2); }
long orc_size_uv(int nx, int ny, int nz) { return (long)(nx + 2) * (ny + 2) * nz; }
long orc_size_w(int nx, int ny, int nz) { return (long)(nx + 2) * (ny + 2) * (nz + 1); }
long orc_size_visc_aug(int nx, int ny, int nz) { return (long)(nx + 4) * (ny + 4) * (nz + 2); }

static double *alloc_nan(size_t n) {
  double *a = (double *)malloc(n * sizeof(double));
  for (size_t i = 0; i < n; i++) a[i] = NAN;
  return a;
}
static double *alloc_zero(size_t n) { return (double *)calloc(n, sizeof(double)); }

/* mpi.f90:110-170 exchange2d on one rank: rows 0 <- ny and ny+1 <- 1 over
 * x = 0..nx+1 for every z plane of the array. */
void orc_exchange2d(int nx, int ny, int zlo, int zhi, double *a) {
  DIMS;
  for (int k = 0; k <= zhi - zlo; k++)
    for (int i = 0; i <= nx + 1; i++) {
      a[IX(i, 0, k)] = a[IX(i, ny, k)];
      a[IX(i, ny + 1, k)] = a[IX(i, 1, k)];
    }
}

/* ------------------------------------------------------------------------
 * weno.f90:175-215  WENO5 (Jiang-Shu), evaluation order as written.
 * ---------------------------------------------------------------------- */
double orc_weno5(double v1, double v2, double v3, double v4, double v5) {
  double t1, t2, t3, s1, s2, s3, a1, a2, a3, w1, w2, w3;
  t1 = v1 - 2.0 * v2 + v3;
  t2 = v1 - 4.0 * v2 + 3.0 * v3;
  s1 = 13.0 / 12.0 * t1 * t1 + 0.25 * t2 * t2;
  t1 = v2 - 2.0 * v3 + v4;
  t2 = v2 - v4;
  s2 = 13.0 / 12.0 * t1 * t1 + 0.25 * t2 * t2;
  t1 = v3 - 2.0 * v4 + v5;
  t2 = 3.0 * v3 - 4.0 * v4 + v5;
  s3 = 13.0 / 12.0 * t1 * t1 + 0.25 * t2 * t2;
  a1 = 0.1 / ((WENO_EPS + s1) * (WENO_EPS + s1));
  a2 = 0.6 / ((WENO_EPS + s2) * (WENO_EPS + s2));
  a3 = 0.3 / ((WENO_EPS + s3) * (WENO_EPS + s3));
  w1 = a1 / (a1 + a2 + a3);
  w2 = a2 / (a1 + a2 + a3);
  w3 = a3 / (a1 + a2 + a3);
  t1 = v1 / 3.0 - 7.0 * v2 / 6.0 + 11.0 * v3 / 6.0;
  t2 = -v2 / 6.0 + 5.0 * v3 / 6.0 + v4 / 3.0;
  t3 = v3 / 3.0 + 5.0 * v4 / 6.0 - v5 / 6.0;
  return w1 * t1 + w2 * t2 + w3 * t3;
}

/* weno.f90:18-172 WENOAppoxConvection: l = maxl = nx+1, n = maxn = nz+1;
 * phi is the 3-ghost phi_augaug array. */
static void weno_approx_convection(int nx, int ny, int nz, const double *phi,
                                   const double *u, const double *v,
                                   const double *w, double *dfx, double *dfy,
                                   double *dfz) {
  DIMS;
  const int l = nx + 1, n = nz + 1;
  OMP_FOR
  for (int k = 0; k <= n - 2; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        if (i >= 3 && i <= l - 3) {
          double v1, v2, v3, v4, v5;
          if (u[IX(i, j, k)] >= 0.0) {
            v1 = phi[IAA(i - 2, j + 1, k + 1)];
            v2 = phi[IAA(i - 1, j + 1, k + 1)];
            v3 = phi[IAA(i, j + 1, k + 1)];
            v4 = phi[IAA(i + 1, j + 1, k + 1)];
            v5 = phi[IAA(i + 2, j + 1, k + 1)];
          } else {
            v1 = phi[IAA(i + 3, j + 1, k + 1)];
            v2 = phi[IAA(i + 2, j + 1, k + 1)];
            v3 = phi[IAA(i + 1, j + 1, k + 1)];
            v4 = phi[IAA(i, j + 1, k + 1)];
            v5 = phi[IAA(i - 1, j + 1, k + 1)];
          }
          dfx[IX(i, j, k)] = orc_weno5(v1, v2, v3, v4, v5);
        } else {
          dfx[IX(i, j, k)] = (u[IX(i, j, k)] >= 0.0) ? phi[IAA(i, j + 1, k + 1)]
                                                     : phi[IAA(i + 1, j + 1, k + 1)];
        }
      }
  /* weno.f90:86-100: the i=0 face (sx==1) */
  for (int k = 0; k <= n - 2; k++)
    for (int j = 1; j <= ny; j++)
      dfx[IX(0, j, k)] = (u[IX(0, j, k)] >= 0.0) ? phi[IAA(0, j + 1, k + 1)]
                                                 : phi[IAA(1, j + 1, k + 1)];
  OMP_FOR
  for (int k = 0; k <= n - 2; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        double v1, v2, v3, v4, v5;
        if (v[IX(i, j, k)] >= 0.0) {
          v1 = phi[IAA(i, j - 2, k + 1)];
          v2 = phi[IAA(i, j - 1, k + 1)];
          v3 = phi[IAA(i, j, k + 1)];
          v4 = phi[IAA(i, j + 1, k + 1)];
          v5 = phi[IAA(i, j + 2, k + 1)];
        } else {
          v1 = phi[IAA(i, j + 3, k + 1)];
          v2 = phi[IAA(i, j + 2, k + 1)];
          v3 = phi[IAA(i, j + 1, k + 1)];
          v4 = phi[IAA(i, j, k + 1)];
          v5 = phi[IAA(i, j - 1, k + 1)];
        }
        dfy[IX(i, j, k)] = orc_weno5(v1, v2, v3, v4, v5);
      }
  OMP_FOR
  for (int k = 0; k <= n - 1; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        if (k >= 3 && k <= n - 3) {
          double v1, v2, v3, v4, v5;
          if (w[IX(i, j, k)] >= 0.0) {
            v1 = phi[IAA(i, j + 1, k - 2)];
            v2 = phi[IAA(i, j + 1, k - 1)];
            v3 = phi[IAA(i, j + 1, k)];
            v4 = phi[IAA(i, j + 1, k + 1)];
            v5 = phi[IAA(i, j + 1, k + 2)];
          } else {
            v1 = phi[IAA(i, j + 1, k + 3)];
            v2 = phi[IAA(i, j + 1, k + 2)];
            v3 = phi[IAA(i, j + 1, k + 1)];
            v4 = phi[IAA(i, j + 1, k)];
            v5 = phi[IAA(i, j + 1, k - 1)];
          }
          dfz[IX(i, j, k)] = orc_weno5(v1, v2, v3, v4, v5);
        } else {
          dfz[IX(i, j, k)] = (phi[IAA(i, j + 1, k)] + phi[IAA(i, j + 1, k + 1)]) / 2.0;
        }
      }
}

/* advect_phi.f90:19-119 do_advect_phi.  u2, v2, w2 are inout: their y-ghost
 * rows are refreshed by the exchanges at :317-322. */
void orc_do_advect_phi(int nx, int ny, int nz, const double *phi2, double *u2,
                       double *v2, double *w2, double *conv2_phi, double dx,
                       double dy, double dz) {
  DIMS;
  const int zp = nz + 2;
  double *aa = alloc_nan((size_t)(nx + 6) * (ny + 6) * zp);
  /* :276-284 interior copy and the two x-boundary planes */
  for (int k = 0; k < zp; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 0; i <= nx + 1; i++) aa[IAA(i, j, k)] = phi2[IX(i, j, k)];
  /* :287-296 exchange2d_augaug1/2/3 (mpi.f90:415-662); augaug3 uses the
   * augaug2 datatype (configure_mpi_petsc.F90:326): x span -1..nx+2. */
  for (int k = 0; k < zp; k++) {
    for (int i = 0; i <= nx + 1; i++) {
      aa[IAA(i, 0, k)] = aa[IAA(i, ny, k)];
      aa[IAA(i, ny + 1, k)] = aa[IAA(i, 1, k)];
    }
    for (int i = -1; i <= nx + 2; i++) {
      aa[IAA(i, -1, k)] = aa[IAA(i, ny - 1, k)];
      aa[IAA(i, ny + 2, k)] = aa[IAA(i, 2, k)];
    }
    for (int i = -1; i <= nx + 2; i++) {
      aa[IAA(i, -2, k)] = aa[IAA(i, ny - 2, k)];
      aa[IAA(i, ny + 3, k)] = aa[IAA(i, 3, k)];
    }
  }
  double *dfx = alloc_nan((size_t)orc_size_uv(nx, ny, nz));
  double *dfy = alloc_nan((size_t)orc_size_uv(nx, ny, nz));
  double *dfz = alloc_nan((size_t)orc_size_w(nx, ny, nz));
  weno_approx_convection(nx, ny, nz, aa, u2, v2, w2, dfx, dfy, dfz);
  orc_exchange2d(nx, ny, 0, nz - 1, dfx);
  orc_exchange2d(nx, ny, 0, nz - 1, dfy);
  orc_exchange2d(nx, ny, 0, nz, dfz);
  orc_exchange2d(nx, ny, 0, nz - 1, u2);
  orc_exchange2d(nx, ny, 0, nz - 1, v2);
  orc_exchange2d(nx, ny, 0, nz, w2);
  memset(conv2_phi, 0, sizeof(double) * (size_t)orc_size_p(nx, ny, nz));
  OMP_FOR
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++)
        conv2_phi[IX(i, j, k)] =
            (u2[IX(i, j - 1, k - 1)] * dfx[IX(i, j - 1, k - 1)] -
             u2[IX(i - 1, j - 1, k - 1)] * dfx[IX(i - 1, j - 1, k - 1)]) / dx +
            (v2[IX(i, j, k - 1)] * dfy[IX(i, j, k - 1)] -
             v2[IX(i, j - 1, k - 1)] * dfy[IX(i, j - 1, k - 1)]) / dy +
            (w2[IX(i, j - 1, k)] * dfz[IX(i, j - 1, k)] -
             w2[IX(i, j - 1, k - 1)] * dfz[IX(i, j - 1, k - 1)]) / dz;
  free(aa);
  free(dfx);
  free(dfy);
  free(dfz);
}

/* ------------------------------------------------------------------------
 * levelset.f90:17-94 get_levelset_status (h = dx in the caller).
 * ---------------------------------------------------------------------- */
void orc_get_levelset_status(int nx, int ny, int nz, const double *phi,
                             double *D, int *istatus, double *sgn, double h) {
  DIMS;
  const size_t np = (size_t)orc_size_p(nx, ny, nz);
  memset(D, 0, np * sizeof(double));
  memset(istatus, 0, np * sizeof(int));
  memset(sgn, 0, np * sizeof(double));
  OMP_FOR
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        const size_t c = IX(i, j, k);
        const double p = phi[c];
        sgn[c] = (p < 0.0) ? -1.0 : ((p > 0.0) ? 1.0 : 0.0);
        double a1 = p * phi[IX(i + 1, j, k)], a2 = p * phi[IX(i - 1, j, k)];
        double a3 = p * phi[IX(i, j + 1, k)], a4 = p * phi[IX(i, j - 1, k)];
        double a5 = p * phi[IX(i, j, k + 1)], a6 = p * phi[IX(i, j, k - 1)];
        double mn = fmin(fmin(fmin(a1, a2), fmin(a3, a4)), fmin(a5, a6));
        istatus[c] = (mn <= 0.0) ? 1 : 0;
        if (istatus[c] == 1) {
          double gx = phi[IX(i + 1, j, k)] - phi[IX(i - 1, j, k)];
          double gy = phi[IX(i, j + 1, k)] - phi[IX(i, j - 1, k)];
          double gz = phi[IX(i, j, k + 1)] - phi[IX(i, j, k - 1)];
          double b1 = sqrt(gx * gx + gy * gy + gz * gz) / 2.0;
          double b2 = fabs(phi[IX(i + 1, j, k)] - p);
          double b3 = fabs(phi[IX(i - 1, j, k)] - p);
          double b4 = fabs(phi[IX(i, j + 1, k)] - p);
          double b5 = fabs(phi[IX(i, j - 1, k)] - p);
          double b6 = fabs(phi[IX(i, j, k + 1)] - p);
          double b7 = fabs(phi[IX(i, j, k - 1)] - p);
          double mx = fmax(fmax(fmax(b1, b2), fmax(b3, b4)), fmax(fmax(b5, b6), fmax(b7, h)));
          D[c] = h * p / mx;
        }
      }
}

/* levelset.f90:97-237 do_levelset_iteration (Russo-Smereka). *err receives
 * the sum of squared updates over k=0..n, j=1..ny, i=1..nx.  (The reference
 * accumulates this with `+` under an OpenMP MAX reduction, which makes its
 * logged value 0 when built with OpenMP; the sum is the evident intent.) */
void orc_do_levelset_iteration(int nx, int ny, int nz, const double *phi,
                               double *pr, const double *D,
                               const int *istatus, const double *sgn, double h,
                               double height, double *err) {
  DIMS;
  const int n = nz + 1;
  const size_t np = (size_t)orc_size_p(nx, ny, nz);
  double *up = alloc_nan(np);
  const double dtau = 0.3 * h;
  OMP_FOR
  for (int k = 1; k <= n - 1; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        const size_t c = IX(i, j, k);
        double dc;
        if (istatus[c] == 1) {
          dc = sgn[c] * fabs(pr[c]) - D[c];
        } else {
          dc = 0.0;
          if (phi[c] > 0.0) {
            double aP = fmax(pr[c] - pr[IX(i - 1, j, k)], 0.0);
            double bM = fmin(pr[IX(i + 1, j, k)] - pr[c], 0.0);
            double cP = fmax(pr[c] - pr[IX(i, j - 1, k)], 0.0);
            double dM = fmin(pr[IX(i, j + 1, k)] - pr[c], 0.0);
            double eP = fmax(pr[c] - pr[IX(i, j, k - 1)], 0.0);
            double fM = fmin(pr[IX(i, j, k + 1)] - pr[c], 0.0);
            dc = sgn[c] * (sqrt(fmax(aP * aP, bM * bM) + fmax(cP * cP, dM * dM) +
                                fmax(eP * eP, fM * fM)) - h);
          } else if (phi[c] < 0.0) {
            double bP = fmax(pr[IX(i + 1, j, k)] - pr[c], 0.0);
            double aM = fmin(pr[c] - pr[IX(i - 1, j, k)], 0.0);
            double dP = fmax(pr[IX(i, j + 1, k)] - pr[c], 0.0);
            double cM = fmin(pr[c] - pr[IX(i, j - 1, k)], 0.0);
            double fP = fmax(pr[IX(i, j, k + 1)] - pr[c], 0.0);
            double eM = fmin(pr[c] - pr[IX(i, j, k - 1)], 0.0);
            /* levelset.f90:274-275: x, then z, then y */
            dc = sgn[c] * (sqrt(fmax(bP * bP, aM * aM) + fmax(fP * fP, eM * eM) +
                                fmax(dP * dP, cM * cM)) - h);
          }
        }
        up[c] = pr[c] - dtau * dc / h;
      }
  /* :288-311 inlet plane uses dz = h (= dx) */
  const double dzh = h;
  for (int k = 1; k <= n - 1; k++)
    for (int j = 1; j <= ny; j++) {
      double z = k * dzh - 0.5 * dzh;
      up[IX(0, j, k)] = z - height;
    }
  for (int k = 1; k <= n - 1; k++)
    for (int j = 1; j <= ny; j++) up[IX(nx + 1, j, k)] = up[IX(nx, j, k)];
  /* :313-336 linear extrapolation of the z ghost planes, x = 0..nx+1 */
  for (int j = 1; j <= ny; j++)
    for (int i = 0; i <= nx + 1; i++) {
      up[IX(i, j, 0)] = 2.0 * up[IX(i, j, 1)] - up[IX(i, j, 2)];
      up[IX(i, j, n)] = 2.0 * up[IX(i, j, n - 1)] - up[IX(i, j, n - 2)];
    }
  double e = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : e)
  for (int k = 0; k <= n; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        double d = pr[IX(i, j, k)] - up[IX(i, j, k)];
        e += d * d;
      }
  *err = e;
  memcpy(pr, up, np * sizeof(double)); /* phi_reinit = phi_reinit_updated (y-ghost rows undefined) */
  free(up);
}

/* two_phase_levelset.f90:20-118 do_tpls.  phi2 is read only. */
void orc_do_tpls(int nx, int ny, int nz, const double *phi2, double *phi3,
                 const double *c0, const double *c1, const double *c2,
                 int levelset, double height, double dx, double dz, double dt,
                 double *err2) {
  DIMS;
  const int maxn = nz + 1;
  const size_t np = (size_t)orc_size_p(nx, ny, nz);
  double *rhs = alloc_nan(np);
  for (size_t c = 0; c < np; c++)
    rhs[c] = (23.0 / 12.0) * c2[c] - (4.0 / 3.0) * c1[c] + (5.0 / 12.0) * c0[c];
  orc_exchange2d(nx, ny, 0, nz + 1, rhs);
  for (int k = 1; k <= maxn - 1; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++)
        phi3[IX(i, j, k)] = phi2[IX(i, j, k)] - dt * rhs[IX(i, j, k)];
  for (int k = 1; k <= maxn - 1; k++) {
    double z_val = k * dz - 0.5 * dz;
    for (int j = 1; j <= ny; j++) phi3[IX(0, j, k)] = z_val - height;
  }
  for (int k = 1; k <= maxn - 1; k++)
    for (int j = 1; j <= ny; j++) phi3[IX(nx + 1, j, k)] = phi3[IX(nx, j, k)];
  for (int j = 1; j <= ny; j++)
    for (int i = 0; i <= nx + 1; i++) {
      phi3[IX(i, j, 0)] = 2.0 * phi3[IX(i, j, 1)] - phi3[IX(i, j, 2)];
      phi3[IX(i, j, maxn)] = 2.0 * phi3[IX(i, j, maxn - 1)] - phi3[IX(i, j, maxn - 2)];
    }
  orc_exchange2d(nx, ny, 0, nz + 1, phi3);
  double *D = alloc_zero(np), *sgn = alloc_zero(np);
  int *ist = (int *)calloc(np, sizeof(int));
  orc_get_levelset_status(nx, ny, nz, phi3, D, ist, sgn, dx);
  double *pr = (double *)malloc(np * sizeof(double));
  memcpy(pr, phi3, np * sizeof(double));
  double e = 0.0;
  for (int it = 1; it <= levelset; it++) {
    orc_exchange2d(nx, ny, 0, nz + 1, pr);
    orc_do_levelset_iteration(nx, ny, nz, phi3, pr, D, ist, sgn, dx, height, &e);
  }
  memcpy(phi3, pr, np * sizeof(double));
  *err2 = e;
  free(rhs);
  free(D);
  free(sgn);
  free(ist);
  free(pr);
}

/* ------------------------------------------------------------------------
 * levelset.f90:241-414 get_csf (fx, fy, fz are inout: only the entries the
 * reference assigns are written; the y-ghost rows are left as they were).
 * ---------------------------------------------------------------------- */
void orc_get_csf(int nx, int ny, int nz, double *fx, double *fy, double *fz,
                 const double *fi, double dx, double dy, double dz,
                 double scap, double smooth_width) {
  DIMS;
  const int n = nz + 1;
  const double max_kappa = 1.0 / fmin(fmin(dx, dy), dz);
  double *curv = alloc_nan((size_t)orc_size_p(nx, ny, nz));
  OMP_FOR
  for (int k = 1; k <= n - 1; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        const double f = fi[IX(i, j, k)];
        double d2x = (fi[IX(i + 1, j, k)] - 2.0 * f + fi[IX(i - 1, j, k)]) / (dx * dx);
        double d2y = (fi[IX(i, j + 1, k)] - 2.0 * f + fi[IX(i, j - 1, k)]) / (dy * dy);
        double d2z = (fi[IX(i, j, k + 1)] - 2.0 * f + fi[IX(i, j, k - 1)]) / (dz * dz);
        double gx = (fi[IX(i + 1, j, k)] - fi[IX(i - 1, j, k)]) / (2.0 * dx);
        double gy = (fi[IX(i, j + 1, k)] - fi[IX(i, j - 1, k)]) / (2.0 * dy);
        double gz = (fi[IX(i, j, k + 1)] - fi[IX(i, j, k - 1)]) / (2.0 * dz);
        double gx_up = (fi[IX(i + 1, j, k + 1)] - fi[IX(i - 1, j, k + 1)]) / (2.0 * dx);
        double gx_dn = (fi[IX(i + 1, j, k - 1)] - fi[IX(i - 1, j, k - 1)]) / (2.0 * dx);
        double d2xz = (gx_up - gx_dn) / (2.0 * dz);
        double gy_up = (fi[IX(i, j + 1, k + 1)] - fi[IX(i, j - 1, k + 1)]) / (2.0 * dy);
        double gy_dn = (fi[IX(i, j + 1, k - 1)] - fi[IX(i, j - 1, k - 1)]) / (2.0 * dy);
        double d2yz = (gy_up - gy_dn) / (2.0 * dz);
        double gx_out = (fi[IX(i + 1, j + 1, k)] - fi[IX(i - 1, j + 1, k)]) / (2.0 * dx);
        double gx_in = (fi[IX(i + 1, j - 1, k)] - fi[IX(i - 1, j - 1, k)]) / (2.0 * dx);
        double d2xy = (gx_out - gx_in) / (2.0 * dy);
        double nrm = gx * gx + gy * gy + gz * gz;
        double kap;
        if (nrm < 1e-10) {
          kap = 0.0;
        } else {
          double term1 = (d2x + d2y + d2z) / pow(nrm, 0.5);
          double term2 = gx * gx * d2x + gy * gy * d2y + gz * gz * d2z;
          double term3 = gx * gy * d2xy + gx * gz * d2xz + gy * gz * d2yz;
          term2 = term2 / pow(nrm, 1.5);
          term3 = 2.0 * term3 / pow(nrm, 1.5);
          kap = -(term1 - term2 - term3);
        }
        if (kap > max_kappa) kap = max_kappa;
        curv[IX(i, j, k)] = kap;
      }
  OMP_FOR
  for (int k = 1; k <= n - 1; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        double gx = (fi[IX(i + 1, j, k)] - fi[IX(i - 1, j, k)]) / (2.0 * dx);
        double gy = (fi[IX(i, j + 1, k)] - fi[IX(i, j - 1, k)]) / (2.0 * dy);
        double gz = (fi[IX(i, j, k + 1)] - fi[IX(i, j, k - 1)]) / (2.0 * dz);
        double p = fi[IX(i, j, k)], dirac;
        if (p < -smooth_width)
          dirac = 0.0;
        else if (p > smooth_width)
          dirac = 0.0;
        else
          dirac = (1.0 / (2.0 * smooth_width)) +
                  (1.0 / (2.0 * smooth_width)) * cos(PI_SP * p / smooth_width);
        double kap = curv[IX(i, j, k)];
        fx[IX(i, j, k)] = dirac * scap * kap * gx;
        fy[IX(i, j, k)] = dirac * scap * kap * gy;
        fz[IX(i, j, k)] = dirac * scap * kap * gz;
      }
  double *f3[3] = {fx, fy, fz};
  for (int q = 0; q < 3; q++) {
    double *f = f3[q];
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        f[IX(i, j, 0)] = 2.0 * f[IX(i, j, 1)] - f[IX(i, j, 2)];
        f[IX(i, j, n)] = 2.0 * f[IX(i, j, n - 1)] - f[IX(i, j, n - 2)];
      }
  }
  for (int q = 0; q < 3; q++) {
    double *f = f3[q];
    for (int k = 0; k <= n; k++)
      for (int j = 1; j <= ny; j++) {
        f[IX(0, j, k)] = 2.0 * f[IX(1, j, k)] - f[IX(2, j, k)];
        f[IX(nx + 1, j, k)] = 2.0 * f[IX(nx, j, k)] - f[IX(nx - 1, j, k)];
      }
  }
  free(curv);
}

/* main_ns_hybrid.F90:629-641: CSF forces averaged onto the u, v, w faces
 * (interior i, j only; the ghost entries of csf_* are left untouched). */
void orc_csf_faces(int nx, int ny, int nz, const double *fx, const double *fy,
                   const double *fz, double *csf_u, double *csf_v,
                   double *csf_w) {
  DIMS;
  for (int k = 0; k <= nz - 1; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++)
        csf_u[IX(i, j, k)] = (fx[IX(i + 1, j + 1, k + 1)] + fx[IX(i, j + 1, k + 1)]) / 2.0;
  for (int k = 0; k <= nz - 1; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++)
        csf_v[IX(i, j, k)] = (fy[IX(i, j + 1, k + 1)] + fy[IX(i, j, k + 1)]) / 2.0;
  for (int k = 0; k <= nz; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++)
        csf_w[IX(i, j, k)] = (fz[IX(i, j + 1, k + 1)] + fz[IX(i, j + 1, k)]) / 2.0;
}

/* ------------------------------------------------------------------------
 * cahn_hilliard_solver.f90:41-382 dim: the diffuse-interface (Cahn-Hilliard)
 * update on one rank (sx=1, ex=nx, sy=1, ey=ny, maxl=nx+1, maxn=nz+1).
 * phi, phi_old: concentration C (p-grid); phi_new: starting guess in,
 * C^{n+1} out; conv_prev: ConvPrevPhi, updated.  bulkE0, d2phi and source0
 * are the routine's automatic arrays (NaN canaries where it leaves them
 * undefined).  The routine's max-norm residual is never used by the
 * reference and is not computed.
 * ---------------------------------------------------------------------- */
static double dim_mob(double c1) { /* dsqrt(c1*c1*(1-|c1|)*(1-|c1|)) */
  return sqrt(c1 * c1 * (1.0 - fabs(c1)) * (1.0 - fabs(c1)));
}

void orc_dim(int nx, int ny, int nz, double dx, double dy, double dz, double dt,
             double epn, double pe, const double *phi, const double *phi_old,
             const double *conv2_phi, double *conv_prev, double *phi_new,
             double height, int max_iteration_dim) {
  DIMS;
  const int maxl = nx + 1, maxn = nz + 1;
  const size_t np = (size_t)orc_size_p(nx, ny, nz);
  const double nmda = 0.25, tao = 0.25, alfa1 = 1.1;
  double *bulk = alloc_nan(np), *d2 = alloc_nan(np), *src = alloc_nan(np);
  const double epn2 = epn * epn;
  /* :110-125 */
  for (int k = 1; k <= maxn - 1; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        const double p = phi[IX(i, j, k)];
        bulk[IX(i, j, k)] = (1.0 - 3.0 * p + 2.0 * p * p) * p / 2.0;
        d2[IX(i, j, k)] = (phi[IX(i + 1, j, k)] - 2.0 * p + phi[IX(i - 1, j, k)]) / dx / dx +
                          (phi[IX(i, j + 1, k)] - 2.0 * p + phi[IX(i, j - 1, k)]) / dy / dy +
                          (phi[IX(i, j, k + 1)] - 2.0 * p + phi[IX(i, j, k - 1)]) / dz / dz;
      }
  /* :128-137 z ghost planes, :140-143 exchange, :146-172 x ghost planes */
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      bulk[IX(i, j, 0)] = bulk[IX(i, j, 1)];
      bulk[IX(i, j, maxn)] = bulk[IX(i, j, maxn - 1)];
      d2[IX(i, j, 0)] = d2[IX(i, j, 1)];
      d2[IX(i, j, maxn)] = d2[IX(i, j, maxn - 1)];
    }
  orc_exchange2d(nx, ny, 0, nz + 1, bulk);
  orc_exchange2d(nx, ny, 0, nz + 1, d2);
  for (int k = 1; k <= maxn - 1; k++)
    for (int j = 1; j <= ny; j++) {
      d2[IX(0, j, k)] = d2[IX(1, j, k)];
      bulk[IX(0, j, k)] = bulk[IX(1, j, k)];
      d2[IX(maxl, j, k)] = d2[IX(maxl - 1, j, k)];
      bulk[IX(maxl, j, k)] = bulk[IX(maxl - 1, j, k)];
    }
  /* :174-233 source term and ConvPrevPhi */
  for (int k = 1; k <= maxn - 1; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        const double p = phi[IX(i, j, k)];
        const double a1 = dim_mob((phi[IX(i - 1, j, k)] + p) / 2.0);
        const double a2 = dim_mob((phi[IX(i + 1, j, k)] + p) / 2.0);
        const double a3 = dim_mob((phi[IX(i, j - 1, k)] + p) / 2.0);
        const double a4 = dim_mob((phi[IX(i, j + 1, k)] + p) / 2.0);
        const double a5 = dim_mob((k + 1 == 2) ? p : (phi[IX(i, j, k - 1)] + p) / 2.0);
        const double a6 = dim_mob((phi[IX(i, j, k + 1)] + p) / 2.0);
        const double bc = bulk[IX(i, j, k)], lc = d2[IX(i, j, k)];
        const double temp1 =
            (a2 * (bulk[IX(i + 1, j, k)] - bc) - a1 * (bc - bulk[IX(i - 1, j, k)])) / dx / dx +
            (a4 * (bulk[IX(i, j + 1, k)] - bc) - a3 * (bc - bulk[IX(i, j - 1, k)])) / dy / dy +
            (a6 * (bulk[IX(i, j, k + 1)] - bc) - a5 * (bc - bulk[IX(i, j, k - 1)])) / dz / dz;
        const double temp2 = (d2[IX(i + 1, j, k)] - 2.0 * lc + d2[IX(i - 1, j, k)]) / dx / dx +
                             (d2[IX(i, j + 1, k)] - 2.0 * lc + d2[IX(i, j - 1, k)]) / dy / dy +
                             (d2[IX(i, j, k + 1)] - 2.0 * lc + d2[IX(i, j, k - 1)]) / dz / dz;
        const double temp3 =
            (a2 * (d2[IX(i + 1, j, k)] - lc) - a1 * (lc - d2[IX(i - 1, j, k)])) / dx / dx +
            (a4 * (d2[IX(i, j + 1, k)] - lc) - a3 * (lc - d2[IX(i, j - 1, k)])) / dy / dy +
            (a6 * (d2[IX(i, j, k + 1)] - lc) - a5 * (lc - d2[IX(i, j, k - 1)])) / dz / dz;
        const double temp4 = (temp1 - epn2 * temp3) / epn - nmda * tao / 2.0 * lc + epn2 * nmda / 2.0 * temp2;
        const double temp5 = temp4 / pe - conv2_phi[IX(i, j, k)];
        src[IX(i, j, k)] = temp5 * 2.0 - conv_prev[IX(i, j, k)];
        conv_prev[IX(i, j, k)] = temp5;
      }
  /* :236-238 (dx**2.d0 folds to dx*dx; dx**4.d0 is a pow) */
  const double a1 = 1.0 / (dx * dx) + 1.0 / (dy * dy) + 1.0 / (dz * dz);
  const double a2 = 2.0 / pow(dx, 4.0) + 2.0 / pow(dy, 4.0) + 2.0 / pow(dz, 4.0);
  const double diagonal = 1.5 + nmda / 2.0 / pe * dt * (2.0 * tao * a1 + epn2 * (4.0 * a1 * a1 + a2));
  /* :241-366 SOR */
  for (int it = 1; it <= max_iteration_dim; it++) {
    for (int k = 1; k <= maxn - 1; k++)
      for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
          const double p = phi_new[IX(i, j, k)];
          d2[IX(i, j, k)] = (phi_new[IX(i + 1, j, k)] - 2.0 * p + phi_new[IX(i - 1, j, k)]) / dx / dx +
                            (phi_new[IX(i, j + 1, k)] - 2.0 * p + phi_new[IX(i, j - 1, k)]) / dy / dy +
                            (phi_new[IX(i, j, k + 1)] - 2.0 * p + phi_new[IX(i, j, k - 1)]) / dz / dz;
        }
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        d2[IX(i, j, 0)] = d2[IX(i, j, 1)];
        d2[IX(i, j, maxn)] = d2[IX(i, j, maxn - 1)];
      }
    orc_exchange2d(nx, ny, 0, nz + 1, d2);
    for (int k = 1; k <= maxn - 1; k++)
      for (int j = 1; j <= ny; j++) {
        d2[IX(0, j, k)] = d2[IX(1, j, k)];
        d2[IX(maxl, j, k)] = d2[IX(maxl - 1, j, k)];
      }
    for (int k = 1; k <= maxn - 1; k++)
      for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
          const double l = d2[IX(i, j, k)];
          bulk[IX(i, j, k)] = (d2[IX(i + 1, j, k)] - 2.0 * l + d2[IX(i - 1, j, k)]) / dx / dx +
                              (d2[IX(i, j + 1, k)] - 2.0 * l + d2[IX(i, j - 1, k)]) / dy / dy +
                              (d2[IX(i, j, k + 1)] - 2.0 * l + d2[IX(i, j, k - 1)]) / dz / dz;
        }
    for (int k = 1; k <= maxn - 1; k++)
      for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
          const size_t c = IX(i, j, k);
          const double some = 2.0 * phi[c] - 0.5 * phi_old[c] - 1.5 * phi_new[c] + dt * src[c] +
                              dt * nmda / 2.0 / pe * (tao * d2[c] - epn2 * bulk[c]);
          double v = phi_new[c] + alfa1 * some / diagonal;
          if (v < 0.0) v = 0.0;
          if (v > 1.0) v = 1.0;
          phi_new[c] = v;
        }
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        phi_new[IX(i, j, 0)] = phi_new[IX(i, j, 1)];
        phi_new[IX(i, j, maxn)] = phi_new[IX(i, j, maxn - 1)];
      }
    orc_exchange2d(nx, ny, 0, nz + 1, phi_new);
    for (int k = 1; k <= maxn - 1; k++)
      for (int j = 1; j <= ny; j++) {
        const double z_val = k * dz - 0.5 * dz;
        phi_new[IX(0, j, k)] = 0.5 + 0.5 * tanh((z_val - height) / (2.0 * sqrt(2.0) * epn));
        phi_new[IX(maxl, j, k)] = phi_new[IX(maxl - 1, j, k)];
      }
  }
  free(bulk);
  free(d2);
  free(src);
}

/* ------------------------------------------------------------------------
 * momentum_allflux.f90:474-521 get_viscosity over i=1..nx, plus
 * main_ns_hybrid.F90:651-718: viscosity2_aug interior copy, the x ghost
 * planes from phi2(0,:,:) and phi2(nx+1,:,:), exchange2d_aug1 (rows 0, ny+1)
 * and exchange2d_aug2 (rows -1, ny+2), both over x = 0..nx+1.  x = -1 and
 * nx+2 stay undefined (NaN).
 * ---------------------------------------------------------------------- */
static double heaviside_visc(double phi_val, double sw, double re,
                             double mu_minus, double mu_plus, double pi) {
  double hv;
  if (phi_val < -sw)
    hv = 0.0;
  else if (phi_val > sw)
    hv = 1.0;
  else
    hv = 0.5 + (phi_val / (2.0 * sw)) + (1.0 / (2.0 * pi)) * sin(pi * phi_val / sw);
  double temp = mu_plus * hv + mu_minus * (1.0 - hv);
  return temp / re;
}

void orc_viscosity_aug(int nx, int ny, int nz, const double *phi2,
                       double *va, double sw, double re, double mu_minus,
                       double mu_plus) {
  DIMS;
  const size_t na = (size_t)orc_size_visc_aug(nx, ny, nz);
  for (size_t c = 0; c < na; c++) va[c] = NAN;
  OMP_FOR
  for (int k = 0; k <= nz + 1; k++)
    for (int j = 1; j <= ny; j++) {
      for (int i = 1; i <= nx; i++)
        va[IVA(i, j, k)] = heaviside_visc(phi2[IX(i, j, k)], sw, re, mu_minus, mu_plus, PI_SP);
      va[IVA(0, j, k)] = heaviside_visc(phi2[IX(0, j, k)], sw, re, mu_minus, mu_plus, PI_MAIN);
      va[IVA(nx + 1, j, k)] =
          heaviside_visc(phi2[IX(nx + 1, j, k)], sw, re, mu_minus, mu_plus, PI_MAIN);
    }
  for (int k = 0; k <= nz + 1; k++) {
    for (int i = 0; i <= nx + 1; i++) {
      va[IVA(i, 0, k)] = va[IVA(i, ny, k)];
      va[IVA(i, ny + 1, k)] = va[IVA(i, 1, k)];
    }
    for (int i = 0; i <= nx + 1; i++) {
      va[IVA(i, -1, k)] = va[IVA(i, ny - 1, k)];
      va[IVA(i, ny + 2, k)] = va[IVA(i, 2, k)];
    }
  }
}

/* ------------------------------------------------------------------------
 * momentum_allflux.f90:224-471 get_conv_all
 * ---------------------------------------------------------------------- */
void orc_get_conv_all(int nx, int ny, int nz, double *cu, double *cv,
                      double *cw, const double *va, const double *u,
                      const double *v, const double *w, double dx, double dy,
                      double dz) {
  DIMS;
  const int maxn = nz + 1, ex_loc = nx - 1;
  memset(cu, 0, sizeof(double) * (size_t)orc_size_uv(nx, ny, nz));
  OMP_FOR
  for (int k = 0; k <= maxn - 2; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= ex_loc; i++) {
        double tempv = (v[IX(i, j, k)] + v[IX(i + 1, j, k)] + v[IX(i, j + 1, k)] + v[IX(i + 1, j + 1, k)]) / 4.0;
        double tempw = (w[IX(i, j, k)] + w[IX(i + 1, j, k)] + w[IX(i, j, k + 1)] + w[IX(i + 1, j, k + 1)]) / 4.0;
        double dudx = 0.5 * (u[IX(i + 1, j, k)] - u[IX(i - 1, j, k)]) / dx;
        double Xc = dudx * u[IX(i, j, k)];
        double ub = u[IX(i, j + 1, k)], vb = u[IX(i, j - 1, k)];
        double dudy = 0.5 * (ub - vb) / dy;
        double Yc = dudy * tempv, dudz;
        if (k == 0)
          dudz = (u[IX(i, j, k)] + u[IX(i, j, k + 1)]) / (2.0 * dz);
        else if (k == maxn - 2)
          dudz = -(u[IX(i, j, k)] + u[IX(i, j, k - 1)]) / (2.0 * dz);
        else
          dudz = 0.5 * (u[IX(i, j, k + 1)] - u[IX(i, j, k - 1)]) / dz;
        double Zc = dudz * tempw;
        double t1 = Xc + Yc + Zc;
        double mpx = va[IVA(i + 1, j + 1, k + 1)], mmx = va[IVA(i, j + 1, k + 1)];
        double mpy = (va[IVA(i + 1, j + 2, k + 1)] + va[IVA(i, j + 2, k + 1)] + va[IVA(i + 1, j + 1, k + 1)] + va[IVA(i, j + 1, k + 1)]) / 4.0;
        double mmy = (va[IVA(i + 1, j, k + 1)] + va[IVA(i, j, k + 1)] + va[IVA(i + 1, j + 1, k + 1)] + va[IVA(i, j + 1, k + 1)]) / 4.0;
        double mpz = (va[IVA(i + 1, j + 1, k + 2)] + va[IVA(i, j + 1, k + 2)] + va[IVA(i + 1, j + 1, k + 1)] + va[IVA(i, j + 1, k + 1)]) / 4.0;
        double mmz = (va[IVA(i + 1, j + 1, k)] + va[IVA(i, j + 1, k)] + va[IVA(i + 1, j + 1, k + 1)] + va[IVA(i, j + 1, k + 1)]) / 4.0;
        double E = mpx * (u[IX(i + 1, j, k)] - u[IX(i, j, k)]) / dx;
        double W = mmx * (u[IX(i, j, k)] - u[IX(i - 1, j, k)]) / dx;
        double N = mpy * (v[IX(i + 1, j + 1, k)] - v[IX(i, j + 1, k)]) / dx;
        double S = mmy * (v[IX(i + 1, j, k)] - v[IX(i, j, k)]) / dx;
        double O = mpz * (w[IX(i + 1, j, k + 1)] - w[IX(i, j, k + 1)]) / dx;
        double I = mmz * (w[IX(i + 1, j, k)] - w[IX(i, j, k)]) / dx;
        double t2 = ((E - W) / dx) + ((N - S) / dy) + ((O - I) / dz);
        cu[IX(i, j, k)] = t1 - t2;
      }
  memset(cv, 0, sizeof(double) * (size_t)orc_size_uv(nx, ny, nz));
  OMP_FOR
  for (int k = 0; k <= maxn - 2; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        double tempu = (u[IX(i - 1, j - 1, k)] + u[IX(i - 1, j, k)] + u[IX(i, j - 1, k)] + u[IX(i, j, k)]) / 4.0;
        double tempw = (w[IX(i, j - 1, k)] + w[IX(i, j, k)] + w[IX(i, j - 1, k + 1)] + w[IX(i, j, k + 1)]) / 4.0;
        double dvdy = 0.5 * (v[IX(i, j + 1, k)] - v[IX(i, j - 1, k)]) / dy;
        double Yc = dvdy * v[IX(i, j, k)];
        double vmx = v[IX(i - 1, j, k)], vpx = v[IX(i + 1, j, k)];
        double dvdx = 0.5 * (vpx - vmx) / dx;
        double Xc = dvdx * tempu, dvdz;
        if (k == 0)
          dvdz = (v[IX(i, j, k)] + v[IX(i, j, k + 1)]) / (2.0 * dz);
        else if (k == maxn - 2)
          dvdz = -(v[IX(i, j, k)] + v[IX(i, j, k - 1)]) / (2.0 * dz);
        else
          dvdz = 0.5 * (v[IX(i, j, k + 1)] - v[IX(i, j, k - 1)]) / dz;
        double Zc = dvdz * tempw;
        double t1 = Xc + Yc + Zc;
        double mpx = (va[IVA(i + 1, j + 1, k + 1)] + va[IVA(i + 1, j, k + 1)] + va[IVA(i, j + 1, k + 1)] + va[IVA(i, j, k + 1)]) / 4.0;
        double mmx = (va[IVA(i - 1, j + 1, k + 1)] + va[IVA(i - 1, j, k + 1)] + va[IVA(i, j + 1, k + 1)] + va[IVA(i, j, k + 1)]) / 4.0;
        double mpy = va[IVA(i, j + 1, k + 1)], mmy = va[IVA(i, j, k + 1)];
        double mpz = (va[IVA(i, j + 1, k + 2)] + va[IVA(i, j, k + 2)] + va[IVA(i, j + 1, k + 1)] + va[IVA(i, j, k + 1)]) / 4.0;
        double mmz = (va[IVA(i, j + 1, k)] + va[IVA(i, j, k)] + va[IVA(i, j + 1, k + 1)] + va[IVA(i, j, k + 1)]) / 4.0;
        double E = mpx * (u[IX(i, j, k)] - u[IX(i, j - 1, k)]) / dy;
        double W = mmx * (u[IX(i - 1, j, k)] - u[IX(i - 1, j - 1, k)]) / dy;
        double N = mpy * (v[IX(i, j + 1, k)] - v[IX(i, j, k)]) / dy;
        double S = mmy * (v[IX(i, j, k)] - v[IX(i, j - 1, k)]) / dy;
        double O = mpz * (w[IX(i, j, k + 1)] - w[IX(i, j - 1, k + 1)]) / dy;
        double I = mmz * (w[IX(i, j, k)] - w[IX(i, j - 1, k)]) / dy;
        double t2 = ((E - W) / dx) + ((N - S) / dy) + ((O - I) / dz);
        cv[IX(i, j, k)] = t1 - t2;
      }
  memset(cw, 0, sizeof(double) * (size_t)orc_size_w(nx, ny, nz));
  OMP_FOR
  for (int k = 1; k <= maxn - 2; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        double tempu = (u[IX(i - 1, j, k - 1)] + u[IX(i - 1, j, k)] + u[IX(i, j, k - 1)] + u[IX(i, j, k)]) / 4.0;
        double tempv = (v[IX(i, j, k - 1)] + v[IX(i, j, k)] + v[IX(i, j + 1, k - 1)] + v[IX(i, j + 1, k)]) / 4.0;
        double ub = w[IX(i, j, k + 1)], vb = w[IX(i, j, k - 1)];
        double dwdz = 0.5 * (ub - vb) / dz;
        double Zc = dwdz * w[IX(i, j, k)];
        double wmx = w[IX(i - 1, j, k)], wpx = w[IX(i + 1, j, k)];
        double dwdx = 0.5 * (wpx - wmx) / dx;
        double Xc = dwdx * tempu;
        ub = w[IX(i, j + 1, k)];
        vb = w[IX(i, j - 1, k)];
        double dwdy = 0.5 * (ub - vb) / dy;
        double Yc = dwdy * tempv;
        double t1 = Xc + Yc + Zc;
        double mpx = (va[IVA(i + 1, j + 1, k + 1)] + va[IVA(i + 1, j + 1, k)] + va[IVA(i, j + 1, k + 1)] + va[IVA(i, j + 1, k)]) / 4.0;
        double mmx = (va[IVA(i - 1, j + 1, k + 1)] + va[IVA(i - 1, j + 1, k)] + va[IVA(i, j + 1, k + 1)] + va[IVA(i, j + 1, k)]) / 4.0;
        double mpy = (va[IVA(i, j + 2, k + 1)] + va[IVA(i, j + 2, k)] + va[IVA(i, j + 1, k + 1)] + va[IVA(i, j + 1, k)]) / 4.0;
        double mmy = (va[IVA(i, j, k + 1)] + va[IVA(i, j, k)] + va[IVA(i, j + 1, k + 1)] + va[IVA(i, j + 1, k)]) / 4.0;
        double mpz = va[IVA(i, j + 1, k + 1)], mmz = va[IVA(i, j + 1, k)];
        double E = mpx * (u[IX(i, j, k)] - u[IX(i, j, k - 1)]) / dz;
        double W = mmx * (u[IX(i - 1, j, k)] - u[IX(i - 1, j, k - 1)]) / dz;
        double N = mpy * (v[IX(i, j + 1, k)] - v[IX(i, j + 1, k - 1)]) / dz;
        double S = mmy * (v[IX(i, j, k)] - v[IX(i, j, k - 1)]) / dz;
        double O = mpz * (w[IX(i, j, k + 1)] - w[IX(i, j, k)]) / dz;
        double I = mmz * (w[IX(i, j, k)] - w[IX(i, j, k - 1)]) / dz;
        double t2 = ((E - W) / dx) + ((N - S) / dy) + ((O - I) / dz);
        cw[IX(i, j, k)] = t1 - t2;
      }
}

/* ------------------------------------------------------------------------
 * Face viscosities shared by get_diffusion_all, do_jacobi_* and do_sor_*
 * (momentum_allflux.f90:91-98,145-152,187-194; jacobi/sor identical forms).
 * ---------------------------------------------------------------------- */
typedef struct { double px, mx, py, my, pz, mz; } faces_t;

static inline faces_t faces_u(const double *va, int nx, int ny, int i, int j, int k) {
  DIMS;
  faces_t f;
  f.px = va[IVA(i + 1, j + 1, k + 1)];
  f.mx = va[IVA(i, j + 1, k + 1)];
  f.py = (va[IVA(i, j + 1, k + 1)] + va[IVA(i + 1, j + 1, k + 1)] + va[IVA(i, j + 2, k + 1)] + va[IVA(i + 1, j + 2, k + 1)]) / 4.0;
  f.my = (va[IVA(i, j + 1, k + 1)] + va[IVA(i + 1, j + 1, k + 1)] + va[IVA(i, j, k + 1)] + va[IVA(i + 1, j, k + 1)]) / 4.0;
  f.pz = (va[IVA(i, j + 1, k + 1)] + va[IVA(i + 1, j + 1, k + 1)] + va[IVA(i, j + 1, k + 2)] + va[IVA(i + 1, j + 1, k + 2)]) / 4.0;
  f.mz = (va[IVA(i, j + 1, k + 1)] + va[IVA(i + 1, j + 1, k + 1)] + va[IVA(i, j + 1, k)] + va[IVA(i + 1, j + 1, k)]) / 4.0;
  return f;
}
static inline faces_t faces_v(const double *va, int nx, int ny, int i, int j, int k) {
  DIMS;
  faces_t f;
  f.px = (va[IVA(i, j + 1, k + 1)] + va[IVA(i, j, k + 1)] + va[IVA(i + 1, j + 1, k + 1)] + va[IVA(i + 1, j, k + 1)]) / 4.0;
  f.mx = (va[IVA(i, j + 1, k + 1)] + va[IVA(i, j, k + 1)] + va[IVA(i - 1, j + 1, k + 1)] + va[IVA(i - 1, j, k + 1)]) / 4.0;
  f.py = va[IVA(i, j + 1, k + 1)];
  f.my = va[IVA(i, j, k + 1)];
  f.pz = (va[IVA(i, j + 1, k + 1)] + va[IVA(i, j, k + 1)] + va[IVA(i, j + 1, k + 2)] + va[IVA(i, j, k + 2)]) / 4.0;
  f.mz = (va[IVA(i, j + 1, k + 1)] + va[IVA(i, j, k + 1)] + va[IVA(i, j + 1, k)] + va[IVA(i, j, k)]) / 4.0;
  return f;
}
static inline faces_t faces_w(const double *va, int nx, int ny, int i, int j, int k) {
  DIMS;
  faces_t f;
  f.px = (va[IVA(i, j + 1, k)] + va[IVA(i, j + 1, k + 1)] + va[IVA(i + 1, j + 1, k)] + va[IVA(i + 1, j + 1, k + 1)]) / 4.0;
  f.mx = (va[IVA(i, j + 1, k)] + va[IVA(i, j + 1, k + 1)] + va[IVA(i - 1, j + 1, k)] + va[IVA(i - 1, j + 1, k + 1)]) / 4.0;
  f.py = (va[IVA(i, j + 1, k)] + va[IVA(i, j + 1, k + 1)] + va[IVA(i, j + 2, k)] + va[IVA(i, j + 2, k + 1)]) / 4.0;
  f.my = (va[IVA(i, j + 1, k)] + va[IVA(i, j + 1, k + 1)] + va[IVA(i, j, k)] + va[IVA(i, j, k + 1)]) / 4.0;
  f.pz = va[IVA(i, j + 1, k + 1)];
  f.mz = va[IVA(i, j + 1, k)];
  return f;
}

/* momentum_allflux.f90:22-214 get_diffusion_all */
void orc_get_diffusion_all(int nx, int ny, int nz, double *du, double *dv,
                           double *dw, const double *va, const double *u,
                           const double *v, const double *w, double dx,
                           double dy, double dz) {
  DIMS;
  const int maxn = nz + 1, ex_loc = nx - 1;
  memset(du, 0, sizeof(double) * (size_t)orc_size_uv(nx, ny, nz));
  OMP_FOR
  for (int k = 0; k <= maxn - 2; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= ex_loc; i++) {
        const double c = u[IX(i, j, k)];
        double umz = (k == 0) ? -2.0 * u[IX(i, j, 0)] + u[IX(i, j, 1)] / 3.0 : u[IX(i, j, k - 1)];
        double upz = (k == maxn - 2) ? -2.0 * u[IX(i, j, maxn - 2)] + u[IX(i, j, maxn - 3)] / 3.0
                                     : u[IX(i, j, k + 1)];
        faces_t f = faces_u(va, nx, ny, i, j, k);
        double E = f.px * ((u[IX(i + 1, j, k)] - c) / dx), W = f.mx * ((c - u[IX(i - 1, j, k)]) / dx);
        double N = f.py * ((u[IX(i, j + 1, k)] - c) / dy), S = f.my * ((c - u[IX(i, j - 1, k)]) / dy);
        double O = f.pz * ((upz - c) / dz), I = f.mz * ((c - umz) / dz);
        du[IX(i, j, k)] = ((E - W) / dx) + ((N - S) / dy) + ((O - I) / dz);
      }
  memset(dv, 0, sizeof(double) * (size_t)orc_size_uv(nx, ny, nz));
  OMP_FOR
  for (int k = 0; k <= maxn - 2; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        const double c = v[IX(i, j, k)];
        double vmz = (k == 0) ? -2.0 * v[IX(i, j, 0)] + v[IX(i, j, 1)] / 3.0 : v[IX(i, j, k - 1)];
        double vpz = (k == maxn - 2) ? -2.0 * v[IX(i, j, maxn - 2)] + v[IX(i, j, maxn - 3)] / 3.0
                                     : v[IX(i, j, k + 1)];
        double vmx = v[IX(i - 1, j, k)], vpx = v[IX(i + 1, j, k)];
        faces_t f = faces_v(va, nx, ny, i, j, k);
        double E = f.px * ((vpx - c) / dx), W = f.mx * ((c - vmx) / dx);
        double N = f.py * ((v[IX(i, j + 1, k)] - c) / dy), S = f.my * ((c - v[IX(i, j - 1, k)]) / dy);
        double O = f.pz * ((vpz - c) / dz), I = f.mz * ((c - vmz) / dz);
        dv[IX(i, j, k)] = ((E - W) / dx) + ((N - S) / dy) + ((O - I) / dz);
      }
  memset(dw, 0, sizeof(double) * (size_t)orc_size_w(nx, ny, nz));
  OMP_FOR
  for (int k = 1; k <= maxn - 2; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        const double c = w[IX(i, j, k)];
        double wmx = w[IX(i - 1, j, k)], wpx = w[IX(i + 1, j, k)];
        faces_t f = faces_w(va, nx, ny, i, j, k);
        double E = f.px * ((wpx - c) / dx), W = f.mx * ((c - wmx) / dx);
        double N = f.py * ((w[IX(i, j + 1, k)] - c) / dy), S = f.my * ((c - w[IX(i, j - 1, k)]) / dy);
        double O = f.pz * ((w[IX(i, j, k + 1)] - c) / dz), I = f.mz * ((c - w[IX(i, j, k - 1)]) / dz);
        dw[IX(i, j, k)] = ((E - W) / dx) + ((N - S) / dy) + ((O - I) / dz);
      }
}

/* One Helmholtz point update, jacobi_iteration_allflux.f90:84-90 (and the
 * identical forms of the v, w, and SOR routines). */
static inline double helm_point(faces_t f, double ax, double ay, double az,
                                double xp, double xm, double yp, double ym,
                                double zp, double zm, double rhs) {
  double diag = 1.0 + (ax / 2.0) * (f.px + f.mx) + (ay / 2.0) * (f.py + f.my) +
                (az / 2.0) * (f.pz + f.mz);
  return (1.0 / diag) * ((ax / 2.0) * (f.px * xp + f.mx * xm) +
                         (ay / 2.0) * (f.py * yp + f.my * ym) +
                         (az / 2.0) * (f.pz * zp + f.mz * zm) + rhs);
}

/* jacobi_iteration_allflux.f90:21-282 do_jacobi_{u,v,w}; comp 0/1/2. */
void orc_do_jacobi(int comp, int nx, int ny, int nz, double *x3,
                   const double *xo, const double *rhs, const double *va,
                   double dx, double dy, double dz, double dt) {
  DIMS;
  const int maxn = nz + 1;
  const double ax = dt / (dx * dx), ay = dt / (dy * dy), az = dt / (dz * dz);
  if (comp == 0) {
    OMP_FOR
    for (int k = 0; k <= maxn - 2; k++)
      for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx - 1; i++) {
          double umz = (k == 0) ? -2.0 * xo[IX(i, j, 0)] + xo[IX(i, j, 1)] / 3.0 : xo[IX(i, j, k - 1)];
          double upz = (k == maxn - 2) ? -2.0 * xo[IX(i, j, maxn - 2)] + xo[IX(i, j, maxn - 3)] / 3.0
                                       : xo[IX(i, j, k + 1)];
          x3[IX(i, j, k)] = helm_point(faces_u(va, nx, ny, i, j, k), ax, ay, az, xo[IX(i + 1, j, k)],
                                       xo[IX(i - 1, j, k)], xo[IX(i, j + 1, k)], xo[IX(i, j - 1, k)],
                                       upz, umz, rhs[IX(i, j, k)]);
        }
  } else if (comp == 1) {
    OMP_FOR
    for (int k = 0; k <= maxn - 2; k++)
      for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
          double vmz = (k == 0) ? -2.0 * xo[IX(i, j, 0)] + xo[IX(i, j, 1)] / 3.0 : xo[IX(i, j, k - 1)];
          double vpz = (k == maxn - 2) ? -2.0 * xo[IX(i, j, maxn - 2)] + xo[IX(i, j, maxn - 3)] / 3.0
                                       : xo[IX(i, j, k + 1)];
          x3[IX(i, j, k)] = helm_point(faces_v(va, nx, ny, i, j, k), ax, ay, az, xo[IX(i + 1, j, k)],
                                       xo[IX(i - 1, j, k)], xo[IX(i, j + 1, k)], xo[IX(i, j - 1, k)],
                                       vpz, vmz, rhs[IX(i, j, k)]);
        }
    for (int k = 0; k <= maxn - 2; k++)
      for (int j = 1; j <= ny; j++) x3[IX(0, j, k)] = x3[IX(1, j, k)];
    for (int k = 0; k <= maxn - 2; k++)
      for (int j = 1; j <= ny; j++) x3[IX(nx + 1, j, k)] = x3[IX(nx, j, k)];
  } else {
    OMP_FOR
    for (int k = 1; k <= maxn - 2; k++)
      for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++)
          x3[IX(i, j, k)] = helm_point(faces_w(va, nx, ny, i, j, k), ax, ay, az, xo[IX(i + 1, j, k)],
                                       xo[IX(i - 1, j, k)], xo[IX(i, j + 1, k)], xo[IX(i, j - 1, k)],
                                       xo[IX(i, j, k + 1)], xo[IX(i, j, k - 1)], rhs[IX(i, j, k)]);
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        x3[IX(i, j, 0)] = 0.0;
        x3[IX(i, j, maxn - 1)] = 0.0;
      }
    for (int k = 1; k <= maxn - 2; k++)
      for (int j = 1; j <= ny; j++) x3[IX(0, j, k)] = x3[IX(1, j, k)];
    for (int j = 1; j <= ny; j++) {
      x3[IX(0, j, 0)] = 0.0;
      x3[IX(0, j, maxn - 1)] = 0.0;
    }
    for (int k = 0; k <= maxn - 1; k++)
      for (int j = 1; j <= ny; j++) x3[IX(nx + 1, j, k)] = x3[IX(nx, j, k)];
  }
}

/* sor_iteration_allflux.f90:19-377 do_sor_{u,v,w}: one red-black half
 * sweep in place, relax = 1.2.  Even iteration_time: 3-D checkerboard
 * mod(k+j+flg,2); odd: 2-D colouring mod(j+flg,2), so a point sees the
 * already-updated point below it in the same column (sequential k order). */
static inline double sor_point(int comp, const double *x, const double *rhs,
                               const double *va, int nx, int ny, int nz, int i,
                               int j, int k, double ax, double ay, double az) {
  DIMS;
  const int maxn = nz + 1;
  faces_t f;
  double zp, zm;
  if (comp == 2) {
    f = faces_w(va, nx, ny, i, j, k);
    zp = x[IX(i, j, k + 1)];
    zm = x[IX(i, j, k - 1)];
  } else {
    f = (comp == 0) ? faces_u(va, nx, ny, i, j, k) : faces_v(va, nx, ny, i, j, k);
    zm = (k == 0) ? -2.0 * x[IX(i, j, 0)] + x[IX(i, j, 1)] / 3.0 : x[IX(i, j, k - 1)];
    zp = (k == maxn - 2) ? -2.0 * x[IX(i, j, maxn - 2)] + x[IX(i, j, maxn - 3)] / 3.0 : x[IX(i, j, k + 1)];
  }
  double res = helm_point(f, ax, ay, az, x[IX(i + 1, j, k)], x[IX(i - 1, j, k)], x[IX(i, j + 1, k)],
                          x[IX(i, j - 1, k)], zp, zm, rhs[IX(i, j, k)]);
  return x[IX(i, j, k)] + 1.2 * (res - x[IX(i, j, k)]);
}

void orc_do_sor(int comp, int nx, int ny, int nz, double *x3,
                const double *rhs, const double *va, double dx, double dy,
                double dz, double dt, int flg, int iteration_time) {
  DIMS;
  const int maxn = nz + 1;
  const double ax = dt / (dx * dx), ay = dt / (dy * dy), az = dt / (dz * dz);
  const int iend = (comp == 0) ? nx - 1 : nx;
  const int k0 = (comp == 2) ? 1 : 0, k1 = maxn - 2;
  if (iteration_time % 2 == 0) {
    OMP_FOR
    for (int k = k0; k <= k1; k++)
      for (int j = 1; j <= ny; j++)
        for (int i = (k + j + flg) % 2 + 1; i <= iend; i += 2)
          x3[IX(i, j, k)] = sor_point(comp, x3, rhs, va, nx, ny, nz, i, j, k, ax, ay, az);
  } else {
    for (int k = k0; k <= k1; k++) {
      OMP_FOR
      for (int j = 1; j <= ny; j++)
        for (int i = (j + flg) % 2 + 1; i <= iend; i += 2)
          x3[IX(i, j, k)] = sor_point(comp, x3, rhs, va, nx, ny, nz, i, j, k, ax, ay, az);
    }
  }
}

/* jacobi_iteration_allflux.f90:285-311 get_difference over i 1..nx,
 * j 1..ny, all z planes. */
static double get_difference(int nx, int ny, int nzplanes, const double *a,
                             const double *b) {
  DIMS;
  double d = 0.0;
  for (int k = 0; k < nzplanes; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        double t = a[IX(i, j, k)] - b[IX(i, j, k)];
        d += t * t;
      }
  return d;
}

/* main_ns_hybrid.F90:756-887, one velocity component: x3 = 0, then
 * max_iteration/2 outer iterations of {x3_old = x3; exchange; Jacobi; BC;
 * exchange; SOR flg=0; exchange; SOR flg=1; BC}, then get_difference. */
void orc_momentum(int comp, int nx, int ny, int nz, double *x3, double *x3_old,
                  const double *rhs, const double *va, const double *pres,
                  int max_iteration, double dx, double dy, double dz,
                  double dt, double *err) {
  DIMS;
  const int maxn = nz + 1;
  const int zpl = (comp == 2) ? nz + 1 : nz;
  const size_t n = (size_t)NX2 * NY2 * zpl;
  memset(x3, 0, n * sizeof(double));
  for (int it = 1; it <= max_iteration / 2; it++) {
    memcpy(x3_old, x3, n * sizeof(double));
    orc_exchange2d(nx, ny, 0, zpl - 1, x3_old);
    orc_do_jacobi(comp, nx, ny, nz, x3, x3_old, rhs, va, dx, dy, dz, dt);
    if (comp == 0) { /* :762-774 */
      for (int k = 0; k <= nz - 1; k++)
        for (int j = 1; j <= ny; j++) {
          x3[IX(0, j, k)] = x3[IX(1, j, k)];
          x3[IX(nx, j, k)] = x3[IX(nx - 1, j, k)] +
                             (dt / dx) * (pres[IX(nx + 1, j, k + 1)] + pres[IX(nx - 1, j, k + 1)] -
                                          2.0 * pres[IX(nx, j, k + 1)]);
          x3[IX(nx + 1, j, k)] = 0.0;
        }
    }
    orc_exchange2d(nx, ny, 0, zpl - 1, x3);
    orc_do_sor(comp, nx, ny, nz, x3, rhs, va, dx, dy, dz, dt, 0, it);
    orc_exchange2d(nx, ny, 0, zpl - 1, x3);
    orc_do_sor(comp, nx, ny, nz, x3, rhs, va, dx, dy, dz, dt, 1, it);
    if (comp == 0) { /* :784-799 */
      for (int k = 0; k <= nz - 1; k++)
        for (int j = 1; j <= ny; j++) {
          x3[IX(0, j, k)] = x3[IX(1, j, k)];
          x3[IX(nx, j, k)] = x3[IX(nx - 1, j, k)] +
                             (dt / dx) * (pres[IX(nx + 1, j, k + 1)] + pres[IX(nx - 1, j, k + 1)] -
                                          2.0 * pres[IX(nx, j, k + 1)]);
          x3[IX(nx + 1, j, k)] = 0.0;
        }
    } else if (comp == 1) { /* :826-836 */
      for (int k = 0; k <= maxn - 2; k++)
        for (int j = 1; j <= ny; j++) x3[IX(0, j, k)] = x3[IX(1, j, k)];
      for (int k = 0; k <= maxn - 2; k++)
        for (int j = 1; j <= ny; j++) x3[IX(nx + 1, j, k)] = x3[IX(nx, j, k)];
    } else { /* :860-879 */
      for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
          x3[IX(i, j, 0)] = 0.0;
          x3[IX(i, j, maxn - 1)] = 0.0;
        }
      for (int k = 1; k <= maxn - 2; k++)
        for (int j = 1; j <= ny; j++) x3[IX(0, j, k)] = x3[IX(1, j, k)];
      for (int j = 1; j <= ny; j++) {
        x3[IX(0, j, 0)] = 0.0;
        x3[IX(0, j, maxn - 1)] = 0.0;
      }
      for (int k = 0; k <= maxn - 1; k++)
        for (int j = 1; j <= ny; j++) x3[IX(nx + 1, j, k)] = x3[IX(nx, j, k)];
    }
  }
  *err = get_difference(nx, ny, zpl, x3, x3_old);
}

/* ------------------------------------------------------------------------
 * pressure.f90:16-56 get_source_pres
 * ---------------------------------------------------------------------- */
void orc_get_source_pres(int nx, int ny, int nz, double *rhs, const double *u3,
                         const double *v3, const double *w3, double dx,
                         double dy, double dz, double dt) {
  DIMS;
  const size_t np = (size_t)orc_size_p(nx, ny, nz);
  memset(rhs, 0, np * sizeof(double));
  OMP_FOR
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++)
        rhs[IX(i, j, k)] = ((u3[IX(i, j - 1, k - 1)] - u3[IX(i - 1, j - 1, k - 1)]) / dx) +
                           ((v3[IX(i, j, k - 1)] - v3[IX(i, j - 1, k - 1)]) / dy) +
                           ((w3[IX(i, j - 1, k)] - w3[IX(i, j - 1, k - 1)]) / dz);
  for (size_t c = 0; c < np; c++) rhs[c] = rhs[c] / dt;
}

/* pressure.f90:59-134 get_uvw_pres */
void orc_get_uvw_pres(int nx, int ny, int nz, double *u3, double *v3,
                      double *w3, const double *p, double dx, double dy,
                      double dz, double dt, const double *u_inlet) {
  DIMS;
  OMP_FOR
  for (int k = 0; k <= nz - 1; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 0; i <= nx + 1; i++) {
        if (i == 0)
          u3[IX(i, j, k)] = u_inlet[k];
        else if (i == nx + 1)
          u3[IX(i, j, k)] = 0.0;
        else
          u3[IX(i, j, k)] = u3[IX(i, j, k)] - (dt / dx) * (p[IX(i + 1, j + 1, k + 1)] - p[IX(i, j + 1, k + 1)]);
      }
  OMP_FOR
  for (int k = 0; k <= nz - 1; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 0; i <= nx + 1; i++)
        v3[IX(i, j, k)] = v3[IX(i, j, k)] - (dt / dy) * (p[IX(i, j + 1, k + 1)] - p[IX(i, j, k + 1)]);
  OMP_FOR
  for (int k = 0; k <= nz; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 0; i <= nx + 1; i++)
        w3[IX(i, j, k)] = w3[IX(i, j, k)] - (dt / dz) * (p[IX(i, j + 1, k + 1)] - p[IX(i, j + 1, k)]);
}

/* ------------------------------------------------------------------------
 * Pressure Poisson: the system PETSc is handed (pressure_solver.F90:234-441)
 * solved exactly.  Unknowns are p(x=0..nx+1, y=1..ny, z=0..nz+1), y periodic.
 *   interior rows (x 1..nx, z 1..nz):  2(1/dx^2+1/dy^2+1/dz^2) p
 *        - (1/dy^2)(p[x-1]+p[x+1]) - (1/dx^2)(p[y-1]+p[y+1])
 *        - (1/dz^2)(p[z-1]+p[z+1]) = -RHS_p         (:391-422; PETSc's i
 *        is physical y and carries 1/dx^2, its j is physical x with 1/dy^2)
 *   ghost rows: (p[0]-p[1])/dy = (dx/dt)(u_inlet(k-1)-u3(0,y-1,k-1))/dy at
 *        the inlet (:280-286), zero-flux 2-point rows elsewhere (:321-390).
 * Eliminating the ghost rows gives a symmetric interior operator with
 * Neumann conditions in x and z and periodic y, singular with the constant
 * null space (:436-439).  The oracle removes the mean of the reduced
 * right-hand side (compatibility projection), solves by separable
 * eigen-decomposition (DCT-II bases in x and z, real Fourier basis in y),
 * fixes the constant so the interior mean equals that of the initial guess,
 * and rebuilds every ghost value from its 2-point row.
 * ---------------------------------------------------------------------- */
static void build_neumann_basis(int n, double *Q, double *lam) {
  for (int k = 0; k < n; k++) {
    double c = (k == 0) ? sqrt(1.0 / n) : sqrt(2.0 / n);
    for (int i = 0; i < n; i++) Q[(size_t)k * n + i] = c * cos(M_PI * k * (i + 0.5) / n);
    double s = sin(M_PI * k / (2.0 * n));
    lam[k] = 4.0 * s * s;
  }
}
static void build_periodic_basis(int n, double *Q, double *lam) {
  int idx = 0;
  for (int i = 0; i < n; i++) Q[i] = sqrt(1.0 / n);
  lam[idx++] = 0.0;
  for (int m = 1; 2 * m < n; m++) {
    double s = sin(M_PI * m / n);
    for (int i = 0; i < n; i++) Q[(size_t)idx * n + i] = sqrt(2.0 / n) * cos(2.0 * M_PI * m * i / n);
    lam[idx++] = 4.0 * s * s;
    for (int i = 0; i < n; i++) Q[(size_t)idx * n + i] = sqrt(2.0 / n) * sin(2.0 * M_PI * m * i / n);
    lam[idx++] = 4.0 * s * s;
  }
  if (n % 2 == 0) {
    for (int i = 0; i < n; i++) Q[(size_t)idx * n + i] = (i % 2 == 0) ? sqrt(1.0 / n) : -sqrt(1.0 / n);
    lam[idx++] = 4.0;
  }
}
/* in-place transform along one axis of an (n0,n1,n2) x-fastest array:
 * out[..a..] = sum_b Q[a][b] in[..b..] (fwd) or Q[b][a] (inverse). */
static void apply_axis(double *f, int n0, int n1, int n2, int axis,
                       const double *Q, int inverse) {
  int n = (axis == 0) ? n0 : (axis == 1) ? n1 : n2;
  size_t stride = (axis == 0) ? 1 : (axis == 1) ? (size_t)n0 : (size_t)n0 * n1;
  int outer1 = (axis == 0) ? n1 : n0, outer2 = (axis == 2) ? n1 : n2;
  OMP_FOR
  for (int o2 = 0; o2 < outer2; o2++) {
    double *tin = (double *)malloc(sizeof(double) * n), *tout = (double *)malloc(sizeof(double) * n);
    for (int o1 = 0; o1 < outer1; o1++) {
      size_t base;
      if (axis == 0) base = (size_t)o1 * n0 + (size_t)o2 * n0 * n1;
      else if (axis == 1) base = (size_t)o1 + (size_t)o2 * n0 * n1;
      else base = (size_t)o1 + (size_t)o2 * n0;
      for (int b = 0; b < n; b++) tin[b] = f[base + b * stride];
      for (int a = 0; a < n; a++) {
        double s = 0.0;
        if (!inverse)
          for (int b = 0; b < n; b++) s += Q[(size_t)a * n + b] * tin[b];
        else
          for (int b = 0; b < n; b++) s += Q[(size_t)b * n + a] * tin[b];
        tout[a] = s;
      }
      for (int a = 0; a < n; a++) f[base + a * stride] = tout[a];
    }
    free(tin);
    free(tout);
  }
}

void orc_pressure_solve(int nx, int ny, int nz, double *pres,
                        const double *rhs_p, const double *u3,
                        const double *u_inlet, double dx, double dy,
                        double dz, double dt, double *rnorm) {
  DIMS;
  const size_t N = (size_t)nx * ny * nz;
  const double cx = 1.0 / (dy * dy), cy = 1.0 / (dx * dx), cz = 1.0 / (dz * dz);
  double *b = (double *)malloc(N * sizeof(double));
  double *bin = (double *)malloc((size_t)ny * nz * sizeof(double));
#define RI(i, j, k) ((size_t)((i) - 1) + (size_t)nx * ((size_t)((j) - 1) + (size_t)ny * (size_t)((k) - 1)))
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++)
      bin[(size_t)(j - 1) + (size_t)ny * (k - 1)] =
          (dx / dt) * (u_inlet[k - 1] - u3[IX(0, j - 1, k - 1)]) / dy;
  double mean_b = 0.0, mean_p0 = 0.0;
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        double v = -rhs_p[IX(i, j, k)];
        if (i == 1) v += bin[(size_t)(j - 1) + (size_t)ny * (k - 1)] / dy;
        b[RI(i, j, k)] = v;
        mean_b += v;
        mean_p0 += pres[IX(i, j, k)];
      }
  mean_b /= (double)N;
  mean_p0 /= (double)N;
  for (size_t c = 0; c < N; c++) b[c] -= mean_b;
  double *bproj = (double *)malloc(N * sizeof(double));
  memcpy(bproj, b, N * sizeof(double));
  double *Qx = (double *)malloc(sizeof(double) * nx * nx), *Qy = (double *)malloc(sizeof(double) * ny * ny),
         *Qz = (double *)malloc(sizeof(double) * nz * nz);
  double *lx = (double *)malloc(sizeof(double) * nx), *ly = (double *)malloc(sizeof(double) * ny),
         *lz = (double *)malloc(sizeof(double) * nz);
  build_neumann_basis(nx, Qx, lx);
  build_periodic_basis(ny, Qy, ly);
  build_neumann_basis(nz, Qz, lz);
  apply_axis(b, nx, ny, nz, 0, Qx, 0);
  apply_axis(b, nx, ny, nz, 1, Qy, 0);
  apply_axis(b, nx, ny, nz, 2, Qz, 0);
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        size_t c = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
        double lam = cx * lx[i] + cy * ly[j] + cz * lz[k];
        b[c] = (i == 0 && j == 0 && k == 0) ? 0.0 : b[c] / lam;
      }
  apply_axis(b, nx, ny, nz, 2, Qz, 1);
  apply_axis(b, nx, ny, nz, 1, Qy, 1);
  apply_axis(b, nx, ny, nz, 0, Qx, 1);
  /* constant: interior mean of the initial guess */
  double mean_s = 0.0;
  for (size_t c = 0; c < N; c++) mean_s += b[c];
  mean_s /= (double)N;
  for (size_t c = 0; c < N; c++) b[c] = b[c] - mean_s + mean_p0;
  /* residual of the reduced, projected system */
  double rr = 0.0;
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        double c = b[RI(i, j, k)];
        double xm = (i > 1) ? b[RI(i - 1, j, k)] : c, xp = (i < nx) ? b[RI(i + 1, j, k)] : c;
        double ym = b[RI(i, (j > 1) ? j - 1 : ny, k)], yp = b[RI(i, (j < ny) ? j + 1 : 1, k)];
        double zm = (k > 1) ? b[RI(i, j, k - 1)] : c, zp = (k < nz) ? b[RI(i, j, k + 1)] : c;
        double Ap = cx * (2.0 * c - xm - xp) + cy * (2.0 * c - ym - yp) + cz * (2.0 * c - zm - zp);
        double r = bproj[RI(i, j, k)] - Ap;
        rr += r * r;
      }
  *rnorm = sqrt(rr);
  /* write back with every ghost from its 2-point row */
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) pres[IX(i, j, k)] = b[RI(i, j, k)];
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++) {
      pres[IX(0, j, k)] = pres[IX(1, j, k)] + dy * bin[(size_t)(j - 1) + (size_t)ny * (k - 1)];
      pres[IX(nx + 1, j, k)] = pres[IX(nx, j, k)];
    }
  for (int j = 1; j <= ny; j++)
    for (int i = 0; i <= nx + 1; i++) {
      pres[IX(i, j, 0)] = pres[IX(i, j, 1)];
      pres[IX(i, j, nz + 1)] = pres[IX(i, j, nz)];
    }
  orc_exchange2d(nx, ny, 0, nz + 1, pres);
#undef RI
  free(b);
  free(bproj);
  free(bin);
  free(Qx);
  free(Qy);
  free(Qz);
  free(lx);
  free(ly);
  free(lz);
}

/* ------------------------------------------------------------------------
 * Whole-step driver: main_ns_hybrid.F90:583-918 and the history rotation
 * :2480-2509.
 * ---------------------------------------------------------------------- */
struct orc_ctx {
  int nx, ny, nz;
  tpls_params prm;
  double *u_inlet;
  double *f[TPLS_F_COUNT];
  /* scratch / intermediates */
  double *fx, *fy, *fz, *csf_u2, *csf_v2, *csf_w2, *va;
  double *conv2_u, *conv2_v, *conv2_w, *diff_u, *diff_v, *diff_w;
  double *rhs_u, *rhs_v, *rhs_w, *u3_old, *v3_old, *w3_old;
  double *dim_c;  /* phi2 + 0.5 / phi2 - 0.5 temporaries of the diffuse-interface step */
  tpls_stats st;
};

static int field_kind(int f) {
  switch (f) {
    case TPLS_F_U2: case TPLS_F_V2: case TPLS_F_CONV0_U: case TPLS_F_CONV1_U:
    case TPLS_F_CONV0_V: case TPLS_F_CONV1_V: case TPLS_F_CSF_U0: case TPLS_F_CSF_U1:
    case TPLS_F_CSF_V0: case TPLS_F_CSF_V1: case TPLS_F_U3: case TPLS_F_V3:
      return 1;
    case TPLS_F_W2: case TPLS_F_CONV0_W: case TPLS_F_CONV1_W: case TPLS_F_CSF_W0:
    case TPLS_F_CSF_W1: case TPLS_F_W3:
      return 2;
    default:
      return 0;
  }
}
static size_t field_size(const orc_ctx *c, int f) {
  int k = field_kind(f);
  return (size_t)((k == 0) ? orc_size_p(c->nx, c->ny, c->nz)
                           : (k == 1) ? orc_size_uv(c->nx, c->ny, c->nz) : orc_size_w(c->nx, c->ny, c->nz));
}

orc_ctx *orc_create(int nx, int ny, int nz, const tpls_params *prm,
                    const double *u_inlet) {
  if (nx < 4 || ny < 3 || nz < 4) return NULL;
  orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
  c->nx = nx;
  c->ny = ny;
  c->nz = nz;
  c->prm = *prm;
  c->u_inlet = (double *)malloc(sizeof(double) * nz);
  memcpy(c->u_inlet, u_inlet, sizeof(double) * nz);
  for (int f = 0; f < TPLS_F_COUNT; f++) c->f[f] = alloc_zero(field_size(c, f));
  size_t np = (size_t)orc_size_p(nx, ny, nz), nuv = (size_t)orc_size_uv(nx, ny, nz),
         nw = (size_t)orc_size_w(nx, ny, nz);
  c->fx = alloc_zero(np);
  c->fy = alloc_zero(np);
  c->fz = alloc_zero(np);
  c->csf_u2 = alloc_zero(nuv);
  c->csf_v2 = alloc_zero(nuv);
  c->csf_w2 = alloc_zero(nw);
  c->va = alloc_zero((size_t)orc_size_visc_aug(nx, ny, nz));
  c->conv2_u = alloc_zero(nuv);
  c->conv2_v = alloc_zero(nuv);
  c->conv2_w = alloc_zero(nw);
  c->diff_u = alloc_zero(nuv);
  c->diff_v = alloc_zero(nuv);
  c->diff_w = alloc_zero(nw);
  c->rhs_u = alloc_zero(nuv);
  c->rhs_v = alloc_zero(nuv);
  c->rhs_w = alloc_zero(nw);
  c->u3_old = alloc_zero(nuv);
  c->v3_old = alloc_zero(nuv);
  c->w3_old = alloc_zero(nw);
  c->dim_c = alloc_zero(np);
  return c;
}

void orc_destroy(orc_ctx *c) {
  if (!c) return;
  for (int f = 0; f < TPLS_F_COUNT; f++) free(c->f[f]);
  double *s[] = {c->u_inlet, c->fx, c->fy, c->fz, c->csf_u2, c->csf_v2, c->csf_w2, c->va,
                 c->conv2_u, c->conv2_v, c->conv2_w, c->diff_u, c->diff_v, c->diff_w,
                 c->rhs_u, c->rhs_v, c->rhs_w, c->u3_old, c->v3_old, c->w3_old, c->dim_c};
  for (size_t q = 0; q < sizeof(s) / sizeof(s[0]); q++) free(s[q]);
  free(c);
}

int orc_set_field(orc_ctx *c, int field, const double *host) {
  if (field < 0 || field >= TPLS_F_COUNT) return TPLS_ERR_ARG;
  memcpy(c->f[field], host, field_size(c, field) * sizeof(double));
  return 0;
}
int orc_get_field(orc_ctx *c, int field, double *host) {
  if (field < 0 || field >= TPLS_F_COUNT) return TPLS_ERR_ARG;
  memcpy(host, c->f[field], field_size(c, field) * sizeof(double));
  return 0;
}
void orc_get_stats(orc_ctx *c, tpls_stats *st) { *st = c->st; }

static double liquid_volume(const orc_ctx *c) {
  const int nx = c->nx, ny = c->ny, nz = c->nz;
  DIMS;
  const double *phi = c->f[TPLS_F_PHI2], sw = c->prm.smooth_width;
  double s = 0.0;
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        double p = phi[IX(i, j, k)], hv;
        if (p < -sw) hv = 0.0;
        else if (p > sw) hv = 1.0;
        else hv = 0.5 + (p / (2.0 * sw)) + (1.0 / (2.0 * PI_SP)) * sin(PI_SP * p / sw);
        s += 1.0 - hv;
      }
  return s * c->prm.dx * c->prm.dy * c->prm.dz;
}

void orc_step(orc_ctx *c, int nsteps) {
  const int nx = c->nx, ny = c->ny, nz = c->nz;
  const tpls_params *P = &c->prm;
  const double dx = P->dx, dy = P->dy, dz = P->dz, dt = P->dt;
  double **F = c->f;
  const size_t np = (size_t)orc_size_p(nx, ny, nz), nuv = (size_t)orc_size_uv(nx, ny, nz),
               nw = (size_t)orc_size_w(nx, ny, nz);
  for (int s = 0; s < nsteps; s++) {
    double *u2 = F[TPLS_F_U2], *v2 = F[TPLS_F_V2], *w2 = F[TPLS_F_W2];
    /* :585 advection */
    orc_do_advect_phi(nx, ny, nz, F[TPLS_F_PHI2], u2, v2, w2, F[TPLS_F_CONV2_PHI], dx, dy, dz);
    if (P->idm == TPLS_IDM_DIM) {
      /* :608-611 diffuse interface: dim(phi2+0.5, phi_old+0.5, ..., phi3), then
       * phi3 = phi3 - 0.5; phi_old equals phi2 at every step (:444, :2508) */
      for (size_t e = 0; e < np; e++) c->dim_c[e] = F[TPLS_F_PHI2][e] + 0.5;
      orc_dim(nx, ny, nz, dx, dy, dz, dt, P->epn, P->pe, c->dim_c, c->dim_c, F[TPLS_F_CONV2_PHI],
              F[TPLS_F_CONVPREV_PHI], F[TPLS_F_PHI3], P->height, P->max_iteration_dim);
      for (size_t e = 0; e < np; e++) F[TPLS_F_PHI3][e] = F[TPLS_F_PHI3][e] - 0.5;
      c->st.err_phi = 0.0;
    } else {
      /* :596 level-set update + redistancing */
      orc_do_tpls(nx, ny, nz, F[TPLS_F_PHI2], F[TPLS_F_PHI3], F[TPLS_F_CONV0_PHI], F[TPLS_F_CONV1_PHI],
                  F[TPLS_F_CONV2_PHI], P->levelset, P->height, dx, dz, dt, &c->st.err_phi);
    }
    /* :618-641 CSF */
    orc_exchange2d(nx, ny, 0, nz + 1, F[TPLS_F_PHI3]);
    orc_get_csf(nx, ny, nz, c->fx, c->fy, c->fz, F[TPLS_F_PHI3], dx, dy, dz, P->scap, P->smooth_width);
    orc_exchange2d(nx, ny, 0, nz + 1, c->fx);
    orc_exchange2d(nx, ny, 0, nz + 1, c->fy);
    orc_exchange2d(nx, ny, 0, nz + 1, c->fz);
    orc_csf_faces(nx, ny, nz, c->fx, c->fy, c->fz, c->csf_u2, c->csf_v2, c->csf_w2);
    /* :646-724 viscosity from phi2 (the pre-advection level set); the
     * diffuse-interface method passes phi2-0.5 (:650, :667, :692) */
    const double *vphi = F[TPLS_F_PHI2];
    if (P->idm == TPLS_IDM_DIM) {
      for (size_t e = 0; e < np; e++) c->dim_c[e] = F[TPLS_F_PHI2][e] - 0.5;
      vphi = c->dim_c;
    }
    orc_viscosity_aug(nx, ny, nz, vphi, c->va, P->smooth_width, P->re, P->mu_minus, P->mu_plus);
    /* :728-735 */
    orc_exchange2d(nx, ny, 0, nz - 1, u2);
    orc_exchange2d(nx, ny, 0, nz - 1, v2);
    orc_exchange2d(nx, ny, 0, nz, w2);
    orc_get_conv_all(nx, ny, nz, c->conv2_u, c->conv2_v, c->conv2_w, c->va, u2, v2, w2, dx, dy, dz);
    orc_get_diffusion_all(nx, ny, nz, c->diff_u, c->diff_v, c->diff_w, c->va, u2, v2, w2, dx, dy, dz);
    /* :743-751 AB3 + CN right-hand sides over the whole arrays */
    struct { double *r, *x, *c2, *c1, *c0, *d, *s2, *s1, *s0; size_t n; } R[3] = {
        {c->rhs_u, u2, c->conv2_u, F[TPLS_F_CONV1_U], F[TPLS_F_CONV0_U], c->diff_u, c->csf_u2,
         F[TPLS_F_CSF_U1], F[TPLS_F_CSF_U0], nuv},
        {c->rhs_v, v2, c->conv2_v, F[TPLS_F_CONV1_V], F[TPLS_F_CONV0_V], c->diff_v, c->csf_v2,
         F[TPLS_F_CSF_V1], F[TPLS_F_CSF_V0], nuv},
        {c->rhs_w, w2, c->conv2_w, F[TPLS_F_CONV1_W], F[TPLS_F_CONV0_W], c->diff_w, c->csf_w2,
         F[TPLS_F_CSF_W1], F[TPLS_F_CSF_W0], nw}};
    for (int q = 0; q < 3; q++)
      for (size_t e = 0; e < R[q].n; e++)
        R[q].r[e] = R[q].x[e] -
                    dt * ((23.0 / 12.0) * R[q].c2[e] - (4.0 / 3.0) * R[q].c1[e] + (5.0 / 12.0) * R[q].c0[e]) +
                    (dt / 2.0) * R[q].d[e] +
                    dt * ((23.0 / 12.0) * R[q].s2[e] - (4.0 / 3.0) * R[q].s1[e] + (5.0 / 12.0) * R[q].s0[e]);
    /* :756-887 momentum sweeps (u uses pres in its outlet condition) */
    orc_momentum(0, nx, ny, nz, F[TPLS_F_U3], c->u3_old, c->rhs_u, c->va, F[TPLS_F_PRES], P->mom_u, dx,
                 dy, dz, dt, &c->st.err_u);
    orc_momentum(1, nx, ny, nz, F[TPLS_F_V3], c->v3_old, c->rhs_v, c->va, F[TPLS_F_PRES], P->mom_v, dx,
                 dy, dz, dt, &c->st.err_v);
    orc_momentum(2, nx, ny, nz, F[TPLS_F_W3], c->w3_old, c->rhs_w, c->va, F[TPLS_F_PRES], P->mom_w, dx,
                 dy, dz, dt, &c->st.err_w);
    /* :889-894 */
    orc_exchange2d(nx, ny, 0, nz - 1, F[TPLS_F_U3]);
    orc_exchange2d(nx, ny, 0, nz - 1, F[TPLS_F_V3]);
    orc_exchange2d(nx, ny, 0, nz, F[TPLS_F_W3]);
    orc_get_source_pres(nx, ny, nz, F[TPLS_F_RHS_P], F[TPLS_F_U3], F[TPLS_F_V3], F[TPLS_F_W3], dx, dy, dz,
                        dt);
    orc_exchange2d(nx, ny, 0, nz + 1, F[TPLS_F_RHS_P]);
    /* :897-913 */
    memcpy(F[TPLS_F_PRES], F[TPLS_F_PRES_OLD], np * sizeof(double));
    orc_pressure_solve(nx, ny, nz, F[TPLS_F_PRES], F[TPLS_F_RHS_P], F[TPLS_F_U3], c->u_inlet, dx, dy, dz,
                       dt, &c->st.p_rnorm);
    c->st.p_its = 0;
    c->st.p_reason = TPLS_KSP_CONVERGED_RTOL;
    /* :918 projection, applied to copies kept as the next step's state */
    memcpy(u2, F[TPLS_F_U3], nuv * sizeof(double));
    memcpy(v2, F[TPLS_F_V3], nuv * sizeof(double));
    memcpy(w2, F[TPLS_F_W3], nw * sizeof(double));
    orc_get_uvw_pres(nx, ny, nz, u2, v2, w2, F[TPLS_F_PRES], dx, dy, dz, dt, c->u_inlet);
    /* :2480-2509 history rotation (u2 <- u3 done above) */
    memcpy(F[TPLS_F_CONV0_U], F[TPLS_F_CONV1_U], nuv * sizeof(double));
    memcpy(F[TPLS_F_CONV0_V], F[TPLS_F_CONV1_V], nuv * sizeof(double));
    memcpy(F[TPLS_F_CONV0_W], F[TPLS_F_CONV1_W], nw * sizeof(double));
    memcpy(F[TPLS_F_CONV1_U], c->conv2_u, nuv * sizeof(double));
    memcpy(F[TPLS_F_CONV1_V], c->conv2_v, nuv * sizeof(double));
    memcpy(F[TPLS_F_CONV1_W], c->conv2_w, nw * sizeof(double));
    memcpy(F[TPLS_F_CSF_U0], F[TPLS_F_CSF_U1], nuv * sizeof(double));
    memcpy(F[TPLS_F_CSF_V0], F[TPLS_F_CSF_V1], nuv * sizeof(double));
    memcpy(F[TPLS_F_CSF_W0], F[TPLS_F_CSF_W1], nw * sizeof(double));
    memcpy(F[TPLS_F_CSF_U1], c->csf_u2, nuv * sizeof(double));
    memcpy(F[TPLS_F_CSF_V1], c->csf_v2, nuv * sizeof(double));
    memcpy(F[TPLS_F_CSF_W1], c->csf_w2, nw * sizeof(double));
    memcpy(F[TPLS_F_CONV0_PHI], F[TPLS_F_CONV1_PHI], np * sizeof(double));
    memcpy(F[TPLS_F_CONV1_PHI], F[TPLS_F_CONV2_PHI], np * sizeof(double));
    memcpy(F[TPLS_F_PRES_OLD], F[TPLS_F_PRES], np * sizeof(double));
    memcpy(F[TPLS_F_PHI2], F[TPLS_F_PHI3], np * sizeof(double));
    c->st.steps_done++;
    c->st.liquid_volume = liquid_volume(c);
  }
}

/* ------------------------------------------------------------------------
 * Base state of the two-layer channel: twophase_initialisation_wave.F90:79-122.
 * visc_oned(k), k = 0..n (n = nz+1), from the smoothed Heaviside of
 * phi = z - height with pi the single-precision literal 3.14159265359
 * (:54); then num_iterations = 10000 in-place Gauss-Seidel sweeps of
 * (d/dz)(mu du/dz) = dpdl over u2_oned(0..n-2) with the wall ghost rule
 * -2 u(0) + u(1)/3 at both ends (:101-120).  Output u_oned(0..nz-1).
 * ---------------------------------------------------------------------- */
void orc_base_profile(int nz, double dz, double reynolds, double dpdl,
                      double mu_minus, double mu_plus, double height,
                      double smooth_width, double *u_oned) {
  const double pi = (double)3.14159265359f;
  const int n = nz + 1;
  double *visc_oned = (double *)malloc(sizeof(double) * (size_t)(n + 1));
  double *u2 = (double *)calloc((size_t)(n - 1), sizeof(double));
  for (int k = 0; k <= n; k++) {
    double z_val = dz * k - (dz / 2.0);
    double phi_val = z_val - height;
    double heaviside_phi;
    if (phi_val < -smooth_width)
      heaviside_phi = 0.0;
    else if (phi_val > smooth_width)
      heaviside_phi = 1.0;
    else
      heaviside_phi = 0.5 + (phi_val / (2.0 * smooth_width)) +
                      (1.0 / (2.0 * pi)) * sin(pi * phi_val / smooth_width);
    double temp = mu_plus * heaviside_phi + mu_minus * (1.0 - heaviside_phi);
    visc_oned[k] = temp / reynolds;
  }
  const double rhs = dpdl;
  for (int it = 1; it <= 10000; it++) {
    for (int k = 0; k <= n - 2; k++) {
      double u_minusz = (k == 0) ? -2.0 * u2[0] + u2[1] / 3.0 : u2[k - 1];
      double u_plusz = (k == n - 2) ? -2.0 * u2[n - 2] + u2[n - 3] / 3.0 : u2[k + 1];
      double mu_minusk = (visc_oned[k] + visc_oned[k + 1]) / 2.0;
      double mu_plusk = (visc_oned[k + 2] + visc_oned[k + 1]) / 2.0;
      double diag_val = (mu_plusk + mu_minusk) / (dz * dz);
      u2[k] = (1.0 / diag_val) * (((mu_plusk * u_plusz + mu_minusk * u_minusz) / (dz * dz)) - rhs);
    }
  }
  for (int k = 0; k < nz; k++) u_oned[k] = u2[k];
  free(visc_oned);
  free(u2);
}
