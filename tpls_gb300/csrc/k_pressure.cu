// k_pressure.cu -- pressure Poisson solve (replaces the PETSc KSPSolve of
// main_ns_hybrid.F90:896-913 with the callbacks of pressure_solver.F90:
// 205-486).
//
// The system PETSc is handed has unknowns on x = 0..nx+1, z = 0..nz+1 and
// periodic y.  Its ghost rows are 2-point rows (zero-flux, or the inlet
// flux (dx/dt)(u_inlet-u3(0))/dy at x = 0), so they are eliminated exactly:
// the interior operator becomes the symmetric 7-point operator with
// Neumann conditions in x and z and periodic y,
//   A p = cx(2p - p[x-1] - p[x+1]) + cy(2p - p[y-1] - p[y+1])
//       + cz(2p - p[z-1] - p[z+1]),  missing x/z neighbours -> p itself,
// with cx = 1/dy^2, cy = 1/dx^2, cz = 1/dz^2 exactly as compute_matrix
// assigns them (PETSc's first index is physical y).  It is singular with
// the constant null space (pressure_solver.F90:436-439): the right-hand
// side is projected to zero mean and the solution keeps the interior mean
// of the initial guess p_old.
//
// Solver: CG preconditioned by one symmetric multigrid V-cycle.
//   levels: cell-centred coarsening of every dimension that is even and
//           >= 4 (y >= 4), down to <= 512 cells or no coarsenable dimension;
//   smoother: damped z-line Jacobi (one tridiagonal solve per (x,y) column
//           with precomputed Thomas factors -- the operator's z couplings
//           are (dx/dz)^2 times stronger than x/y on the channel grids);
//   transfer: trilinear prolongation P, restriction R = P^T / 2^d;
//   coarse operator: rediscretisation; coarsest grid: dense FP64
//           pseudo-inverse built from the separable eigen-decomposition.
// All reductions are deterministic (per-block partials summed in a fixed
// order), so a solve's iterates do not depend on timing.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "tpls_pressure.h"

namespace tpls {

constexpr int PB = 256;  // threads per block for 1-D pressure kernels

struct PLevel {
  int nx, ny, nz, n;
  int cxs, cys, czs;     // this level was coarsened in x/y/z from the finer one
  double cx, cy, cz;
  double *b = nullptr, *e = nullptr, *e2 = nullptr, *r = nullptr, *t = nullptr;
  double *thomas = nullptr;  // [3 classes][nz][2] = (cprime, inv_den)
};

struct PoissonSolver {
  int nx, ny, nz, N;
  std::vector<PLevel> lv;
  double *cinv = nullptr;  // coarsest pseudo-inverse (nc x nc), or null
  int coarse_sweeps = 0;
  double *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *bvec = nullptr;
  double *bin = nullptr;     // inlet ghost-row data (ny*nz)
  double *part = nullptr;    // reduction partials (3 * rblk)
  unsigned *counter = nullptr;  // last-block ticket of the reductions
  double *s = nullptr;       // device scalars
  double *s_host = nullptr;  // pinned mirror
  int rblk;                  // blocks of the grid-stride reduction kernels
  double omega = 0.8;
};

// device scalars of the CG iteration
enum { S_SUMB = 0, S_SUMX0, S_BB, S_RR, S_RZ, S_ZMEAN, S_BETA, S_ALPHA, S_SUMX, S_COUNT };

static inline int nblocks(int n) { return (n + PB - 1) / PB; }

// ---------------------------------------------------------------------------
// Reductions: a fixed grid of rblk blocks, each thread accumulating a fixed
// strided subset, one partial per block, and the last block to finish (by
// an atomic ticket) summing the partials in a fixed order.  The result does
// not depend on scheduling.  Returns true in the last block, with the sums
// in tot[] of thread 0.
template <int NQ>
__device__ __forceinline__ bool reduce_last(double (&v)[NQ], double *part, unsigned *counter,
                                            double (&tot)[NQ]) {
  __shared__ double sh[NQ][PB / 32];
  __shared__ bool last;
  const int nblk = gridDim.x;
  for (int q = 0; q < NQ; q++) {
    double a = v[q];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) sh[q][threadIdx.x >> 5] = a;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 0; q < NQ; q++) {
      double a = 0.0;
      for (int w = 0; w < PB / 32; w++) a += sh[q][w];
      part[(size_t)q * nblk + blockIdx.x] = a;
    }
    __threadfence();
    last = (atomicAdd(counter, 1u) == (unsigned)(nblk - 1));
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  for (int q = 0; q < NQ; q++) {
    double a = 0.0;
    for (int b = threadIdx.x; b < nblk; b += PB) a += __ldcg(part + (size_t)q * nblk + b);
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) sh[q][threadIdx.x >> 5] = a;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 0; q < NQ; q++) {
      double a = 0.0;
      for (int w = 0; w < PB / 32; w++) a += sh[q][w];
      tot[q] = a;
    }
    *counter = 0u;
  }
  return true;
}

__device__ __forceinline__ double applyA(const double *__restrict__ e, int i, int j, int k, int nx,
                                         int ny, int nz, double cx, double cy, double cz) {
  const int c = i + nx * (j + ny * k);
  const double v = e[c];
  const double xm = (i > 0) ? e[c - 1] : v, xp = (i < nx - 1) ? e[c + 1] : v;
  const double ym = e[c + nx * ((j > 0) ? -1 : ny - 1)];
  const double yp = e[c + nx * ((j < ny - 1) ? 1 : 1 - ny)];
  const double zm = (k > 0) ? e[c - nx * ny] : v, zp = (k < nz - 1) ? e[c + nx * ny] : v;
  return cx * (2.0 * v - xm - xp) + cy * (2.0 * v - ym - yp) + cz * (2.0 * v - zm - zp);
}

#define GRID_STRIDE(c, N) for (int c = blockIdx.x * PB + threadIdx.x; c < (N); c += gridDim.x * PB)

// b (compact interior) = -RHS_p + inlet contribution; x0 = p_old interior;
// sums of b and x0.
__global__ void __launch_bounds__(PB)
    k_build_b(Geo g, double dxdt_over_dy, double rdy, const double *__restrict__ rhs_p,
              const double *__restrict__ u3, const double *__restrict__ uin,
              const double *__restrict__ pold, double *__restrict__ b, double *__restrict__ x0,
              double *__restrict__ bin, double *part, unsigned *counter, double *s) {
  const int nx = g.nx, ny = g.ny, nz = g.nz, N = nx * ny * nz;
  double v[2] = {0.0, 0.0};
  GRID_STRIDE(c, N) {
    const int i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
    const int pc = TPLS_IDX(g, i + 1, j + 1, k + 1);
    double bb = -rhs_p[pc];
    if (i == 0) {
      // pressure_solver.F90:280-286: b(i,0,k) = (dx/dt)(u_inlet(k-1)-u3(0,i,k-1))/dy
      const int ju = (j == 0) ? ny : j;  // u row (j+1)-1; row 0 is the copy of row ny
      const double bi = dxdt_over_dy * (uin[k] - u3[TPLS_IDX(g, 0, ju, k)]);
      bin[j + ny * k] = bi;
      bb += bi * rdy;
    }
    b[c] = bb;
    const double p0 = pold[pc];
    x0[c] = p0;
    v[0] += bb;
    v[1] += p0;
  }
  double tot[2];
  if (reduce_last<2>(v, part, counter, tot) && threadIdx.x == 0) {
    s[S_SUMB] = tot[0];
    s[S_SUMX0] = tot[1];
  }
}

// b -= mean(b); r = b - A x; ||b||^2, ||r||^2
__global__ void __launch_bounds__(PB)
    k_init_r(int nx, int ny, int nz, double cx, double cy, double cz, double invN, double *s,
             double *__restrict__ b, const double *__restrict__ x, double *__restrict__ r, double *part,
             unsigned *counter) {
  const int N = nx * ny * nz;
  const double mb = s[S_SUMB] * invN;
  double v[2] = {0.0, 0.0};
  GRID_STRIDE(c, N) {
    const int i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
    const double bb = b[c] - mb;
    b[c] = bb;
    const double rr = bb - applyA(x, i, j, k, nx, ny, nz, cx, cy, cz);
    r[c] = rr;
    v[0] += bb * bb;
    v[1] += rr * rr;
  }
  double tot[2];
  if (reduce_last<2>(v, part, counter, tot) && threadIdx.x == 0) {
    s[S_BB] = tot[0];
    s[S_RR] = tot[1];
  }
}

// sum z, sum r, r.z -> mean(z), rz_new = r.(z - mean z), beta = rz_new/rz
__global__ void __launch_bounds__(PB)
    k_zdot(int N, double invN, int first, const double *__restrict__ r, const double *__restrict__ z,
           double *part, unsigned *counter, double *s) {
  double v[3] = {0.0, 0.0, 0.0};
  GRID_STRIDE(c, N) {
    const double zz = z[c], rr = r[c];
    v[0] += zz;
    v[1] += rr;
    v[2] += rr * zz;
  }
  double tot[3];
  if (reduce_last<3>(v, part, counter, tot) && threadIdx.x == 0) {
    const double zm = tot[0] * invN;
    const double rzn = tot[2] - zm * tot[1];
    s[S_BETA] = first ? 0.0 : rzn / s[S_RZ];
    s[S_ZMEAN] = zm;
    s[S_RZ] = rzn;
  }
}

// p = (z - mean z) + beta p
__global__ void __launch_bounds__(PB)
    k_pupdate(int N, const double *__restrict__ s, const double *__restrict__ z, double *__restrict__ p) {
  const double zm = s[S_ZMEAN], beta = s[S_BETA];
  const int c = blockIdx.x * PB + threadIdx.x;
  if (c < N) p[c] = (z[c] - zm) + beta * p[c];
}

// q = A p; p.q -> alpha = rz / p.q
__global__ void __launch_bounds__(PB)
    k_apply_dot(int nx, int ny, int nz, double cx, double cy, double cz, const double *__restrict__ p,
                double *__restrict__ q, double *part, unsigned *counter, double *s) {
  const int N = nx * ny * nz;
  double v[1] = {0.0};
  GRID_STRIDE(c, N) {
    const int i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
    const double a = applyA(p, i, j, k, nx, ny, nz, cx, cy, cz);
    q[c] = a;
    v[0] += p[c] * a;
  }
  double tot[1];
  if (reduce_last<1>(v, part, counter, tot) && threadIdx.x == 0) s[S_ALPHA] = s[S_RZ] / tot[0];
}

// x += alpha p; r -= alpha q; ||r||^2
__global__ void __launch_bounds__(PB)
    k_axpy(int N, double *s, const double *__restrict__ p, const double *__restrict__ q,
           double *__restrict__ x, double *__restrict__ r, double *part, unsigned *counter) {
  const double alpha = s[S_ALPHA];
  double v[1] = {0.0};
  GRID_STRIDE(c, N) {
    x[c] += alpha * p[c];
    const double rr = r[c] - alpha * q[c];
    r[c] = rr;
    v[0] += rr * rr;
  }
  double tot[1];
  if (reduce_last<1>(v, part, counter, tot) && threadIdx.x == 0) s[S_RR] = tot[0];
}

__global__ void __launch_bounds__(PB)
    k_sumx(int N, const double *__restrict__ x, double *part, unsigned *counter, double *s) {
  double v[1] = {0.0};
  GRID_STRIDE(c, N) v[0] += x[c];
  double tot[1];
  if (reduce_last<1>(v, part, counter, tot) && threadIdx.x == 0) s[S_SUMX] = tot[0];
}

// write the solution back into the full p-grid array with every ghost
// value rebuilt from its 2-point row, and the constant fixed.
__global__ void k_writeback(Geo g, double dy, double invN, const double *__restrict__ s,
                            const double *__restrict__ x, const double *__restrict__ bin,
                            double *__restrict__ pres) {
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 4 + threadIdx.y, k = blockIdx.z;
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  if (i > nx + 1 || j > ny + 1) return;
  const double shift = (s[S_SUMX0] - s[S_SUMX]) * invN;
  const int jj = wrapy(j, ny) - 1;
  const int kk = (k == 0) ? 0 : ((k == nz + 1) ? nz - 1 : k - 1);  // z ghost planes copy
  double v;
  if (i == 0) {
    v = x[nx * (jj + ny * kk)] + shift + dy * bin[jj + ny * kk];
  } else {
    const int ii = (i == nx + 1) ? nx - 1 : i - 1;
    v = x[ii + nx * (jj + ny * kk)] + shift;
  }
  pres[TPLS_IDX(g, i, j, k)] = v;
}

// ---------------------------------------------------------------------------
// multigrid kernels
struct LevArgs {
  int nx, ny, nz;
  double cx, cy, cz;
};

// one damped z-line Jacobi sweep: eo = (1-w) ei + w Dline^{-1}(b - N ei);
// zero_init: ei == 0.
constexpr int LJB = 64;  // threads per block of the line smoother (one column each)

__global__ void __launch_bounds__(LJB)
    k_line_jacobi(LevArgs L, double omega, double one_m_omega, int zero_init,
                  const double *__restrict__ thomas, const double *__restrict__ b,
                  const double *__restrict__ ei, double *__restrict__ t, double *__restrict__ eo) {
  const int col = blockIdx.x * LJB + threadIdx.x;
  const int nx = L.nx, ny = L.ny, nz = L.nz;
  if (col >= nx * ny) return;
  const int i = col % nx, j = col / nx;
  const int cls = (nx == 1) ? 1 : ((i == 0) ? 0 : ((i == nx - 1) ? 2 : 1));
  const double *th = thomas + (size_t)cls * nz * 2;
  const int plane = nx * ny;
  const int jm = (j > 0) ? -nx : nx * (ny - 1), jp = (j < ny - 1) ? nx : -nx * (ny - 1);
  double y = 0.0;
  for (int k = 0; k < nz; k++) {
    const int c = col + plane * k;
    double rhs = b[c];
    if (!zero_init) {
      double nb = L.cy * (ei[c + jm] + ei[c + jp]);
      if (i > 0) nb += L.cx * ei[c - 1];
      if (i < nx - 1) nb += L.cx * ei[c + 1];
      rhs += nb;
    }
    y = (rhs + L.cz * y) * th[2 * k + 1];
    t[c] = y;
  }
  double xn = 0.0;
  for (int k = nz - 1; k >= 0; k--) {
    const int c = col + plane * k;
    xn = t[c] - ((k < nz - 1) ? th[2 * k] * xn : 0.0);
    eo[c] = zero_init ? omega * xn : one_m_omega * ei[c] + omega * xn;
  }
}

// The same sweep for 32 columns per block in three phases: all threads
// assemble the line right-hand sides into shared memory, one warp runs the
// Thomas forward/backward substitution in shared memory, all threads write
// the damped result.  Dynamic shared memory: nz * 32 doubles.
constexpr int LJ2_T = 256;

__global__ void __launch_bounds__(LJ2_T)
    k_line_jacobi2(LevArgs L, double omega, double one_m_omega, int zero_init,
                   const double *__restrict__ thomas, const double *__restrict__ b,
                   const double *__restrict__ ei, double *__restrict__ eo) {
  extern __shared__ double buf[];  // [nz][32]
  const int nx = L.nx, ny = L.ny, nz = L.nz, ncol = nx * ny, plane = nx * ny;
  const int col0 = blockIdx.x * 32;
  for (int t = threadIdx.x; t < nz * 32; t += LJ2_T) {
    const int k = t >> 5, cl = t & 31, col = col0 + cl;
    double rhs = 0.0;
    if (col < ncol) {
      const int c = col + plane * k;
      rhs = b[c];
      if (!zero_init) {
        const int i = col % nx, j = col / nx;
        const int jm = (j > 0) ? -nx : nx * (ny - 1), jp = (j < ny - 1) ? nx : -nx * (ny - 1);
        double nb = L.cy * (ei[c + jm] + ei[c + jp]);
        if (i > 0) nb += L.cx * ei[c - 1];
        if (i < nx - 1) nb += L.cx * ei[c + 1];
        rhs += nb;
      }
    }
    buf[t] = rhs;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int col = col0 + threadIdx.x;
    if (col < ncol) {
      const int i = col % nx;
      const int cls = (nx == 1) ? 1 : ((i == 0) ? 0 : ((i == nx - 1) ? 2 : 1));
      const double *th = thomas + (size_t)cls * nz * 2;
      double y = 0.0;
      for (int k = 0; k < nz; k++) {
        y = (buf[k * 32 + threadIdx.x] + L.cz * y) * th[2 * k + 1];
        buf[k * 32 + threadIdx.x] = y;
      }
      double xn = y;
      for (int k = nz - 2; k >= 0; k--) {
        xn = buf[k * 32 + threadIdx.x] - th[2 * k] * xn;
        buf[k * 32 + threadIdx.x] = xn;
      }
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nz * 32; t += LJ2_T) {
    const int k = t >> 5, col = col0 + (t & 31);
    if (col < ncol) {
      const int c = col + plane * k;
      eo[c] = zero_init ? omega * buf[t] : one_m_omega * ei[c] + omega * buf[t];
    }
  }
}

__global__ void k_residual(LevArgs L, const double *__restrict__ b, const double *__restrict__ e,
                           double *__restrict__ r) {
  const int c = blockIdx.x * PB + threadIdx.x;
  const int nx = L.nx, ny = L.ny, nz = L.nz;
  if (c >= nx * ny * nz) return;
  const int i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
  r[c] = b[c] - applyA(e, i, j, k, nx, ny, nz, L.cx, L.cy, L.cz);
}

// 1-D restriction stencil: fine indices and weights contributing to coarse c
__device__ __forceinline__ int rstencil(int c, int nc, int coarsened, int periodic, int *f,
                                        double *w) {
  if (!coarsened) {
    f[0] = c;
    w[0] = 1.0;
    return 1;
  }
  const int nf = 2 * nc;
  int m = 0;
  f[m] = 2 * c;
  w[m++] = (!periodic && c == 0) ? 1.0 : 0.75;
  f[m] = 2 * c + 1;
  w[m++] = (!periodic && c == nc - 1) ? 1.0 : 0.75;
  if (c > 0) { f[m] = 2 * c - 1; w[m++] = 0.25; }
  else if (periodic) { f[m] = nf - 1; w[m++] = 0.25; }
  if (c < nc - 1) { f[m] = 2 * c + 2; w[m++] = 0.25; }
  else if (periodic) { f[m] = 0; w[m++] = 0.25; }
  return m;
}

__global__ void k_restrict(LevArgs F, LevArgs C, int cxs, int cys, int czs, double scale,
                           const double *__restrict__ rf, double *__restrict__ bc) {
  const int c = blockIdx.x * PB + threadIdx.x;
  if (c >= C.nx * C.ny * C.nz) return;
  const int I = c % C.nx, J = (c / C.nx) % C.ny, K = c / (C.nx * C.ny);
  int fx[4], fy[4], fz[4];
  double wx[4], wy[4], wz[4];
  const int mx = rstencil(I, C.nx, cxs, 0, fx, wx);
  const int my = rstencil(J, C.ny, cys, 1, fy, wy);
  const int mz = rstencil(K, C.nz, czs, 0, fz, wz);
  double acc = 0.0;
  for (int a = 0; a < mz; a++)
    for (int bq = 0; bq < my; bq++) {
      const double wzy = wz[a] * wy[bq];
      const double *row = rf + F.nx * (fy[bq] + F.ny * fz[a]);
      double sx = 0.0;
      for (int q = 0; q < mx; q++) sx += wx[q] * row[fx[q]];
      acc += wzy * sx;
    }
  bc[c] = acc * scale;
}

// 1-D prolongation: coarse indices and weights for fine f
__device__ __forceinline__ int pstencil(int f, int nc, int coarsened, int periodic, int *c,
                                        double *w) {
  if (!coarsened) {
    c[0] = f;
    w[0] = 1.0;
    return 1;
  }
  const int c0 = f >> 1;
  int c1 = (f & 1) ? c0 + 1 : c0 - 1;
  if (c1 < 0 || c1 >= nc) {
    if (!periodic) {
      c[0] = c0;
      w[0] = 1.0;
      return 1;
    }
    c1 = (c1 < 0) ? c1 + nc : c1 - nc;
  }
  c[0] = c0;
  w[0] = 0.75;
  c[1] = c1;
  w[1] = 0.25;
  return 2;
}

__global__ void k_prolong_add(LevArgs F, LevArgs C, int cxs, int cys, int czs,
                              const double *__restrict__ ec, double *__restrict__ ef) {
  const int c = blockIdx.x * PB + threadIdx.x;
  if (c >= F.nx * F.ny * F.nz) return;
  const int i = c % F.nx, j = (c / F.nx) % F.ny, k = c / (F.nx * F.ny);
  int cx[2], cy[2], cz[2];
  double wx[2], wy[2], wz[2];
  const int mx = pstencil(i, C.nx, cxs, 0, cx, wx);
  const int my = pstencil(j, C.ny, cys, 1, cy, wy);
  const int mz = pstencil(k, C.nz, czs, 0, cz, wz);
  double acc = 0.0;
  for (int a = 0; a < mz; a++)
    for (int bq = 0; bq < my; bq++) {
      const double *row = ec + C.nx * (cy[bq] + C.ny * cz[a]);
      double sx = 0.0;
      for (int q = 0; q < mx; q++) sx += wx[q] * row[cx[q]];
      acc += wz[a] * wy[bq] * sx;
    }
  ef[c] += acc;
}

// coarsest grid: e = Cinv b (one block)
__global__ void k_coarse_solve(int n, const double *__restrict__ cinv, const double *__restrict__ b,
                               double *__restrict__ e) {
  __shared__ double sb[512];
  for (int a = threadIdx.x; a < n; a += blockDim.x) sb[a] = b[a];
  __syncthreads();
  for (int a = threadIdx.x; a < n; a += blockDim.x) {
    const double *row = cinv + (size_t)a * n;
    double acc = 0.0;
    for (int q = 0; q < n; q++) acc += row[q] * sb[q];
    e[a] = acc;
  }
}

// ---------------------------------------------------------------------------
// host side

static void neumann_basis(int n, std::vector<double> &Q, std::vector<double> &lam) {
  Q.assign((size_t)n * n, 0.0);
  lam.assign(n, 0.0);
  for (int k = 0; k < n; k++) {
    const double c = (k == 0) ? sqrt(1.0 / n) : sqrt(2.0 / n);
    for (int i = 0; i < n; i++) Q[(size_t)k * n + i] = c * cos(M_PI * k * (i + 0.5) / n);
    const double s = sin(M_PI * k / (2.0 * n));
    lam[k] = 4.0 * s * s;
  }
}
static void periodic_basis(int n, std::vector<double> &Q, std::vector<double> &lam) {
  Q.assign((size_t)n * n, 0.0);
  lam.assign(n, 0.0);
  int idx = 0;
  for (int i = 0; i < n; i++) Q[i] = sqrt(1.0 / n);
  lam[idx++] = 0.0;
  for (int m = 1; 2 * m < n; m++) {
    const double s = sin(M_PI * m / n);
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

// dense pseudo-inverse of the separable level operator
static std::vector<double> coarse_pinv(const PLevel &L) {
  std::vector<double> Qx, Qy, Qz, lx, ly, lz;
  neumann_basis(L.nx, Qx, lx);
  periodic_basis(L.ny, Qy, ly);
  neumann_basis(L.nz, Qz, lz);
  const int n = L.n;
  std::vector<double> M((size_t)n * n, 0.0);
  for (int mz = 0; mz < L.nz; mz++)
    for (int my = 0; my < L.ny; my++)
      for (int mx = 0; mx < L.nx; mx++) {
        const double lam = L.cx * lx[mx] + L.cy * ly[my] + L.cz * lz[mz];
        if (mx == 0 && my == 0 && mz == 0) continue;
        const double il = 1.0 / lam;
        std::vector<double> v(n);
        for (int k = 0; k < L.nz; k++)
          for (int j = 0; j < L.ny; j++)
            for (int i = 0; i < L.nx; i++)
              v[i + L.nx * (j + L.ny * k)] =
                  Qx[(size_t)mx * L.nx + i] * Qy[(size_t)my * L.ny + j] * Qz[(size_t)mz * L.nz + k];
        for (int a = 0; a < n; a++) {
          const double va = v[a] * il;
          double *row = &M[(size_t)a * n];
          for (int b = 0; b < n; b++) row[b] += va * v[b];
        }
      }
  return M;
}

// Thomas factors of the z-line matrix per x-class (first, interior, last)
static std::vector<double> thomas_factors(const PLevel &L) {
  std::vector<double> th((size_t)3 * L.nz * 2);
  for (int cls = 0; cls < 3; cls++) {
    double nbx = 2.0;
    if (L.nx == 1) nbx = 0.0;
    else if (cls != 1) nbx = 1.0;
    const double dxy = L.cx * nbx + 2.0 * L.cy;
    double cprev = 0.0;
    for (int k = 0; k < L.nz; k++) {
      double nbz = 2.0;
      if (L.nz == 1) nbz = 0.0;
      else if (k == 0 || k == L.nz - 1) nbz = 1.0;
      const double d = dxy + L.cz * nbz;
      const double den = (k == 0) ? d : d + L.cz * cprev;  // d - a*c'_{k-1}, a = -cz
      const double cp = -L.cz / den;
      th[((size_t)cls * L.nz + k) * 2 + 0] = cp;
      th[((size_t)cls * L.nz + k) * 2 + 1] = 1.0 / den;
      cprev = cp;
    }
  }
  return th;
}

#define PCK(x)                        \
  do {                                \
    cudaError_t e_ = (x);             \
    if (e_ != cudaSuccess) return e_; \
  } while (0)

cudaError_t poisson_create(const Geo &g, double cx, double cy, double cz,
                           PoissonSolver **out) {
  PoissonSolver *S = new PoissonSolver();
  S->nx = g.nx;
  S->ny = g.ny;
  S->nz = g.nz;
  S->N = g.nx * g.ny * g.nz;
  PLevel L0;
  L0.nx = g.nx;
  L0.ny = g.ny;
  L0.nz = g.nz;
  L0.n = S->N;
  L0.cxs = L0.cys = L0.czs = 0;
  L0.cx = cx;
  L0.cy = cy;
  L0.cz = cz;
  S->lv.push_back(L0);
  while (true) {
    const PLevel &f = S->lv.back();
    if (f.n <= 512) break;
    PLevel c;
    c.cxs = (f.nx % 2 == 0 && f.nx >= 4);
    c.cys = (f.ny % 2 == 0 && f.ny >= 4);
    c.czs = (f.nz % 2 == 0 && f.nz >= 4);
    if (!c.cxs && !c.cys && !c.czs) break;
    c.nx = c.cxs ? f.nx / 2 : f.nx;
    c.ny = c.cys ? f.ny / 2 : f.ny;
    c.nz = c.czs ? f.nz / 2 : f.nz;
    c.n = c.nx * c.ny * c.nz;
    c.cx = c.cxs ? f.cx / 4.0 : f.cx;
    c.cy = c.cys ? f.cy / 4.0 : f.cy;
    c.cz = c.czs ? f.cz / 4.0 : f.cz;
    S->lv.push_back(c);
  }
  for (size_t l = 0; l < S->lv.size(); l++) {
    PLevel &L = S->lv[l];
    const size_t bytes = sizeof(double) * (size_t)L.n;
    if (l > 0) PCK(cudaMalloc(&L.b, bytes));
    PCK(cudaMalloc(&L.e, bytes));
    PCK(cudaMalloc(&L.e2, bytes));
    PCK(cudaMalloc(&L.r, bytes));
    PCK(cudaMalloc(&L.t, bytes));
    std::vector<double> th = thomas_factors(L);
    PCK(cudaMalloc(&L.thomas, th.size() * sizeof(double)));
    PCK(cudaMemcpy(L.thomas, th.data(), th.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  PCK(cudaFuncSetAttribute(k_line_jacobi2, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  const PLevel &C = S->lv.back();
  if (C.n <= 512) {
    std::vector<double> M = coarse_pinv(C);
    PCK(cudaMalloc(&S->cinv, M.size() * sizeof(double)));
    PCK(cudaMemcpy(S->cinv, M.data(), M.size() * sizeof(double), cudaMemcpyHostToDevice));
  } else {
    S->coarse_sweeps = 40;
  }
  const size_t nb = sizeof(double) * (size_t)S->N;
  PCK(cudaMalloc(&S->x, nb));
  PCK(cudaMalloc(&S->r, nb));
  PCK(cudaMalloc(&S->z, nb));
  PCK(cudaMalloc(&S->p, nb));
  PCK(cudaMalloc(&S->q, nb));
  PCK(cudaMalloc(&S->bvec, nb));
  PCK(cudaMalloc(&S->bin, sizeof(double) * (size_t)g.ny * g.nz));
  S->rblk = nblocks(S->N) < 1216 ? nblocks(S->N) : 1216;  // 8 blocks per SM on 152 SMs
  PCK(cudaMalloc(&S->part, sizeof(double) * (size_t)S->rblk * 3));
  PCK(cudaMalloc(&S->counter, sizeof(unsigned)));
  PCK(cudaMemset(S->counter, 0, sizeof(unsigned)));
  PCK(cudaMalloc(&S->s, sizeof(double) * S_COUNT));
  PCK(cudaMemset(S->s, 0, sizeof(double) * S_COUNT));
  PCK(cudaMallocHost(&S->s_host, sizeof(double) * S_COUNT));
  *out = S;
  return cudaSuccess;
}

void poisson_destroy(PoissonSolver *S) {
  if (!S) return;
  for (PLevel &L : S->lv) {
    cudaFree(L.b);
    cudaFree(L.e);
    cudaFree(L.e2);
    cudaFree(L.r);
    cudaFree(L.t);
    cudaFree(L.thomas);
  }
  cudaFree(S->cinv);
  cudaFree(S->x);
  cudaFree(S->r);
  cudaFree(S->z);
  cudaFree(S->p);
  cudaFree(S->q);
  cudaFree(S->bvec);
  cudaFree(S->bin);
  cudaFree(S->part);
  cudaFree(S->counter);
  cudaFree(S->s);
  cudaFreeHost(S->s_host);
  delete S;
}

int poisson_levels(const PoissonSolver *S) { return (int)S->lv.size(); }

static LevArgs largs(const PLevel &L) {
  LevArgs a;
  a.nx = L.nx;
  a.ny = L.ny;
  a.nz = L.nz;
  a.cx = L.cx;
  a.cy = L.cy;
  a.cz = L.cz;
  return a;
}

static void line_sweep(const PLevel &L, const LevArgs &A, double w, double w1, int zero_init,
                       const double *b, const double *ei, double *eo, cudaStream_t st) {
  const size_t smem = sizeof(double) * 32 * (size_t)L.nz;
  if (smem <= 200 * 1024) {
    k_line_jacobi2<<<(L.nx * L.ny + 31) / 32, LJ2_T, smem, st>>>(A, w, w1, zero_init, L.thomas, b, ei, eo);
  } else {
    k_line_jacobi<<<(L.nx * L.ny + LJB - 1) / LJB, LJB, 0, st>>>(A, w, w1, zero_init, L.thomas, b, ei, L.t,
                                                                 eo);
  }
}

// one symmetric V-cycle: out = M b0.  Every level pre-smooths into its
// scratch e2 (one damped line-Jacobi sweep from zero), restricts the
// residual, adds the prolonged coarse correction into e2 and post-smooths
// from e2 into its result buffer (out on the finest level, e elsewhere).
static cudaError_t vcycle(PoissonSolver *S, const double *b0, double *out, cudaStream_t st, long *nl) {
  const int nlev = (int)S->lv.size();
  const double w = S->omega, w1 = 1.0 - S->omega;
  for (int l = 0; l < nlev; l++) {
    PLevel &L = S->lv[l];
    const double *b = (l == 0) ? b0 : L.b;
    double *res = (l == 0) ? out : L.e;
    const LevArgs A = largs(L);
    if (l == nlev - 1) {
      if (S->cinv) {
        k_coarse_solve<<<1, 256, 0, st>>>(L.n, S->cinv, b, res);
        (*nl)++;
      } else {
        double *cur = L.e2, *oth = res;
        line_sweep(L, A, w, w1, 1, b, nullptr, cur, st);
        (*nl)++;
        for (int sw = 1; sw < S->coarse_sweeps; sw++) {
          line_sweep(L, A, w, w1, 0, b, cur, oth, st);
          (*nl)++;
          double *tmp = cur;
          cur = oth;
          oth = tmp;
        }
        if (cur != res) PCK(cudaMemcpyAsync(res, cur, sizeof(double) * L.n, cudaMemcpyDeviceToDevice, st));
      }
      PCK(cudaGetLastError());
      break;
    }
    line_sweep(L, A, w, w1, 1, b, nullptr, L.e2, st);
    k_residual<<<nblocks(L.n), PB, 0, st>>>(A, b, L.e2, L.r);
    const PLevel &C = S->lv[l + 1];
    const double scale = 1.0 / (double)((C.cxs ? 2 : 1) * (C.cys ? 2 : 1) * (C.czs ? 2 : 1));
    k_restrict<<<nblocks(C.n), PB, 0, st>>>(A, largs(C), C.cxs, C.cys, C.czs, scale, L.r, C.b);
    *nl += 3;
    PCK(cudaGetLastError());
  }
  for (int l = nlev - 2; l >= 0; l--) {
    PLevel &L = S->lv[l];
    const PLevel &C = S->lv[l + 1];
    const double *b = (l == 0) ? b0 : L.b;
    double *res = (l == 0) ? out : L.e;
    const LevArgs A = largs(L);
    k_prolong_add<<<nblocks(L.n), PB, 0, st>>>(A, largs(C), C.cxs, C.cys, C.czs, C.e, L.e2);
    line_sweep(L, A, w, w1, 0, b, L.e2, res, st);
    *nl += 2;
    PCK(cudaGetLastError());
  }
  return cudaSuccess;
}

cudaError_t poisson_solve(PoissonSolver *S, const Geo &g, const Phys &ph,
                          const double *rhs_p, const double *u3,
                          const double *u_inlet, const double *pres_old,
                          double *pres, double rtol, int maxits, int *its,
                          double *rnorm, double *bnorm, int *reason,
                          cudaStream_t st, long *nl) {
  const int N = S->N, rb = S->rblk;
  const double invN = 1.0 / (double)N;
  const PLevel &F = S->lv[0];
  k_build_b<<<rb, PB, 0, st>>>(g, (ph.dx / ph.dt) / ph.dy, 1.0 / ph.dy, rhs_p, u3, u_inlet, pres_old,
                               S->bvec, S->x, S->bin, S->part, S->counter, S->s);
  k_init_r<<<rb, PB, 0, st>>>(F.nx, F.ny, F.nz, F.cx, F.cy, F.cz, invN, S->s, S->bvec, S->x, S->r, S->part,
                              S->counter);
  *nl += 2;
  PCK(cudaGetLastError());
  PCK(cudaMemcpyAsync(S->s_host, S->s, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, st));
  PCK(cudaStreamSynchronize(st));
  const double bb = sqrt(S->s_host[S_BB]);
  double rr = sqrt(S->s_host[S_RR]);
  *bnorm = bb;
  int it = 0, rsn = 0;
  const double target = rtol * bb;
  if (!(rr == rr)) rsn = TPLS_KSP_DIVERGED_NAN;
  else if (rr <= target || bb == 0.0) rsn = TPLS_KSP_CONVERGED_RTOL;
  const int nb = nblocks(N);
  while (rsn == 0) {
    PCK(vcycle(S, S->r, S->z, st, nl));
    k_zdot<<<rb, PB, 0, st>>>(N, invN, it == 0, S->r, S->z, S->part, S->counter, S->s);
    k_pupdate<<<nb, PB, 0, st>>>(N, S->s, S->z, S->p);
    k_apply_dot<<<rb, PB, 0, st>>>(F.nx, F.ny, F.nz, F.cx, F.cy, F.cz, S->p, S->q, S->part, S->counter, S->s);
    k_axpy<<<rb, PB, 0, st>>>(N, S->s, S->p, S->q, S->x, S->r, S->part, S->counter);
    *nl += 4;
    PCK(cudaGetLastError());
    it++;
    PCK(cudaMemcpyAsync(S->s_host + S_RR, S->s + S_RR, sizeof(double), cudaMemcpyDeviceToHost, st));
    PCK(cudaStreamSynchronize(st));
    rr = sqrt(S->s_host[S_RR]);
    if (!(rr == rr)) rsn = TPLS_KSP_DIVERGED_NAN;
    else if (rr <= target) rsn = TPLS_KSP_CONVERGED_RTOL;
    else if (it >= maxits) rsn = TPLS_KSP_DIVERGED_ITS;
  }
  k_sumx<<<rb, PB, 0, st>>>(N, S->x, S->part, S->counter, S->s);
  dim3 grd((g.nx + 2 + 31) / 32, (g.ny + 2 + 3) / 4, g.nz + 2);
  k_writeback<<<grd, dim3(32, 4), 0, st>>>(g, ph.dy, invN, S->s, S->x, S->bin, pres);
  *nl += 2;
  PCK(cudaGetLastError());
  *its = it;
  *rnorm = rr;
  *reason = rsn;
  return cudaSuccess;
}

}  // namespace tpls
