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

// Level vectors are stored in the level type of the solver (double, or
// float for the FP32 preconditioner of the FP32-mixed form); void pointers
// here, typed at each launch.
struct PLevel {
  int nx, ny, nz, n;
  int cxs, cys, czs;     // this level was coarsened in x/y/z from the finer one
  double cx, cy, cz;
  void *b = nullptr, *e = nullptr, *e2 = nullptr, *r = nullptr, *t = nullptr;
  void *thomas = nullptr;  // [3 classes][nz][2] = (cprime, inv_den)
  int point = 0;  // near-isotropic level: red-black Gauss-Seidel instead of z-lines
  double invd[3][3];  // point smoother: 1/diagonal by x class (first, interior, last) and z class
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
  int fp32 = 0;              // multigrid levels in FP32 (CG stays FP64)
  cudaStream_t side = nullptr;  // capture stream of the WHILE body
};

// device scalars of the CG iteration
// S_IT: iterations of the current solve; S_REASON: its KSP-style reason (0
// while iterating); S_WORST: lowest reason since the last stats read;
// S_ITS_TOTAL: iterations since the solver was created.
enum {
  S_SUMB = 0, S_SUMX0, S_BB, S_RR, S_RZ, S_ZMEAN, S_BETA, S_ALPHA, S_SUMX,
  S_TARGET, S_IT, S_REASON, S_WORST, S_ITS_TOTAL, S_COUNT
};

// Convergence test of pressure_solver.F90's KSP settings on the device, by
// the last block of a reduction: NaN, ||r|| <= rtol ||b||, or maxits.  With a
// graph, the WHILE node's condition is set here, so a captured solve needs
// no host round trip.
struct CgCtl {
  int maxits;
  int use_cond;
  cudaGraphConditionalHandle cond;
};

__device__ __forceinline__ void cg_decide(double *s, double rr2, int it, const CgCtl &ctl, bool init) {
  const double rr = sqrt(rr2);
  int rsn = 0;
  if (!(rr == rr)) rsn = TPLS_KSP_DIVERGED_NAN;
  else if (rr <= s[S_TARGET] || (init && s[S_BB] == 0.0)) rsn = TPLS_KSP_CONVERGED_RTOL;
  else if (!init && it >= ctl.maxits) rsn = TPLS_KSP_DIVERGED_ITS;
  s[S_IT] = (double)it;
  s[S_REASON] = (double)rsn;
  if (rsn != 0) {
    if ((double)rsn < s[S_WORST]) s[S_WORST] = (double)rsn;
    s[S_ITS_TOTAL] += (double)it;
  }
  if (ctl.use_cond) cudaGraphSetConditional(ctl.cond, rsn == 0 ? 1u : 0u);
}

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

template <typename R, typename TE>
__device__ __forceinline__ R applyA(const TE *__restrict__ e, int i, int j, int k, int nx, int ny, int nz,
                                    R cx, R cy, R cz) {
  const int c = i + nx * (j + ny * k);
  const R v = (R)e[c];
  const R xm = (i > 0) ? (R)e[c - 1] : v, xp = (i < nx - 1) ? (R)e[c + 1] : v;
  const R ym = (R)e[c + nx * ((j > 0) ? -1 : ny - 1)];
  const R yp = (R)e[c + nx * ((j < ny - 1) ? 1 : 1 - ny)];
  const R zm = (k > 0) ? (R)e[c - nx * ny] : v, zp = (k < nz - 1) ? (R)e[c + nx * ny] : v;
  // (2cx + 2cy + 2cz) v - cx (xm + xp) - cy (ym + yp) - cz (zm + zp): seven
  // FP64 operations (the FP64 pipe bounds these kernels on GB300)
  const R d = (R)2 * (cx + cy + cz);
  R a = d * v;
  a = fma(-cx, xm + xp, a);
  a = fma(-cy, ym + yp, a);
  return fma(-cz, zm + zp, a);
}

#define GRID_STRIDE(c, N) for (int c = blockIdx.x * PB + threadIdx.x; c < (N); c += gridDim.x * PB)
// rows (j, k) of the compact nx*ny*nz grid handed to warps in a fixed
// order, lanes striding over i; row = j + ny k, c = i + nx row
#define ROW_LOOP(nx, ny, nz)                                                                          \
  for (int row = blockIdx.x * (PB / 32) + (int)(threadIdx.x >> 5); row < (ny) * (nz);                \
       row += gridDim.x * (PB / 32))                                                                 \
    for (int j = row % (ny), k = row / (ny), i = (int)(threadIdx.x & 31); i < (nx); i += 32)

// b (compact interior) = -RHS_p + inlet contribution; x0 = p_old interior;
// sums of b and x0.
template <typename TU>
__global__ void __launch_bounds__(PB)
    k_build_b(Geo g, double dxdt_over_dy, double rdy, const double *__restrict__ rhs_p,
              const TU *__restrict__ u3, const double *__restrict__ uin,
              const double *__restrict__ pold, double *__restrict__ b, double *__restrict__ x0,
              double *__restrict__ bin, double *part, unsigned *counter, double *s) {
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  double v[2] = {0.0, 0.0};
  ROW_LOOP(nx, ny, nz) {
    const int c = i + nx * row;
    const int pc = TPLS_IDX(g, i + 1, j + 1, k + 1);
    double bb = -rhs_p[pc];
    if (i == 0) {
      // pressure_solver.F90:280-286: b(i,0,k) = (dx/dt)(u_inlet(k-1)-u3(0,i,k-1))/dy
      const int ju = (j == 0) ? ny : j;  // u row (j+1)-1; row 0 is the copy of row ny
      const double bi = dxdt_over_dy * (uin[k] - (double)u3[TPLS_IDX(g, 0, ju, k)]);
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
    k_init_r(int nx, int ny, int nz, double cx, double cy, double cz, double invN, double rtol, CgCtl ctl,
             double *s, double *__restrict__ b, const double *__restrict__ x, double *__restrict__ r, double *part,
             unsigned *counter) {
  const double mb = s[S_SUMB] * invN;
  double v[2] = {0.0, 0.0};
  ROW_LOOP(nx, ny, nz) {
    const int c = i + nx * row;
    const double bb = b[c] - mb;
    b[c] = bb;
    const double rr = bb - applyA<double, double>(x, i, j, k, nx, ny, nz, cx, cy, cz);
    r[c] = rr;
    v[0] += bb * bb;
    v[1] += rr * rr;
  }
  double tot[2];
  if (reduce_last<2>(v, part, counter, tot) && threadIdx.x == 0) {
    s[S_BB] = tot[0];
    s[S_RR] = tot[1];
    s[S_TARGET] = rtol * sqrt(tot[0]);
    cg_decide(s, tot[1], 0, ctl, true);
  }
}

// sum z, sum r, r.z -> mean(z), rz_new = r.(z - mean z), beta = rz_new/rz
__global__ void __launch_bounds__(PB)
    k_zdot(int N, double invN, const double *__restrict__ r, const double *__restrict__ z, double *part,
           unsigned *counter, double *s) {
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
    s[S_BETA] = (s[S_IT] == 0.0) ? 0.0 : rzn / s[S_RZ];
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
  double v[1] = {0.0};
  ROW_LOOP(nx, ny, nz) {
    const int c = i + nx * row;
    const double a = applyA<double, double>(p, i, j, k, nx, ny, nz, cx, cy, cz);
    q[c] = a;
    v[0] += p[c] * a;
  }
  double tot[1];
  if (reduce_last<1>(v, part, counter, tot) && threadIdx.x == 0) s[S_ALPHA] = s[S_RZ] / tot[0];
}

// x += alpha p; r -= alpha q; ||r||^2
__global__ void __launch_bounds__(PB)
    k_axpy(int N, CgCtl ctl, double *s, const double *__restrict__ p, const double *__restrict__ q,
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
  if (reduce_last<1>(v, part, counter, tot) && threadIdx.x == 0) {
    s[S_RR] = tot[0];
    cg_decide(s, tot[0], (int)s[S_IT] + 1, ctl, false);
  }
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
// multigrid kernels.  R is the arithmetic type of the level (double, or
// float for the FP32 preconditioner); TB, TE, TO the storage types of the
// right-hand side, the input iterate and the output (the finest level of
// the FP32 preconditioner reads the FP64 CG residual and writes the FP64
// preconditioned vector directly).
template <typename R>
struct LevArgs {
  int nx, ny, nz;
  R cx, cy, cz;
};

// one damped z-line Jacobi sweep: eo = (1-w) ei + w Dline^{-1}(b - N ei);
// zero_init: ei == 0.
constexpr int LJB = 64;  // threads per block of the line smoother (one column each)

template <typename R, typename TB, typename TE, typename TO>
__global__ void __launch_bounds__(LJB)
    k_line_jacobi(LevArgs<R> L, R omega, R one_m_omega, int zero_init, const R *__restrict__ thomas,
                  const TB *__restrict__ b, const TE *__restrict__ ei, R *__restrict__ t, TO *__restrict__ eo) {
  const int col = blockIdx.x * LJB + threadIdx.x;
  const int nx = L.nx, ny = L.ny, nz = L.nz;
  if (col >= nx * ny) return;
  const int i = col % nx, j = col / nx;
  const int cls = (nx == 1) ? 1 : ((i == 0) ? 0 : ((i == nx - 1) ? 2 : 1));
  const R *th = thomas + (size_t)cls * nz * 2;
  const int plane = nx * ny;
  const int jm = (j > 0) ? -nx : nx * (ny - 1), jp = (j < ny - 1) ? nx : -nx * (ny - 1);
  R y = (R)0;
  for (int k = 0; k < nz; k++) {
    const int c = col + plane * k;
    R rhs = (R)b[c];
    if (!zero_init) {
      R nb = L.cy * ((R)ei[c + jm] + (R)ei[c + jp]);
      if (i > 0) nb += L.cx * (R)ei[c - 1];
      if (i < nx - 1) nb += L.cx * (R)ei[c + 1];
      rhs += nb;
    }
    y = (rhs + L.cz * y) * th[2 * k + 1];
    t[c] = y;
  }
  R xn = (R)0;
  for (int k = nz - 1; k >= 0; k--) {
    const int c = col + plane * k;
    xn = t[c] - ((k < nz - 1) ? th[2 * k] * xn : (R)0);
    eo[c] = (TO)(zero_init ? omega * xn : one_m_omega * (R)ei[c] + omega * xn);
  }
}

// The same sweep for 32 columns per block in three phases: all threads
// assemble the line right-hand sides into shared memory, one warp runs the
// Thomas forward/backward substitution in shared memory, all threads write
// the damped result.  Dynamic shared memory: nz * 32 values of R.
constexpr int LJ2_T = 256;

template <typename R, typename TB, typename TE, typename TO>
__global__ void __launch_bounds__(LJ2_T)
    k_line_jacobi2(LevArgs<R> L, R omega, R one_m_omega, int zero_init, const R *__restrict__ thomas,
                   const TB *__restrict__ b, const TE *__restrict__ ei, TO *__restrict__ eo) {
  extern __shared__ __align__(16) unsigned char lj2_raw[];
  R *buf = reinterpret_cast<R *>(lj2_raw);  // [nz][32]
  const int nx = L.nx, ny = L.ny, nz = L.nz, ncol = nx * ny, plane = nx * ny;
  const int col0 = blockIdx.x * 32;
  // every thread keeps one column (LJ2_T is a multiple of 32)
  const int mycol = col0 + (threadIdx.x & 31);
  const int ci = mycol % nx, cj = mycol / nx;
  const int jm = (cj > 0) ? -nx : nx * (ny - 1), jp = (cj < ny - 1) ? nx : -nx * (ny - 1);
  for (int t = threadIdx.x; t < nz * 32; t += LJ2_T) {
    const int k = t >> 5;
    R rhs = (R)0;
    if (mycol < ncol) {
      const int c = mycol + plane * k;
      rhs = (R)b[c];
      if (!zero_init) {
        R nb = L.cy * ((R)ei[c + jm] + (R)ei[c + jp]);
        if (ci > 0) nb += L.cx * (R)ei[c - 1];
        if (ci < nx - 1) nb += L.cx * (R)ei[c + 1];
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
      const R *th = thomas + (size_t)cls * nz * 2;
      R y = (R)0;
      for (int k = 0; k < nz; k++) {
        y = (buf[k * 32 + threadIdx.x] + L.cz * y) * th[2 * k + 1];
        buf[k * 32 + threadIdx.x] = y;
      }
      R xn = y;
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
      eo[c] = (TO)(zero_init ? omega * buf[t] : one_m_omega * (R)ei[c] + omega * buf[t]);
    }
  }
}

// point kernels of the V-cycle run on 3-D grids of 32x8 blocks (x, y) and
// one z plane per grid z index
constexpr int MG_BX = 32, MG_BY = 8;
static inline dim3 mg_grid(int nx, int ny, int nz) {
  return dim3((nx + MG_BX - 1) / MG_BX, (ny + MG_BY - 1) / MG_BY, nz);
}

// Red-black Gauss-Seidel half-sweep for near-isotropic levels (where
// z-lines buy nothing): points with (i + j + k) % 2 == colour get
// e = (b + sum of neighbour couplings) / diagonal; with `copy`, the other
// colour is copied from ein to eout so that eout holds the whole iterate.
// One thread per x pair.  zero_init: ein is zero (first half-sweep from a
// zero start).
template <typename R>
struct InvD {
  R v[3][3];
};

template <typename R, typename TB, typename TE, typename TO>
__global__ void k_rbgs(LevArgs<R> L, InvD<R> inv, int colour, int zero_init, int copy, const TB *__restrict__ b,
                       const TE *ein, TO *eout) {
  const int nx = L.nx, ny = L.ny, nz = L.nz;
  const int i2 = blockIdx.x * MG_BX + threadIdx.x, j = blockIdx.y * MG_BY + threadIdx.y, k = blockIdx.z;
  if (2 * i2 >= nx || j >= ny) return;
  const int plane = nx * ny;
  const int jm = (j > 0) ? -nx : nx * (ny - 1), jp = (j < ny - 1) ? nx : -nx * (ny - 1);
  const int zc = (nz == 1) ? 1 : ((k == 0) ? 0 : ((k == nz - 1) ? 2 : 1));
  for (int q = 0; q < 2; q++) {
    const int i = 2 * i2 + q;
    if (i >= nx) break;
    const int c = i + nx * j + plane * k;
    if (((i + j + k) & 1) == colour) {
      R acc = (R)b[c];
      if (!zero_init) {
        R sx = (R)0, sz = (R)0;
        if (i > 0) sx += (R)ein[c - 1];
        if (i < nx - 1) sx += (R)ein[c + 1];
        if (k > 0) sz += (R)ein[c - plane];
        if (k < nz - 1) sz += (R)ein[c + plane];
        acc = fma(L.cx, sx, acc);
        acc = fma(L.cy, (R)ein[c + jm] + (R)ein[c + jp], acc);
        acc = fma(L.cz, sz, acc);
      }
      const int xc = (nx == 1) ? 1 : ((i == 0) ? 0 : ((i == nx - 1) ? 2 : 1));
      eout[c] = (TO)(acc * inv.v[xc][zc]);
    } else if (copy) {
      eout[c] = (TO)ein[c];
    }
  }
}

template <typename R, typename TB, typename TE>
__global__ void k_residual(LevArgs<R> L, const TB *__restrict__ b, const TE *__restrict__ e, R *__restrict__ r) {
  const int nx = L.nx, ny = L.ny, nz = L.nz;
  const int i = blockIdx.x * MG_BX + threadIdx.x, j = blockIdx.y * MG_BY + threadIdx.y, k = blockIdx.z;
  if (i >= nx || j >= ny) return;
  const int c = i + nx * (j + ny * k);
  r[c] = (R)b[c] - applyA<R, TE>(e, i, j, k, nx, ny, nz, L.cx, L.cy, L.cz);
}

// 1-D restriction stencil: fine indices and weights contributing to coarse c
template <typename R>
__device__ __forceinline__ int rstencil(int c, int nc, int coarsened, int periodic, int *f, R *w) {
  if (!coarsened) {
    f[0] = c;
    w[0] = (R)1;
    return 1;
  }
  const int nf = 2 * nc;
  int m = 0;
  f[m] = 2 * c;
  w[m++] = (!periodic && c == 0) ? (R)1 : (R)0.75;
  f[m] = 2 * c + 1;
  w[m++] = (!periodic && c == nc - 1) ? (R)1 : (R)0.75;
  if (c > 0) { f[m] = 2 * c - 1; w[m++] = (R)0.25; }
  else if (periodic) { f[m] = nf - 1; w[m++] = (R)0.25; }
  if (c < nc - 1) { f[m] = 2 * c + 2; w[m++] = (R)0.25; }
  else if (periodic) { f[m] = 0; w[m++] = (R)0.25; }
  return m;
}

// 1-D prolongation: coarse indices and weights for fine f
template <typename R>
__device__ __forceinline__ int pstencil(int f, int nc, int coarsened, int periodic, int *c, R *w) {
  if (!coarsened) {
    c[0] = f;
    w[0] = (R)1;
    return 1;
  }
  const int c0 = f >> 1;
  int c1 = (f & 1) ? c0 + 1 : c0 - 1;
  if (c1 < 0 || c1 >= nc) {
    if (!periodic) {
      c[0] = c0;
      w[0] = (R)1;
      return 1;
    }
    c1 = (c1 < 0) ? c1 + nc : c1 - nc;
  }
  c[0] = c0;
  w[0] = (R)0.75;
  c[1] = c1;
  w[1] = (R)0.25;
  return 2;
}

// Separable transfers: P = Px (x) Py (x) Pz and R = P^T / 2^d applied one
// axis at a time through intermediate grids, 2 (P) or 4 (R) multiply-adds
// per output point instead of the 8 (P) or 64 (R) of the direct 3-D
// stencils.  (nx, ny, nz) are the output dimensions; the input has the same
// dimensions except `nin` along axis `ax`.
template <typename R>
__global__ void k_prolong_axis(int ax, int periodic, int nx, int ny, int nz, int nin, const R *__restrict__ in,
                               R *__restrict__ out, int add) {
  const int i = blockIdx.x * MG_BX + threadIdx.x, j = blockIdx.y * MG_BY + threadIdx.y, k = blockIdx.z;
  if (i >= nx || j >= ny) return;
  const int f = (ax == 0) ? i : ((ax == 1) ? j : k);
  int cc[2];
  R w[2];
  const int m = pstencil<R>(f, nin, 1, periodic, cc, w);
  const int inx = (ax == 0) ? nin : nx, iny = (ax == 1) ? nin : ny;
  R acc = (R)0;
  for (int q = 0; q < m; q++) {
    const int ii = (ax == 0) ? cc[q] : i, jj = (ax == 1) ? cc[q] : j, kk = (ax == 2) ? cc[q] : k;
    acc = fma(w[q], in[ii + inx * (jj + iny * kk)], acc);
  }
  const int o = i + nx * (j + ny * k);
  out[o] = add ? out[o] + acc : acc;
}

template <typename R>
__global__ void k_restrict_axis(int ax, int periodic, int nx, int ny, int nz, int nin, R scale,
                                const R *__restrict__ in, R *__restrict__ out) {
  const int i = blockIdx.x * MG_BX + threadIdx.x, j = blockIdx.y * MG_BY + threadIdx.y, k = blockIdx.z;
  if (i >= nx || j >= ny) return;
  const int cidx = (ax == 0) ? i : ((ax == 1) ? j : k);
  const int nco = (ax == 0) ? nx : ((ax == 1) ? ny : nz);
  int ff[4];
  R w[4];
  const int m = rstencil<R>(cidx, nco, 1, periodic, ff, w);
  const int inx = (ax == 0) ? nin : nx, iny = (ax == 1) ? nin : ny;
  R acc = (R)0;
  for (int q = 0; q < m; q++) {
    const int ii = (ax == 0) ? ff[q] : i, jj = (ax == 1) ? ff[q] : j, kk = (ax == 2) ? ff[q] : k;
    acc = fma(w[q], in[ii + inx * (jj + iny * kk)], acc);
  }
  out[i + nx * (j + ny * k)] = acc * scale;
}

// coarsest grid: e = Cinv b (one block; the pseudo-inverse and the
// products stay FP64 in both forms)
template <typename T>
__global__ void k_coarse_solve(int n, const double *__restrict__ cinv, const T *__restrict__ b, T *__restrict__ e) {
  __shared__ double sb[512];
  for (int a = threadIdx.x; a < n; a += blockDim.x) sb[a] = (double)b[a];
  __syncthreads();
  for (int a = threadIdx.x; a < n; a += blockDim.x) {
    const double *row = cinv + (size_t)a * n;
    double acc = 0.0;
    for (int q = 0; q < n; q++) acc += row[q] * sb[q];
    e[a] = (T)acc;
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

template <typename R, typename TB, typename TE, typename TO>
static cudaError_t lj2_attr() {
  return cudaFuncSetAttribute(k_line_jacobi2<R, TB, TE, TO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              200 * 1024);
}

cudaError_t poisson_create(const Geo &g, double cx, double cy, double cz, int fp32,
                           PoissonSolver **out) {
  PoissonSolver *S = new PoissonSolver();
  S->fp32 = fp32 ? 1 : 0;
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
  const size_t esz = S->fp32 ? sizeof(float) : sizeof(double);
  for (size_t l = 0; l < S->lv.size(); l++) {
    PLevel &L = S->lv[l];
    {
      const double cmax = fmax(fmax(L.cx, L.cy), L.cz), cmin = fmin(fmin(L.cx, L.cy), L.cz);
      // red-black needs an even periodic y extent (j = 0 and ny - 1 are
      // neighbours); otherwise, or when z couplings dominate, z-lines
      L.point = (cmax <= 2.0 * cmin && L.ny % 2 == 0) ? 1 : 0;
      for (int a = 0; a < 3; a++)
        for (int q = 0; q < 3; q++) {
          const double nbx = (L.nx == 1) ? 0.0 : ((a == 1) ? 2.0 : 1.0);
          const double nbz = (L.nz == 1) ? 0.0 : ((q == 1) ? 2.0 : 1.0);
          L.invd[a][q] = 1.0 / (L.cx * nbx + 2.0 * L.cy + L.cz * nbz);
        }
    }
    const size_t bytes = esz * (size_t)L.n;
    if (l > 0) PCK(cudaMalloc(&L.b, bytes));
    PCK(cudaMalloc(&L.e, bytes));
    PCK(cudaMalloc(&L.e2, bytes));
    PCK(cudaMalloc(&L.r, bytes));
    PCK(cudaMalloc(&L.t, bytes));
    std::vector<double> th = thomas_factors(L);
    if (S->fp32) {
      std::vector<float> thf(th.begin(), th.end());
      PCK(cudaMalloc(&L.thomas, thf.size() * sizeof(float)));
      PCK(cudaMemcpy(L.thomas, thf.data(), thf.size() * sizeof(float), cudaMemcpyHostToDevice));
    } else {
      PCK(cudaMalloc(&L.thomas, th.size() * sizeof(double)));
      PCK(cudaMemcpy(L.thomas, th.data(), th.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
  }
  if (S->fp32) {
    PCK((lj2_attr<float, double, float, float>()));
    PCK((lj2_attr<float, double, float, double>()));
    PCK((lj2_attr<float, float, float, float>()));
  } else {
    PCK((lj2_attr<double, double, double, double>()));
  }
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
  if (S->side) cudaStreamDestroy(S->side);
  delete S;
}

int poisson_levels(const PoissonSolver *S) { return (int)S->lv.size(); }

size_t poisson_footprint(const Geo &g, int fp32, size_t (*rnd)(size_t)) {
  // the level sizes poisson_create builds, without allocating
  const size_t esz = fp32 ? sizeof(float) : sizeof(double);
  size_t tot = 0;
  int nx = g.nx, ny = g.ny, nz = g.nz, l = 0;
  while (true) {
    const size_t n = (size_t)nx * ny * nz;
    tot += (l > 0 ? 5 : 4) * rnd(esz * n) + rnd(esz * 3 * nz * 2);
    if (n <= 512) {
      tot += rnd(sizeof(double) * n * n);
      break;
    }
    const int cx = (nx % 2 == 0 && nx >= 4), cy = (ny % 2 == 0 && ny >= 4), cz = (nz % 2 == 0 && nz >= 4);
    if (!cx && !cy && !cz) break;
    nx = cx ? nx / 2 : nx;
    ny = cy ? ny / 2 : ny;
    nz = cz ? nz / 2 : nz;
    l++;
  }
  const size_t N = (size_t)g.nx * g.ny * g.nz;
  tot += 6 * rnd(sizeof(double) * N) + rnd(sizeof(double) * (size_t)g.ny * g.nz);
  tot += rnd(sizeof(double) * 3 * 1216) + rnd(sizeof(unsigned)) + rnd(sizeof(double) * S_COUNT);
  return tot;
}

template <typename R>
static LevArgs<R> largs(const PLevel &L) {
  LevArgs<R> a;
  a.nx = L.nx;
  a.ny = L.ny;
  a.nz = L.nz;
  a.cx = (R)L.cx;
  a.cy = (R)L.cy;
  a.cz = (R)L.cz;
  return a;
}

template <typename R, typename TB, typename TE, typename TO>
static void line_sweep(const PLevel &L, R w, R w1, int zero_init, const TB *b, const TE *ei, TO *eo,
                       cudaStream_t st) {
  const LevArgs<R> A = largs<R>(L);
  const R *th = static_cast<const R *>(L.thomas);
  const size_t smem = sizeof(R) * 32 * (size_t)L.nz;
  if (smem <= 200 * 1024) {
    k_line_jacobi2<R, TB, TE, TO><<<(L.nx * L.ny + 31) / 32, LJ2_T, smem, st>>>(A, w, w1, zero_init, th, b, ei, eo);
  } else {
    k_line_jacobi<R, TB, TE, TO><<<(L.nx * L.ny + LJB - 1) / LJB, LJB, 0, st>>>(A, w, w1, zero_init, th, b, ei,
                                                                                static_cast<R *>(L.t), eo);
  }
}

// R = P^T / 2^d over the coarsened axes in the order x, y, z; the
// intermediate grids live in the fine level's scratch t (n values: the
// first intermediate uses its first n/2, the second the next n/4).
template <typename R>
static cudaError_t restrict_chain(const PLevel &F, const PLevel &C, const R *rf, R *t, R *bc, cudaStream_t st,
                                  long *nl) {
  int d[3] = {F.nx, F.ny, F.nz};
  const int cd[3] = {C.nx, C.ny, C.nz};
  const int cs[3] = {C.cxs, C.cys, C.czs};
  int last = -1, nax = 0;
  for (int a = 0; a < 3; a++)
    if (cs[a]) last = a, nax++;
  const R scale = (R)(1.0 / (double)(1 << nax));
  const R *src = rf;
  R *bufs[2] = {t, t + (size_t)F.n / 2};
  int b = 0;
  for (int a = 0; a < 3; a++) {
    if (!cs[a]) continue;
    const int nin = d[a];
    d[a] = cd[a];
    R *dst = (a == last) ? bc : bufs[b++];
    k_restrict_axis<R><<<mg_grid(d[0], d[1], d[2]), dim3(MG_BX, MG_BY), 0, st>>>(
        a, a == 1, d[0], d[1], d[2], nin, (a == last) ? scale : (R)1, src, dst);
    (*nl)++;
    src = dst;
  }
  return cudaGetLastError();
}

// ef += P ec over the coarsened axes in the order z, y, x.
template <typename R>
static cudaError_t prolong_chain(const PLevel &F, const PLevel &C, const R *ec, R *t, R *ef, cudaStream_t st,
                                 long *nl) {
  int d[3] = {C.nx, C.ny, C.nz};
  const int fd[3] = {F.nx, F.ny, F.nz};
  const int cs[3] = {C.cxs, C.cys, C.czs};
  int last = -1;
  for (int a = 2; a >= 0; a--)
    if (cs[a]) last = a;
  const R *src = ec;
  R *bufs[2] = {t + (size_t)F.n / 2, t};  // the smaller intermediate first
  int b = 0;
  for (int a = 2; a >= 0; a--) {
    if (!cs[a]) continue;
    const int nin = d[a];
    d[a] = fd[a];
    const bool fin = (a == last);
    R *dst = fin ? ef : bufs[b++];
    k_prolong_axis<R><<<mg_grid(d[0], d[1], d[2]), dim3(MG_BX, MG_BY), 0, st>>>(a, a == 1, d[0], d[1], d[2], nin,
                                                                                src, dst, fin ? 1 : 0);
    (*nl)++;
    src = dst;
  }
  return cudaGetLastError();
}

template <typename R>
static InvD<R> invd_of(const PLevel &L) {
  InvD<R> v;
  for (int a = 0; a < 3; a++)
    for (int q = 0; q < 3; q++) v.v[a][q] = (R)L.invd[a][q];
  return v;
}

// pre-smoothing from a zero start into e2: z-line Jacobi, or red then black
template <typename R, typename TB>
static void pre_smooth(const PLevel &L, R w, R w1, const TB *b, R *e2, cudaStream_t st, long *nl) {
  if (!L.point) {
    line_sweep<R, TB, R, R>(L, w, w1, 1, b, nullptr, e2, st);
    (*nl)++;
    return;
  }
  const LevArgs<R> A = largs<R>(L);
  const dim3 grd = mg_grid((L.nx + 1) / 2, L.ny, L.nz);
  k_rbgs<R, TB, R, R><<<grd, dim3(MG_BX, MG_BY), 0, st>>>(A, invd_of<R>(L), 0, 1, 0, b, e2, e2);
  k_rbgs<R, TB, R, R><<<grd, dim3(MG_BX, MG_BY), 0, st>>>(A, invd_of<R>(L), 1, 0, 0, b, e2, e2);
  *nl += 2;
}

// post-smoothing of e2 into res: z-line Jacobi, or black (in place) then red
// (with the black values copied), the adjoint order of the pre-smoothing
template <typename R, typename TB, typename TO>
static void post_smooth(const PLevel &L, R w, R w1, const TB *b, R *e2, TO *res, cudaStream_t st, long *nl) {
  if (!L.point) {
    line_sweep<R, TB, R, TO>(L, w, w1, 0, b, e2, res, st);
    (*nl)++;
    return;
  }
  const LevArgs<R> A = largs<R>(L);
  const dim3 grd = mg_grid((L.nx + 1) / 2, L.ny, L.nz);
  k_rbgs<R, TB, R, R><<<grd, dim3(MG_BX, MG_BY), 0, st>>>(A, invd_of<R>(L), 1, 0, 0, b, e2, e2);
  k_rbgs<R, TB, R, TO><<<grd, dim3(MG_BX, MG_BY), 0, st>>>(A, invd_of<R>(L), 0, 0, 1, b, e2, res);
  *nl += 2;
}

// one symmetric V-cycle: out = M b0.  Every level pre-smooths into its
// scratch e2 (one damped line-Jacobi sweep from zero), restricts the
// residual, adds the prolonged coarse correction into e2 and post-smooths
// from e2 into its result buffer (out on the finest level, e elsewhere).
// R: level type; the finest level reads b0 and writes out in FP64.
template <typename R>
static cudaError_t vcycle(PoissonSolver *S, const double *b0, double *out, cudaStream_t st, long *nl) {
  const int nlev = (int)S->lv.size();
  const R w = (R)S->omega, w1 = (R)(1.0 - S->omega);
  auto lvp = [](void *p) { return static_cast<R *>(p); };
  if (nlev == 1) {
    PLevel &L = S->lv[0];
    if (S->cinv) {
      k_coarse_solve<double><<<1, 256, 0, st>>>(L.n, S->cinv, b0, out);
      (*nl)++;
      return cudaGetLastError();
    }
    // single level without a dense inverse: damped line-Jacobi sweeps
    R *cur = lvp(L.e2), *oth = lvp(L.e);
    line_sweep<R, double, R, R>(L, w, w1, 1, b0, nullptr, cur, st);
    (*nl)++;
    for (int sw = 1; sw < S->coarse_sweeps - 1; sw++) {
      line_sweep<R, double, R, R>(L, w, w1, 0, b0, cur, oth, st);
      (*nl)++;
      R *tmp = cur;
      cur = oth;
      oth = tmp;
    }
    line_sweep<R, double, R, double>(L, w, w1, 0, b0, cur, out, st);
    (*nl)++;
    return cudaGetLastError();
  }
  for (int l = 0; l < nlev; l++) {
    PLevel &L = S->lv[l];
    const R *b = lvp(L.b);
    R *res = lvp(L.e);
    if (l == nlev - 1) {
      if (S->cinv) {
        k_coarse_solve<R><<<1, 256, 0, st>>>(L.n, S->cinv, b, res);
        (*nl)++;
      } else {
        R *cur = lvp(L.e2), *oth = res;
        line_sweep<R, R, R, R>(L, w, w1, 1, b, nullptr, cur, st);
        (*nl)++;
        for (int sw = 1; sw < S->coarse_sweeps; sw++) {
          line_sweep<R, R, R, R>(L, w, w1, 0, b, cur, oth, st);
          (*nl)++;
          R *tmp = cur;
          cur = oth;
          oth = tmp;
        }
        if (cur != res) PCK(cudaMemcpyAsync(res, cur, sizeof(R) * L.n, cudaMemcpyDeviceToDevice, st));
      }
      PCK(cudaGetLastError());
      break;
    }
    const LevArgs<R> A = largs<R>(L);
    if (l == 0) {
      pre_smooth<R, double>(L, w, w1, b0, lvp(L.e2), st, nl);
      k_residual<R, double, R><<<mg_grid(L.nx, L.ny, L.nz), dim3(MG_BX, MG_BY), 0, st>>>(A, b0, lvp(L.e2),
                                                                                    lvp(L.r));
    } else {
      pre_smooth<R, R>(L, w, w1, b, lvp(L.e2), st, nl);
      k_residual<R, R, R><<<mg_grid(L.nx, L.ny, L.nz), dim3(MG_BX, MG_BY), 0, st>>>(A, b, lvp(L.e2), lvp(L.r));
    }
    const PLevel &C = S->lv[l + 1];
    PCK(restrict_chain<R>(L, C, lvp(L.r), lvp(L.t), lvp(C.b), st, nl));
    *nl += 1;
    PCK(cudaGetLastError());
  }
  for (int l = nlev - 2; l >= 0; l--) {
    PLevel &L = S->lv[l];
    const PLevel &C = S->lv[l + 1];
    const LevArgs<R> A = largs<R>(L);
    PCK(prolong_chain<R>(L, C, lvp(C.e), lvp(L.t), lvp(L.e2), st, nl));
    if (l == 0)
      post_smooth<R, double, double>(L, w, w1, b0, lvp(L.e2), out, st, nl);
    else
      post_smooth<R, R, R>(L, w, w1, lvp(L.b), lvp(L.e2), lvp(L.e), st, nl);
    PCK(cudaGetLastError());
  }
  return cudaSuccess;
}

// The solve in three parts: set-up (b, x0 = p_old, r0 and the first
// convergence test), one PCG iteration (V-cycle, z.r, p update, A p, x and r
// updates, convergence test), and the write-back of p with its ghosts.
static cudaError_t solve_begin(PoissonSolver *S, const Geo &g, const Phys &ph, const double *rhs_p,
                               const void *u3, int u3_fp32, const double *u_inlet, const double *pres_old,
                               double rtol, const CgCtl &ctl, cudaStream_t st, long *nl) {
  const int N = S->N, rb = S->rblk;
  const PLevel &F = S->lv[0];
  if (u3_fp32)
    k_build_b<float><<<rb, PB, 0, st>>>(g, (ph.dx / ph.dt) / ph.dy, 1.0 / ph.dy, rhs_p,
                                        static_cast<const float *>(u3), u_inlet, pres_old, S->bvec, S->x, S->bin,
                                        S->part, S->counter, S->s);
  else
    k_build_b<double><<<rb, PB, 0, st>>>(g, (ph.dx / ph.dt) / ph.dy, 1.0 / ph.dy, rhs_p,
                                         static_cast<const double *>(u3), u_inlet, pres_old, S->bvec, S->x, S->bin,
                                         S->part, S->counter, S->s);
  k_init_r<<<rb, PB, 0, st>>>(F.nx, F.ny, F.nz, F.cx, F.cy, F.cz, 1.0 / (double)N, rtol, ctl, S->s, S->bvec,
                              S->x, S->r, S->part, S->counter);
  *nl += 2;
  return cudaGetLastError();
}

static cudaError_t solve_iteration(PoissonSolver *S, const CgCtl &ctl, cudaStream_t st, long *nl) {
  const int N = S->N, rb = S->rblk;
  const PLevel &F = S->lv[0];
  PCK(S->fp32 ? vcycle<float>(S, S->r, S->z, st, nl) : vcycle<double>(S, S->r, S->z, st, nl));
  k_zdot<<<rb, PB, 0, st>>>(N, 1.0 / (double)N, S->r, S->z, S->part, S->counter, S->s);
  k_pupdate<<<nblocks(N), PB, 0, st>>>(N, S->s, S->z, S->p);
  k_apply_dot<<<rb, PB, 0, st>>>(F.nx, F.ny, F.nz, F.cx, F.cy, F.cz, S->p, S->q, S->part, S->counter, S->s);
  k_axpy<<<rb, PB, 0, st>>>(N, ctl, S->s, S->p, S->q, S->x, S->r, S->part, S->counter);
  *nl += 4;
  return cudaGetLastError();
}

static cudaError_t solve_end(PoissonSolver *S, const Geo &g, const Phys &ph, double *pres, cudaStream_t st,
                             long *nl) {
  k_sumx<<<S->rblk, PB, 0, st>>>(S->N, S->x, S->part, S->counter, S->s);
  dim3 grd((g.nx + 2 + 31) / 32, (g.ny + 2 + 3) / 4, g.nz + 2);
  k_writeback<<<grd, dim3(32, 4), 0, st>>>(g, ph.dy, 1.0 / (double)S->N, S->s, S->x, S->bin, pres);
  *nl += 2;
  return cudaGetLastError();
}

cudaError_t poisson_solve(PoissonSolver *S, const Geo &g, const Phys &ph,
                          const double *rhs_p, const void *u3, int u3_fp32,
                          const double *u_inlet, const double *pres_old,
                          double *pres, double rtol, int maxits, int *its,
                          double *rnorm, double *bnorm, int *reason,
                          cudaStream_t st, long *nl) {
  const CgCtl ctl = {maxits, 0, 0};
  PCK(solve_begin(S, g, ph, rhs_p, u3, u3_fp32, u_inlet, pres_old, rtol, ctl, st, nl));
  while (true) {
    PCK(cudaMemcpyAsync(S->s_host, S->s, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, st));
    PCK(cudaStreamSynchronize(st));
    if (S->s_host[S_REASON] != 0.0) break;
    PCK(solve_iteration(S, ctl, st, nl));
  }
  PCK(solve_end(S, g, ph, pres, st, nl));
  *its = (int)S->s_host[S_IT];
  *rnorm = sqrt(S->s_host[S_RR]);
  *bnorm = sqrt(S->s_host[S_BB]);
  *reason = (int)S->s_host[S_REASON];
  return cudaSuccess;
}

cudaError_t poisson_solve_capture(PoissonSolver *S, const Geo &g, const Phys &ph,
                                  const double *rhs_p, const void *u3, int u3_fp32,
                                  const double *u_inlet, const double *pres_old,
                                  double *pres, double rtol, int maxits,
                                  cudaStream_t st, long *nl_static, long *nl_body) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t graph = nullptr;
  PCK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &graph, nullptr, nullptr, nullptr));
  if (cs != cudaStreamCaptureStatusActive || !graph) return cudaErrorStreamCaptureUnmatched;
  CgCtl ctl = {maxits, 1, 0};
  PCK(cudaGraphConditionalHandleCreate(&ctl.cond, graph, 0, 0));
  PCK(solve_begin(S, g, ph, rhs_p, u3, u3_fp32, u_inlet, pres_old, rtol, ctl, st, nl_static));
  const cudaGraphNode_t *deps = nullptr;
  size_t ndeps = 0;
  PCK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &graph, &deps, nullptr, &ndeps));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = ctl.cond;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  PCK(cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  if (!S->side) PCK(cudaStreamCreateWithFlags(&S->side, cudaStreamNonBlocking));
  PCK(cudaStreamBeginCaptureToGraph(S->side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  const cudaError_t eb = solve_iteration(S, ctl, S->side, nl_body);
  cudaGraph_t out = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(S->side, &out);
  PCK(eb);
  PCK(ee);
  PCK(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  return solve_end(S, g, ph, pres, st, nl_static);
}

cudaError_t poisson_read(PoissonSolver *S, cudaStream_t st, int *its, double *rnorm, double *bnorm,
                         int *reason, int *worst, double *its_total) {
  PCK(cudaMemcpyAsync(S->s_host, S->s, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, st));
  PCK(cudaStreamSynchronize(st));
  *its = (int)S->s_host[S_IT];
  *rnorm = sqrt(S->s_host[S_RR]);
  *bnorm = sqrt(S->s_host[S_BB]);
  *reason = (int)S->s_host[S_REASON];
  *worst = (int)S->s_host[S_WORST];
  *its_total = S->s_host[S_ITS_TOTAL];
  return cudaSuccess;
}

cudaError_t poisson_reset_worst(PoissonSolver *S, cudaStream_t st) {
  static const double zero = 0.0;
  return cudaMemcpyAsync(S->s + S_WORST, &zero, sizeof(double), cudaMemcpyHostToDevice, st);
}

}  // namespace tpls
