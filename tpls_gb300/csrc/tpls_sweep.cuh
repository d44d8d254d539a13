// tpls_sweep.cuh -- device helpers shared by the Crank-Nicolson sweep
// kernels (boundary rows of main_ns_hybrid.F90:756-887 and the fused
// periodic ghost-row copies), templated on the storage type of the
// velocity being relaxed (double, or float in the FP32-mixed form).
#pragma once
#include "tpls_kernels.h"
#include "tpls_pair.cuh"

namespace tpls {

struct Helm {
  double ax2, ay2, az2;  // dt/(2 d^2)
  double dtdx;           // dt/dx (u outlet condition)
  float dtdxf;           // the same, rounded, for the FP32 defect-form sweeps
  double rdx, rdy, rdz;  // 1/dx, 1/dy, 1/dz
};

template <typename T>
struct FcT {
  T px, mx, py, my, pz, mz;
};
using Fc = FcT<double>;


// face viscosities, momentum_allflux.f90:91-98 (u), :145-152 (v), :187-194 (w)
template <typename T>
__device__ __forceinline__ FcT<T> faces(int comp, const Geo &g, const T *__restrict__ mu, int i, int j,
                                        int k) {
  const int sy = g.sy, sz = g.szm;
  FcT<T> f;
  if (comp == 0) {
    const T *m = mu + TPLS_IDXM(g, i, j + 1, k + 1);
    const T a = m[0], b = m[1];
    f.px = b;
    f.mx = a;
    f.py = (a + b + m[sy] + m[1 + sy]) * (T)0.25;
    f.my = (a + b + m[-sy] + m[1 - sy]) * (T)0.25;
    f.pz = (a + b + m[sz] + m[1 + sz]) * (T)0.25;
    f.mz = (a + b + m[-sz] + m[1 - sz]) * (T)0.25;
  } else if (comp == 1) {
    const T *m = mu + TPLS_IDXM(g, i, j + 1, k + 1);
    const T a = m[0], b = m[-sy];
    f.px = (a + b + m[1] + m[1 - sy]) * (T)0.25;
    f.mx = (a + b + m[-1] + m[-1 - sy]) * (T)0.25;
    f.py = a;
    f.my = b;
    f.pz = (a + b + m[sz] + m[sz - sy]) * (T)0.25;
    f.mz = (a + b + m[-sz] + m[-sz - sy]) * (T)0.25;
  } else {
    const T *m = mu + TPLS_IDXM(g, i, j + 1, k);
    const T a = m[0], b = m[sz];
    f.px = (a + b + m[1] + m[1 + sz]) * (T)0.25;
    f.mx = (a + b + m[-1] + m[-1 + sz]) * (T)0.25;
    f.py = (a + b + m[sy] + m[sy + sz]) * (T)0.25;
    f.my = (a + b + m[-sy] + m[-sy + sz]) * (T)0.25;
    f.pz = b;
    f.mz = a;
  }
  return f;
}

// Slot of point (i, j, k) (linear index c, 1 <= i <= nx) in the coefficient
// record arrays.  Each (j, k) row keeps the records of odd i in its first
// half and of even i in its second half (the row pitch sy is a multiple of
// 4), so a red-black half-sweep, which relaxes one i parity per row, reads
// one contiguous half-row of records instead of every other 64-byte record.
__device__ __forceinline__ int rec_slot(const Geo &g, int c, int i) {
  return c - i + ((i & 1) ? ((i - 1) >> 1) : ((g.sy >> 1) + (i >> 1) - 1));
}

// Write a value and, when ghost rows are fused (even ny), its periodic copy.
template <typename T>
__device__ __forceinline__ void put(const Geo &g, T *x, int i, int j, int k, T v, int fuse) {
  x[TPLS_IDX(g, i, j, k)] = v;
  if (fuse) {
    if (j == g.ny) x[TPLS_IDX(g, i, 0, k)] = v;
    if (j == 1) x[TPLS_IDX(g, i, g.ny + 1, k)] = v;
  }
}

// Boundary rows.  The FP64 form iterates on x itself (X = null); the
// FP32-mixed sweeps iterate on d = x - X, X the FP64 velocity state of the
// step (u2, v2 or w2), so that FP32 rounding acts on the small correction
// instead of on the velocity.  A boundary relation of x becomes one of d
// whose FP64 parts are differences of nearby X (and P) values, taken from
// FP32 pairs (integer splitting, tpls_pair.cuh): the FP32 sweeps issue no
// FP64 instruction, which on GB300's FP64 pipe made the boundary threads
// the critical path of every sweep.
//
// copy x(it) = x(is) (inlet / outlet copies)
__device__ __forceinline__ void bc_copy(const Geo &g, double *x, const double *, int it, int, int j, int k,
                                        double vs, int fuse) {
  put(g, x, it, j, k, vs, fuse);
}
__device__ __forceinline__ void bc_copy(const Geo &g, float *x, const double *X, int it, int is, int j, int k,
                                        float ds, int fuse) {
  const F2 a = split_bits(X[TPLS_IDX(g, is, j, k)]), b = split_bits(X[TPLS_IDX(g, it, j, k)]);
  put(g, x, it, j, k, ds + dif(a, b), fuse);
}
// x(i, j, k) = 0 (u fictitious point, w walls)
__device__ __forceinline__ void bc_zero(const Geo &g, double *x, const double *, int i, int j, int k, int fuse) {
  put(g, x, i, j, k, 0.0, fuse);
}
__device__ __forceinline__ void bc_zero(const Geo &g, float *x, const double *X, int i, int j, int k, int fuse) {
  put(g, x, i, j, k, -round_bits(X[TPLS_IDX(g, i, j, k)]), fuse);
}

// u outlet, main_ns_hybrid.F90:768-776 (the pressure row index is the u row
// index j, as written in the reference):
//   x(nx) = x(nx-1) + dt/dx (P(nx+1) + P(nx-1) - 2 P(nx))
__device__ __forceinline__ double u_outlet(const Geo &g, const Helm &h, const double *P, double unm1, int j,
                                           int k) {
  const int nx = g.nx;
  return unm1 + h.dtdx * (P[TPLS_IDX(g, nx + 1, j, k + 1)] + P[TPLS_IDX(g, nx - 1, j, k + 1)] -
                          2.0 * P[TPLS_IDX(g, nx, j, k + 1)]);
}
__device__ __forceinline__ void bc_u_outlet(const Geo &g, const Helm &h, const double *P, double *x,
                                            const double *, int j, int k, double vm1, int fuse) {
  put(g, x, g.nx, j, k, u_outlet(g, h, P, vm1, j, k), fuse);
}
// defect form: d(nx) = d(nx-1) + (X(nx-1) - X(nx)) + dt/dx ((P+ - P0) - (P0 - P-))
__device__ __forceinline__ void bc_u_outlet(const Geo &g, const Helm &h, const double *P, float *x,
                                            const double *X, int j, int k, float dm1, int fuse) {
  const int nx = g.nx;
  const F2 pp = split_bits(P[TPLS_IDX(g, nx + 1, j, k + 1)]), p0 = split_bits(P[TPLS_IDX(g, nx, j, k + 1)]);
  const F2 pm = split_bits(P[TPLS_IDX(g, nx - 1, j, k + 1)]);
  const F2 xa = split_bits(X[TPLS_IDX(g, nx - 1, j, k)]), xb = split_bits(X[TPLS_IDX(g, nx, j, k)]);
  put(g, x, nx, j, k, dm1 + dif(xa, xb) + h.dtdxf * (dif(pp, p0) - dif(p0, pm)), fuse);
}

// Post-sweep boundary rows of the Jacobi sweep at point (i, j, k) with new
// value v (main_ns_hybrid.F90:784-799 u, :826-836 v, :860-879 w).
template <typename T>
__device__ __forceinline__ void jacobi_bc(int comp, const Geo &g, const Helm &h, T *x, const double *X,
                                          const double *P, int i, int j, int k, T v, int fuse) {
  if (comp == 0) {
    if (i == 1) bc_copy(g, x, X, 0, 1, j, k, v, fuse);
    if (i == g.nx - 1) {
      bc_u_outlet(g, h, P, x, X, j, k, v, fuse);
      bc_zero(g, x, X, g.nx + 1, j, k, fuse);
    }
  } else if (comp == 1) {
    if (i == 1) bc_copy(g, x, X, 0, 1, j, k, v, fuse);
    if (i == g.nx) bc_copy(g, x, X, g.nx + 1, g.nx, j, k, v, fuse);
  } else {
    const int nz = g.nz;
    if (k == 1) bc_zero(g, x, X, i, j, 0, fuse);
    if (k == nz - 1) bc_zero(g, x, X, i, j, nz, fuse);
    if (i == 1) {
      bc_copy(g, x, X, 0, 1, j, k, v, fuse);
      if (k == 1) bc_zero(g, x, X, 0, j, 0, fuse);
      if (k == nz - 1) bc_zero(g, x, X, 0, j, nz, fuse);
    }
    if (i == g.nx) {
      bc_copy(g, x, X, g.nx + 1, g.nx, j, k, v, fuse);
      if (k == 1) bc_zero(g, x, X, g.nx + 1, j, 0, fuse);
      if (k == nz - 1) bc_zero(g, x, X, g.nx + 1, j, nz, fuse);
    }
  }
}

// Post-sweep boundary rows of a red-black half-sweep, written by the thread
// that owns the first / last x pair: the inlet copy x(0) = x(1), for u the
// pressure outlet x(nx) and the fictitious point x(nx+1) = 0, for v and w
// the outlet copy.  A value of the colour not relaxed in this half-sweep is
// read (it is final already).
template <typename T>
__device__ __forceinline__ void sor_bc(int comp, const Geo &g, const Helm &h, T *x, const double *X,
                                       const double *P, int i2, int i, int iend, T v, int j, int k, int fuse) {
  if (i2 == 0) {
    const T v1 = (i == 1) ? v : x[TPLS_IDX(g, 1, j, k)];
    bc_copy(g, x, X, 0, 1, j, k, v1, fuse);
  }
  if (i2 == (iend - 1) / 2) {
    const T ve = (i == iend) ? v : x[TPLS_IDX(g, iend, j, k)];
    if (comp == 0) {
      bc_u_outlet(g, h, P, x, X, j, k, ve, fuse);
      bc_zero(g, x, X, g.nx + 1, j, k, fuse);
    } else {
      bc_copy(g, x, X, g.nx + 1, iend, j, k, ve, fuse);
    }
  }
}

// One batch member's arguments of the FP32 sweeps, for the multi-instance
// launches of a batch (device array, one entry per member).
struct SweepMember {
  Geo g;
  Helm h;
  MuCoef s[3];          // per component: viscosity, b, scales, boundary offsets
  float *x[3][2];       // per component: the defect iterate pair
  const double *X[3];   // per component: the FP64 base state (u2, v2, w2)
  const double *P;      // pressure (u outlet)
  int fuse;             // periodic ghost rows written by the sweeps (even ny)
};
// Tiles of the single-instance FP32 Jacobi / checkerboard grid (4 rows per
// block) and of the odd half-sweep grid of component comp.
int sweep4_tiles(int comp, const Geo &g);
int odd_tiles(int comp, const Geo &g);
// One launch of the FP32 Jacobi (mode 0) or checkerboard (mode 1) sweep of
// component comp over all n members: prefix[m] = first tile of member m,
// prefix[n] = total_tiles (device array); Jacobi reads x[comp][src] and
// writes x[comp][1-src], the half-sweep relaxes x[comp][src]; ctr = two
// zeroed unsigned counters (left zero by the launch); nblocks = persistent
// blocks.
cudaError_t launch_sweep4_multi(int mode, int comp, const SweepMember *mem, const int *prefix, int n,
                                int total_tiles, int src, int flg, int bc, unsigned *ctr, int nblocks,
                                cudaStream_t st);
// The odd half-sweep (2-D colouring) of component comp over all members.
cudaError_t launch_odd_multi(int comp, const SweepMember *mem, const int *prefix, int n, int total_tiles,
                             int src, int flg, int bc, unsigned *ctr, int nblocks, cudaStream_t st);

// FP32 Jacobi (mode 0) and checkerboard half-sweep (mode 1) with four x
// points per thread (k_sweep32.cu); tile = rows per block choice.
cudaError_t launch_sweep4(int mode, int comp, const Geo &g, const Helm &h, const float *xo, float *x,
                          const MuCoef &s, const double *P, const double *X, int flg, int bc, int fuse, int tile,
                          cudaStream_t st);

static inline Helm helm_of(const Phys &ph) {
  Helm h;
  h.ax2 = (ph.dt / (ph.dx * ph.dx)) / 2.0;
  h.ay2 = (ph.dt / (ph.dy * ph.dy)) / 2.0;
  h.az2 = (ph.dt / (ph.dz * ph.dz)) / 2.0;
  h.dtdx = ph.dt / ph.dx;
  h.dtdxf = (float)h.dtdx;
  h.rdx = 1.0 / ph.dx;
  h.rdy = 1.0 / ph.dy;
  h.rdz = 1.0 / ph.dz;
  return h;
}

}  // namespace tpls
