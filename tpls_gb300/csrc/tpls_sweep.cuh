// tpls_sweep.cuh -- device helpers shared by the Crank-Nicolson sweep
// kernels (boundary rows of main_ns_hybrid.F90:756-887 and the fused
// periodic ghost-row copies), templated on the storage type of the
// velocity being relaxed (double, or float in the FP32-mixed form).
#pragma once
#include "tpls_kernels.h"

namespace tpls {

struct Helm {
  double ax2, ay2, az2;  // dt/(2 d^2)
  double dtdx;           // dt/dx (u outlet condition)
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

// Defect form.  The FP32-mixed sweeps iterate on d = x - X, X the FP64
// velocity state of the step (u2, v2 or w2), so that FP32 rounding acts on
// the small correction instead of on the velocity; the FP64 form passes
// X = null and iterates on x itself.  Interior updates are the same affine
// map in both (the records' b is shifted accordingly); boundary rows are
// evaluated in x space in FP64 and stored back as x - X.
template <typename T>
__device__ __forceinline__ double xval(const Geo &g, const double *X, T d, int i, int j, int k) {
  return X ? (double)d + X[TPLS_IDX(g, i, j, k)] : (double)d;
}
template <typename T>
__device__ __forceinline__ void bput(const Geo &g, T *x, const double *X, int i, int j, int k, double v,
                                     int fuse) {
  put(g, x, i, j, k, (T)(X ? v - X[TPLS_IDX(g, i, j, k)] : v), fuse);
}

// u outlet, main_ns_hybrid.F90:768-776 (the pressure row index is the u row
// index j, as written in the reference); x space, FP64.
__device__ __forceinline__ double u_outlet(const Geo &g, const Helm &h, const double *P, double unm1, int j,
                                           int k) {
  const int nx = g.nx;
  return unm1 + h.dtdx * (P[TPLS_IDX(g, nx + 1, j, k + 1)] + P[TPLS_IDX(g, nx - 1, j, k + 1)] -
                          2.0 * P[TPLS_IDX(g, nx, j, k + 1)]);
}

// Post-sweep boundary rows (main_ns_hybrid.F90:784-799 u, :826-836 v,
// :860-879 w), written by the thread that owns the first / last x pair:
// the inlet copy x(0) = x(1), for u the pressure outlet x(nx) and the
// fictitious point x(nx+1) = 0, for v and w the outlet copy.  A value of the
// colour not relaxed in this half-sweep is read (it is final already).
template <typename T>
__device__ __forceinline__ void sor_bc(int comp, const Geo &g, const Helm &h, T *x, const double *X,
                                       const double *P, int i2, int i, int iend, T v, int j, int k, int fuse) {
  if (i2 == 0) {
    const T v1 = (i == 1) ? v : x[TPLS_IDX(g, 1, j, k)];
    bput(g, x, X, 0, j, k, xval(g, X, v1, 1, j, k), fuse);
  }
  if (i2 == (iend - 1) / 2) {
    const T ve = (i == iend) ? v : x[TPLS_IDX(g, iend, j, k)];
    const double vex = xval(g, X, ve, iend, j, k);
    if (comp == 0) {
      bput(g, x, X, g.nx, j, k, u_outlet(g, h, P, vex, j, k), fuse);
      bput(g, x, X, g.nx + 1, j, k, 0.0, fuse);
    } else {
      bput(g, x, X, g.nx + 1, j, k, vex, fuse);
    }
  }
}

static inline Helm helm_of(const Phys &ph) {
  Helm h;
  h.ax2 = (ph.dt / (ph.dx * ph.dx)) / 2.0;
  h.ay2 = (ph.dt / (ph.dy * ph.dy)) / 2.0;
  h.az2 = (ph.dt / (ph.dz * ph.dz)) / 2.0;
  h.dtdx = ph.dt / ph.dx;
  return h;
}

}  // namespace tpls
