// k_momentum.cu -- momentum operator and Crank-Nicolson sweeps
// (momentum_allflux.f90:22-471, jacobi_iteration_allflux.f90:21-311,
// sor_iteration_allflux.f90:19-377, main_ns_hybrid.F90:629-641,743-887).
//
// Velocity components are addressed in the reference's staggered index
// space: u(i,j,k) sits between p-cells (i,j+1,k+1) and (i+1,j+1,k+1),
// v(i,j,k) between (i,j,k+1) and (i,j+1,k+1), w(i,j,k) between (i,j+1,k)
// and (i,j+1,k+1); the viscosity field mu is on the p-grid with two
// periodic ghost rows, so every face viscosity of the reference is read
// directly.
//
// Red-black SOR: for an even iteration_time the colouring is the 3-D
// checkerboard mod(k+j+flg,2), every point of a colour is independent and
// one thread updates one point.  For an odd iteration_time the colouring is
// mod(j+flg,2) in every plane, so the reference's sequential loop lets a
// point see the already-relaxed point below it: one thread marches each
// (i,j) column upward, carrying the relaxed value in a register.
// Periodic ghost rows are written by the thread that writes the row they
// copy (legal for even ny: no point of the colour being relaxed reads a
// ghost row written in the same half-sweep); for odd ny the caller runs a
// separate exchange after each half-sweep instead.
#include "tpls_sweep.cuh"
#include "tpls_pair.cuh"

namespace tpls {

// jacobi_iteration_allflux.f90:84-90 (same form in every Jacobi/SOR routine)
__device__ __forceinline__ double helm(const Fc &f, const Helm &h, double xp, double xm,
                                       double yp, double ym, double zp, double zm,
                                       double rhs) {
  const double diag =
      1.0 + h.ax2 * (f.px + f.mx) + h.ay2 * (f.py + f.my) + h.az2 * (f.pz + f.mz);
  return (h.ax2 * (f.px * xp + f.mx * xm) + h.ay2 * (f.py * yp + f.my * ym) +
          h.az2 * (f.pz * zp + f.mz * zm) + rhs) /
         diag;
}

// ---------------------------------------------------------------------------
// get_conv_all / get_diffusion_all point forms.
template <typename T>
struct CDT {
  T conv, diff;
};

// INTERIOR: the caller knows 0 < k < nz-1, so the wall-level forms of u and
// v (k = 0, nz-1) are left out at compile time (if-converted, their FP64
// instructions would occupy GB300's FP64 pipe on every level).
template <typename T, bool INTERIOR = false>
__device__ __forceinline__ CDT<T> conv_diff(int comp, const Geo &g, T rdx, T rdy, T rdz,
                                            const T *__restrict__ U, const T *__restrict__ V,
                                            const T *__restrict__ W, const FcT<T> &f, int i, int j,
                                            int k) {
  const int sy = g.sy, sz = g.sz, nzu = g.nz;  // u/v have planes 0..nz-1
  const int c = TPLS_IDX(g, i, j, k);
  const T h = (T)0.5, two = (T)2, third = (T)(1.0 / 3.0);
  const bool kb = !INTERIOR && k == 0, kt = !INTERIOR && k == nzu - 1;
  CDT<T> r;
  if (comp == 0) {
    const T x = U[c];
    const T tempv = (V[c] + V[c + 1] + V[c + sy] + V[c + 1 + sy]) * (T)0.25;
    const T tempw = (W[c] + W[c + 1] + W[c + sz] + W[c + 1 + sz]) * (T)0.25;
    const T Xc = h * (U[c + 1] - U[c - 1]) * rdx * x;
    const T Yc = h * (U[c + sy] - U[c - sy]) * rdy * tempv;
    T dz_;
    if (kb) dz_ = (x + U[c + sz]) * (h * rdz);
    else if (kt) dz_ = -(x + U[c - sz]) * (h * rdz);
    else dz_ = h * (U[c + sz] - U[c - sz]) * rdz;
    const T t1 = Xc + Yc + dz_ * tempw;
    const T E = f.px * (U[c + 1] - x) * rdx, Wt = f.mx * (x - U[c - 1]) * rdx;
    const T N = f.py * (V[c + 1 + sy] - V[c + sy]) * rdx, S = f.my * (V[c + 1] - V[c]) * rdx;
    const T O = f.pz * (W[c + 1 + sz] - W[c + sz]) * rdx, I = f.mz * (W[c + 1] - W[c]) * rdx;
    r.conv = t1 - ((E - Wt) * rdx + (N - S) * rdy + (O - I) * rdz);
    // loads only the planes each form uses (no plane -1 at k = 0, no plane nz at k = nz-1)
    const T umz = kb ? -two * x + U[c + sz] * third : U[c - sz];
    const T upz = kt ? -two * x + U[c - sz] * third : U[c + sz];
    r.diff = (f.px * (U[c + 1] - x) - f.mx * (x - U[c - 1])) * (rdx * rdx) +
             (f.py * (U[c + sy] - x) - f.my * (x - U[c - sy])) * (rdy * rdy) +
             (f.pz * (upz - x) - f.mz * (x - umz)) * (rdz * rdz);
  } else if (comp == 1) {
    const T x = V[c];
    const T tempu = (U[c - 1 - sy] + U[c - 1] + U[c - sy] + U[c]) * (T)0.25;
    const T tempw = (W[c - sy] + W[c] + W[c - sy + sz] + W[c + sz]) * (T)0.25;
    const T Yc = h * (V[c + sy] - V[c - sy]) * rdy * x;
    const T Xc = h * (V[c + 1] - V[c - 1]) * rdx * tempu;
    T dz_;
    if (kb) dz_ = (x + V[c + sz]) * (h * rdz);
    else if (kt) dz_ = -(x + V[c - sz]) * (h * rdz);
    else dz_ = h * (V[c + sz] - V[c - sz]) * rdz;
    const T t1 = Xc + Yc + dz_ * tempw;
    const T E = f.px * (U[c] - U[c - sy]) * rdy, Wt = f.mx * (U[c - 1] - U[c - 1 - sy]) * rdy;
    const T N = f.py * (V[c + sy] - x) * rdy, S = f.my * (x - V[c - sy]) * rdy;
    const T O = f.pz * (W[c + sz] - W[c - sy + sz]) * rdy, I = f.mz * (W[c] - W[c - sy]) * rdy;
    r.conv = t1 - ((E - Wt) * rdx + (N - S) * rdy + (O - I) * rdz);
    // loads only the planes each form uses (no plane -1 at k = 0, no plane nz at k = nz-1)
    const T vmz = kb ? -two * x + V[c + sz] * third : V[c - sz];
    const T vpz = kt ? -two * x + V[c - sz] * third : V[c + sz];
    r.diff = (f.px * (V[c + 1] - x) - f.mx * (x - V[c - 1])) * (rdx * rdx) +
             (f.py * (V[c + sy] - x) - f.my * (x - V[c - sy])) * (rdy * rdy) +
             (f.pz * (vpz - x) - f.mz * (x - vmz)) * (rdz * rdz);
  } else {
    const T x = W[c];
    const T tempu = (U[c - 1 - sz] + U[c - 1] + U[c - sz] + U[c]) * (T)0.25;
    const T tempv = (V[c - sz] + V[c] + V[c + sy - sz] + V[c + sy]) * (T)0.25;
    const T Zc = h * (W[c + sz] - W[c - sz]) * rdz * x;
    const T Xc = h * (W[c + 1] - W[c - 1]) * rdx * tempu;
    const T Yc = h * (W[c + sy] - W[c - sy]) * rdy * tempv;
    const T t1 = Xc + Yc + Zc;
    const T E = f.px * (U[c] - U[c - sz]) * rdz, Wt = f.mx * (U[c - 1] - U[c - 1 - sz]) * rdz;
    const T N = f.py * (V[c + sy] - V[c + sy - sz]) * rdz, S = f.my * (V[c] - V[c - sz]) * rdz;
    const T O = f.pz * (W[c + sz] - x) * rdz, I = f.mz * (x - W[c - sz]) * rdz;
    r.conv = t1 - ((E - Wt) * rdx + (N - S) * rdy + (O - I) * rdz);
    r.diff = (f.px * (W[c + 1] - x) - f.mx * (x - W[c - 1])) * (rdx * rdx) +
             (f.py * (W[c + sy] - x) - f.my * (x - W[c - sy])) * (rdy * rdy) +
             (f.pz * (W[c + sz] - x) - f.mz * (x - W[c - sz])) * (rdz * rdz);
  }
  return r;
}

constexpr int MB_X = 32, MB_Y = 4;

// Domain of a component's conv/diff (get_conv_all ranges) and of the
// right-hand side kernel (whole face range the history arrays carry).
__device__ __forceinline__ bool cd_valid(int comp, const Geo &g, int i, int k) {
  if (comp == 0) return i <= g.nx - 1;
  if (comp == 2) return k >= 1 && k <= g.nz - 1;
  return true;
}

// The sweep coefficients of one point, divided by the Helmholtz diagonal
// (jacobi_iteration_allflux.f90:84-90): x_new = cxp x[i+1] + cxm x[i-1] +
// cyp x[j+1] + cym x[j-1] + czp x[k+1] + czm x[k-1] + rhs/diag.  For u and v
// the wall ghost rule `-2 x(0) + x(1)/3` (and its top mirror) is folded in:
// at k = 0 the czm slot multiplies the point itself and czp absorbs czm/3;
// at k = nz-1 the czp slot multiplies the point itself and czm absorbs
// czp/3.  One 64-byte record per point: (cxp, cxm, cyp, cym, czp, czm, b,
// 1.2 czm), the last the factor of the odd half-sweep's column recurrence.
__device__ __forceinline__ void store_rec(double *rec, double a0, double a1, double a2, double a3, double a4,
                                          double a5, double a6) {
  double2 *o = reinterpret_cast<double2 *>(rec);
  o[0] = make_double2(a0, a1);
  o[1] = make_double2(a2, a3);
  o[2] = make_double2(a4, a5);
  o[3] = make_double2(a6, 1.2 * a5);
}

// The record of one point of the FP64 sweeps.
template <bool INTERIOR>
__device__ __forceinline__ void write_coef(int comp, const Geo &g, const Helm &h, const FcT<double> &f,
                                           double rhs, int k, double *__restrict__ rec) {
  const double ax2 = h.ax2, ay2 = h.ay2, az2 = h.az2;
  const double diag = 1.0 + ax2 * (f.px + f.mx) + ay2 * (f.py + f.my) + az2 * (f.pz + f.mz);
  const double r = 1.0 / diag;
  double czp = az2 * f.pz * r, czm = az2 * f.mz * r;
  if (!INTERIOR && comp != 2) {
    if (k == 0) {
      czp += czm * (1.0 / 3.0);
      czm = -2.0 * czm;
    } else if (k == g.nz - 1) {
      czm += czp * (1.0 / 3.0);
      czp = -2.0 * czp;
    }
  }
  store_rec(rec, ax2 * f.px * r, ax2 * f.mx * r, ay2 * f.py * r, ay2 * f.my * r, czp, czm, rhs * r);
}

// FP64 stencils.  TR = double: the FP64 form's right-hand side and 64-byte
// sweep records (X64 = the component's FP64 state u2, v2 or w2); TR = float:
// the FP32-mixed form with FP64 stencils, which stores the defect b alone.
template <typename T, typename TR, bool INTERIOR>
__device__ __forceinline__ void mom_rhs_point(int comp, const Geo &g, const Phys &ph, const Helm &hm,
                                              const T *__restrict__ U, const T *__restrict__ V,
                                              const T *__restrict__ W, const double *__restrict__ X64,
                                              const T *__restrict__ mu, const T *__restrict__ fc,
                                              const double *__restrict__ c1, const double *__restrict__ c0,
                                              const double *__restrict__ s1, const double *__restrict__ s0,
                                              double *__restrict__ conv2, double *__restrict__ csf2,
                                              double *__restrict__ rhs, double *__restrict__ diff_out,
                                              TR *__restrict__ coef, int i, int j, int k) {
  const int c = TPLS_IDX(g, i, j, k);
  CDT<T> cd = {(T)0, (T)0};
  const bool valid = cd_valid(comp, g, i, k);
  FcT<T> f;
  if (valid) {
    f = faces(comp, g, mu, i, j, k);
    // 1/dx, 1/dy, 1/dz from the host (the same IEEE quotients, not three FP64
    // divisions per point on GB300's FP64 pipe)
    cd = conv_diff<T, INTERIOR>(comp, g, (T)hm.rdx, (T)hm.rdy, (T)hm.rdz, U, V, W, f, i, j, k);
  }
  // main_ns_hybrid.F90:629-641 face averages of the CSF force
  double s2;
  if (comp == 0) s2 = ((double)fc[TPLS_IDX(g, i + 1, j + 1, k + 1)] + (double)fc[TPLS_IDX(g, i, j + 1, k + 1)]) * 0.5;
  else if (comp == 1) s2 = ((double)fc[TPLS_IDX(g, i, j + 1, k + 1)] + (double)fc[TPLS_IDX(g, i, j, k + 1)]) * 0.5;
  else s2 = ((double)fc[TPLS_IDX(g, i, j + 1, k + 1)] + (double)fc[TPLS_IDX(g, i, j + 1, k)]) * 0.5;
  const double dt = ph.dt, conv = (double)cd.conv, diff = (double)cd.diff;
  if constexpr (sizeof(TR) == sizeof(float)) {
    // FP32 defect-form sweeps: b = R / diag with R = dt (diff - AB3(conv) +
    // AB3(csf)), the defect equation's right-hand side (see k_mom_rhs_pair),
    // here in FP64; the sweeps rebuild the coefficients themselves
    conv2[c] = conv;
    csf2[c] = s2;
    if (coef && valid) {
      const double abc = (23.0 / 12.0) * conv - (4.0 / 3.0) * c1[c] + (5.0 / 12.0) * c0[c];
      const double abs_ = (23.0 / 12.0) * s2 - (4.0 / 3.0) * s1[c] + (5.0 / 12.0) * s0[c];
      const double diag =
          1.0 + hm.ax2 * (f.px + f.mx) + hm.ay2 * (f.py + f.my) + hm.az2 * (f.pz + f.mz);
      coef[rec_slot(g, c, i)] = (TR)(dt * (diff - abc + abs_) / diag);
    }
  } else {
    const double X = X64[c];
    // main_ns_hybrid.F90:743-751 (AB3 convection and CSF, CN diffusion)
    const double r = X - dt * ((23.0 / 12.0) * conv - (4.0 / 3.0) * c1[c] + (5.0 / 12.0) * c0[c]) +
                     (dt / 2.0) * diff +
                     dt * ((23.0 / 12.0) * s2 - (4.0 / 3.0) * s1[c] + (5.0 / 12.0) * s0[c]);
    conv2[c] = conv;
    csf2[c] = s2;
    if (rhs) rhs[c] = r;
    if (diff_out) diff_out[c] = diff;
    if (coef && valid) write_coef<INTERIOR>(comp, g, hm, f, r, k, coef + 8 * (size_t)rec_slot(g, c, i));
  }
}

// CC: the velocity component at compile time.  The wall levels of u and v
// (k = 0, nz-1) take their own copy of the point code by a block-uniform
// branch, so the interior levels carry none of the wall forms.
template <typename T, typename TR, int CC>
__global__ void __launch_bounds__(MB_X *MB_Y)
    k_mom_rhs(Geo g, Phys ph, Helm hm, const T *__restrict__ U, const T *__restrict__ V,
              const T *__restrict__ W, const double *__restrict__ X64, const T *__restrict__ mu,
              const T *__restrict__ fc, const double *__restrict__ c1, const double *__restrict__ c0,
              const double *__restrict__ s1, const double *__restrict__ s0, double *__restrict__ conv2,
              double *__restrict__ csf2, double *__restrict__ rhs, double *__restrict__ diff_out,
              TR *__restrict__ coef) {
  const int i = blockIdx.x * MB_X + threadIdx.x + 1, j = blockIdx.y * MB_Y + threadIdx.y + 1;
  const int k = blockIdx.z;
  if (i > g.nx || j > g.ny) return;
  if (CC != 2 && (k == 0 || k == g.nz - 1))
    mom_rhs_point<T, TR, false>(CC, g, ph, hm, U, V, W, X64, mu, fc, c1, c0, s1, s0, conv2, csf2, rhs, diff_out,
                                coef, i, j, k);
  else
    mom_rhs_point<T, TR, true>(CC, g, ph, hm, U, V, W, X64, mu, fc, c1, c0, s1, s0, conv2, csf2, rhs, diff_out,
                               coef, i, j, k);
}

template <typename T, typename TR = T>
static cudaError_t mom_rhs(int comp, const Geo &g, const Phys &ph, const T *u2, const T *v2, const T *w2,
                           const double *x64, const T *mu, const T *fcsf, const double *c1, const double *c0,
                           const double *s1, const double *s0, double *conv2, double *csf2, double *rhs,
                           double *diff_out, TR *coef, cudaStream_t st) {
  const int nk = (comp == 2) ? g.nz + 1 : g.nz;
  dim3 grd((g.nx + MB_X - 1) / MB_X, (g.ny + MB_Y - 1) / MB_Y, nk);
  const Helm hm = helm_of(ph);
  if (comp == 0)
    k_mom_rhs<T, TR, 0><<<grd, dim3(MB_X, MB_Y), 0, st>>>(g, ph, hm, u2, v2, w2, x64, mu, fcsf, c1, c0, s1, s0,
                                                          conv2, csf2, rhs, diff_out, coef);
  else if (comp == 1)
    k_mom_rhs<T, TR, 1><<<grd, dim3(MB_X, MB_Y), 0, st>>>(g, ph, hm, u2, v2, w2, x64, mu, fcsf, c1, c0, s1, s0,
                                                          conv2, csf2, rhs, diff_out, coef);
  else
    k_mom_rhs<T, TR, 2><<<grd, dim3(MB_X, MB_Y), 0, st>>>(g, ph, hm, u2, v2, w2, x64, mu, fcsf, c1, c0, s1, s0,
                                                          conv2, csf2, rhs, diff_out, coef);
  return cudaGetLastError();
}

cudaError_t launch_mom_rhs(int comp, const Geo &g, const Phys &ph,
                           const double *u2, const double *v2,
                           const double *w2, const double *mu,
                           const double *fcsf, const double *c1,
                           const double *c0, const double *s1,
                           const double *s0, double *conv2, double *csf2,
                           double *rhs, double *diff_out, double *coef, cudaStream_t st) {
  const double *x64 = (comp == 0) ? u2 : (comp == 1) ? v2 : w2;
  return mom_rhs<double>(comp, g, ph, u2, v2, w2, x64, mu, fcsf, c1, c0, s1, s0, conv2, csf2, rhs, diff_out,
                         coef, st);
}

cudaError_t launch_mom_rhs64r32(int comp, const Geo &g, const Phys &ph, const double *u2, const double *v2,
                                const double *w2, const double *mu, const double *fcsf, const double *c1,
                                const double *c0, const double *s1, const double *s0, double *conv2,
                                double *csf2, float *bdef, cudaStream_t st) {
  const double *x64 = (comp == 0) ? u2 : (comp == 1) ? v2 : w2;
  return mom_rhs<double, float>(comp, g, ph, u2, v2, w2, x64, mu, fcsf, c1, c0, s1, s0, conv2, csf2, nullptr,
                                nullptr, bdef, st);
}
// ---------------------------------------------------------------------------
// FP32 momentum stencils of the FP32-mixed form on the FP64 velocity state.
//
// Each FP64 value is split by integer operations into an FP32 pair
// (hi = the value truncated to 24 significant bits, lo = the FP32 rounding
// of the remainder), so no FP64 instruction is issued: on GB300 FP64
// arithmetic and FP64<->FP32 conversions share a pipe 64x slower than FP32.
// Neighbour differences are formed as (hi_a - hi_b) + (lo_a - lo_b), which
// carries the FP32 precision of the difference itself instead of that of
// the O(|u|) values: the stencils' cancellations (first and second
// differences of a smooth field) then cost 1e-7 of the difference, not of
// |u|.  Sums and products use the pair rounded to FP32.
__device__ __forceinline__ F2 ld2(const double *__restrict__ p) { return split_bits(__ldg(p)); }

// float constants of one step (computed on the host in FP64, then rounded)
struct MomF {
  float rdx, rdy, rdz, dt, ax2, ay2, az2;
  double dt64;
};

// get_conv_all / get_diffusion_all point forms (momentum_allflux.f90:22-471)
// on split values; the same operations as conv_diff with every difference
// of two velocity values taken from the pairs.  At the walls (u, v: k = 0
// and nz-1) the ghost value -2 x + x(k+-1)/3 enters as the difference
// x(k+-1)/3 - 3 x.
__device__ __forceinline__ CDT<float> conv_diff_pair(int comp, const Geo &g, const MomF &m,
                                                     const double *__restrict__ U, const double *__restrict__ V,
                                                     const double *__restrict__ W, const FcT<float> &f, int i,
                                                     int j, int k) {
  const int sy = g.sy, sz = g.sz, nzu = g.nz;
  const int c = TPLS_IDX(g, i, j, k);
  const float h = 0.5f, third = (float)(1.0 / 3.0), rdx = m.rdx, rdy = m.rdy, rdz = m.rdz;
  CDT<float> r;
  if (comp == 0 || comp == 1) {
    const double *S = comp == 0 ? U : V;
    const F2 x = ld2(S + c), xe = ld2(S + c + 1), xw = ld2(S + c - 1), xn = ld2(S + c + sy), xs = ld2(S + c - sy);
    float dT, dB, dzc;  // x(k+1) - x, x - x(k-1) (ghosts at the walls), centred z difference term
    if (k == 0) {
      const F2 xt = ld2(S + c + sz);
      dT = dif(xt, x);
      dB = (3.0f * x.h - xt.h * third) + (3.0f * x.l - xt.l * third);
      dzc = (val(x) + val(xt)) * (h * rdz);
    } else if (k == nzu - 1) {
      const F2 xb = ld2(S + c - sz);
      dB = dif(x, xb);
      dT = (xb.h * third - 3.0f * x.h) + (xb.l * third - 3.0f * x.l);
      dzc = -(val(x) + val(xb)) * (h * rdz);
    } else {
      const F2 xt = ld2(S + c + sz), xb = ld2(S + c - sz);
      dT = dif(xt, x);
      dB = dif(x, xb);
      dzc = h * dif(xt, xb) * rdz;
    }
    const float dE = dif(xe, x), dW = dif(x, xw), dN = dif(xn, x), dS = dif(x, xs);
    float t1, E, Wt, N, Sf, O, I;
    if (comp == 0) {
      const F2 v0 = ld2(V + c), v1 = ld2(V + c + 1), v2 = ld2(V + c + sy), v3 = ld2(V + c + 1 + sy);
      const F2 w0 = ld2(W + c), w1 = ld2(W + c + 1), w2 = ld2(W + c + sz), w3 = ld2(W + c + 1 + sz);
      const float tempv = (val(v0) + val(v1) + val(v2) + val(v3)) * 0.25f;
      const float tempw = (val(w0) + val(w1) + val(w2) + val(w3)) * 0.25f;
      const float Xc = h * dif(xe, xw) * rdx * val(x);
      const float Yc = h * dif(xn, xs) * rdy * tempv;
      t1 = Xc + Yc + dzc * tempw;
      E = f.px * dE * rdx;
      Wt = f.mx * dW * rdx;
      N = f.py * dif(v3, v2) * rdx;
      Sf = f.my * dif(v1, v0) * rdx;
      O = f.pz * dif(w3, w2) * rdx;
      I = f.mz * dif(w1, w0) * rdx;
    } else {
      const F2 u0 = ld2(U + c - 1 - sy), u1 = ld2(U + c - 1), u2 = ld2(U + c - sy), u3 = ld2(U + c);
      const F2 w0 = ld2(W + c - sy), w1 = ld2(W + c), w2 = ld2(W + c - sy + sz), w3 = ld2(W + c + sz);
      const float tempu = (val(u0) + val(u1) + val(u2) + val(u3)) * 0.25f;
      const float tempw = (val(w0) + val(w1) + val(w2) + val(w3)) * 0.25f;
      const float Yc = h * dif(xn, xs) * rdy * val(x);
      const float Xc = h * dif(xe, xw) * rdx * tempu;
      t1 = Xc + Yc + dzc * tempw;
      E = f.px * dif(u3, u2) * rdy;
      Wt = f.mx * dif(u1, u0) * rdy;
      N = f.py * dN * rdy;
      Sf = f.my * dS * rdy;
      O = f.pz * dif(w3, w2) * rdy;
      I = f.mz * dif(w1, w0) * rdy;
    }
    r.conv = t1 - ((E - Wt) * rdx + (N - Sf) * rdy + (O - I) * rdz);
    r.diff = (f.px * dE - f.mx * dW) * (rdx * rdx) + (f.py * dN - f.my * dS) * (rdy * rdy) +
             (f.pz * dT - f.mz * dB) * (rdz * rdz);
  } else {
    const F2 x = ld2(W + c), xe = ld2(W + c + 1), xw = ld2(W + c - 1), xn = ld2(W + c + sy), xs = ld2(W + c - sy);
    const F2 xt = ld2(W + c + sz), xb = ld2(W + c - sz);
    const F2 u0 = ld2(U + c - 1 - sz), u1 = ld2(U + c - 1), u2 = ld2(U + c - sz), u3 = ld2(U + c);
    const F2 v0 = ld2(V + c - sz), v1 = ld2(V + c), v2 = ld2(V + c + sy - sz), v3 = ld2(V + c + sy);
    const float tempu = (val(u0) + val(u1) + val(u2) + val(u3)) * 0.25f;
    const float tempv = (val(v0) + val(v1) + val(v2) + val(v3)) * 0.25f;
    const float Zc = h * dif(xt, xb) * rdz * val(x);
    const float Xc = h * dif(xe, xw) * rdx * tempu;
    const float Yc = h * dif(xn, xs) * rdy * tempv;
    const float t1 = Xc + Yc + Zc;
    const float dE = dif(xe, x), dW = dif(x, xw), dN = dif(xn, x), dS = dif(x, xs);
    const float dT = dif(xt, x), dB = dif(x, xb);
    const float E = f.px * dif(u3, u2) * rdz, Wt = f.mx * dif(u1, u0) * rdz;
    const float N = f.py * dif(v3, v2) * rdz, Sf = f.my * dif(v1, v0) * rdz;
    const float O = f.pz * dT * rdz, I = f.mz * dB * rdz;
    r.conv = t1 - ((E - Wt) * rdx + (N - Sf) * rdy + (O - I) * rdz);
    r.diff = (f.px * dE - f.mx * dW) * (rdx * rdx) + (f.py * dN - f.my * dS) * (rdy * rdy) +
             (f.pz * dT - f.mz * dB) * (rdz * rdz);
  }
  return r;
}

// Right-hand side of the FP32-mixed form's sweeps with FP32 stencils.
// The sweeps solve for the defect d = x - X (X the FP64 state of the
// component): with diag x - sum(a_n x_n) = rhs and diag = 1 + sum(a_n), the
// defect equation's right-hand side is
//   R = (rhs - X) + sum(a_n (X_n - X)) = dt (diff - AB3(conv) + AB3(csf)),
// because sum(a_n (X_n - X)) = (dt/2) diff for the same ghost-substituted
// neighbours (main_ns_hybrid.F90:743-751 for rhs).  conv and diff come from
// the FP32 pair stencils; the CSF force, the AB3 histories and R stay FP64
// (eleven FP64 operations per point): the CSF force is large at the
// interface, where it is balanced by the pressure gradient outside R, so its
// rounding is not relative to the step's increment.  Stored: b = R / diag,
// one float per point in record-slot order (the sweeps recompute the
// coefficients from mu).  conv is stored into its FP64 history exactly.
__global__ void __launch_bounds__(MB_X *MB_Y)
    k_mom_rhs_pair(int comp, Geo g, MomF m, const double *__restrict__ U, const double *__restrict__ V,
                   const double *__restrict__ W, const float *__restrict__ mu, const double *__restrict__ fc,
                   const double *__restrict__ c1, const double *__restrict__ c0, const double *__restrict__ s1,
                   const double *__restrict__ s0, double *__restrict__ conv2, double *__restrict__ csf2,
                   float *__restrict__ bdef) {
  const int i = blockIdx.x * MB_X + threadIdx.x + 1, j = blockIdx.y * MB_Y + threadIdx.y + 1;
  const int k = blockIdx.z;
  if (i > g.nx || j > g.ny) return;
  const int c = TPLS_IDX(g, i, j, k);
  CDT<float> cd = {0.0f, 0.0f};
  const bool valid = cd_valid(comp, g, i, k);
  FcT<float> f;
  if (valid) {
    f = faces<float>(comp, g, mu, i, j, k);
    cd = conv_diff_pair(comp, g, m, U, V, W, f, i, j, k);
  }
  // main_ns_hybrid.F90:629-641 face averages of the CSF force
  double s2;
  if (comp == 0) s2 = (fc[TPLS_IDX(g, i + 1, j + 1, k + 1)] + fc[TPLS_IDX(g, i, j + 1, k + 1)]) * 0.5;
  else if (comp == 1) s2 = (fc[TPLS_IDX(g, i, j + 1, k + 1)] + fc[TPLS_IDX(g, i, j, k + 1)]) * 0.5;
  else s2 = (fc[TPLS_IDX(g, i, j + 1, k + 1)] + fc[TPLS_IDX(g, i, j + 1, k)]) * 0.5;
  const double conv = widen_bits(cd.conv);
  conv2[c] = conv;
  csf2[c] = s2;
  if (!valid) return;
  const double abc = (23.0 / 12.0) * conv - (4.0 / 3.0) * c1[c] + (5.0 / 12.0) * c0[c];
  const double abs_ = (23.0 / 12.0) * s2 - (4.0 / 3.0) * s1[c] + (5.0 / 12.0) * s0[c];
  const double R = m.dt64 * (widen_bits(cd.diff) - abc + abs_);
  const float diag = 1.0f + m.ax2 * (f.px + f.mx) + m.ay2 * (f.py + f.my) + m.az2 * (f.pz + f.mz);
  bdef[rec_slot(g, c, i)] = round_bits(R) / diag;
}

cudaError_t launch_mom_rhs_pair(int comp, const Geo &g, const Phys &ph, const double *u2, const double *v2,
                                const double *w2, const float *mu, const double *fcsf, const double *c1,
                                const double *c0, const double *s1, const double *s0, double *conv2,
                                double *csf2, float *bdef, cudaStream_t st) {
  const Helm hm = helm_of(ph);
  MomF m;
  m.rdx = (float)(1.0 / ph.dx);
  m.rdy = (float)(1.0 / ph.dy);
  m.rdz = (float)(1.0 / ph.dz);
  m.dt = (float)ph.dt;
  m.dt64 = ph.dt;
  m.ax2 = (float)hm.ax2;
  m.ay2 = (float)hm.ay2;
  m.az2 = (float)hm.az2;
  const int nk = (comp == 2) ? g.nz + 1 : g.nz;
  dim3 grd((g.nx + MB_X - 1) / MB_X, (g.ny + MB_Y - 1) / MB_Y, nk);
  k_mom_rhs_pair<<<grd, dim3(MB_X, MB_Y), 0, st>>>(comp, g, m, u2, v2, w2, mu, fcsf, c1, c0, s1, s0, conv2, csf2,
                                                   bdef);
  return cudaGetLastError();
}

// standalone get_conv_all / get_diffusion_all: out = conv or diff on the
// component's domain (other entries are left untouched; the caller zeroes).
__global__ void k_conv_diff(int comp, int want_conv, Geo g, Phys ph, const double *__restrict__ U,
                            const double *__restrict__ V, const double *__restrict__ W,
                            const double *__restrict__ mu, double *__restrict__ out) {
  const int i = blockIdx.x * MB_X + threadIdx.x + 1, j = blockIdx.y * MB_Y + threadIdx.y + 1;
  const int k = blockIdx.z;
  if (i > g.nx || j > g.ny || !cd_valid(comp, g, i, k)) return;
  const Fc f = faces(comp, g, mu, i, j, k);
  CDT<double> cd = conv_diff<double>(comp, g, 1.0 / ph.dx, 1.0 / ph.dy, 1.0 / ph.dz, U, V, W, f, i, j, k);
  out[TPLS_IDX(g, i, j, k)] = want_conv ? cd.conv : cd.diff;
}

cudaError_t launch_conv_diff(int comp, int want_conv, const Geo &g,
                             const Phys &ph, const double *u2,
                             const double *v2, const double *w2,
                             const double *mu, double *out, cudaStream_t st) {
  const int nk = (comp == 2) ? g.nz + 1 : g.nz;
  dim3 grd((g.nx + MB_X - 1) / MB_X, (g.ny + MB_Y - 1) / MB_Y, nk);
  k_conv_diff<<<grd, dim3(MB_X, MB_Y), 0, st>>>(comp, want_conv, g, ph, u2, v2, w2, mu, out);
  return cudaGetLastError();
}

// z neighbours for u/v with the wall ghost rule `-2*x(0)+x(1)/3`
// (jacobi_iteration_allflux.f90:63-73)
__device__ __forceinline__ double zm_uv(const double *x, int c, int k, int sz) {
  return (k == 0) ? -2.0 * x[c] + x[c + sz] * (1.0 / 3.0) : x[c - sz];
}
__device__ __forceinline__ double zp_uv(const double *x, int c, int k, int nzu, int sz) {
  return (k == nzu - 1) ? -2.0 * x[c] + x[c - sz] * (1.0 / 3.0) : x[c + sz];
}

// jacobi_iteration_allflux.f90:21-282 with the routine's own boundary rows
// (v, w) and, for bc=1, the driver's u boundary rows (:762-776).
__global__ void __launch_bounds__(MB_X *MB_Y)
    k_jacobi(int comp, Geo g, Helm h, const double *__restrict__ xo,
             const double *__restrict__ rhs, const double *__restrict__ mu,
             const double *__restrict__ P, double *__restrict__ x, int bc, int fuse) {
  const int i = blockIdx.x * MB_X + threadIdx.x + 1, j = blockIdx.y * MB_Y + threadIdx.y + 1;
  const int k = blockIdx.z + (comp == 2 ? 1 : 0);
  const int iend = (comp == 0) ? g.nx - 1 : g.nx;
  if (i > iend || j > g.ny) return;
  const int c = TPLS_IDX(g, i, j, k), sy = g.sy, sz = g.sz;
  const Fc f = faces(comp, g, mu, i, j, k);
  double zp, zm;
  if (comp == 2) {
    zp = xo[c + sz];
    zm = xo[c - sz];
  } else {
    zp = zp_uv(xo, c, k, g.nz, sz);
    zm = zm_uv(xo, c, k, sz);
  }
  const double v = helm(f, h, xo[c + 1], xo[c - 1], xo[c + sy], xo[c - sy], zp, zm, rhs[c]);
  put(g, x, i, j, k, v, fuse);
  if (comp == 0) {
    if (bc) {
      if (i == 1) put(g, x, 0, j, k, v, fuse);
      if (i == g.nx - 1) {
        put(g, x, g.nx, j, k, u_outlet(g, h, P, v, j, k), fuse);
        put(g, x, g.nx + 1, j, k, 0.0, fuse);
      }
    }
  } else if (comp == 1) {  // jacobi_iteration_allflux.f90:178-189
    if (i == 1) put(g, x, 0, j, k, v, fuse);
    if (i == g.nx) put(g, x, g.nx + 1, j, k, v, fuse);
  } else {  // jacobi_iteration_allflux.f90:257-279
    const int nz = g.nz;
    if (k == 1) put(g, x, i, j, 0, 0.0, fuse);
    if (k == nz - 1) put(g, x, i, j, nz, 0.0, fuse);
    if (i == 1) {
      put(g, x, 0, j, k, v, fuse);
      if (k == 1) put(g, x, 0, j, 0, 0.0, fuse);
      if (k == nz - 1) put(g, x, 0, j, nz, 0.0, fuse);
    }
    if (i == g.nx) {
      put(g, x, g.nx + 1, j, k, v, fuse);
      if (k == 1) put(g, x, g.nx + 1, j, 0, 0.0, fuse);
      if (k == nz - 1) put(g, x, g.nx + 1, j, nz, 0.0, fuse);
    }
  }
}

cudaError_t launch_jacobi(int comp, const Geo &g, const Phys &ph,
                          const double *xo, const double *rhs,
                          const double *mu, const double *pres, double *x,
                          int bc, int fuse_ghosts, cudaStream_t st) {
  Helm h;
  h.ax2 = (ph.dt / (ph.dx * ph.dx)) / 2.0;
  h.ay2 = (ph.dt / (ph.dy * ph.dy)) / 2.0;
  h.az2 = (ph.dt / (ph.dz * ph.dz)) / 2.0;
  h.dtdx = ph.dt / ph.dx;
  const int nk = (comp == 2) ? g.nz - 1 : g.nz;
  const int iend = (comp == 0) ? g.nx - 1 : g.nx;
  dim3 grd((iend + MB_X - 1) / MB_X, (g.ny + MB_Y - 1) / MB_Y, nk);
  k_jacobi<<<grd, dim3(MB_X, MB_Y), 0, st>>>(comp, g, h, xo, rhs, mu, pres, x, bc, fuse_ghosts);
  return cudaGetLastError();
}

// sor_iteration_allflux.f90:54-99 (and v, w): 3-D checkerboard half-sweep.
__global__ void __launch_bounds__(MB_X *MB_Y)
    k_sor_even(int comp, Geo g, Helm h, double *__restrict__ x, const double *__restrict__ rhs,
               const double *__restrict__ mu, const double *__restrict__ P, int flg, int bc,
               int fuse) {
  const int i2 = blockIdx.x * MB_X + threadIdx.x, j = blockIdx.y * MB_Y + threadIdx.y + 1;
  const int k = blockIdx.z + (comp == 2 ? 1 : 0);
  const int iend = (comp == 0) ? g.nx - 1 : g.nx;
  if (i2 > (iend - 1) / 2 || j > g.ny) return;
  const int i = 2 * i2 + 1 + ((k + j + flg) & 1);
  double v = 0.0;
  if (i <= iend) {
    const int c = TPLS_IDX(g, i, j, k), sy = g.sy, sz = g.sz;
    const Fc f = faces(comp, g, mu, i, j, k);
    double zp, zm;
    if (comp == 2) {
      zp = x[c + sz];
      zm = x[c - sz];
    } else {
      zp = zp_uv(x, c, k, g.nz, sz);
      zm = zm_uv(x, c, k, sz);
    }
    const double xc = x[c];
    const double res = helm(f, h, x[c + 1], x[c - 1], x[c + sy], x[c - sy], zp, zm, rhs[c]);
    v = xc + 1.2 * (res - xc);
    put(g, x, i, j, k, v, fuse);
  }
  if (bc) sor_bc(comp, g, h, x, (const double *)nullptr, P, i2, i, iend, v, j, k, fuse);
}

// sor_iteration_allflux.f90:100-146 (and v, w): 2-D colouring, sequential
// in k within each column.
__global__ void __launch_bounds__(MB_X *MB_Y)
    k_sor_odd(int comp, Geo g, Helm h, double *__restrict__ x, const double *__restrict__ rhs,
              const double *__restrict__ mu, const double *__restrict__ P, int flg, int bc,
              int fuse) {
  const int i2 = blockIdx.x * MB_X + threadIdx.x, j = blockIdx.y * MB_Y + threadIdx.y + 1;
  const int iend = (comp == 0) ? g.nx - 1 : g.nx;
  if (i2 > (iend - 1) / 2 || j > g.ny) return;
  const int i = 2 * i2 + 1 + ((j + flg) & 1);
  const bool act = (i <= iend);
  const int sy = g.sy, sz = g.sz, nz = g.nz;
  const int k0 = (comp == 2) ? 1 : 0, k1 = nz - 1;
  double prev = 0.0;  // relaxed value at k-1 in this column
  for (int k = k0; k <= k1; k++) {
    double v = 0.0;
    if (act) {
      const int c = TPLS_IDX(g, i, j, k);
      const Fc f = faces(comp, g, mu, i, j, k);
      const double xc = x[c];
      double zp, zm;
      if (comp == 2) {
        zm = (k == k0) ? x[c - sz] : prev;
        zp = x[c + sz];
      } else {
        zm = (k == 0) ? -2.0 * xc + x[c + sz] * (1.0 / 3.0) : prev;
        zp = (k == nz - 1) ? -2.0 * xc + prev * (1.0 / 3.0) : x[c + sz];
      }
      const double res = helm(f, h, x[c + 1], x[c - 1], x[c + sy], x[c - sy], zp, zm, rhs[c]);
      v = xc + 1.2 * (res - xc);
      put(g, x, i, j, k, v, fuse);
      prev = v;
    }
    if (bc) sor_bc(comp, g, h, x, (const double *)nullptr, P, i2, i, iend, v, j, k, fuse);
  }
}

cudaError_t launch_sor(int comp, const Geo &g, const Phys &ph, double *x,
                       const double *rhs, const double *mu,
                       const double *pres, int flg, int iteration_time,
                       int bc, int fuse_ghosts, cudaStream_t st) {
  Helm h;
  h.ax2 = (ph.dt / (ph.dx * ph.dx)) / 2.0;
  h.ay2 = (ph.dt / (ph.dy * ph.dy)) / 2.0;
  h.az2 = (ph.dt / (ph.dz * ph.dz)) / 2.0;
  h.dtdx = ph.dt / ph.dx;
  const int iend = (comp == 0) ? g.nx - 1 : g.nx;
  const int npairs = (iend + 1) / 2;
  if (iteration_time % 2 == 0) {
    const int nk = (comp == 2) ? g.nz - 1 : g.nz;
    dim3 grd((npairs + MB_X - 1) / MB_X, (g.ny + MB_Y - 1) / MB_Y, nk);
    k_sor_even<<<grd, dim3(MB_X, MB_Y), 0, st>>>(comp, g, h, x, rhs, mu, pres, flg, bc, fuse_ghosts);
  } else {
    dim3 grd((npairs + MB_X - 1) / MB_X, (g.ny + MB_Y - 1) / MB_Y, 1);
    k_sor_odd<<<grd, dim3(MB_X, MB_Y), 0, st>>>(comp, g, h, x, rhs, mu, pres, flg, bc, fuse_ghosts);
  }
  return cudaGetLastError();
}

// get_difference: per-block partials of sum (a-b)^2 over i 1..nx, j 1..ny,
// planes 0..nzp-1.
// Sum of squared differences of two iterates (the sweeps' convergence
// diagnostic), one partial per block.  FP64 iterates are differenced and
// summed in FP64; FP32 iterates in FP32 up to the warp sums (exactly
// widened), so the FP32 form issues no FP64 instruction per point.
template <typename T>
__global__ void k_diff2(Geo g, const T *__restrict__ a, const T *__restrict__ b, double *__restrict__ part) {
  const int i = blockIdx.x * MB_X + threadIdx.x + 1, j = blockIdx.y * MB_Y + threadIdx.y + 1;
  const int k = blockIdx.z;
  T e = (T)0;
  if (i <= g.nx && j <= g.ny) {
    const int c = TPLS_IDX(g, i, j, k);
    const T d = a[c] - b[c];
    e = d * d;
  }
  __shared__ double s[MB_X * MB_Y / 32];
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
  const int t = threadIdx.y * MB_X + threadIdx.x;
  if constexpr (sizeof(T) == sizeof(float)) {
    if ((t & 31) == 0) s[t >> 5] = widen_bits(e);
  } else {
    if ((t & 31) == 0) s[t >> 5] = e;
  }
  __syncthreads();
  if (t == 0) {
    double acc = 0.0;
    for (int q = 0; q < MB_X * MB_Y / 32; q++) acc += s[q];
    part[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = acc;
  }
}

int diff2_blocks(const Geo &g, int nzp) {
  return ((g.nx + MB_X - 1) / MB_X) * ((g.ny + MB_Y - 1) / MB_Y) * nzp;
}

template <typename T>
static cudaError_t diff2(const Geo &g, const T *a, const T *b, int nzp, double *part, cudaStream_t st) {
  dim3 grd((g.nx + MB_X - 1) / MB_X, (g.ny + MB_Y - 1) / MB_Y, nzp);
  k_diff2<T><<<grd, dim3(MB_X, MB_Y), 0, st>>>(g, a, b, part);
  return cudaGetLastError();
}
cudaError_t launch_diff2(const Geo &g, const double *a, const double *b, int nzp, double *part,
                         cudaStream_t st) {
  return diff2(g, a, b, nzp, part, st);
}
cudaError_t launch_diff2(const Geo &g, const float *a, const float *b, int nzp, double *part,
                         cudaStream_t st) {
  return diff2(g, a, b, nzp, part, st);
}

// ---------------------------------------------------------------------------
// pressure.f90:16-56 get_source_pres on the full p-grid (zero outside the
// interior, ghost rows included, as the routine itself leaves them).
template <typename T>
__global__ void k_source(Geo g, double rdx, double rdy, double rdz, double rdt, const T *__restrict__ U,
                         const T *__restrict__ V, const T *__restrict__ W, double *__restrict__ rhs) {
  const int i = blockIdx.x * MB_X + threadIdx.x, j = blockIdx.y * MB_Y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.nx + 1 || j > g.ny + 1) return;
  double r = 0.0;
  if (i >= 1 && i <= g.nx && j >= 1 && j <= g.ny && k >= 1 && k <= g.nz) {
    const int jj = j, jm = (jj == 1) ? g.ny : jj - 1;
    r = (((double)U[TPLS_IDX(g, i, jm, k - 1)] - (double)U[TPLS_IDX(g, i - 1, jm, k - 1)]) * rdx +
         ((double)V[TPLS_IDX(g, i, jj, k - 1)] - (double)V[TPLS_IDX(g, i, jm, k - 1)]) * rdy +
         ((double)W[TPLS_IDX(g, i, jm, k)] - (double)W[TPLS_IDX(g, i, jm, k - 1)]) * rdz) *
        rdt;
  }
  rhs[TPLS_IDX(g, i, j, k)] = r;
}

template <typename T>
static cudaError_t source(const Geo &g, const Phys &ph, const T *u3, const T *v3, const T *w3, double *rhs_p,
                          cudaStream_t st) {
  dim3 grd((g.nx + 2 + MB_X - 1) / MB_X, (g.ny + 2 + MB_Y - 1) / MB_Y, g.nz + 2);
  k_source<T><<<grd, dim3(MB_X, MB_Y), 0, st>>>(g, 1.0 / ph.dx, 1.0 / ph.dy, 1.0 / ph.dz, 1.0 / ph.dt, u3, v3,
                                                w3, rhs_p);
  return cudaGetLastError();
}
cudaError_t launch_source(const Geo &g, const Phys &ph, const double *u3, const double *v3, const double *w3,
                          double *rhs_p, cudaStream_t st) {
  return source(g, ph, u3, v3, w3, rhs_p, st);
}

// pressure.f90:59-134 get_uvw_pres, written out of place into the next
// state's velocity arrays over x 0..nx+1 and every row (ghost rows as
// periodic copies).
template <typename T>
__global__ void k_project(Geo g, double dtdx, double dtdy, double dtdz, const T *__restrict__ U,
                          const T *__restrict__ V, const T *__restrict__ W, const double *__restrict__ P,
                          const double *__restrict__ uin, double *__restrict__ uo,
                          double *__restrict__ vo, double *__restrict__ wo) {
  const int i = blockIdx.x * MB_X + threadIdx.x, j = blockIdx.y * MB_Y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.nx + 1 || j > g.ny + 1) return;
  const int jj = wrapy(j, g.ny);
  const int c = TPLS_IDX(g, i, j, k), cc = TPLS_IDX(g, i, jj, k);
  const int sy = g.sy, sz = g.sz;
  if (k <= g.nz - 1) {
    double u;
    if (i == 0) u = uin[k];
    else if (i == g.nx + 1) u = 0.0;
    else u = (double)U[cc] - dtdx * (P[cc + 1 + sy + sz] - P[cc + sy + sz]);
    uo[c] = u;
    vo[c] = (double)V[cc] - dtdy * (P[cc + sy + sz] - P[cc + sz]);
  }
  wo[c] = (double)W[cc] - dtdz * (P[cc + sy + sz] - P[cc + sy]);
}

template <typename T>
static cudaError_t project(const Geo &g, const Phys &ph, const T *u3, const T *v3, const T *w3, const double *p,
                           const double *u_inlet, double *u_out, double *v_out, double *w_out, cudaStream_t st) {
  dim3 grd((g.nx + 2 + MB_X - 1) / MB_X, (g.ny + 2 + MB_Y - 1) / MB_Y, g.nz + 1);
  k_project<T><<<grd, dim3(MB_X, MB_Y), 0, st>>>(g, ph.dt / ph.dx, ph.dt / ph.dy, ph.dt / ph.dz, u3, v3, w3, p,
                                                 u_inlet, u_out, v_out, w_out);
  return cudaGetLastError();
}
cudaError_t launch_project(const Geo &g, const Phys &ph, const double *u3, const double *v3, const double *w3,
                           const double *p, const double *u_inlet, double *u_out, double *v_out, double *w_out,
                           cudaStream_t st) {
  return project(g, ph, u3, v3, w3, p, u_inlet, u_out, v_out, w_out, st);
}


}  // namespace tpls
