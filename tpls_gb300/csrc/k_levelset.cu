// k_levelset.cu -- level-set update, Russo-Smereka redistancing, CSF
// surface tension and viscosity (two_phase_levelset.f90:20-118,
// levelset.f90:17-414, momentum_allflux.f90:474-521,
// main_ns_hybrid.F90:646-724).
//
// Every kernel is a gather over the full halo'd index space: a thread
// computes its own output element, including ghost planes, by evaluating
// the reference's boundary rule (copy, linear extrapolation, inlet value)
// on the interior values it needs.  That replaces the reference's sequence
// of interior pass + boundary passes + exchange2d with one launch, with
// identical values.
#include <cstring>
#include <type_traits>

#include "tpls_kernels.h"
#include "tpls_pair.cuh"

namespace tpls {

constexpr int LS_BX = 32, LS_BY = 8;

static inline dim3 full_grid(const Geo &g, int nzp) {
  return dim3((g.nx + 2 + LS_BX - 1) / LS_BX, (g.ny + 2 + LS_BY - 1) / LS_BY, nzp);
}

// ---------------------------------------------------------------------------
// two_phase_levelset.f90:56-95: phi3 = phi2 - dt*AB3(conv) on the interior,
// inlet value z-height at i=0, outlet copy at i=nx+1, linear extrapolation
// of the z ghost planes, periodic y rows.
__device__ __forceinline__ double ab3_val(const Geo &g, const Phys &ph, const double *phi2,
                                          const double *c0, const double *c1,
                                          const double *c2, int i, int j, int k) {
  if (i == 0) return (k * ph.dz - 0.5 * ph.dz) - ph.height;
  const int ii = (i == g.nx + 1) ? g.nx : i;
  const int c = TPLS_IDX(g, ii, j, k);
  return phi2[c] - ph.dt * ((23.0 / 12.0) * c2[c] - (4.0 / 3.0) * c1[c] + (5.0 / 12.0) * c0[c]);
}

__global__ void k_ls_ab3(Geo g, Phys ph, const double *__restrict__ phi2,
                         const double *__restrict__ c0, const double *__restrict__ c1,
                         const double *__restrict__ c2, double *__restrict__ phi3) {
  const int i = blockIdx.x * LS_BX + threadIdx.x, j = blockIdx.y * LS_BY + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.nx + 1 || j > g.ny + 1) return;
  const int jj = wrapy(j, g.ny);
  double v;
  if (k == 0)
    v = 2.0 * ab3_val(g, ph, phi2, c0, c1, c2, i, jj, 1) - ab3_val(g, ph, phi2, c0, c1, c2, i, jj, 2);
  else if (k == g.nz + 1)
    v = 2.0 * ab3_val(g, ph, phi2, c0, c1, c2, i, jj, g.nz) -
        ab3_val(g, ph, phi2, c0, c1, c2, i, jj, g.nz - 1);
  else
    v = ab3_val(g, ph, phi2, c0, c1, c2, i, jj, k);
  phi3[TPLS_IDX(g, i, j, k)] = v;
}

cudaError_t launch_ls_ab3(const Geo &g, const Phys &ph, const double *phi2,
                          const double *c0, const double *c1, const double *c2,
                          double *phi3, cudaStream_t st) {
  k_ls_ab3<<<full_grid(g, g.nz + 2), dim3(LS_BX, LS_BY), 0, st>>>(g, ph, phi2, c0, c1, c2, phi3);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// levelset.f90:17-94 get_levelset_status with h = dx.  flags packs the
// indicator istatus (bit 0) and sign(phi)+1 (bits 1-2); D and flags are 0
// outside the interior.
// p*q <= 0 for the rounded FP64 product, from the operands' bits: a zero
// operand or differing signs, as long as the product cannot underflow to
// zero (both magnitudes >= 2^-511, biased exponent >= 512).  Returns 1 for
// <= 0, 0 for > 0 and 2 when an operand is too small to decide by bits.
__device__ __forceinline__ int prod_le0_bits(double p, double q) {
  const int ha = __double2hiint(p), hb = __double2hiint(q);
  if (((ha & 0x7fffffff) | __double2loint(p)) == 0 || ((hb & 0x7fffffff) | __double2loint(q)) == 0) return 1;
  if (((ha >> 20) & 0x7ff) >= 512 && ((hb >> 20) & 0x7ff) >= 512) return ((ha ^ hb) < 0) ? 1 : 0;
  return 2;
}

// levelset.f90:60-71 the reference's test itself, for points with an operand
// below 2^-511 (a call, so the other points carry none of its FP64
// instructions)
__device__ __noinline__ int status_products(double p, double pxp, double pxm, double pyp, double pym, double pzp,
                                            double pzm) {
  const double mn = fmin(fmin(fmin(p * pxp, p * pxm), fmin(p * pyp, p * pym)), fmin(p * pzp, p * pzm));
  return (mn <= 0.0) ? 1 : 0;
}

// levelset.f90:75-85 the distance estimate D of an interface point.  A
// call: about 6% of the warps hold an interface point, and if-converted into
// the kernel its ~30 FP64 instructions would occupy the FP64 pipe in all.
__device__ __noinline__ double status_distance(double h, double p, double pxp, double pxm, double pyp,
                                               double pym, double pzp, double pzm) {
  const double gx = pxp - pxm, gy = pyp - pym, gz = pzp - pzm;
  const double b1 = sqrt(gx * gx + gy * gy + gz * gz) * 0.5;
  double mx = dmax_bits(dmax_bits(fabs(pxp - p), fabs(pxm - p)), dmax_bits(fabs(pyp - p), fabs(pym - p)));
  mx = dmax_bits(dmax_bits(mx, dmax_bits(fabs(pzp - p), fabs(pzm - p))), dmax_bits(b1, h));
  return h * p / mx;
}

template <typename T>
__global__ void k_ls_status(Geo g, double h, const double *__restrict__ phi, T *__restrict__ D,
                            signed char *__restrict__ flags) {
  const int i = blockIdx.x * LS_BX + threadIdx.x, j = blockIdx.y * LS_BY + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.nx + 1 || j > g.ny + 1) return;
  const int c = TPLS_IDX(g, i, j, k);
  if (i < 1 || i > g.nx || j < 1 || j > g.ny || k < 1 || k > g.nz) {
    D[c] = (T)0;
    flags[c] = 0;
    return;
  }
  // FP64 in both forms: the status flags are discrete decisions, so the
  // FP32-mixed form takes them from the same arithmetic as the FP64 form
  // and only stores D in FP32.  Signs, the test min(p*q) <= 0 and the
  // maxima are taken from the bit patterns (exact; GB300's FP64 pipe keeps
  // only the band's arithmetic).
  const double p = phi[c];
  const double pxp = phi[c + 1], pxm = phi[c - 1], pyp = phi[c + g.sy], pym = phi[c - g.sy];
  const double pzp = phi[c + g.sz], pzm = phi[c - g.sz];
  const int ph = __double2hiint(p);
  const int sgn = (((ph & 0x7fffffff) | __double2loint(p)) == 0) ? 0 : ((ph < 0) ? -1 : 1);
  const int q = prod_le0_bits(p, pxp) | prod_le0_bits(p, pxm) | prod_le0_bits(p, pyp) |
                prod_le0_bits(p, pym) | prod_le0_bits(p, pzp) | prod_le0_bits(p, pzm);
  const int st = (q & 2) ? status_products(p, pxp, pxm, pyp, pym, pzp, pzm) : (q & 1);
  const double d = st ? status_distance(h, p, pxp, pxm, pyp, pym, pzp, pzm) : 0.0;
  D[c] = (T)d;
  flags[c] = (signed char)(st | ((sgn + 1) << 1));
}

cudaError_t launch_ls_status(const Geo &g, const Phys &ph, const double *phi3,
                             double *D, signed char *flags, cudaStream_t st) {
  k_ls_status<double><<<full_grid(g, g.nz + 2), dim3(LS_BX, LS_BY), 0, st>>>(g, ph.dx, phi3, D, flags);
  return cudaGetLastError();
}
cudaError_t launch_ls_status(const Geo &g, const Phys &ph, const double *phi3, float *D, signed char *flags,
                             cudaStream_t st) {
  k_ls_status<float><<<full_grid(g, g.nz + 2), dim3(LS_BX, LS_BY), 0, st>>>(g, ph.dx, phi3, D, flags);
  return cudaGetLastError();
}

// v with its sign bit flipped when m is the sign mask (exact negation by an
// integer operation on the high word)
__device__ __forceinline__ double neg_if(double v, int m) {
  return __hiloint2double(__double2hiint(v) ^ m, __double2loint(v));
}

// ---------------------------------------------------------------------------
// levelset.f90:97-237 do_levelset_iteration: one Godunov pseudo-time step
// with dtau = 0.3h (h = dx), then the inlet value (with dz = h), the outlet
// copy, linear z extrapolation, periodic y.  err_part (optional) receives
// one partial of sum((pr - pr_new)^2) per block over i 1..nx, j 1..ny,
// k 0..nz+1.
// RT: type of the updated value.  The FP32-mixed form keeps the iterate in
// FP64 (RT = double) and evaluates only the increment ktau*dc in FP32, so the
// iterate accumulates no FP32 rounding across the iterations and steps.
// dc of the update at point c, p = its value, pr a loader of the stencil
// values in the arithmetic type TC.
template <typename TC, typename LD>
__device__ __forceinline__ TC rs_dc(const Geo &g, TC h, const LD &pr, TC p, const TC *__restrict__ D, int f,
                                   int c) {
  // s = sign(phi) + 1.  The products sg * X of the reference (sg = -1, 0, 1)
  // are written as selects and negations, which are exact: no int-to-FP64
  // conversion, compare or multiply on GB300's FP64 pipe.
  const int s = (f >> 1) & 3;
  const TC zero = (TC)0;
  if (f & 1) {
    const TC ap = fabs(p);
    return ((s == 2) ? ap : ((s == 0) ? -ap : zero)) - D[c];
  }
  if constexpr (sizeof(TC) == sizeof(double)) {
    // One evaluation for both signs (a warp straddling the interface would
    // otherwise run both, and predicated-off FP64 instructions still hold
    // the FP64 pipe).  With sigma = sign(phi) and m its sign mask:
    //   phi > 0: a = max(p - min(l, r), 0)
    //   phi < 0: a = max(max(l, r) - p, 0) = max((-p) - min(-l, -r), 0),
    // exactly ((-p) - (-M) = M - p in IEEE arithmetic), and
    // dc = sigma (sqrt(ax^2 + ay^2 + az^2) - h), the sum taken in the
    // reference's order: x, y, z for phi > 0 and x, z, y for phi < 0
    // (levelset.f90:274-275).
    // max(aP^2, bM^2) with aP = max(p - p[i-1], 0), bM = min(p[i+1] - p, 0)
    // equals max(p - min(p[i-1], p[i+1]), 0)^2 bit for bit (rounding of a
    // difference and of a square are monotone), likewise in y and z.
    if (s == 1) return zero;
    const int m = (s == 0) ? (int)0x80000000 : 0;
    const double sp = neg_if(p, m);
    const double ax = dpos_bits(sp - dmin_bits(neg_if(pr[c - 1], m), neg_if(pr[c + 1], m)));
    const double ay = dpos_bits(sp - dmin_bits(neg_if(pr[c - g.sy], m), neg_if(pr[c + g.sy], m)));
    const double az = dpos_bits(sp - dmin_bits(neg_if(pr[c - g.sz], m), neg_if(pr[c + g.sz], m)));
    const double a2 = (s == 2) ? ay : az, a3 = (s == 2) ? az : ay;
    return neg_if(sqrt(ax * ax + a2 * a2 + a3 * a3) - h, m);
  } else {
    if (s == 2) {
      const TC ax = fmaxf(p - fminf(pr[c - 1], pr[c + 1]), zero);
      const TC ay = fmaxf(p - fminf(pr[c - g.sy], pr[c + g.sy]), zero);
      const TC az = fmaxf(p - fminf(pr[c - g.sz], pr[c + g.sz]), zero);
      return sqrt(ax * ax + ay * ay + az * az) - h;
    }
    if (s == 0) {
      const TC ax = fmaxf(fmaxf(pr[c - 1], pr[c + 1]) - p, zero);
      const TC ay = fmaxf(fmaxf(pr[c - g.sy], pr[c + g.sy]) - p, zero);
      const TC az = fmaxf(fmaxf(pr[c - g.sz], pr[c + g.sz]) - p, zero);
      return -(sqrt(ax * ax + az * az + ay * ay) - h);
    }
    return zero;
  }
}

template <typename TC, typename TI>
struct LdCvt {
  const TI *p;
  __device__ __forceinline__ TC operator[](int q) const { return (TC)p[q]; }
};

template <typename TC, typename TI, typename RT>
__device__ __forceinline__ RT rs_update(const Geo &g, TC h, TC ktau, const TI *__restrict__ pr0,
                                        const TC *__restrict__ D, const signed char *__restrict__ flags,
                                        int i, int j, int k) {
  const int c = TPLS_IDX(g, i, j, k);
  const LdCvt<TC, TI> pr{pr0};
  const TC p = pr[c];
  const TC dc = rs_dc<TC>(g, h, pr, p, D, flags[c], c);
  if constexpr (sizeof(RT) == sizeof(TC)) return p - ktau * dc;
  else return (RT)pr0[c] - (RT)(ktau * dc);
}

// levelset.f90 inlet value (k - 1/2) h - height at i = 0.  A call, not
// inline code: if-converted it would put its FP64 instructions on every
// lane's FP64 pipe, and only one column of the grid takes it.
__device__ __noinline__ double ls_inlet(double h, double height, int k) {
  return (k * h - 0.5 * h) - height;
}

template <typename TC, typename TI, typename RT>
__device__ __forceinline__ RT rs_val(const Geo &g, const Phys &ph, TC h, TC ktau, const TI *pr, const TC *D,
                                     const signed char *flags, int i, int j, int k) {
  if (i == 0) return (RT)ls_inlet((double)h, ph.height, k);
  return rs_update<TC, TI, RT>(g, h, ktau, pr, D, flags, (i == g.nx + 1) ? g.nx : i, j, k);
}

// TI/TO: storage of the input/output iterate; TC: arithmetic (double for
// the FP64 form; float for the FP32-mixed form, whose first iteration reads
// the FP64 phi3 and whose last writes the FP64 state).
// ERR: the launch also writes the error partials (the last iteration only;
// a compile-time switch, so the other iterations carry no predicated-off
// FP64 instructions for it).
template <typename TC, typename TI, typename TO, bool ERR>
__global__ void __launch_bounds__(LS_BX *LS_BY)
    k_ls_iter(Geo g, Phys ph, TC h, TC ktau, const TI *__restrict__ pr, const TC *__restrict__ D,
              const signed char *__restrict__ flags, TO *__restrict__ out, double *__restrict__ err_part) {
  const int i = blockIdx.x * LS_BX + threadIdx.x, j = blockIdx.y * LS_BY + threadIdx.y;
  const int k = blockIdx.z;
  double e = 0.0;
  if (i <= g.nx + 1 && j <= g.ny + 1) {
    const int jj = wrapy(j, g.ny);
    using RT = typename std::conditional<sizeof(TO) == sizeof(double), double, TC>::type;
    RT v;
    if (k == 0)
      v = (RT)2 * rs_val<TC, TI, RT>(g, ph, h, ktau, pr, D, flags, i, jj, 1) -
          rs_val<TC, TI, RT>(g, ph, h, ktau, pr, D, flags, i, jj, 2);
    else if (k == g.nz + 1)
      v = (RT)2 * rs_val<TC, TI, RT>(g, ph, h, ktau, pr, D, flags, i, jj, g.nz) -
          rs_val<TC, TI, RT>(g, ph, h, ktau, pr, D, flags, i, jj, g.nz - 1);
    else
      v = rs_val<TC, TI, RT>(g, ph, h, ktau, pr, D, flags, i, jj, k);
    const int c = TPLS_IDX(g, i, j, k);
    if (ERR && i >= 1 && i <= g.nx && j >= 1 && j <= g.ny) {
      const double d = (double)pr[c] - (double)v;
      e = d * d;
    }
    out[c] = (TO)v;
  }
  if constexpr (ERR) {
    __shared__ double s[LS_BX * LS_BY / 32];
    for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
    const int t = threadIdx.y * LS_BX + threadIdx.x;
    if ((t & 31) == 0) s[t >> 5] = e;
    __syncthreads();
    if (t == 0) {
      double a = 0.0;
      for (int q = 0; q < LS_BX * LS_BY / 32; q++) a += s[q];
      err_part[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = a;
    }
  }
}

// FP32-mixed redistancing: the iterate is carried as a float pair
// (hi, lo) with hi + lo holding ~48 bits of the FP64 value.  The stencil
// takes its differences from the pairs (FP32 arithmetic, no FP64
// instruction on the common path), and the increment is added into the pair
// with an error-free two-sum, so the iterate accumulates no FP32 rounding
// over the iterations (FP64<->FP32 conversions run on GB300's FP64 pipe,
// which made an FP64 iterate cost as much as FP64 arithmetic).  IN64: the
// input is the FP64 phi3 (first iteration), split by integer operations;
// OUT64: the output is the FP64 state (last).
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF two_sum(float a, float b) {
  const float s = a + b;
  const float bp = s - a;
  return FF{s, (a - (s - bp)) + (b - bp)};
}
__device__ __forceinline__ FF ff_split(double v) {
  const float hi = (float)v;
  return FF{hi, (float)(v - (double)hi)};
}
__device__ __forceinline__ double ff_dbl(const FF &v) { return (double)v.hi + (double)v.lo; }

template <bool IN64>
struct FFSrc {
  const double *x64;
  const float *hi, *lo;
  // the stencil value as a pair: split by integer operations from the FP64
  // phi3 on the first iteration, the stored pair afterwards
  __device__ __forceinline__ F2 pair(int q) const {
    if (IN64) return split_bits(x64[q]);
    return F2{hi[q], lo[q]};
  }
  __device__ __forceinline__ double exact(int q) const { return IN64 ? x64[q] : (double)hi[q] + (double)lo[q]; }
};

// rs_dc on pairs: the one-sided differences of the Godunov gradient are
// taken from the pairs ((hi_a - hi_b) + (lo_a - lo_b)), so they carry FP32
// precision relative to the difference, not to |phi|; the rest is FP32.
template <bool IN64>
__device__ __forceinline__ float rs_dc_pair(const Geo &g, float h, const FFSrc<IN64> &src, F2 p,
                                            const float *__restrict__ D, int f, int c) {
  const float sg = (float)(((f >> 1) & 3) - 1);
  if (f & 1) return sg * fabsf(val(p)) - D[c];
  if (sg > 0.0f) {  // max(p - min(p[i-1], p[i+1]), 0), likewise y, z (see rs_dc)
    const float ax = fmaxf(dif(p, pmin(src.pair(c - 1), src.pair(c + 1))), 0.0f);
    const float ay = fmaxf(dif(p, pmin(src.pair(c - g.sy), src.pair(c + g.sy))), 0.0f);
    const float az = fmaxf(dif(p, pmin(src.pair(c - g.sz), src.pair(c + g.sz))), 0.0f);
    return sg * (sqrtf(ax * ax + ay * ay + az * az) - h);
  }
  if (sg < 0.0f) {
    const float ax = fmaxf(dif(pmax(src.pair(c - 1), src.pair(c + 1)), p), 0.0f);
    const float ay = fmaxf(dif(pmax(src.pair(c - g.sy), src.pair(c + g.sy)), p), 0.0f);
    const float az = fmaxf(dif(pmax(src.pair(c - g.sz), src.pair(c + g.sz)), p), 0.0f);
    return sg * (sqrtf(ax * ax + az * az + ay * ay) - h);
  }
  return 0.0f;
}

// inlet row (levelset.f90:168-177), FP64, out of line (see below)
__device__ __noinline__ FF ff_inlet(float h, double height, int k) {
  return ff_split((k * (double)h - 0.5 * (double)h) - height);
}

template <bool IN64>
__device__ __forceinline__ FF ff_val(const Geo &g, const Phys &ph, float h, float ktau, const FFSrc<IN64> &src,
                                     const float *D, const signed char *flags, int i, int j, int k) {
  if (i == 0) return ff_inlet(h, ph.height, k);
  if (i == g.nx + 1) i = g.nx;
  const int c = TPLS_IDX(g, i, j, k);
  const F2 p = src.pair(c);
  const float inc = ktau * rs_dc_pair<IN64>(g, h, src, p, D, flags[c], c);
  return two_sum(p.h, p.l - inc);
}

// The FP64 paths of the float-pair iteration (the extrapolated ghost planes,
// the residual of the last iteration) are kept out of line: if-converted
// into the kernel body their FP64 instructions would be issued, predicated
// off, for every point and fill GB300's slow FP64 pipe.
template <bool IN64>
__device__ __noinline__ FF ff_ghost_plane(const Geo &g, const Phys &ph, float h, float ktau, const FFSrc<IN64> &src,
                                          const float *D, const signed char *flags, int i, int jj, int k) {
  const int k1 = (k == 0) ? 1 : g.nz, k2 = (k == 0) ? 2 : g.nz - 1;
  return ff_split(2.0 * ff_dbl(ff_val<IN64>(g, ph, h, ktau, src, D, flags, i, jj, k1)) -
                  ff_dbl(ff_val<IN64>(g, ph, h, ktau, src, D, flags, i, jj, k2)));
}

template <bool IN64, bool OUT64>
__global__ void __launch_bounds__(LS_BX *LS_BY)
    k_ls_iter_ff(Geo g, Phys ph, float h, float ktau, FFSrc<IN64> src, const float *__restrict__ D,
                 const signed char *__restrict__ flags, double *__restrict__ out64, float *__restrict__ ohi,
                 float *__restrict__ olo, double *__restrict__ err_part) {
  const int i = blockIdx.x * LS_BX + threadIdx.x, j = blockIdx.y * LS_BY + threadIdx.y;
  const int k = blockIdx.z;
  float e = 0.0f;
  if (i <= g.nx + 1 && j <= g.ny + 1) {
    const int jj = wrapy(j, g.ny);
    const int c = TPLS_IDX(g, i, j, k);
    FF v;
    if (k == 0 || k == g.nz + 1)  // linear extrapolation, in FP64
      v = ff_ghost_plane<IN64>(g, ph, h, ktau, src, D, flags, i, jj, k);
    else
      v = ff_val<IN64>(g, ph, h, ktau, src, D, flags, i, jj, k);
    if (err_part && i >= 1 && i <= g.nx && j >= 1 && j <= g.ny) {  // the iteration's change, from pairs
      const float d = dif(src.pair(c), F2{v.hi, v.lo});
      e = d * d;
    }
    if (OUT64) {  // exact widening by integer operations, one FP64 add
      out64[c] = widen_bits(v.hi) + widen_bits(v.lo);
    } else {
      ohi[c] = v.hi;
      olo[c] = v.lo;
    }
  }
  if (err_part) {
    __shared__ double s[LS_BX * LS_BY / 32];
    for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
    const int t = threadIdx.y * LS_BX + threadIdx.x;
    if ((t & 31) == 0) s[t >> 5] = widen_bits(e);
    __syncthreads();
    if (t == 0) {
      double a = 0.0;
      for (int q = 0; q < LS_BX * LS_BY / 32; q++) a += s[q];
      err_part[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = a;
    }
  }
}

int ls_iter_blocks(const Geo &g) {
  dim3 gr = full_grid(g, g.nz + 2);
  return (int)(gr.x * gr.y * gr.z);
}

template <typename TC, typename TI, typename TO>
static cudaError_t ls_iter(const Geo &g, const Phys &ph, const TI *pr, const TC *D, const signed char *flags,
                           TO *pr_new, double *err_part, cudaStream_t st) {
  const double h = ph.dx, dtau = 0.3 * h;
  if (err_part)
    k_ls_iter<TC, TI, TO, true><<<full_grid(g, g.nz + 2), dim3(LS_BX, LS_BY), 0, st>>>(
        g, ph, (TC)h, (TC)(dtau / h), pr, D, flags, pr_new, err_part);
  else
    k_ls_iter<TC, TI, TO, false><<<full_grid(g, g.nz + 2), dim3(LS_BX, LS_BY), 0, st>>>(
        g, ph, (TC)h, (TC)(dtau / h), pr, D, flags, pr_new, err_part);
  return cudaGetLastError();
}
cudaError_t launch_ls_iter(const Geo &g, const Phys &ph, const double *pr, const double *D,
                           const signed char *flags, double *pr_new, double *err_part, cudaStream_t st) {
  return ls_iter<double, double, double>(g, ph, pr, D, flags, pr_new, err_part, st);
}
cudaError_t launch_ls_iter_ff(const Geo &g, const Phys &ph, const double *in64, const float *hi,
                              const float *lo, const float *D, const signed char *flags, double *out64,
                              float *ohi, float *olo, double *err_part, cudaStream_t st) {
  const float h = (float)ph.dx, ktau = (float)(0.3 * ph.dx / ph.dx);
  const dim3 grd = full_grid(g, g.nz + 2), blk(LS_BX, LS_BY);
  if (in64) {
    const FFSrc<true> src{in64, nullptr, nullptr};
    if (out64)
      k_ls_iter_ff<true, true><<<grd, blk, 0, st>>>(g, ph, h, ktau, src, D, flags, out64, nullptr, nullptr,
                                                   err_part);
    else
      k_ls_iter_ff<true, false><<<grd, blk, 0, st>>>(g, ph, h, ktau, src, D, flags, nullptr, ohi, olo, err_part);
  } else {
    const FFSrc<false> src{nullptr, hi, lo};
    if (out64)
      k_ls_iter_ff<false, true><<<grd, blk, 0, st>>>(g, ph, h, ktau, src, D, flags, out64, nullptr, nullptr,
                                                    err_part);
    else
      k_ls_iter_ff<false, false><<<grd, blk, 0, st>>>(g, ph, h, ktau, src, D, flags, nullptr, ohi, olo,
                                                     err_part);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// levelset.f90:241-414 get_csf: curvature (clipped at 1/min(dx,dy,dz)),
// smoothed Dirac delta, CSF force; x and z ghost planes by linear
// extrapolation; periodic y rows.  Outside the smoothing band the Dirac
// delta is 0 and the force is 0 without evaluating the curvature.
struct F3 {
  double x, y, z;
};

template <typename T>
__device__ __forceinline__ F3 csf_point(const Geo &g, const Phys &ph, double max_kappa,
                                        const double *__restrict__ fi0, int i, int j, int k) {
  const int c = TPLS_IDX(g, i, j, k);
  struct Ld {
    const double *p;
    __device__ T operator[](int q) const { return (T)p[q]; }
  } fi{fi0};
  const double p64 = fi0[c];
  F3 r = {0.0, 0.0, 0.0};
  // band decision on the FP64 value in both forms, by order keys of the bit
  // patterns (exact; no FP64 compare)
  const long long kp = dkey(p64);
  if (kp < dkey(-ph.sw) || kp > dkey(ph.sw)) return r;
  const T p = (T)p64;
  const int sy = g.sy, sz = g.sz;
  const T rdx = (T)(1.0 / ph.dx), rdy = (T)(1.0 / ph.dy), rdz = (T)(1.0 / ph.dz);
  const T r2dx = (T)0.5 * rdx, r2dy = (T)0.5 * rdy, r2dz = (T)0.5 * rdz, two = (T)2;
  const T d2x = (fi[c + 1] - two * p + fi[c - 1]) * (rdx * rdx);
  const T d2y = (fi[c + sy] - two * p + fi[c - sy]) * (rdy * rdy);
  const T d2z = (fi[c + sz] - two * p + fi[c - sz]) * (rdz * rdz);
  const T gx = (fi[c + 1] - fi[c - 1]) * r2dx;
  const T gy = (fi[c + sy] - fi[c - sy]) * r2dy;
  const T gz = (fi[c + sz] - fi[c - sz]) * r2dz;
  const T d2xz = ((fi[c + 1 + sz] - fi[c - 1 + sz]) - (fi[c + 1 - sz] - fi[c - 1 - sz])) * (r2dx * r2dz);
  const T d2yz = ((fi[c + sy + sz] - fi[c - sy + sz]) - (fi[c + sy - sz] - fi[c - sy - sz])) * (r2dy * r2dz);
  const T d2xy = ((fi[c + 1 + sy] - fi[c - 1 + sy]) - (fi[c + 1 - sy] - fi[c - 1 - sy])) * (r2dx * r2dy);
  const T nrm = gx * gx + gy * gy + gz * gz;
  T kap;
  if (nrm < (T)1e-10) {
    kap = (T)0;
  } else {
    const T s = sqrt(nrm);             // nrm**0.5
    const T inv15 = (T)1 / (nrm * s);  // nrm**(-1.5)
    const T term1 = (d2x + d2y + d2z) / s;
    const T term2 = (gx * gx * d2x + gy * gy * d2y + gz * gz * d2z) * inv15;
    const T term3 = two * (gx * gy * d2xy + gx * gz * d2xz + gy * gz * d2yz) * inv15;
    kap = -(term1 - term2 - term3);
  }
  if (kap > (T)max_kappa) kap = (T)max_kappa;
  const T a = (T)(1.0 / (2.0 * ph.sw));
  const T dirac = a + a * cos((T)TPLS_PI_SP * p / (T)ph.sw);
  const T m = dirac * (T)ph.scap * kap;
  r.x = (double)(m * gx);
  r.y = (double)(m * gy);
  r.z = (double)(m * gz);
  return r;
}

__device__ __forceinline__ F3 lin2(F3 a, F3 b) {  // 2a - b
  F3 r = {2.0 * a.x - b.x, 2.0 * a.y - b.y, 2.0 * a.z - b.z};
  return r;
}

// value on the i = 1..nx columns including the extrapolated z ghost planes
template <typename T>
__device__ __forceinline__ F3 csf_colval(const Geo &g, const Phys &ph, double mk,
                                         const double *fi, int i, int j, int k) {
  if (k == 0) return lin2(csf_point<T>(g, ph, mk, fi, i, j, 1), csf_point<T>(g, ph, mk, fi, i, j, 2));
  if (k == g.nz + 1)
    return lin2(csf_point<T>(g, ph, mk, fi, i, j, g.nz), csf_point<T>(g, ph, mk, fi, i, j, g.nz - 1));
  return csf_point<T>(g, ph, mk, fi, i, j, k);
}

// T: arithmetic of the curvature (double, or float in the FP32-mixed form);
// TO: storage of the force components.
template <typename T, typename TO>
__global__ void k_csf(Geo g, Phys ph, double mk, const double *__restrict__ fi,
                      TO *__restrict__ fx, TO *__restrict__ fy, TO *__restrict__ fz) {
  const int i = blockIdx.x * LS_BX + threadIdx.x, j = blockIdx.y * LS_BY + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.nx + 1 || j > g.ny + 1) return;
  const int jj = wrapy(j, g.ny);
  F3 v;
  if (i == 0)
    v = lin2(csf_colval<T>(g, ph, mk, fi, 1, jj, k), csf_colval<T>(g, ph, mk, fi, 2, jj, k));
  else if (i == g.nx + 1)
    v = lin2(csf_colval<T>(g, ph, mk, fi, g.nx, jj, k), csf_colval<T>(g, ph, mk, fi, g.nx - 1, jj, k));
  else
    v = csf_colval<T>(g, ph, mk, fi, i, jj, k);
  const int c = TPLS_IDX(g, i, j, k);
  fx[c] = (TO)v.x;
  fy[c] = (TO)v.y;
  fz[c] = (TO)v.z;
}

cudaError_t launch_csf(const Geo &g, const Phys &ph, const double *phi3,
                       double *fx, double *fy, double *fz, cudaStream_t st) {
  const double mk = 1.0 / fmin(fmin(ph.dx, ph.dy), ph.dz);
  k_csf<double, double><<<full_grid(g, g.nz + 2), dim3(LS_BX, LS_BY), 0, st>>>(g, ph, mk, phi3, fx, fy, fz);
  return cudaGetLastError();
}
cudaError_t launch_csf(const Geo &g, const Phys &ph, const double *phi3, float *fx, float *fy, float *fz,
                       cudaStream_t st) {
  const double mk = 1.0 / fmin(fmin(ph.dx, ph.dy), ph.dz);
  // curvature stays FP64: its second differences of phi (~dx^2 |phi''|)
  // would lose ~1e-3 of their value to FP32 cancellation, a coherent error
  // in the surface-tension force at the interface; the force is stored FP32
  k_csf<double, float><<<full_grid(g, g.nz + 2), dim3(LS_BX, LS_BY), 0, st>>>(g, ph, mk, phi3, fx, fy, fz);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// momentum_allflux.f90:474-521 get_viscosity on x = 0..nx+1 (the ghost
// planes of main_ns_hybrid.F90:653-710 use the same formula and the same
// single-precision pi) and the 2-row periodic-y augmentation.
// Outside the band |p| <= sw the smoothed Heaviside is exactly 0 or 1 and the
// viscosity exactly mu_minus/re or mu_plus/re (the host's IEEE quotients,
// mlo and mhi); the band test compares order keys of the bit patterns
// (klo = key(-sw), khi = key(sw)), so those points use no FP64 instruction.
template <typename T, bool OFF>
__global__ void k_visc(Geo g, Phys ph, const double *__restrict__ phi, double off, long long klo,
                       long long khi, double mlo, double mhi, T *__restrict__ mu) {
  const int i = blockIdx.x * LS_BX + threadIdx.x, j = blockIdx.y * LS_BY + threadIdx.y - 1;
  const int k = blockIdx.z;
  if (i > g.nx + 1 || j > g.ny + 2) return;
  // off: -0.5 for the diffuse-interface method, which passes phi2-0.5
  // (main_ns_hybrid.F90:650, :667, :692); 0 for the level set, where adding
  // it would change nothing but the sign of a zero (OFF false: no add)
  double p = phi[TPLS_IDX(g, i, wrapy(j, g.ny), k)];
  if constexpr (OFF) p += off;
  const long long kp = dkey(p);
  double m;
  if (kp < klo) {
    m = mlo;
  } else if (kp > khi) {
    m = mhi;
  } else {
    const double hv = 0.5 + (p / (2.0 * ph.sw)) + (1.0 / (2.0 * TPLS_PI_SP)) * sin(TPLS_PI_SP * p / ph.sw);
    m = (ph.mu_plus * hv + ph.mu_minus * (1.0 - hv)) / ph.re;
  }
  mu[TPLS_IDXM(g, i, j, k)] = (T)m;
}

static long long host_dkey(double a) {
  long long b;
  memcpy(&b, &a, sizeof b);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

cudaError_t launch_visc(const Geo &g, const Phys &ph, const double *phi2,
                        double *mu, cudaStream_t st, double phi_offset) {
  dim3 grd((g.nx + 2 + LS_BX - 1) / LS_BX, (g.ny + 4 + LS_BY - 1) / LS_BY, g.nz + 2);
  const long long klo = host_dkey(-ph.sw), khi = host_dkey(ph.sw);
  const double mlo = ph.mu_minus / ph.re, mhi = ph.mu_plus / ph.re;
  if (phi_offset != 0.0)
    k_visc<double, true><<<grd, dim3(LS_BX, LS_BY), 0, st>>>(g, ph, phi2, phi_offset, klo, khi, mlo, mhi, mu);
  else
    k_visc<double, false><<<grd, dim3(LS_BX, LS_BY), 0, st>>>(g, ph, phi2, phi_offset, klo, khi, mlo, mhi, mu);
  return cudaGetLastError();
}
// The FP32 viscosity of the FP32-mixed form: the same formula in FP32 on
// phi rounded to FP32 by integer operations (the smoothed Heaviside is
// continuous at |phi| = sw, so the band test needs no FP64 either).
struct ViscF {
  float sw, half_rsw, pi_rsw, half_rpi, mp, mm;
};
__global__ void k_visc32(Geo g, ViscF v, const double *__restrict__ phi, float *__restrict__ mu) {
  const int i = blockIdx.x * LS_BX + threadIdx.x, j = blockIdx.y * LS_BY + threadIdx.y - 1;
  const int k = blockIdx.z;
  if (i > g.nx + 1 || j > g.ny + 2) return;
  const float p = round_bits(phi[TPLS_IDX(g, i, wrapy(j, g.ny), k)]);
  float hv;
  if (p < -v.sw)
    hv = 0.0f;
  else if (p > v.sw)
    hv = 1.0f;
  else
    hv = 0.5f + p * v.half_rsw + v.half_rpi * sinf(v.pi_rsw * p);
  mu[TPLS_IDXM(g, i, j, k)] = v.mp * hv + v.mm * (1.0f - hv);
}

cudaError_t launch_visc(const Geo &g, const Phys &ph, const double *phi2, float *mu, cudaStream_t st) {
  dim3 grd((g.nx + 2 + LS_BX - 1) / LS_BX, (g.ny + 4 + LS_BY - 1) / LS_BY, g.nz + 2);
  ViscF v;
  v.sw = (float)ph.sw;
  v.half_rsw = (float)(1.0 / (2.0 * ph.sw));
  v.pi_rsw = (float)(TPLS_PI_SP / ph.sw);
  v.half_rpi = (float)(1.0 / (2.0 * TPLS_PI_SP));
  v.mp = (float)(ph.mu_plus / ph.re);
  v.mm = (float)(ph.mu_minus / ph.re);
  k_visc32<<<grd, dim3(LS_BX, LS_BY), 0, st>>>(g, v, phi2, mu);
  return cudaGetLastError();
}

}  // namespace tpls
