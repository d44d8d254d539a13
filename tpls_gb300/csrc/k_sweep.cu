// k_sweep.cu -- Jacobi and red-black SOR sweeps of the Crank-Nicolson
// Helmholtz solve on precomputed per-point coefficient records
// (jacobi_iteration_allflux.f90:21-282, sor_iteration_allflux.f90:19-377,
// boundary rows of main_ns_hybrid.F90:756-887).
//
// k_mom_rhs writes, once per timestep, one record per point of a velocity
// component: the six neighbour coefficients and rhs/diag, already divided
// by the Helmholtz diagonal, and the odd half-sweep's factor 1.2 czm (see
// write_coef in k_momentum.cu).  A sweep
// point is then x_new = sum(c_n x_n) + b: seven FMAs instead of the face
// averages, diagonal and division of the reference's form, evaluated once
// per step instead of once per sweep: on GB300's FP64 pipe the 64-byte
// record is the cheaper side of that trade.  The FP32 sweeps of the
// FP32-mixed form take the other side: FP32 arithmetic is 64x faster, so
// they recompute the coefficients per point from the FP32 viscosity and read
// only b (4 bytes), cutting a Jacobi point from ~40 to ~16 bytes of traffic.
// Templated on the arithmetic type and the coefficient source (records, or
// MuCoef).
#include "tpls_sweep.cuh"

namespace tpls {

// bz = 1.2 zm, the factor of the odd half-sweep's column recurrence.  The
// FP64 records carry it in their eighth slot (written by k_mom_rhs by the
// same multiplication, so the values are identical), loaded with b instead
// of computed in every odd half-sweep on the FP64 pipe.
template <typename T>
struct Rec {
  T xp, xm, yp, ym, zp, zm, b, bz;
};

// record of point c of the FP64 sweeps (8 doubles; `stream` = evict-first loads)
__device__ __forceinline__ Rec<double> load_rec(const double *__restrict__ coef, int c, bool stream) {
  const double2 *r = reinterpret_cast<const double2 *>(coef + 8 * (size_t)c);
  const double2 a = stream ? __ldcs(r) : __ldg(r), b = stream ? __ldcs(r + 1) : __ldg(r + 1);
  const double2 d = stream ? __ldcs(r + 2) : __ldg(r + 2), e = stream ? __ldcs(r + 3) : __ldg(r + 3);
  Rec<double> q = {a.x, a.y, b.x, b.y, d.x, d.y, e.x, e.y};
  return q;
}

template <typename T>
__device__ __forceinline__ T rec_apply(const Rec<T> &q, T xp, T xm, T yp, T ym, T zp, T zm) {
  T v = fma(q.xp, xp, q.b);
  v = fma(q.xm, xm, v);
  v = fma(q.yp, yp, v);
  v = fma(q.ym, ym, v);
  v = fma(q.zp, zp, v);
  return fma(q.zm, zm, v);
}

// Coefficients of point (i, j, k): the FP64 form reads its record; the FP32
// sweeps recompute the six coefficients from the FP32 viscosity exactly as
// the right-hand side kernels do (face averages, diagonal, wall rule folded
// into the z slots for u and v) and read b alone.
__device__ __forceinline__ Rec<double> get_rec(int, const Geo &g, const double *__restrict__ coef, int c, int i,
                                               int, int, bool stream) {
  return load_rec(coef, rec_slot(g, c, i), stream);
}
__device__ __forceinline__ Rec<float> get_rec(int comp, const Geo &g, const MuCoef &s, int c, int i, int j, int k,
                                              bool stream) {
  const FcT<float> f = faces<float>(comp, g, s.mu, i, j, k);
  const float diag = 1.0f + s.ax2 * (f.px + f.mx) + s.ay2 * (f.py + f.my) + s.az2 * (f.pz + f.mz);
  const float r = __fdividef(1.0f, diag);  // diag >= 1: the fast reciprocal is within 2 ulp
  float czp = s.az2 * f.pz * r, czm = s.az2 * f.mz * r;
  if (comp != 2) {
    if (k == 0) {
      czp += czm * (float)(1.0 / 3.0);
      czm = -2.0f * czm;
    } else if (k == g.nz - 1) {
      czm += czp * (float)(1.0 / 3.0);
      czp = -2.0f * czp;
    }
  }
  const float *bp = s.b + rec_slot(g, c, i);
  Rec<float> q = {s.ax2 * f.px * r, s.ax2 * f.mx * r, s.ay2 * f.py * r, s.ay2 * f.my * r, czp, czm,
                  stream ? __ldcs(bp) : __ldg(bp), 1.2f * czm};
  return q;
}

// The per-routine entries' coefficients (sor_iteration_allflux.f90 on host
// arrays): face viscosities of the FP64 viscosity_aug and the right-hand
// side, divided by the Helmholtz diagonal, the wall rule folded into the z
// slots as in the records.
__device__ __forceinline__ Rec<double> get_rec(int comp, const Geo &g, const RefCoef &s, int c, int i, int j, int k,
                                               bool) {
  const FcT<double> f = faces<double>(comp, g, s.mu, i, j, k);
  const double diag = 1.0 + s.ax2 * (f.px + f.mx) + s.ay2 * (f.py + f.my) + s.az2 * (f.pz + f.mz);
  const double r = 1.0 / diag;
  double czp = s.az2 * f.pz * r, czm = s.az2 * f.mz * r;
  if (comp != 2) {
    if (k == 0) {
      czp += czm * (1.0 / 3.0);
      czm = -2.0 * czm;
    } else if (k == g.nz - 1) {
      czm += czp * (1.0 / 3.0);
      czp = -2.0 * czp;
    }
  }
  Rec<double> q = {s.ax2 * f.px * r, s.ax2 * f.mx * r, s.ay2 * f.py * r, s.ay2 * f.my * r, czp, czm, s.rhs[c] * r, 1.2 * czm};
  return q;
}

// Jacobi: x = J(xo) on the component's interior with its boundary rows.
template <typename T, typename CS, int CC, int SW_X, int SW_Y>
__global__ void __launch_bounds__(SW_X *SW_Y)
    k_jacobi_c(int comp_, Geo g, Helm h, const T *__restrict__ xo, const CS coef,
               const double *__restrict__ P, const double *__restrict__ X, T *__restrict__ x, int fuse) {
  const int comp = (CC >= 0) ? CC : comp_;
  const int i = blockIdx.x * SW_X + threadIdx.x + 1, j = blockIdx.y * SW_Y + threadIdx.y + 1;
  const int k = blockIdx.z + (comp == 2 ? 1 : 0);
  const int iend = (comp == 0) ? g.nx - 1 : g.nx;
  if (i > iend || j > g.ny) return;
  const int c = TPLS_IDX(g, i, j, k), sy = g.sy, sz = g.sz;
  const Rec<T> q = get_rec(comp, g, coef, c, i, j, k, false);
  const T xc = xo[c];
  T zp, zm;
  if (comp == 2) {
    zp = xo[c + sz];
    zm = xo[c - sz];
  } else {  // walls folded into the record: the z slot multiplies the point itself
    zp = (k == g.nz - 1) ? xc : xo[c + sz];
    zm = (k == 0) ? xc : xo[c - sz];
  }
  const T v = rec_apply(q, xo[c + 1], xo[c - 1], xo[c + sy], xo[c - sy], zp, zm);
  put(g, x, i, j, k, v, fuse);
  const bool edge = (i == 1) || (i >= g.nx - 1) || (comp == 2 && (k == 1 || k == g.nz - 1));
  if (edge) jacobi_bc(comp, g, h, x, X, P, i, j, k, v, fuse);
}

// 3-D checkerboard half-sweep (even iteration_time), one thread per point
// of the colour.
template <typename T, typename CS, int CC, int SW_X, int SW_Y>
__global__ void __launch_bounds__(SW_X *SW_Y)
    k_sor_even_c(int comp_, Geo g, Helm h, T *__restrict__ x, const CS coef,
                 const double *__restrict__ P, const double *__restrict__ X, int flg, int bc, int fuse) {
  const int comp = (CC >= 0) ? CC : comp_;
  const int i2 = blockIdx.x * SW_X + threadIdx.x, j = blockIdx.y * SW_Y + threadIdx.y + 1;
  const int k = blockIdx.z + (comp == 2 ? 1 : 0);
  const int iend = (comp == 0) ? g.nx - 1 : g.nx;
  if (i2 > (iend - 1) / 2 || j > g.ny) return;
  const int i = 2 * i2 + 1 + ((k + j + flg) & 1);
  T v = 0;
  if (i <= iend) {
    const int c = TPLS_IDX(g, i, j, k), sy = g.sy, sz = g.sz;
    const Rec<T> q = get_rec(comp, g, coef, c, i, j, k, false);
    const T xc = x[c];
    T zp, zm;
    if (comp == 2) {
      zp = x[c + sz];
      zm = x[c - sz];
    } else {
      zp = (k == g.nz - 1) ? xc : x[c + sz];
      zm = (k == 0) ? xc : x[c - sz];
    }
    const T res = rec_apply(q, x[c + 1], x[c - 1], x[c + sy], x[c - sy], zp, zm);
    v = xc + (T)1.2 * (res - xc);
    put(g, x, i, j, k, v, fuse);
  }
  if (bc) sor_bc(comp, g, h, x, X, P, i2, i, iend, v, j, k, fuse);
}

// Odd-iteration half-sweep (2-D colouring, sequential in k).  Within such a
// half-sweep every value a point reads is the pre-sweep value except the
// relaxed point below it in its own column, so the update is the recurrence
//   x_new(k) = A(k) + B(k) x_new(k-1),
//   A = x + 1.2 (partial - x),  B = 1.2 czm   (partial = all terms but czm),
// with A and B known before the sweep; the column is split into chunks whose
// recurrences run in parallel from a zero start and are then joined:
// x = y + P x_in, with y the chunk-local solution, P the product of the B
// factors since the chunk start and x_in the value entering the chunk.
// Coefficient records are streamed (evict-first) so the x field stays
// resident in L2.
//
// The kernel walks the column in super-chunks of SOC_SC levels with a
// carried value, so shared memory stays bounded for any column length (36 KB for
// FP64) and several blocks share an SM.  Per super-chunk:
//   1. produce: A and B of every (level, column) pair, a warp per level and
//      a lane per column, all pairs independent (their loads overlap);
//   2. scan: warp w runs the recurrence over its SOC_SC/SOC_W levels from a
//      zero start, keeping y(k) and P(k) = prod B in place of A and B;
//   3. each warp folds the chunk ends below it and the carried value into
//      x_in and writes x = y + P x_in with the boundary rows; the last
//      level's x is carried into the next super-chunk.
// The rounding differs from the level-by-level order (the oracle's) by a
// few ulp.
constexpr int SOC_W = 8, SOC_SC = 64;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ double ld_acquire_f64(const double *p) {
  double v;
  asm volatile("ld.acquire.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Phases 1 and 2 of one super-chunk (levels kc .. kc+n-1) of a tile: A and B
// of every (level, column) pair into sA/sB, then each warp's chunk scanned
// in place (y and P), its ends into ey/ep.  Synchronises the block.  The
// form of the FP32 sweeps (latency-bound): a warp per level, all (level,
// column) pairs independent so that their loads overlap.
template <typename T, typename CS>
__device__ __forceinline__ void odd_produce_scan_levels(int comp, const Geo &g, const CS &coef,
                                                        const T *__restrict__ x, int i, int j, bool act, int k0,
                                                        int kc, int n, T (*sA)[32], T (*sB)[32], T (*ey)[32],
                                                        T (*ep)[32]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int sy_ = g.sy, sz = g.sz, nz = g.nz;
  constexpr int PER = SOC_SC / SOC_W;
#pragma unroll 4
  for (int r = 0; r < PER; r++) {
    const int lk = w + r * SOC_W, k = kc + lk;
    if (lk < n) {
      T A = 0, B = 0;
      if (act) {
        const int c = TPLS_IDX(g, i, j, k);
        const Rec<T> q = get_rec(comp, g, coef, c, i, j, k, true);
        const T xc = x[c];
        T zp;
        if (comp == 2) zp = x[c + sz];
        else zp = (k == nz - 1) ? xc : x[c + sz];
        T part = fma(q.xp, x[c + 1], q.b);
        part = fma(q.xm, x[c - 1], part);
        part = fma(q.yp, x[c + sy_], part);
        part = fma(q.ym, x[c - sy_], part);
        part = fma(q.zp, zp, part);
        if (k == k0) {  // the point below is a wall value (w) or the point itself (u, v)
          const T zm = (comp == 2) ? x[c - sz] : xc;
          A = xc + (T)1.2 * (fma(q.zm, zm, part) - xc);
        } else {
          A = xc + (T)1.2 * (part - xc);
          B = (T)1.2 * q.zm;
        }
      }
      sA[lk][lane] = A;
      sB[lk][lane] = B;
    }
  }
  __syncthreads();
  const int lb = w * PER, le = min(n, lb + PER);
  T yv = 0, pv = 1;
  for (int lk = lb; lk < le; lk++) {
    const T B = sB[lk][lane];
    yv = fma(B, yv, sA[lk][lane]);
    pv = B * pv;
    sA[lk][lane] = yv;
    sB[lk][lane] = pv;
  }
  ey[w][lane] = yv;  // an empty chunk passes x_in through (y 0, P 1)
  ep[w][lane] = pv;
  __syncthreads();
}

// The same for the FP64 sweeps (bound by the FP64 pipe): each warp marches
// up its own PER consecutive levels and steps its chunk's recurrence as it
// goes, B read from the record (bz), the point above a level becoming the
// next level's centre value, no block barrier between production and scan.
// The operations per level and their order are those above, so both forms
// give the results of the whole-column form bit for bit.  With B from the
// record and the segment kernel's once-per-block fold, this form measured
// 10% faster than the level form for the FP64 sweeps at 256x128x192 and
// 11% slower for the FP32 sweeps at 512x256x256.
template <typename T, typename CS>
__device__ __forceinline__ void odd_produce_scan(int comp, const Geo &g, const CS &coef, const T *__restrict__ x,
                                                 int i, int j, bool act, int k0, int kc, int n,
                                                 T (*sA)[32], T (*sB)[32], T (*ey)[32], T (*ep)[32]) {
  if constexpr (sizeof(T) == 4) {
    odd_produce_scan_levels<T, CS>(comp, g, coef, x, i, j, act, k0, kc, n, sA, sB, ey, ep);
  } else {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int sy_ = g.sy, sz = g.sz, nz = g.nz;
    constexpr int PER = SOC_SC / SOC_W;
    const int lb = w * PER, le = min(n, lb + PER);
    T yv = 0, pv = 1;
    int c = act ? TPLS_IDX(g, i, j, kc + lb) : 0;
    T xc = (act && lb < le) ? x[c] : (T)0;
#pragma unroll
    for (int l = 0; l < PER; l++) {
      const int lk = lb + l, k = kc + lk;
      if (lk < le) {
        T A = 0, B = 0;
        if (act) {
          const Rec<T> q = get_rec(comp, g, coef, c, i, j, k, true);
          T zp;
          if (comp == 2) zp = x[c + sz];
          else zp = (k == nz - 1) ? xc : x[c + sz];
          T part = fma(q.xp, x[c + 1], q.b);
          part = fma(q.xm, x[c - 1], part);
          part = fma(q.yp, x[c + sy_], part);
          part = fma(q.ym, x[c - sy_], part);
          part = fma(q.zp, zp, part);
          if (k == k0) {
            const T zm = (comp == 2) ? x[c - sz] : xc;
            A = xc + (T)1.2 * (fma(q.zm, zm, part) - xc);
          } else {
            A = xc + (T)1.2 * (part - xc);
            B = q.bz;
          }
          xc = zp;  // x(k+1), the centre of the next level (unused after k = nz-1)
          c += sz;
        }
        yv = fma(B, yv, A);
        pv = B * pv;
        sA[lk][lane] = yv;
        sB[lk][lane] = pv;
      }
    }
    ey[w][lane] = yv;  // an empty chunk passes x_in through (y 0, P 1)
    ep[w][lane] = pv;
    __syncthreads();
  }
}

// x at the super-chunk's last level given the value entering it (what phase
// 3 writes there, by the same operations); 0 for a column outside the grid.
template <typename T>
__device__ __forceinline__ T odd_last_value(T xin, int n, bool col_in, T (*sA)[32], T (*sB)[32], T (*ey)[32],
                                            T (*ep)[32]) {
  const int lane = threadIdx.x & 31;
  constexpr int PER = SOC_SC / SOC_W;
  const int wl = (n - 1) / PER;
  for (int v = 0; v < wl; v++) xin = fma(ep[v][lane], xin, ey[v][lane]);
  return col_in ? fma(sB[n - 1][lane], xin, sA[n - 1][lane]) : (T)0;
}

// Phase 3: each warp writes x = y + P x_in from the value entering its own
// chunk (given in xin for FP64; for FP32 xin enters the super-chunk and the
// warp folds the chunk ends below its own into it first), then the
// boundary rows of its levels.  Returns x at the super-chunk's last level
// for the warp that owns it (0 elsewhere).
template <typename T>
__device__ __forceinline__ T odd_write(int comp, const Geo &g, const Helm &h, T *__restrict__ x,
                                       const double *__restrict__ X, const double *__restrict__ P, int bc,
                                       int fuse, int i2, int i, int j, int iend, int npair, int kc, int n, T xin,
                                       T (*sA)[32], T (*sB)[32], T (*ey)[32], T (*ep)[32]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  constexpr int PER = SOC_SC / SOC_W;
  const int lb = w * PER, le = min(n, lb + PER);
  T last = 0;
  if constexpr (sizeof(T) == 4)
    for (int v = 0; v < w; v++) xin = fma(ep[v][lane], xin, ey[v][lane]);
  if (i2 < npair) {
    for (int lk = lb; lk < le; lk++) {
      T v = 0;
      if (i <= iend) {
        v = fma(sB[lk][lane], xin, sA[lk][lane]);
        put(g, x, i, j, kc + lk, v, fuse);
      }
      sA[lk][lane] = v;  // kept for the boundary rows below
      if (lk == n - 1) last = v;
    }
    // boundary rows of these levels, by the owners of the first and last
    // pairs, after the writes: the point each boundary copies (relaxed
    // here, or of the other colour and final) is loaded for all levels at
    // once instead of level by level.  Nothing in this sweep reads the
    // boundary values of these levels.
    if (bc && (i2 == 0 || i2 == (iend - 1) / 2)) {
      const int ib = (i2 == 0) ? 1 : iend;
      T src[PER];
#pragma unroll
      for (int l = 0; l < PER; l++)
        src[l] = (lb + l < le) ? ((i != ib) ? x[TPLS_IDX(g, ib, j, kc + lb + l)] : sA[lb + l][lane]) : (T)0;
#pragma unroll
      for (int l = 0; l < PER; l++)
        if (lb + l < le) sor_bc(comp, g, h, x, X, P, i2, ib, iend, src[l], j, kc + lb + l, fuse);
    }
  }
  return last;
}

// One tile: 32 columns (x pairs from bx*32) of row j = by+1, the whole
// column.  Every thread of the block runs it (it synchronises the block).
// The segment kernel below runs the same phases by the helpers above, one
// super-chunk per block.
template <typename T, typename CS, int CC>
__device__ __forceinline__ void sor_odd_c4_tile(int comp_, const Geo &g, const Helm &h, T *__restrict__ x,
                                                const CS &coef, const double *__restrict__ P,
                                                const double *__restrict__ X, int flg, int bc, int fuse, int bx,
                                                int by) {
  const int comp = (CC >= 0) ? CC : comp_;
  __shared__ T sA[SOC_SC][32], sB[SOC_SC][32];
  __shared__ T ey[SOC_W][32], ep[SOC_W][32], scarry[32];
  const int j = by + 1;
  const int iend = (comp == 0) ? g.nx - 1 : g.nx;
  const int npair = (iend + 1) / 2;
  const int par = (j + flg) & 1;
  const int k0 = (comp == 2) ? 1 : 0, k1 = g.nz - 1;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int i2 = bx * 32 + lane, i = 2 * i2 + 1 + par;
  const bool act = (i2 < npair) && (i <= iend);
  const int sy_ = g.sy, sz = g.sz, nz = g.nz;
  constexpr int PER = SOC_SC / SOC_W;
  T carry = 0;  // x of the level below the super-chunk (k0 has B = 0)
  for (int kc = k0; kc <= k1; kc += SOC_SC) {
    const int n = min(SOC_SC, k1 - kc + 1);
    // 1. produce
#pragma unroll 4
    for (int r = 0; r < PER; r++) {
      const int lk = w + r * SOC_W, k = kc + lk;
      if (lk < n) {
        T A = 0, B = 0;
        if (act) {
          const int c = TPLS_IDX(g, i, j, k);
          const Rec<T> q = get_rec(comp, g, coef, c, i, j, k, true);
          const T xc = x[c];
          T zp;
          if (comp == 2) zp = x[c + sz];
          else zp = (k == nz - 1) ? xc : x[c + sz];
          T part = fma(q.xp, x[c + 1], q.b);
          part = fma(q.xm, x[c - 1], part);
          part = fma(q.yp, x[c + sy_], part);
          part = fma(q.ym, x[c - sy_], part);
          part = fma(q.zp, zp, part);
          if (k == k0) {  // the point below is a wall value (w) or the point itself (u, v)
            const T zm = (comp == 2) ? x[c - sz] : xc;
            A = xc + (T)1.2 * (fma(q.zm, zm, part) - xc);
          } else {
            A = xc + (T)1.2 * (part - xc);
            B = (sizeof(T) == 8) ? q.bz : (T)1.2 * q.zm;
          }
        }
        sA[lk][lane] = A;
        sB[lk][lane] = B;
      }
    }
    __syncthreads();
    // 2. scan of this warp's levels
    const int lb = w * PER, le = min(n, lb + PER);
    T yv = 0, pv = 1;
    for (int lk = lb; lk < le; lk++) {
      const T B = sB[lk][lane];
      yv = fma(B, yv, sA[lk][lane]);
      pv = B * pv;
      sA[lk][lane] = yv;
      sB[lk][lane] = pv;
    }
    ey[w][lane] = yv;  // an empty chunk passes x_in through (y 0, P 1)
    ep[w][lane] = pv;
    __syncthreads();
    // 3. fold and write
    T xin = carry;
    for (int v = 0; v < w; v++) xin = fma(ep[v][lane], xin, ey[v][lane]);
    if (i2 < npair) {
      for (int lk = lb; lk < le; lk++) {
        T v = 0;
        if (i <= iend) {
          v = fma(sB[lk][lane], xin, sA[lk][lane]);
          put(g, x, i, j, kc + lk, v, fuse);
        }
        sA[lk][lane] = v;  // kept for the boundary rows below
        if (lk == n - 1) scarry[lane] = v;
      }
      // boundary rows of these levels, by the owners of the first and last
      // pairs, after the writes: the point each boundary copies (relaxed
      // here, or of the other colour and final) is loaded for all levels at
      // once instead of level by level.  Nothing in this sweep reads the
      // boundary values of these levels.
      if (bc && (i2 == 0 || i2 == (iend - 1) / 2)) {
        const int ib = (i2 == 0) ? 1 : iend;
        T src[PER];
#pragma unroll
        for (int l = 0; l < PER; l++)
          src[l] = (lb + l < le) ? ((i != ib) ? x[TPLS_IDX(g, ib, j, kc + lb + l)] : sA[lb + l][lane]) : (T)0;
#pragma unroll
        for (int l = 0; l < PER; l++)
          if (lb + l < le) sor_bc(comp, g, h, x, X, P, i2, ib, iend, src[l], j, kc + lb + l, fuse);
      }
    }
    __syncthreads();
    carry = scarry[lane];
  }
}

// Odd half-sweep with one block per super-chunk of a tile (segment), for
// columns of 3 or more segments (FP64 records, the FP32 sweeps and the
// per-routine entries alike), so a launch has nz/64 times the blocks of
// the whole-column form and the blocks' load, scan and write phases
// overlap.
// The value entering a segment is the last value of the segment below it:
// segments are taken in ticket order, lowest segment of every tile first,
// so the block a segment waits for took its ticket earlier and is running;
// it publishes that value (the same operations as the whole-column form,
// so the results are bit-identical to it) as soon as it has its own
// entering value, before it writes.  The wait is bounded: if it runs out
// the block counts it in *kto, takes NaN as its entering value (the step's
// pressure solve then reports DIVERGED_NAN) and still publishes, so no
// later segment waits on it.
template <typename T, typename CS, int CC>
__global__ void __launch_bounds__(SOC_W * 32, sizeof(T) == 4 ? 6 : 5)  // 40 / 48 registers: 6 / 5 blocks per SM
    k_sor_odd_seg(int comp_, Geo g, Helm h, T *__restrict__ x, const CS coef, const double *__restrict__ P,
                  const double *__restrict__ X, int flg, int bc, int fuse, OddChain oc, int gx, int limit) {
  const int comp = (CC >= 0) ? CC : comp_;
  __shared__ T sA[SOC_SC][32], sB[SOC_SC][32];
  // the value entering each warp's chunk (FP64), or the segment's (FP32)
  __shared__ T ey[SOC_W][32], ep[SOC_W][32], sxin[sizeof(T) == 8 ? SOC_W : 1][32];
  __shared__ unsigned s_t, s_ep;
  if (threadIdx.x == 0) {
    s_t = atomicAdd(&oc.ctr[0], 1u);
    s_ep = ld_acquire_u32(&oc.ctr[2]);
  }
  __syncthreads();
  const unsigned t = s_t, epoch = s_ep;
  const int nct = gx * g.ny;
  const int seg = (int)(t / (unsigned)nct), ct = (int)(t - (unsigned)seg * nct);
  const int bx = ct % gx, j = ct / gx + 1;
  const int iend = (comp == 0) ? g.nx - 1 : g.nx;
  const int npair = (iend + 1) / 2;
  const int par = (j + flg) & 1;
  const int k0 = (comp == 2) ? 1 : 0, k1 = g.nz - 1;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int i2 = bx * 32 + lane, i = 2 * i2 + 1 + par;
  const bool act = (i2 < npair) && (i <= iend);
  const int kc = k0 + seg * SOC_SC, n = min(SOC_SC, k1 - kc + 1);
  constexpr int PER = SOC_SC / SOC_W;
  odd_produce_scan<T, CS>(comp, g, coef, x, i, j, act, k0, kc, n, sA, sB, ey, ep);
  if (w == 0) {
    T xin = 0;  // k0 has B = 0
    if (seg > 0) {
      // every lane acquires the flag itself (one transaction per poll for
      // the warp) before reading its column's value
      const unsigned pt = t - (unsigned)nct;  // the segment below, same columns
      bool ok = true;
      int it = 0;
      while (ld_acquire_u32(&oc.flag[pt]) != epoch + 1u)
        if (++it >= limit) {
          ok = false;
          break;
        }
      xin = ok ? (T)ld_acquire_f64(&oc.incl[(size_t)pt * 32 + lane]) : (T)__longlong_as_double(0x7ff8000000000000ll);
      if (__any_sync(0xffffffffu, !ok) && lane == 0) atomicAdd(oc.kto, 1.0);
    }
    if constexpr (sizeof(T) == 8) {
      // FP64: the value entering every warp's chunk, the chunk ends below
      // it folded in order, once for the block instead of once per warp
      T xw = xin;
#pragma unroll
      for (int v = 0; v < SOC_W; v++) {
        sxin[v][lane] = xw;
        if (v + 1 < SOC_W) xw = fma(ep[v][lane], xw, ey[v][lane]);
      }
      if (seg < (k1 - k0) / SOC_SC) {  // a segment above waits for this one
        oc.incl[(size_t)t * 32 + lane] =
            act ? fma(sB[n - 1][lane], sxin[(n - 1) / PER][lane], sA[n - 1][lane]) : (T)0;
        __threadfence();
        __syncwarp();
        if (lane == 0) st_release_u32(&oc.flag[t], epoch + 1u);
      }
    } else {
      if (seg < (k1 - k0) / SOC_SC) {  // a segment above waits for this one
        oc.incl[(size_t)t * 32 + lane] = (double)odd_last_value<T>(xin, n, i2 < npair && i <= iend, sA, sB, ey, ep);
        __threadfence();
        __syncwarp();
        if (lane == 0) st_release_u32(&oc.flag[t], epoch + 1u);
      }
      sxin[0][lane] = xin;
    }
  }
  __syncthreads();
  odd_write<T>(comp, g, h, x, X, P, bc, fuse, i2, i, j, iend, npair, kc, n, sxin[sizeof(T) == 8 ? w : 0][lane], sA,
               sB, ey, ep);
  if (threadIdx.x == 0) {  // the last block to leave resets the tickets and starts a new epoch
    __threadfence();
    if (atomicAdd(&oc.ctr[1], 1u) == gridDim.x - 1) {
      oc.ctr[0] = 0u;
      oc.ctr[1] = 0u;
      __threadfence();
      atomicAdd(&oc.ctr[2], 1u);
    }
  }
}

template <typename T, typename CS, int CC>
__global__ void __launch_bounds__(SOC_W * 32)
    k_sor_odd_c4(int comp_, Geo g, Helm h, T *__restrict__ x, const CS coef,
                 const double *__restrict__ P, const double *__restrict__ X, int flg, int bc, int fuse) {
  sor_odd_c4_tile<T, CS, CC>(comp_, g, h, x, coef, P, X, flg, bc, fuse, blockIdx.x, blockIdx.y);
}

// Multi-instance odd half-sweep of the FP32 sweeps of a batch: the tiles of
// every member (32 columns of one row each) taken in order by an atomic
// ticket, as k_sweep4_multi.
template <int CC>
__global__ void __launch_bounds__(SOC_W * 32)
    k_odd_multi(const SweepMember *__restrict__ mem, const int *__restrict__ prefix, int n, int src, int flg,
                int bc, unsigned *ctr) {
  __shared__ int s_t;
  const int total = prefix[n];
  for (;;) {
    if (threadIdx.x == 0) s_t = (int)atomicAdd(&ctr[0], 1u);
    __syncthreads();
    const int t = s_t;
    __syncthreads();
    if (t >= total) break;
    int m = 0;
    while (prefix[m + 1] <= t) m++;
    const SweepMember &M = mem[m];
    const int iend = (CC == 0) ? M.g.nx - 1 : M.g.nx;
    const int gx = ((iend + 1) / 2 + 31) / 32;
    const int lt = t - prefix[m];
    sor_odd_c4_tile<float, MuCoef, CC>(CC, M.g, M.h, M.x[CC][src], M.s[CC], M.P, M.X[CC], flg, bc, M.fuse,
                                       lt % gx, lt / gx);
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&ctr[1], 1u) == gridDim.x - 1) {
      ctr[0] = 0u;
      ctr[1] = 0u;
    }
  }
}

int odd_tiles(int comp, const Geo &g) {
  const int iend = (comp == 0) ? g.nx - 1 : g.nx;
  return (((iend + 1) / 2 + 31) / 32) * g.ny;
}

cudaError_t launch_odd_multi(int comp, const SweepMember *mem, const int *prefix, int n, int total_tiles, int src,
                             int flg, int bc, unsigned *ctr, int nblocks, cudaStream_t st) {
  const int nb = total_tiles < nblocks ? total_tiles : nblocks;
  if (nb <= 0) return cudaSuccess;
  if (comp == 0) k_odd_multi<0><<<nb, SOC_W * 32, 0, st>>>(mem, prefix, n, src, flg, bc, ctr);
  else if (comp == 1) k_odd_multi<1><<<nb, SOC_W * 32, 0, st>>>(mem, prefix, n, src, flg, bc, ctr);
  else k_odd_multi<2><<<nb, SOC_W * 32, 0, st>>>(mem, prefix, n, src, flg, bc, ctr);
  return cudaGetLastError();
}

cudaError_t sweep_init() { return cudaSuccess; }

template <typename T, typename CS, int CC, int BX, int BY>
static void jacobi_v(int comp, const Geo &g, const Helm &h, const T *xo, CS coef, const double *pres,
                     const double *X, T *x, int fuse, cudaStream_t st) {
  const int nk = (comp == 2) ? g.nz - 1 : g.nz;
  const int iend = (comp == 0) ? g.nx - 1 : g.nx;
  dim3 grd((iend + BX - 1) / BX, (g.ny + BY - 1) / BY, nk);
  k_jacobi_c<T, CS, CC, BX, BY><<<grd, dim3(BX, BY), 0, st>>>(comp, g, h, xo, coef, pres, X, x, fuse);
}

// tile: the block shape (threads over i, or i pairs, by threads over j) the
// autotuner chooses among for the Jacobi and even-SOR kernels: 0 = 32x4 (the
// default), 1 = 32x8, 2 = 64x4, 3 = 16x8.
template <typename T, typename CS, int CC>
static cudaError_t jacobi_c(int comp, const Geo &g, const Phys &ph, const T *xo, CS coef, const double *pres,
                            const double *X, T *x, int fuse, int tile, cudaStream_t st) {
  const Helm h = helm_of(ph);
  switch (tile) {
    case 1: jacobi_v<T, CS, CC, 32, 8>(comp, g, h, xo, coef, pres, X, x, fuse, st); break;
    case 2: jacobi_v<T, CS, CC, 64, 4>(comp, g, h, xo, coef, pres, X, x, fuse, st); break;
    case 3: jacobi_v<T, CS, CC, 16, 8>(comp, g, h, xo, coef, pres, X, x, fuse, st); break;
    default: jacobi_v<T, CS, CC, 32, 4>(comp, g, h, xo, coef, pres, X, x, fuse, st); break;
  }
  return cudaGetLastError();
}

template <typename T, typename CS, int CC, int BX, int BY>
static void even_v(int comp, const Geo &g, const Helm &h, T *x, CS coef, const double *pres, const double *X,
                   int flg, int bc, int fuse, cudaStream_t st) {
  const int iend = (comp == 0) ? g.nx - 1 : g.nx;
  const int npairs = (iend + 1) / 2;
  const int nk = (comp == 2) ? g.nz - 1 : g.nz;
  dim3 grd((npairs + BX - 1) / BX, (g.ny + BY - 1) / BY, nk);
  k_sor_even_c<T, CS, CC, BX, BY><<<grd, dim3(BX, BY), 0, st>>>(comp, g, h, x, coef, pres, X, flg, bc, fuse);
}

int odd_chain_segments(const Geo &g) {
  const int gx = (((g.nx + 1) / 2) + 31) / 32;  // v and w have the most pairs
  return ((g.nz - 1) / SOC_SC + 1) * gx * g.ny;
}

template <typename T, typename CS, int CC>
static cudaError_t sor_c(int comp, const Geo &g, const Phys &ph, T *x, CS coef, const double *pres,
                         const double *X, int flg, int iteration_time, int bc, int fuse, int tile_even,
                         int tile_odd, cudaStream_t st, const OddChain *oc = nullptr) {
  const int iend = (comp == 0) ? g.nx - 1 : g.nx;
  const int npairs = (iend + 1) / 2;
  const Helm h = helm_of(ph);
  if (iteration_time % 2 == 0) {
    switch (tile_even) {
      case 1: even_v<T, CS, CC, 32, 8>(comp, g, h, x, coef, pres, X, flg, bc, fuse, st); break;
      case 2: even_v<T, CS, CC, 64, 4>(comp, g, h, x, coef, pres, X, flg, bc, fuse, st); break;
      case 3: even_v<T, CS, CC, 16, 8>(comp, g, h, x, coef, pres, X, flg, bc, fuse, st); break;
      default: even_v<T, CS, CC, 32, 4>(comp, g, h, x, coef, pres, X, flg, bc, fuse, st); break;
    }
  } else {
    (void)tile_odd;
    const int gx = (npairs + 31) / 32;
    const int k0 = (comp == 2) ? 1 : 0, nseg = (g.nz - 1 - k0) / SOC_SC + 1;
    // one block per segment, chained, for columns of 3 or more segments:
    // with 2, half the blocks wait on the other half for a larger share of
    // their time than the extra blocks save (measured slower on the batched
    // workload's grids, nz <= 128; faster at nz = 192 and 256)
    if (oc && nseg >= 3 && oc->cap >= nseg * gx * g.ny) {
      k_sor_odd_seg<T, CS, CC><<<nseg * gx * g.ny, SOC_W * 32, 0, st>>>(comp, g, h, x, coef, pres, X, flg, bc,
                                                                       fuse, *oc, gx, 1 << 20);
    } else {  // one block per 32 columns of a row, the column in super-chunks
      dim3 grd(gx, g.ny, 1);
      k_sor_odd_c4<T, CS, CC><<<grd, SOC_W * 32, 0, st>>>(comp, g, h, x, coef, pres, X, flg, bc, fuse);
    }
  }
  return cudaGetLastError();
}

cudaError_t launch_sor_ref_odd(int comp, const Geo &g, const Phys &ph, double *x, const double *rhs,
                               const double *mu, int flg, cudaStream_t st, const OddChain *oc) {
  const Helm h = helm_of(ph);
  RefCoef r;
  r.mu = mu;
  r.rhs = rhs;
  r.ax2 = h.ax2;
  r.ay2 = h.ay2;
  r.az2 = h.az2;
  return sor_c<double, RefCoef, -1>(comp, g, ph, x, r, nullptr, nullptr, flg, 1, 0, 0, 0, 0, st, oc);
}

MuCoef mu_coef(const Phys &ph, const float *mu, const float *b, const float4 *bco) {
  const Helm h = helm_of(ph);
  MuCoef m;
  m.mu = mu;
  m.b = b;
  m.bco = bco;
  m.ax2 = (float)h.ax2;
  m.ay2 = (float)h.ay2;
  m.az2 = (float)h.az2;
  return m;
}

cudaError_t launch_jacobi_c(int comp, const Geo &g, const Phys &ph, const double *xo, const double *coef,
                            const double *pres, double *x, int fuse, cudaStream_t st, const SweepTiles &t) {
  return jacobi_c<double, const double *, -1>(comp, g, ph, xo, coef, pres, nullptr, x, fuse, t.jac, st);
}
cudaError_t launch_jacobi_c(int comp, const Geo &g, const Phys &ph, const float *xo, const MuCoef &coef,
                            const double *pres, const double *X, float *x, int fuse, cudaStream_t st,
                            const SweepTiles &t) {
  return launch_sweep4(0, comp, g, helm_of(ph), xo, x, coef, pres, X, 0, 1, fuse, t.jac, st);
}
cudaError_t launch_sor_c(int comp, const Geo &g, const Phys &ph, double *x, const double *coef,
                         const double *pres, int flg, int iteration_time, int bc, int fuse, cudaStream_t st,
                         const SweepTiles &t, const OddChain *oc) {
  return sor_c<double, const double *, -1>(comp, g, ph, x, coef, pres, nullptr, flg, iteration_time, bc, fuse, t.even,
                                          t.odd, st, oc);
}
cudaError_t launch_sor_c(int comp, const Geo &g, const Phys &ph, float *x, const MuCoef &coef,
                         const double *pres, const double *X, int flg, int iteration_time, int bc, int fuse,
                         cudaStream_t st, const SweepTiles &t, const OddChain *oc) {
  if (iteration_time % 2 == 0)  // checkerboard half-sweep: four x points per thread (k_sweep32.cu)
    return launch_sweep4(1, comp, g, helm_of(ph), x, x, coef, pres, X, flg, bc, fuse, t.even, st);
  if (comp == 0)
    return sor_c<float, MuCoef, 0>(comp, g, ph, x, coef, pres, X, flg, iteration_time, bc, fuse, t.even, t.odd, st, oc);
  if (comp == 1)
    return sor_c<float, MuCoef, 1>(comp, g, ph, x, coef, pres, X, flg, iteration_time, bc, fuse, t.even, t.odd, st, oc);
  return sor_c<float, MuCoef, 2>(comp, g, ph, x, coef, pres, X, flg, iteration_time, bc, fuse, t.even, t.odd, st, oc);
}

// defect form: d = -X before the first sweep (the sweeps start from x = 0),
// x = X + d after the last (conversions by integer operations, tpls_pair.cuh)
__global__ void k_defect_init(const double *__restrict__ X, float *__restrict__ d, size_t n) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    d[q] = -round_bits(X[q]);
}
__global__ void k_defect_apply(const double *__restrict__ X, const float *__restrict__ d, double *__restrict__ x,
                               size_t n) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    x[q] = X[q] + widen_bits(d[q]);
}
cudaError_t launch_defect_init(const double *X, float *d, size_t n, cudaStream_t st) {
  k_defect_init<<<1216, 256, 0, st>>>(X, d, n);
  return cudaGetLastError();
}
cudaError_t launch_defect_apply(const double *X, const float *d, double *x, size_t n, cudaStream_t st) {
  k_defect_apply<<<1216, 256, 0, st>>>(X, d, x, n);
  return cudaGetLastError();
}

}  // namespace tpls
