// k_advect.cu -- level-set advection: WENO5 face values and the
// conservative flux divergence (advect_phi.f90:19-119, weno.f90:18-215).
//
// One thread per (i,j) column of p-cells, marching a chunk of 16 z levels
// (one z-face below the chunk is computed at its start).  Each face value
// is computed once: the x-face left of a thread is its left neighbour's
// right face and the y-face below is the lower row's upper face, both
// through a shared tile (the block's left and bottom edge faces computed by
// one warp each), and the z-face below is the previous level's z-face held
// in a register.
// The periodic-y halo of the reference's 3-ghost phi_augaug copy becomes a
// wrapped row index; no augmented array is built.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include "tpls_kernels.h"
#include "tpls_pair.cuh"

namespace tpls {

// weno.f90:175-215 (Jiang-Shu WENO5).  The three nonlinear weights
// a_i/(a1+a2+a3) with a_i = c_i/q_i are formed with one division:
// w_i = c_i*prod_{j!=i} q_j / sum_m c_m*prod_{j!=m} q_j.
template <typename T>
__device__ __forceinline__ T weno5(T v1, T v2, T v3, T v4, T v5) {
  const T eps = (T)TPLS_WENO_EPS, two = (T)2, three = (T)3, four = (T)4;
  const T c13 = (T)(13.0 / 12.0), c14 = (T)0.25;
  T t1 = v1 - two * v2 + v3, t2 = v1 - four * v2 + three * v3;
  T q1 = eps + (c13 * t1 * t1 + c14 * t2 * t2);
  t1 = v2 - two * v3 + v4;
  t2 = v2 - v4;
  T q2 = eps + (c13 * t1 * t1 + c14 * t2 * t2);
  t1 = v3 - two * v4 + v5;
  t2 = three * v3 - four * v4 + v5;
  T q3 = eps + (c13 * t1 * t1 + c14 * t2 * t2);
  q1 *= q1;
  q2 *= q2;
  q3 *= q3;
  const T n1 = (T)0.1 * (q2 * q3), n2 = (T)0.6 * (q1 * q3), n3 = (T)0.3 * (q1 * q2);
  const T p1 = v1 * (T)(1.0 / 3.0) - v2 * (T)(7.0 / 6.0) + v3 * (T)(11.0 / 6.0);
  const T p2 = -v2 * (T)(1.0 / 6.0) + v3 * (T)(5.0 / 6.0) + v4 * (T)(1.0 / 3.0);
  const T p3 = v3 * (T)(1.0 / 3.0) + v4 * (T)(5.0 / 6.0) - v5 * (T)(1.0 / 6.0);
  return (n1 * p1 + n2 * p2 + n3 * p3) / (n1 + n2 + n3);
}

// vel >= 0 (-0 included) from the sign bit for FP64, so the upwind choice
// takes no FP64 compare; a NaN velocity (a diverged state) may pick either
// stencil.
__device__ __forceinline__ bool upwind_pos(double v) {
  const int hi = __double2hiint(v);
  return hi >= 0 || (hi == (int)0x80000000 && __double2loint(v) == 0);
}
__device__ __forceinline__ bool upwind_pos(float v) { return v >= 0.0f; }

// The upwind WENO5 value on the face between c0 and p1 of a line of six
// points m2 m1 c0 p1 p2 p3: the stencil m2..p2 when the face velocity is
// >= 0, else p3..m1 (weno.f90:52-60, 64-72).  The stencil is selected before
// the one weno5 evaluation, so a warp whose lanes see both signs does not
// run weno5 twice.
template <typename T>
__device__ __forceinline__ T weno_up(bool pos, T m2, T m1, T c0, T p1, T p2, T p3) {
  return weno5(pos ? m2 : p3, pos ? m1 : p2, pos ? c0 : p1, pos ? p1 : c0, pos ? p2 : m1);
}

// dfx at u-index (iu, jp-1, kp-1): phi along x at p-row jp, level kp.
// WENO for 3 <= iu <= nx-2, first-order upwind otherwise (weno.f90:45-100).
template <typename T>
__device__ __forceinline__ T xface(const Geo &g, const T *__restrict__ phi,
                                        const T *__restrict__ u, int iu, int jp,
                                        int kp) {
  const int ju = (jp - 1 == 0) ? g.ny : jp - 1;
  const T vel = u[TPLS_IDX(g, iu, ju, kp - 1)];
  const T *row = phi + TPLS_IDX(g, 0, jp, kp);
  if (iu >= 3 && iu <= g.nx - 2)
    return weno_up(upwind_pos(vel), row[iu - 2], row[iu - 1], row[iu], row[iu + 1], row[iu + 2], row[iu + 3]);
  return (upwind_pos(vel)) ? row[iu] : row[iu + 1];
}

// dfy at v-index (ip, jv, kp-1): phi along y at x=ip, level kp, periodic
// rows (weno.f90:105-132; row 0 is the exchanged copy of row ny).
template <typename T>
__device__ __forceinline__ T yface(const Geo &g, const T *__restrict__ phi,
                                        const T *__restrict__ v, int ip, int jv,
                                        int kp) {
  const int ny = g.ny;
  if (jv == 0) jv = ny;
  const T vel = v[TPLS_IDX(g, ip, jv, kp - 1)];
  const T *col = phi + TPLS_IDX(g, ip, 0, kp);
  const int sy = g.sy;
#define PY(jj) col[sy * wrapy((jj), ny)]
  return weno_up(upwind_pos(vel), PY(jv - 2), PY(jv - 1), PY(jv), PY(jv + 1), PY(jv + 2), PY(jv + 3));
#undef PY
}

constexpr int ADV_BX = 32, ADV_BY = 8;
constexpr int ADV_KC = 16;  // z levels per thread (column chunk)

// One block covers 32 x 8 columns and a chunk of ADV_KC levels.  At each
// level every thread computes the x-face right of its cell and the y-face
// above it; the faces left of the block's first column (8, one per row) are
// computed by eight lanes of warp 1 and those below its first row (32) by
// warp 0, so the extra faces cost about two warp evaluations per block and
// level instead of one per warp.  Faces pass through a double-buffered
// shared tile (one barrier per level).  The z-faces come from a six-point
// window of the column held in registers, one new load per level.
template <typename T>
__global__ void __launch_bounds__(ADV_BX *ADV_BY, 4)
    k_advect(Geo g, T rdx, T rdy, T rdz, const T *__restrict__ phi, const T *__restrict__ u,
             const T *__restrict__ v, const T *__restrict__ w, double *__restrict__ conv) {
  __shared__ T xs[2][ADV_BY][ADV_BX + 1];  // x-faces iu = i0-1 .. i0+31 per row
  __shared__ T ys[2][ADV_BY + 1][ADV_BX];  // y-faces jv = j0-1 .. j0+7 per column
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i0 = blockIdx.x * ADV_BX + 1, j0 = blockIdx.y * ADV_BY + 1;
  const int i = i0 + tx, j = j0 + ty;
  const int k0 = blockIdx.z * ADV_KC + 1, k1 = min(k0 + ADV_KC - 1, g.nz);
  const bool act = (i <= g.nx) && (j <= g.ny);
  const int ic = act ? i : 1, jc = act ? j : 1;  // clamped for inactive lanes
  const int jm = (jc == 1) ? g.ny : jc - 1;      // u/v/w row index j-1 (wrapped)
  // the row whose left x-face this lane computes when it is one of warp 1's
  // first eight lanes (clamped like jc)
  const int jx = (j0 + tx <= g.ny) ? j0 + tx : 1;
  // z window c0..c5 = phi(ic, jc, kw-2 .. kw+3) for the z-face kw (w-index),
  // indices clamped to the array's 0..nz+1; the clamped entries are read only
  // where the face is the arithmetic mean of c2 and c3 (kw < 3 or kw > nz-2)
  const T *col = phi + TPLS_IDX(g, ic, jc, 0);
  const int sz = g.sz, nzp1 = g.nz + 1;
  auto zld = [&](int kk) { return col[(size_t)sz * min(max(kk, 0), nzp1)]; };
  // dfz at w-index (ic, jc-1, kw): WENO for 3 <= kw <= nz-2, arithmetic mean
  // otherwise (weno.f90:136-166)
  auto zface = [&](int kw, T c0, T c1, T c2, T c3, T c4, T c5) -> T {
    if (kw >= 3 && kw <= g.nz - 2) return weno_up(upwind_pos(w[TPLS_IDX(g, ic, jm, kw)]), c0, c1, c2, c3, c4, c5);
    return (c2 + c3) / (T)2;
  };
  T c0 = zld(k0 - 3), c1 = zld(k0 - 2), c2 = zld(k0 - 1), c3 = zld(k0), c4 = zld(k0 + 1), c5 = zld(k0 + 2);
  T zlo = zface(k0 - 1, c0, c1, c2, c3, c4, c5);
  for (int k = k0; k <= k1; k++) {
    const int b = k & 1;
    c0 = c1;
    c1 = c2;
    c2 = c3;
    c3 = c4;
    c4 = c5;
    c5 = zld(k + 3);
    const T xo = xface(g, phi, u, ic, jc, k);
    const T yo = yface(g, phi, v, ic, jc, k);
    xs[b][ty][tx + 1] = xo;
    ys[b][ty + 1][tx] = yo;
    if (ty == 0)
      ys[b][0][tx] = yface(g, phi, v, ic, jc - 1, k);
    else if (ty == 1 && tx < ADV_BY)
      xs[b][tx][0] = xface(g, phi, u, i0 - 1, jx, k);
    const T zo = zface(k, c0, c1, c2, c3, c4, c5);
    __syncthreads();
    if (act) {
      const T xl = xs[b][ty][tx], yl = ys[b][ty][tx];
      const T fxp = u[TPLS_IDX(g, i, jm, k - 1)] * xo;
      const T fxm = u[TPLS_IDX(g, i - 1, jm, k - 1)] * xl;
      const T fyp = v[TPLS_IDX(g, i, j, k - 1)] * yo;
      const T fym = v[TPLS_IDX(g, i, jm, k - 1)] * yl;
      const T fzp = w[TPLS_IDX(g, i, jm, k)] * zo;
      const T fzm = w[TPLS_IDX(g, i, jm, k - 1)] * zlo;
      conv[TPLS_IDX(g, i, j, k)] = (double)((fxp - fxm) * rdx + (fyp - fym) * rdy + (fzp - fzm) * rdz);
    }
    zlo = zo;
  }
}

// ---------------------------------------------------------------------------
// The FP32 advection with phi staged by TMA.  A block (32 x 8 cells of
// AT_TZ levels) loads the phi tile with its 3-cell halos into shared memory
// by cp.async.bulk.tensor: one load per y row (AT_NR rows j0-3 .. j0+10),
// each a 40 x 1 x AT_NZ box of the FP32 phi copy, so the periodic y wrap of
// the reference's phi_augaug is just the row coordinate; the x start is the
// tile's first halo column rounded down to a 16-byte boundary, and levels
// outside the array read as zero (only the arithmetic-mean z-faces sit near
// them, and those read levels 0..nz+1).  The loads complete on one mbarrier;
// every thread then evaluates the same faces as k_advect<float>, operation
// for operation, from shared memory, so the result is bit-identical.  The
// velocities are read from global memory as before.
//
// The wait on the mbarrier is bounded (`limit` polls): when it runs out the
// block adds 1 to *kto, writes NaN into its output cells (the step's
// pressure solve then reports DIVERGED_NAN), waits again, bounded, for any
// copy still in flight, and returns.  arm = 0 issues no load (the
// self-test of that path: nothing completes the barrier).
constexpr int AT_BX = 32, AT_BY = 8, AT_TZ = 8;
constexpr int AT_W = 40;               // staged x extent (floats)
constexpr int AT_NR = AT_BY + 6;       // staged rows
constexpr int AT_NZ = AT_TZ + 6;       // staged levels
constexpr int AT_SLAB = 576;           // floats per row slab (40 x 14 = 560, padded to 128 bytes)
static_assert(AT_W * AT_NZ <= AT_SLAB && (AT_SLAB * 4) % 128 == 0, "slab layout");
constexpr unsigned AT_TX_BYTES = AT_NR * AT_W * AT_NZ * 4;

__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, int limit) {
  for (int it = 0; it < limit; it++) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__global__ void __launch_bounds__(AT_BX *AT_BY)
    k_advect_tma(const __grid_constant__ CUtensorMap phimap, Geo g, float rdx, float rdy, float rdz,
                 const float *__restrict__ u, const float *__restrict__ v, const float *__restrict__ w,
                 double *__restrict__ conv, double *kto, int arm, int limit) {
  __shared__ __align__(128) float sphi[AT_NR * AT_SLAB];
  __shared__ float xs[2][AT_BY][AT_BX + 1];
  __shared__ float ys[2][AT_BY + 1][AT_BX];
  __shared__ __align__(8) unsigned long long bar;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * AT_BX + tx;
  const int i0 = blockIdx.x * AT_BX + 1, j0 = blockIdx.y * AT_BY + 1;
  const int k0 = blockIdx.z * AT_TZ + 1, k1 = min(k0 + AT_TZ - 1, g.nz);
  const int x0 = blockIdx.x * AT_BX;  // row-start element of the slab: XOFF + i0 - 4, 16-byte aligned
  const unsigned sbar = smem_addr(&bar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0 && arm) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sbar), "r"(AT_TX_BYTES) : "memory");
    const unsigned long long map = reinterpret_cast<unsigned long long>(&phimap);
    for (int r = 0; r < AT_NR; r++) {
      const int jw = ((j0 - 4 + r) % g.ny + g.ny) % g.ny + 1;  // periodic row in 1..ny for any ny
      asm volatile(
          "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
          "[%5];" ::"r"(smem_addr(sphi + r * AT_SLAB)),
          "l"(map), "r"(x0), "r"(jw), "r"(k0 - 3), "r"(sbar)
          : "memory");
    }
  }
  const bool ok = __syncthreads_and(mbar_wait(sbar, 0, limit));
  const int i = i0 + tx, j = j0 + ty;
  const bool act = (i <= g.nx) && (j <= g.ny);
  if (!ok) {
    if (tid == 0) atomicAdd(kto, 1.0);
    if (act)
      for (int k = k0; k <= k1; k++) conv[TPLS_IDX(g, i, j, k)] = __longlong_as_double(0x7ff8000000000000ll);
    if (arm) mbar_wait(sbar, 0, limit);  // copies still in flight land before the block leaves
    return;
  }
  // phi at (x index ii, row r of the staged tile, level kk)
  auto PH = [&](int ii, int r, int kk) { return sphi[r * AT_SLAB + (kk - k0 + 3) * AT_W + (ii + XOFF - x0)]; };
  // Velocity indices are clamped into the grid for lanes outside it; the
  // staged indices of such a lane stay its own tile position (in the
  // staged tile, results unused), so every shared-memory read is in range.
  const int ic = act ? i : 1, jc = act ? j : 1;
  const int ii = i0 + tx, jj = j0 + ty;  // staged column / row of this thread (= i, j when active)
  const int jm = (jc == 1) ? g.ny : jc - 1;
  const int jx = (j0 + tx <= g.ny) ? j0 + tx : 1;
  const int rown = ty + 3;  // staged row of this thread's cell row
  // dfx at u-index iu (staged column iu, velocity column iv) of staged row r
  // (velocity p-row jp), level kp (as xface)
  auto xf = [&](int iu, int iv, int r, int jp, int kp) -> float {
    const int ju = (jp - 1 == 0) ? g.ny : jp - 1;
    const float vel = u[TPLS_IDX(g, iv, ju, kp - 1)];
    if (iu >= 3 && iu <= g.nx - 2)
      return weno_up(upwind_pos(vel), PH(iu - 2, r, kp), PH(iu - 1, r, kp), PH(iu, r, kp), PH(iu + 1, r, kp),
                     PH(iu + 2, r, kp), PH(iu + 3, r, kp));
    return (upwind_pos(vel)) ? PH(iu, r, kp) : PH(iu + 1, r, kp);
  };
  // dfy at staged v-index jv (rows jv-2..jv+3 staged at jv-2-(j0-3)) and
  // velocity v-index jvv, staged column ip, velocity column ipv, level kp
  // (as yface)
  auto yf = [&](int ip, int ipv, int jv, int jvv, int kp) -> float {
    const int rb = jv - j0 + 1;
    const float vel = v[TPLS_IDX(g, ipv, (jvv == 0) ? g.ny : jvv, kp - 1)];
    return weno_up(upwind_pos(vel), PH(ip, rb, kp), PH(ip, rb + 1, kp), PH(ip, rb + 2, kp), PH(ip, rb + 3, kp),
                   PH(ip, rb + 4, kp), PH(ip, rb + 5, kp));
  };
  auto zf = [&](int kw, float c0, float c1, float c2, float c3, float c4, float c5) -> float {
    if (kw >= 3 && kw <= g.nz - 2) return weno_up(upwind_pos(w[TPLS_IDX(g, ic, jm, kw)]), c0, c1, c2, c3, c4, c5);
    return (c2 + c3) / 2.0f;
  };
  float c0 = PH(ii, rown, k0 - 3), c1 = PH(ii, rown, k0 - 2), c2 = PH(ii, rown, k0 - 1), c3 = PH(ii, rown, k0);
  float c4 = PH(ii, rown, k0 + 1), c5 = PH(ii, rown, k0 + 2);
  float zlo = zf(k0 - 1, c0, c1, c2, c3, c4, c5);
  for (int k = k0; k <= k1; k++) {
    const int b = k & 1;
    c0 = c1;
    c1 = c2;
    c2 = c3;
    c3 = c4;
    c4 = c5;
    c5 = PH(ii, rown, k + 3);
    const float xo = xf(ii, ic, rown, jc, k);
    const float yo = yf(ii, ic, jj, jc, k);
    xs[b][ty][tx + 1] = xo;
    ys[b][ty + 1][tx] = yo;
    if (ty == 0)
      ys[b][0][tx] = yf(ii, ic, j0 - 1, jc - 1, k);
    else if (ty == 1 && tx < AT_BY)
      xs[b][tx][0] = xf(i0 - 1, i0 - 1, tx + 3, jx, k);
    const float zo = zf(k, c0, c1, c2, c3, c4, c5);
    __syncthreads();
    if (act) {
      const float xl = xs[b][ty][tx], yl = ys[b][ty][tx];
      const float fxp = u[TPLS_IDX(g, i, jm, k - 1)] * xo;
      const float fxm = u[TPLS_IDX(g, i - 1, jm, k - 1)] * xl;
      const float fyp = v[TPLS_IDX(g, i, j, k - 1)] * yo;
      const float fym = v[TPLS_IDX(g, i, jm, k - 1)] * yl;
      const float fzp = w[TPLS_IDX(g, i, jm, k)] * zo;
      const float fzm = w[TPLS_IDX(g, i, jm, k - 1)] * zlo;
      conv[TPLS_IDX(g, i, j, k)] = (double)((fxp - fxm) * rdx + (fyp - fym) * rdy + (fzp - fzm) * rdz);
    }
    zlo = zo;
  }
}

// Tensor map of the FP32 phi copy for k_advect_tma: 3-D (x row elements,
// y rows 0..ny+1, z planes 0..nz+1) over the whole pitched allocation.
cudaError_t advect_tma_map(const Geo &g, const float *phi32, void *map128) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess) return e;
    if (q != cudaDriverEntryPointSuccess || !fn) return cudaErrorNotSupported;
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  const float *base = phi32 - XOFF;  // the allocation: row starts on 16-byte boundaries
  const cuuint64_t dims[3] = {(cuuint64_t)g.sy, (cuuint64_t)(g.ny + 2), (cuuint64_t)(g.nz + 2)};
  const cuuint64_t strides[2] = {(cuuint64_t)g.sy * 4, (cuuint64_t)g.sz * 4};
  const cuuint32_t box[3] = {AT_W, 1, AT_NZ}, es[3] = {1, 1, 1};
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (strides[0] & 15) || (strides[1] & 15)) return cudaErrorInvalidValue;
  const CUresult r = encode(reinterpret_cast<CUtensorMap *>(map128), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                            const_cast<float *>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t launch_advect_tma(const Geo &g, const Phys &ph, const void *map128, const float *u2, const float *v2,
                              const float *w2, double *conv2_phi, double *kto, cudaStream_t st, int arm, int limit,
                              int one_block) {
  dim3 blk(AT_BX, AT_BY), grd((g.nx + AT_BX - 1) / AT_BX, (g.ny + AT_BY - 1) / AT_BY, (g.nz + AT_TZ - 1) / AT_TZ);
  if (one_block) grd = dim3(1, 1, 1);
  const CUtensorMap &m = *reinterpret_cast<const CUtensorMap *>(map128);
  k_advect_tma<<<grd, blk, 0, st>>>(m, g, (float)(1.0 / ph.dx), (float)(1.0 / ph.dy), (float)(1.0 / ph.dz), u2, v2,
                                    w2, conv2_phi, kto, arm, limit);
  return cudaGetLastError();
}

cudaError_t launch_advect(const Geo &g, const Phys &ph, const double *phi2,
                          const double *u2, const double *v2,
                          const double *w2, double *conv2_phi,
                          cudaStream_t st) {
  dim3 blk(ADV_BX, ADV_BY),
      grd((g.nx + ADV_BX - 1) / ADV_BX, (g.ny + ADV_BY - 1) / ADV_BY, (g.nz + ADV_KC - 1) / ADV_KC);
  k_advect<double><<<grd, blk, 0, st>>>(g, 1.0 / ph.dx, 1.0 / ph.dy, 1.0 / ph.dz, phi2, u2, v2, w2,
                                        conv2_phi);
  return cudaGetLastError();
}

cudaError_t launch_advect(const Geo &g, const Phys &ph, const float *phi2, const float *u2, const float *v2,
                          const float *w2, double *conv2_phi, cudaStream_t st) {
  dim3 blk(ADV_BX, ADV_BY),
      grd((g.nx + ADV_BX - 1) / ADV_BX, (g.ny + ADV_BY - 1) / ADV_BY, (g.nz + ADV_KC - 1) / ADV_KC);
  k_advect<float><<<grd, blk, 0, st>>>(g, (float)(1.0 / ph.dx), (float)(1.0 / ph.dy), (float)(1.0 / ph.dz), phi2,
                                       u2, v2, w2, conv2_phi);
  return cudaGetLastError();
}

// elementwise FP64 -> FP32 copy over n elements (the FP32 shadows of the
// FP64 state used by the FP32-mixed form)
__global__ void k_to_float(const double *__restrict__ a, float *__restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = round_bits(a[i]);  // integer split: no FP64-pipe conversion
}
cudaError_t launch_to_float(const double *a, float *b, size_t n, cudaStream_t st) {
  k_to_float<<<1216, 256, 0, st>>>(a, b, n);
  return cudaGetLastError();
}

// exchange2d on one GPU: rows 0 <- ny, ny+1 <- 1 over x = 0..nx+1.
template <typename T>
__global__ void k_exchange(Geo g, T *a, int nzp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (i > g.nx + 1 || k >= nzp) return;
  a[TPLS_IDX(g, i, 0, k)] = a[TPLS_IDX(g, i, g.ny, k)];
  a[TPLS_IDX(g, i, g.ny + 1, k)] = a[TPLS_IDX(g, i, 1, k)];
}

cudaError_t launch_exchange(const Geo &g, double *a, int nzp, cudaStream_t st) {
  dim3 blk(128), grd((g.nx + 2 + 127) / 128, nzp);
  k_exchange<double><<<grd, blk, 0, st>>>(g, a, nzp);
  return cudaGetLastError();
}
cudaError_t launch_exchange(const Geo &g, float *a, int nzp, cudaStream_t st) {
  dim3 blk(128), grd((g.nx + 2 + 127) / 128, nzp);
  k_exchange<float><<<grd, blk, 0, st>>>(g, a, nzp);
  return cudaGetLastError();
}

// Deterministic final reduction of per-block partials (one block).
__global__ void k_finish_sum(const double *part, int nparts, double *out, int nout) {
  __shared__ double s[256];
  for (int o = 0; o < nout; o++) {
    double acc = 0.0;
    for (int p = threadIdx.x; p < nparts; p += blockDim.x) acc += part[(size_t)o * nparts + p];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[o] = s[0];
    __syncthreads();
  }
}

// Sums of contiguous chunks of the partials, one block per chunk, each in a
// fixed order (the first stage of finish_sum for long partial arrays).
__global__ void k_chunk_sum(const double *__restrict__ part, int nparts, int chunk, double *__restrict__ out) {
  __shared__ double s[256];
  const int lo = blockIdx.x * chunk, hi = min(nparts, lo + chunk);
  double acc = 0.0;
  for (int p = lo + (int)threadIdx.x; p < hi; p += blockDim.x) acc += part[p];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = s[0];
}

static int chunk_blocks(int nparts) { return min(FS_TAIL, (nparts + 2047) / 2048); }

int finish_sum_kernels(int nparts, int nout) { return (nout == 1 && nparts > FS_ONE_BLOCK) ? 2 : 1; }

cudaError_t finish_sum(double *part, int nparts, double *out, int nout, cudaStream_t st) {
  if (finish_sum_kernels(nparts, nout) == 2) {
    const int nb = chunk_blocks(nparts), chunk = (nparts + nb - 1) / nb;
    k_chunk_sum<<<nb, 256, 0, st>>>(part, nparts, chunk, part + nparts);
    k_finish_sum<<<1, 256, 0, st>>>(part + nparts, nb, out, 1);
  } else {
    k_finish_sum<<<1, 256, 0, st>>>(part, nparts, out, nout);
  }
  return cudaGetLastError();
}

}  // namespace tpls
