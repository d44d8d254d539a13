// k_advect.cu -- level-set advection: WENO5 face values and the
// conservative flux divergence (advect_phi.f90:19-119, weno.f90:18-215).
//
// One thread per (i,j) column of p-cells, marching a chunk of 16 z levels
// (one z-face below the chunk is computed at its start).  Each face
// value is computed once: the x-face below a thread comes from its lower
// lane by warp shuffle (lane 0 computes it), the y-face below from the row
// below through shared memory (row 0 of the block computes it), and the
// z-face below is the previous level's z-face held in a register.
// The periodic-y halo of the reference's 3-ghost phi_augaug copy becomes a
// wrapped row index; no augmented array is built.
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

// dfx at u-index (iu, jp-1, kp-1): phi along x at p-row jp, level kp.
// WENO for 3 <= iu <= nx-2, first-order upwind otherwise (weno.f90:45-100).
template <typename T>
__device__ __forceinline__ T xface(const Geo &g, const T *__restrict__ phi,
                                        const T *__restrict__ u, int iu, int jp,
                                        int kp) {
  const int ju = (jp - 1 == 0) ? g.ny : jp - 1;
  const T vel = u[TPLS_IDX(g, iu, ju, kp - 1)];
  const T *row = phi + TPLS_IDX(g, 0, jp, kp);
  if (iu >= 3 && iu <= g.nx - 2) {
    if (vel >= (T)0) return weno5(row[iu - 2], row[iu - 1], row[iu], row[iu + 1], row[iu + 2]);
    return weno5(row[iu + 3], row[iu + 2], row[iu + 1], row[iu], row[iu - 1]);
  }
  return (vel >= (T)0) ? row[iu] : row[iu + 1];
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
  if (vel >= (T)0) return weno5(PY(jv - 2), PY(jv - 1), PY(jv), PY(jv + 1), PY(jv + 2));
  return weno5(PY(jv + 3), PY(jv + 2), PY(jv + 1), PY(jv), PY(jv - 1));
#undef PY
}

// dfz at w-index (ip, jp-1, kw): phi along z at x=ip, row jp.  WENO for
// 3 <= kw <= nz-2, arithmetic mean otherwise (weno.f90:136-166).
template <typename T>
__device__ __forceinline__ T zface(const Geo &g, const T *__restrict__ phi,
                                        const T *__restrict__ w, int ip, int jp,
                                        int kw) {
  const int ju = (jp - 1 == 0) ? g.ny : jp - 1;
  const T *col = phi + TPLS_IDX(g, ip, jp, 0);
  const int sz = g.sz;
  if (kw >= 3 && kw <= g.nz - 2) {
    const T vel = w[TPLS_IDX(g, ip, ju, kw)];
    if (vel >= (T)0)
      return weno5(col[sz * (kw - 2)], col[sz * (kw - 1)], col[sz * kw], col[sz * (kw + 1)],
                   col[sz * (kw + 2)]);
    return weno5(col[sz * (kw + 3)], col[sz * (kw + 2)], col[sz * (kw + 1)], col[sz * kw],
                 col[sz * (kw - 1)]);
  }
  return (col[sz * kw] + col[sz * (kw + 1)]) / (T)2;
}

constexpr int ADV_BX = 32, ADV_BY = 8;
constexpr int ADV_KC = 16;  // z levels per thread (column chunk)

template <typename T>
__global__ void __launch_bounds__(ADV_BX *ADV_BY)
    k_advect(Geo g, T rdx, T rdy, T rdz, const T *__restrict__ phi, const T *__restrict__ u,
             const T *__restrict__ v, const T *__restrict__ w, double *__restrict__ conv) {
  __shared__ T yf_s[ADV_BY][ADV_BX];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i = blockIdx.x * ADV_BX + tx + 1;
  const int j = blockIdx.y * ADV_BY + ty + 1;
  const int k0 = blockIdx.z * ADV_KC + 1, k1 = min(k0 + ADV_KC - 1, g.nz);
  const bool act = (i <= g.nx) && (j <= g.ny);
  const int ic = act ? i : 1, jc = act ? j : 1;  // clamped for inactive lanes
  const int jm = (jc == 1) ? g.ny : jc - 1;      // u/v/w row index j-1 (wrapped)
  T zlo = zface(g, phi, w, ic, jc, k0 - 1);
  for (int k = k0; k <= k1; k++) {
    const T xo = xface(g, phi, u, ic, jc, k);
    T xl = __shfl_up_sync(0xffffffffu, xo, 1);
    if (tx == 0) xl = xface(g, phi, u, ic - 1, jc, k);
    const T yo = yface(g, phi, v, ic, jc, k);
    yf_s[ty][tx] = yo;
    __syncthreads();
    const T yl = (ty > 0) ? yf_s[ty - 1][tx] : yface(g, phi, v, ic, jc - 1, k);
    const T zo = zface(g, phi, w, ic, jc, k);
    if (act) {
      const T fxp = u[TPLS_IDX(g, i, jm, k - 1)] * xo;
      const T fxm = u[TPLS_IDX(g, i - 1, jm, k - 1)] * xl;
      const T fyp = v[TPLS_IDX(g, i, j, k - 1)] * yo;
      const T fym = v[TPLS_IDX(g, i, jm, k - 1)] * yl;
      const T fzp = w[TPLS_IDX(g, i, jm, k)] * zo;
      const T fzm = w[TPLS_IDX(g, i, jm, k - 1)] * zlo;
      conv[TPLS_IDX(g, i, j, k)] = (double)((fxp - fxm) * rdx + (fyp - fym) * rdy + (fzp - fzm) * rdz);
    }
    zlo = zo;
    __syncthreads();
  }
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
