// k_sweep32.cu -- FP32 defect-form Jacobi sweep and 3-D checkerboard
// half-sweep (even iteration_time) of the FP32-mixed form
// (jacobi_iteration_allflux.f90:21-282, sor_iteration_allflux.f90:19-146,
// boundary rows of main_ns_hybrid.F90:756-887).
//
// A thread owns four consecutive x points of one (j, k) row, i = 4q+1 ..
// 4q+4.  Every row it needs is one aligned 16-byte load (rows are PX floats
// with x = 1 on a 16-byte boundary); the x-1 / x+4 neighbours come from the
// adjacent lanes by warp shuffles (the first lane, and the last active one,
// load theirs).  A thread issues all of its loads before it waits for any:
// the iterate's row and its four neighbour rows, the five or six viscosity
// rows of the face averages and b (one aligned 8-byte load per x parity).
//
// Arithmetic per point: the reference's update
//   x = (1/diag) (a_x (mu+ x+ + mu- x-) + a_y (...) + a_z (...) + rhs)
// with the face viscosities of momentum_allflux.f90 (a single cell value on
// the component's own axis, a four-cell average on the other two), written
// as x = r (cx tx + cy ty + cz tz) + b, r = 1/diag, t = mu+ x+ + mu- x-, the
// 1/4 of the averages folded into the per-axis constants cx, cy, cz and the
// four-cell sums built from pair sums shared by neighbouring points; b is
// stored already divided by diag.  The no-slip ghost value -2 u(0) + u(1)/3
// of u and v (momentum_allflux.f90:79-89) enters as the missing z
// neighbour.  The boundary rows (inlet and outlet copies, the u pressure
// outlet and fictitious point) add a per-row offset that is constant for the
// whole momentum solve, computed once per component and step
// (launch_bc32_prep).
#include "tpls_sweep.cuh"

namespace tpls {
namespace {

constexpr unsigned FULL = 0xffffffffu;
enum { M_JAC = 0, M_EVEN = 1 };

// Four x points of a row and their x-1 (l) and x+4 (r) neighbours.
struct Row {
  float4 v;
  float l, r;
};

__device__ __forceinline__ float el(const Row &w, int e) {
  return e == 0 ? w.v.x : (e == 1 ? w.v.y : (e == 2 ? w.v.z : w.v.w));
}
// element e = -1 .. 4 (the x-1 and x+4 neighbours at the ends)
__device__ __forceinline__ float ex(const Row &w, int e) { return e < 0 ? w.l : (e > 3 ? w.r : el(w, e)); }

// Row segment at p (i = 4q+1 of the row), in two steps so that a thread
// issues every load before it waits for any: issue() loads the 16 bytes and,
// for the lanes that own them, the x-1 / x+4 neighbours (lane 0 its left one;
// the last lane, or the last active group, its right one); halo() then
// takes the other lanes' neighbours from the adjacent lanes.  halo() is
// called by every lane of the warp (the shuffles need all of them);
// inactive lanes load nothing.
template <bool L, bool R, bool NC>
__device__ __forceinline__ void issue(Row &w, const float *p, bool act, bool own_l, bool own_r) {
  w.v = make_float4(0.f, 0.f, 0.f, 0.f);
  w.l = w.r = 0.f;
  if (act) {
    const float4 *p4 = reinterpret_cast<const float4 *>(p);
    w.v = NC ? __ldg(p4) : *p4;
    if (L && own_l) w.l = NC ? __ldg(p - 1) : p[-1];
    if (R && own_r) w.r = NC ? __ldg(p + 4) : p[4];
  }
}
template <bool L, bool R>
__device__ __forceinline__ void halo(Row &w, bool own_l, bool own_r) {
  if (L) {
    const float t = __shfl_up_sync(FULL, w.v.w, 1);
    if (!own_l) w.l = t;
  }
  if (R) {
    const float t = __shfl_down_sync(FULL, w.v.x, 1);
    if (!own_r) w.r = t;
  }
}

// Viscosity rows of one level, as the face averages of faces() in
// tpls_sweep.cuh read them (u: 5 rows, v and w: 6).
struct MuRows {
  Row r[6];
};

template <int CC>
__device__ __forceinline__ void issue_mu(MuRows &m, const Geo &g, const float *__restrict__ mu, int i0, int j, int k,
                                         bool act, bool ol, bool orr) {
  const int sy = g.sy, sz = g.szm;
  if (CC == 0) {
    const float *b = mu + TPLS_IDXM(g, i0, j + 1, k + 1);
    issue<false, true, true>(m.r[0], b, act, ol, orr);       // (j+1, k+1)
    issue<false, true, true>(m.r[1], b + sy, act, ol, orr);  // (j+2, k+1)
    issue<false, true, true>(m.r[2], b - sy, act, ol, orr);  // (j, k+1)
    issue<false, true, true>(m.r[3], b + sz, act, ol, orr);  // (j+1, k+2)
    issue<false, true, true>(m.r[4], b - sz, act, ol, orr);  // (j+1, k)
  } else if (CC == 1) {
    const float *b = mu + TPLS_IDXM(g, i0, j + 1, k + 1);
    issue<true, true, true>(m.r[0], b, act, ol, orr);              // (j+1, k+1)
    issue<true, true, true>(m.r[1], b - sy, act, ol, orr);         // (j, k+1)
    issue<false, false, true>(m.r[2], b + sz, act, ol, orr);       // (j+1, k+2)
    issue<false, false, true>(m.r[3], b + sz - sy, act, ol, orr);  // (j, k+2)
    issue<false, false, true>(m.r[4], b - sz, act, ol, orr);       // (j+1, k)
    issue<false, false, true>(m.r[5], b - sz - sy, act, ol, orr);  // (j, k)
  } else {
    const float *b = mu + TPLS_IDXM(g, i0, j + 1, k);
    issue<true, true, true>(m.r[0], b, act, ol, orr);              // (j+1, k)
    issue<true, true, true>(m.r[1], b + sz, act, ol, orr);         // (j+1, k+1)
    issue<false, false, true>(m.r[2], b + sy, act, ol, orr);       // (j+2, k)
    issue<false, false, true>(m.r[3], b + sy + sz, act, ol, orr);  // (j+2, k+1)
    issue<false, false, true>(m.r[4], b - sy, act, ol, orr);       // (j, k)
    issue<false, false, true>(m.r[5], b - sy + sz, act, ol, orr);  // (j, k+1)
  }
}
template <int CC>
__device__ __forceinline__ void halo_mu(MuRows &m, bool ol, bool orr) {
  if (CC == 0) {
#pragma unroll
    for (int r = 0; r < 5; r++) halo<false, true>(m.r[r], ol, orr);
  } else {
    halo<true, true>(m.r[0], ol, orr);
    halo<true, true>(m.r[1], ol, orr);
  }
}

// Face viscosities of the four points, unscaled: a single cell value on the
// component's own axis, the four-cell sum (the average times 4) on the
// other two.  p / m: + and - faces per axis.
struct Faces {
  float px[4], mx[4], py[4], my[4], pz[4], mz[4];
};

template <int CC>
__device__ __forceinline__ void faces4(const MuRows &m, Faces &f) {
  if (CC == 0) {
    // u: x faces mu(i), mu(i+1); pair sums along x of the other rows
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const float a = el(m.r[0], e), b = ex(m.r[0], e + 1), s0 = a + b;
      f.px[e] = b;
      f.mx[e] = a;
      f.py[e] = s0 + (el(m.r[1], e) + ex(m.r[1], e + 1));
      f.my[e] = s0 + (el(m.r[2], e) + ex(m.r[2], e + 1));
      f.pz[e] = s0 + (el(m.r[3], e) + ex(m.r[3], e + 1));
      f.mz[e] = s0 + (el(m.r[4], e) + ex(m.r[4], e + 1));
    }
  } else {
    // v: s0 = mu(j+1) + mu(j) at the same i; w: s0 = mu(k) + mu(k+1)
    float s0[6];
#pragma unroll
    for (int e = -1; e <= 4; e++) s0[e + 1] = ex(m.r[0], e) + ex(m.r[1], e);
#pragma unroll
    for (int e = 0; e < 4; e++) {
      f.px[e] = s0[e + 1] + s0[e + 2];
      f.mx[e] = s0[e + 1] + s0[e];
      if (CC == 1) {
        f.py[e] = el(m.r[0], e);
        f.my[e] = el(m.r[1], e);
        f.pz[e] = s0[e + 1] + (el(m.r[2], e) + el(m.r[3], e));
        f.mz[e] = s0[e + 1] + (el(m.r[4], e) + el(m.r[5], e));
      } else {
        f.py[e] = s0[e + 1] + (el(m.r[2], e) + el(m.r[3], e));
        f.my[e] = s0[e + 1] + (el(m.r[4], e) + el(m.r[5], e));
        f.pz[e] = el(m.r[1], e);
        f.mz[e] = el(m.r[0], e);
      }
    }
  }
}

// b of the four points (record-slot order: odd i in the first half of the
// row, even i in the second, so each parity's two values are one aligned
// 8-byte load: the b arrays carry no x offset); `par` < 0 loads all four,
// else the two points of that x parity.
__device__ __forceinline__ void load_b(const Geo &g, const float *__restrict__ b, int q, int i0, int iend, int j, int k,
                                       int par, bool act, float *out) {
  const float *rb = b + g.sy * j + g.sz * k + 2 * q;
  out[0] = out[1] = out[2] = out[3] = 0.f;
  if (act && par != 1) {  // i = 4q+1, 4q+3
    const float2 v = __ldg(reinterpret_cast<const float2 *>(rb));
    out[0] = v.x;
    out[2] = v.y;
  }
  if (act && par != 0 && i0 + 1 <= iend) {  // i = 4q+2, 4q+4
    const float2 v = __ldg(reinterpret_cast<const float2 *>(rb + (g.sy >> 1)));
    out[1] = v.x;
    out[3] = v.y;
  }
}

// One tile (block (bx, by, bz) of the single-instance grid) of the sweep;
// the single-instance kernel runs one per block, the multi-instance kernel
// of a batch any tile of any member.
template <int CC, int MODE, int BY>
__device__ __forceinline__ void sweep4_tile(const Geo &g, const Helm &h, const float *__restrict__ xo, float *x,
                                            const MuCoef &s, const double *__restrict__ X, int flg, int bc,
                                            int fuse, int bx, int by, int bz) {
  const int lane = threadIdx.x, q = bx * 32 + lane;
  const int j = by * BY + threadIdx.y + 1;
  if (j > g.ny) return;  // uniform per warp
  const int nx = g.nx, nz = g.nz, sy = g.sy, sz = g.sz;
  const int k = bz + ((CC == 2) ? 1 : 0);
  const int iend = (CC == 0) ? nx - 1 : nx;
  const int G = (iend + 3) >> 2;
  const bool act = q < G;
  const bool ol = (lane == 0), orr = (lane == 31) || (q + 1 >= G);
  const int i0 = 4 * q + 1;
  const bool full = act && (i0 + 3 <= iend);
  constexpr bool NC = (MODE == M_JAC);  // only the Jacobi source is read-only
  const float *xr = (MODE == M_JAC) ? xo : x;
  const float *pc = xr + (i0 + sy * j + sz * k);
  // every load of the thread first, then the shuffles
  const bool has_zp = (CC == 2) || (k + 1 <= nz - 1), has_zm = (CC == 2) || (k >= 1);
  Row cc, yp, ym, zp, zm;
  MuRows m;
  issue<true, true, NC>(cc, pc, act, ol, orr);
  issue<false, false, NC>(yp, pc + sy, act, ol, orr);
  issue<false, false, NC>(ym, pc - sy, act, ol, orr);
  issue<false, false, NC>(zp, pc + sz, act && has_zp, ol, orr);
  issue<false, false, NC>(zm, pc - sz, act && has_zm, ol, orr);
  issue_mu<CC>(m, g, s.mu, i0, j, k, act, ol, orr);
  const int par = (MODE == M_JAC) ? -1 : ((k + j + flg) & 1);
  float bv[4];
  load_b(g, s.b, q, i0, iend, j, k, par, act, bv);
  halo<true, true>(cc, ol, orr);
  halo_mu<CC>(m, ol, orr);
  Faces f;
  faces4<CC>(m, f);
  // per-axis scale: dt/(2 d^2), and a quarter of it for the averaged faces
  const float cx = (CC == 0) ? s.ax2 : 0.25f * s.ax2;
  const float cy = (CC == 1) ? s.ay2 : 0.25f * s.ay2;
  const float cz = (CC == 2) ? s.az2 : 0.25f * s.az2;
  float out[4] = {cc.v.x, cc.v.y, cc.v.z, cc.v.w};
#pragma unroll
  for (int e = 0; e < 4; e++) {
    const bool upd = act && (i0 + e <= iend) && (MODE == M_JAC || (e & 1) == par);
    if (upd) {
      const float xc = el(cc, e);
      float zpv = el(zp, e), zmv = el(zm, e);
      if (CC != 2) {  // no-slip ghost value -2 x(0) + x(1)/3 below k = 0 and above k = nz-1
        if (k == 0) zmv = fmaf(zpv, 1.0f / 3.0f, -2.0f * xc);
        if (k == nz - 1) zpv = fmaf(zmv, 1.0f / 3.0f, -2.0f * xc);
      }
      float d = fmaf(cx, f.px[e] + f.mx[e], 1.0f);
      d = fmaf(cy, f.py[e] + f.my[e], d);
      d = fmaf(cz, f.pz[e] + f.mz[e], d);
      const float r = __fdividef(1.0f, d);  // d >= 1: the fast reciprocal is within 2 ulp
      const float tx = fmaf(f.px[e], ex(cc, e + 1), f.mx[e] * ex(cc, e - 1));
      const float ty = fmaf(f.py[e], el(yp, e), f.my[e] * el(ym, e));
      const float tz = fmaf(f.pz[e], zpv, f.mz[e] * zmv);
      const float t = fmaf(cx, tx, fmaf(cy, ty, cz * tz));
      const float v = fmaf(r, t, bv[e]);
      out[e] = (MODE == M_JAC) ? v : xc + 1.2f * (v - xc);
    }
  }
  // store: whole groups as one 16-byte store (in the half-sweep the other
  // colour's values are rewritten unchanged: nothing else writes them in
  // this launch), ragged ends point by point
  float *po = x + (i0 + sy * j + sz * k);
  if (full) {
    const float4 o = make_float4(out[0], out[1], out[2], out[3]);
    *reinterpret_cast<float4 *>(po) = o;
    if (fuse && j == g.ny) *reinterpret_cast<float4 *>(po - sy * g.ny) = o;
    if (fuse && j == 1) *reinterpret_cast<float4 *>(po + sy * g.ny) = o;
  } else if (act) {
#pragma unroll
    for (int e = 0; e < 4; e++)
      if (i0 + e <= iend && (MODE == M_JAC || (e & 1) == par)) put(g, x, i0 + e, j, k, out[e], fuse);
  }
  if (!act || (MODE != M_JAC && !bc)) return;
  // boundary rows (the post-sweep ones of main_ns_hybrid.F90:784-799,
  // 826-836, 860-879): x(0) = x(1) + off.x; u: x(nx) = x(nx-1) + off.y and
  // x(nx+1) = off.z; v, w: x(nx+1) = x(nx) + off.y.  x(1) and x(iend) are
  // this thread's out values (relaxed now, or the other colour's final ones)
  const bool first = (q == 0), last = (i0 + 3 >= iend);
  if (first || last) {
    const float4 off = s.bco[j + (g.ny + 2) * k];
    if (first) put(g, x, 0, j, k, out[0] + off.x, fuse);
    if (last) {
      const int e = iend - i0;
      const float ve = e == 0 ? out[0] : (e == 1 ? out[1] : (e == 2 ? out[2] : out[3]));
      if (CC == 0) {
        put(g, x, nx, j, k, ve + off.y, fuse);
        put(g, x, nx + 1, j, k, off.z, fuse);
      } else {
        put(g, x, nx + 1, j, k, ve + off.y, fuse);
      }
    }
  }
  // w: the wall rows k = 0 and nz (x = 0, so d = -X there), rewritten by
  // the Jacobi sweep next to them for the ping-pong buffer
  if (CC == 2 && MODE == M_JAC && (k == 1 || k == nz - 1)) {
    const int kw = (k == 1) ? 0 : nz;
#pragma unroll
    for (int e = 0; e < 4; e++)
      if (i0 + e <= iend) bc_zero(g, x, X, i0 + e, j, kw, fuse);
    if (first) bc_zero(g, x, X, 0, j, kw, fuse);
    if (last) bc_zero(g, x, X, nx + 1, j, kw, fuse);
  }
}

template <int CC, int MODE, int BY>
__global__ void __launch_bounds__(32 * BY)
    k_sweep4(Geo g, Helm h, const float *__restrict__ xo, float *x, MuCoef s, const double *__restrict__ X,
             int flg, int bc, int fuse) {
  sweep4_tile<CC, MODE, BY>(g, h, xo, x, s, X, flg, bc, fuse, blockIdx.x, blockIdx.y, blockIdx.z);
}

// tiles of the single-instance grid of component CC (4 rows per block)
__host__ __device__ inline void sweep4_grid(int cc, const Geo &g, int *gx, int *gy, int *gz) {
  const int iend = (cc == 0) ? g.nx - 1 : g.nx;
  *gx = ((iend + 3) / 4 + 31) / 32;
  *gy = (g.ny + 3) / 4;
  *gz = (cc == 2) ? g.nz - 1 : g.nz;
}

// Multi-instance form: one persistent launch runs the sweep of component CC
// for every member of a batch.  The work is the list of all members' tiles
// (prefix[m] = first tile of member m); blocks take tiles in order by an
// atomic ticket, so uneven members share the GPU without one launch each.
// No block waits for another; the last block to leave resets the ticket
// for the next launch.
template <int CC, int MODE>
__global__ void __launch_bounds__(128)
    k_sweep4_multi(const SweepMember *__restrict__ mem, const int *__restrict__ prefix, int n, int src, int flg,
                   int bc, unsigned *ctr) {
  __shared__ int s_t;
  const int total = prefix[n];
  for (;;) {
    if (threadIdx.x == 0 && threadIdx.y == 0) s_t = (int)atomicAdd(&ctr[0], 1u);
    __syncthreads();
    const int t = s_t;
    __syncthreads();
    if (t >= total) break;
    int m = 0;
    while (prefix[m + 1] <= t) m++;
    const SweepMember &M = mem[m];
    int gx, gy, gz;
    sweep4_grid(CC, M.g, &gx, &gy, &gz);
    const int lt = t - prefix[m];
    const int bx = lt % gx, by = (lt / gx) % gy, bz = lt / (gx * gy);
    const float *xo = M.x[CC][src];
    float *xd = (MODE == M_JAC) ? M.x[CC][1 - src] : M.x[CC][src];
    sweep4_tile<CC, MODE, 4>(M.g, M.h, xo, xd, M.s[CC], M.X[CC], flg, bc, M.fuse, bx, by, bz);
  }
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    __threadfence();
    if (atomicAdd(&ctr[1], 1u) == gridDim.x - 1) {
      ctr[0] = 0u;
      ctr[1] = 0u;
    }
  }
}

template <int CC, int MODE, int BY>
cudaError_t launch4(const Geo &g, const Helm &h, const float *xo, float *x, const MuCoef &s, const double *X,
                    int flg, int bc, int fuse, cudaStream_t st) {
  const int iend = (CC == 0) ? g.nx - 1 : g.nx;
  const int G = (iend + 3) / 4;
  const int nk = (CC == 2) ? g.nz - 1 : g.nz;
  dim3 grd((G + 31) / 32, (g.ny + BY - 1) / BY, nk);
  k_sweep4<CC, MODE, BY><<<grd, dim3(32, BY), 0, st>>>(g, h, xo, x, s, X, flg, bc, fuse);
  return cudaGetLastError();
}

// tile: rows per block (0: 4, 1: 8, 2: 2, 3: 1)
template <int CC, int MODE>
cudaError_t launch4_t(int tile, const Geo &g, const Helm &h, const float *xo, float *x, const MuCoef &s,
                      const double *X, int flg, int bc, int fuse, cudaStream_t st) {
  switch (tile) {
    case 1: return launch4<CC, MODE, 8>(g, h, xo, x, s, X, flg, bc, fuse, st);
    case 2: return launch4<CC, MODE, 2>(g, h, xo, x, s, X, flg, bc, fuse, st);
    case 3: return launch4<CC, MODE, 1>(g, h, xo, x, s, X, flg, bc, fuse, st);
    default: return launch4<CC, MODE, 4>(g, h, xo, x, s, X, flg, bc, fuse, st);
  }
}

template <int MODE>
cudaError_t by_comp(int comp, int tile, const Geo &g, const Helm &h, const float *xo, float *x, const MuCoef &s,
                    const double *X, int flg, int bc, int fuse, cudaStream_t st) {
  if (comp == 0) return launch4_t<0, MODE>(tile, g, h, xo, x, s, X, flg, bc, fuse, st);
  if (comp == 1) return launch4_t<1, MODE>(tile, g, h, xo, x, s, X, flg, bc, fuse, st);
  return launch4_t<2, MODE>(tile, g, h, xo, x, s, X, flg, bc, fuse, st);
}

// one thread per (j, k) row of the component
__global__ void k_bc32_prep(int comp, Geo g, Helm h, const double *__restrict__ X, const double *__restrict__ P,
                            float4 *__restrict__ bco) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1, k = blockIdx.y;
  if (j > g.ny) return;
  const int nx = g.nx;
  auto xs = [&](int i) { return split_bits(X[TPLS_IDX(g, i, j, k)]); };
  float4 o = make_float4(dif(xs(1), xs(0)), 0.f, 0.f, 0.f);
  if (comp == 0) {
    const F2 pp = split_bits(P[TPLS_IDX(g, nx + 1, j, k + 1)]), p0 = split_bits(P[TPLS_IDX(g, nx, j, k + 1)]);
    const F2 pm = split_bits(P[TPLS_IDX(g, nx - 1, j, k + 1)]);
    o.y = dif(xs(nx - 1), xs(nx)) + h.dtdxf * (dif(pp, p0) - dif(p0, pm));
    o.z = -round_bits(X[TPLS_IDX(g, nx + 1, j, k)]);
  } else {
    o.y = dif(xs(nx), xs(nx + 1));
  }
  bco[j + (g.ny + 2) * k] = o;
}

}  // namespace

cudaError_t launch_sweep4(int mode, int comp, const Geo &g, const Helm &h, const float *xo, float *x,
                          const MuCoef &s, const double *, const double *X, int flg, int bc, int fuse, int tile,
                          cudaStream_t st) {
  if (mode == M_JAC) return by_comp<M_JAC>(comp, tile, g, h, xo, x, s, X, flg, bc, fuse, st);
  return by_comp<M_EVEN>(comp, tile, g, h, xo, x, s, X, flg, bc, fuse, st);
}

int sweep4_tiles(int comp, const Geo &g) {
  int gx, gy, gz;
  sweep4_grid(comp, g, &gx, &gy, &gz);
  return gx * gy * gz;
}

cudaError_t launch_sweep4_multi(int mode, int comp, const SweepMember *mem, const int *prefix, int n,
                                int total_tiles, int src, int flg, int bc, unsigned *ctr, int nblocks,
                                cudaStream_t st) {
  const int nb = total_tiles < nblocks ? total_tiles : nblocks;
  if (nb <= 0) return cudaSuccess;
  const dim3 blk(32, 4);
#define TPLS_M4(C, M) k_sweep4_multi<C, M><<<nb, blk, 0, st>>>(mem, prefix, n, src, flg, bc, ctr)
  if (mode == M_JAC) {
    if (comp == 0) TPLS_M4(0, M_JAC);
    else if (comp == 1) TPLS_M4(1, M_JAC);
    else TPLS_M4(2, M_JAC);
  } else {
    if (comp == 0) TPLS_M4(0, M_EVEN);
    else if (comp == 1) TPLS_M4(1, M_EVEN);
    else TPLS_M4(2, M_EVEN);
  }
#undef TPLS_M4
  return cudaGetLastError();
}

cudaError_t launch_bc32_prep(int comp, const Geo &g, const Phys &ph, const double *X, const double *P,
                             float4 *bco, cudaStream_t st) {
  const int nk = (comp == 2) ? g.nz + 1 : g.nz;
  dim3 grd((g.ny + 127) / 128, nk);
  k_bc32_prep<<<grd, 128, 0, st>>>(comp, g, helm_of(ph), X, P, bco);
  return cudaGetLastError();
}

}  // namespace tpls
