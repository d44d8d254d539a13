// k_dim.cu -- the diffuse-interface (Cahn-Hilliard) update of
// cahn_hilliard_solver.f90:41-382 (`dim`), the alternative to the level-set
// update + redistancing selected by idm = dim (main_ns_hybrid.F90:595-612).
//
// One thread per p-grid position.  The routine fills ghost values by copies
// (z planes from k = 1 / nz, periodic y rows, x columns from i = 1 / nx) and
// an inlet profile; a ghost thread here recomputes the value at its source
// position with the same arithmetic instead of waiting for the owner, so
// each phase is one launch.  Positions the routine leaves untouched keep
// their previous value, as the reference's arrays do.  The iterate is
// double-buffered (the update of a point reads only that point, but ghost
// threads read their source points).  FP64 throughout: this is the FP64
// form's path.
#include "tpls_kernels.h"

namespace tpls {

constexpr int DM_BX = 32, DM_BY = 4;

// Where a position's value comes from in the routine's copy rules:
// kind 0 = computed at (si, sj, sk), 1 = not set by the rule (keeps its
// value / undefined).  Interior, the x ghost columns (j 1..ny, k 1..nz), the
// y ghost rows (i 1..nx, k 1..nz) and the z ghost planes (i 1..nx, j 1..ny)
// map to an interior source; corners and edges are not set.
struct Src {
  int set, i, j, k;
};
__device__ __forceinline__ Src first_order_src(const Geo &g, int i, int j, int k) {
  const bool ix = i >= 1 && i <= g.nx, jy = j >= 1 && j <= g.ny, kz = k >= 1 && k <= g.nz;
  Src s = {0, i, j, k};
  if (ix && jy && kz) s.set = 1;
  else if (jy && kz) { s.set = 1; s.i = (i == 0) ? 1 : g.nx; }
  else if (ix && kz) { s.set = 1; s.j = (j == 0) ? g.ny : 1; }
  else if (ix && jy) { s.set = 1; s.k = (k == 0) ? 1 : g.nz; }
  return s;
}

// 7-point Laplacian of a (plus a constant add, the driver's phi2 + 0.5 taken
// on the fly) at an interior point, divisions by dx^2 as multiplications by
// the host's 1/dx/dx
__device__ __forceinline__ double lap7(const Geo &g, const DimK &q, const double *__restrict__ a, double add,
                                       int c) {
  const double p = a[c] + add;
  return ((a[c + 1] + add) - 2.0 * p + (a[c - 1] + add)) * q.rdx2 +
         ((a[c + g.sy] + add) - 2.0 * p + (a[c - g.sy] + add)) * q.rdy2 +
         ((a[c + g.sz] + add) - 2.0 * p + (a[c - g.sz] + add)) * q.rdz2;
}

// dsqrt(c1*c1*(1-|c1|)*(1-|c1|))
__device__ __forceinline__ double mob(double c1) { return sqrt(c1 * c1 * (1.0 - fabs(c1)) * (1.0 - fabs(c1))); }

// :110-172 bulkE0 and d2phi of C = phi + add, with their ghost copies
__global__ void __launch_bounds__(DM_BX *DM_BY)
    k_dim_prep(Geo g, DimK q, const double *__restrict__ phi, double add, double *__restrict__ e0,
               double *__restrict__ l0) {
  const int i = blockIdx.x * DM_BX + threadIdx.x, j = blockIdx.y * DM_BY + threadIdx.y, k = blockIdx.z;
  if (i > g.nx + 1 || j > g.ny + 1) return;
  const Src s = first_order_src(g, i, j, k);
  if (!s.set) return;
  const int c = TPLS_IDX(g, i, j, k), cs = TPLS_IDX(g, s.i, s.j, s.k);
  const double p = phi[cs] + add;
  e0[c] = (1.0 - 3.0 * p + 2.0 * p * p) * p / 2.0;
  l0[c] = lap7(g, q, phi, add, cs);
}

// :174-233 source0 = 2 temp5 - ConvPrevPhi, ConvPrevPhi = temp5 (interior)
__global__ void __launch_bounds__(DM_BX *DM_BY)
    k_dim_source(Geo g, DimK q, const double *__restrict__ phi, double add, const double *__restrict__ e0,
                 const double *__restrict__ l0, const double *__restrict__ conv2, double *__restrict__ cprev,
                 double *__restrict__ src) {
  const int i = blockIdx.x * DM_BX + threadIdx.x + 1, j = blockIdx.y * DM_BY + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > g.nx || j > g.ny) return;
  const int c = TPLS_IDX(g, i, j, k), sy = g.sy, sz = g.sz;
  const double p = phi[c] + add;
  const double a1 = mob(((phi[c - 1] + add) + p) / 2.0), a2 = mob(((phi[c + 1] + add) + p) / 2.0);
  const double a3 = mob(((phi[c - sy] + add) + p) / 2.0), a4 = mob(((phi[c + sy] + add) + p) / 2.0);
  const double a5 = mob((k == 1) ? p : ((phi[c - sz] + add) + p) / 2.0);
  const double a6 = mob(((phi[c + sz] + add) + p) / 2.0);
  const double bc = e0[c], lc = l0[c];
  const double temp1 = (a2 * (e0[c + 1] - bc) - a1 * (bc - e0[c - 1])) * q.rdx2 +
                       (a4 * (e0[c + sy] - bc) - a3 * (bc - e0[c - sy])) * q.rdy2 +
                       (a6 * (e0[c + sz] - bc) - a5 * (bc - e0[c - sz])) * q.rdz2;
  const double temp2 = (l0[c + 1] - 2.0 * lc + l0[c - 1]) * q.rdx2 + (l0[c + sy] - 2.0 * lc + l0[c - sy]) * q.rdy2 +
                       (l0[c + sz] - 2.0 * lc + l0[c - sz]) * q.rdz2;
  const double temp3 = (a2 * (l0[c + 1] - lc) - a1 * (lc - l0[c - 1])) * q.rdx2 +
                       (a4 * (l0[c + sy] - lc) - a3 * (lc - l0[c - sy])) * q.rdy2 +
                       (a6 * (l0[c + sz] - lc) - a5 * (lc - l0[c - sz])) * q.rdz2;
  const double temp4 = (temp1 - q.epn2 * temp3) * q.repn - q.c_nt2 * lc + q.c_en2 * temp2;
  const double temp5 = temp4 * q.rpe - conv2[c];
  src[c] = temp5 * 2.0 - cprev[c];
  cprev[c] = temp5;
}

// :243-283 d2phi = grad^2(phiNew) with its ghost copies
__global__ void __launch_bounds__(DM_BX *DM_BY)
    k_dim_lap(Geo g, DimK q, const double *__restrict__ pin, double *__restrict__ l) {
  const int i = blockIdx.x * DM_BX + threadIdx.x, j = blockIdx.y * DM_BY + threadIdx.y, k = blockIdx.z;
  if (i > g.nx + 1 || j > g.ny + 1) return;
  const Src s = first_order_src(g, i, j, k);
  if (!s.set) return;
  l[TPLS_IDX(g, i, j, k)] = lap7(g, q, pin, 0.0, TPLS_IDX(g, s.i, s.j, s.k));
}

// the relaxed value at an interior point (:286-317): bulkE0 = grad^2(d2phi)
// there, the update and the clamp to [0, 1]
__device__ __forceinline__ double dim_upd(const Geo &g, const DimK &q, const double *__restrict__ phi,
                                          double add, const double *__restrict__ phio, double addo,
                                          const double *__restrict__ src, const double *__restrict__ pin,
                                          const double *__restrict__ l, int c) {
  const double b = lap7(g, q, l, 0.0, c);
  const double some = 2.0 * (phi[c] + add) - 0.5 * (phio[c] + addo) - 1.5 * pin[c] + q.dt * src[c] +
                      q.kc * (q.tao * l[c] - q.epn2 * b);
  double v = pin[c] + q.alfa1 * some * q.rdiag;
  if (v < 0.0) v = 0.0;
  if (v > 1.0) v = 1.0;
  return v;
}

// one SOR iteration's new iterate, every position (:286-360): interior
// updates, the z ghost copies, the periodic y rows (taken after the z copies
// and before this iteration's x columns), the inlet profile and the outlet
// copy; positions no rule sets keep the old value
__global__ void __launch_bounds__(DM_BX *DM_BY)
    k_dim_update(Geo g, DimK q, const double *__restrict__ phi, double add, const double *__restrict__ phio,
                 double addo, const double *__restrict__ src, const double *__restrict__ pin,
                 const double *__restrict__ l, double *__restrict__ pout) {
  const int i = blockIdx.x * DM_BX + threadIdx.x, j = blockIdx.y * DM_BY + threadIdx.y, k = blockIdx.z;
  if (i > g.nx + 1 || j > g.ny + 1) return;
  const bool ix = i >= 1 && i <= g.nx, jy = j >= 1 && j <= g.ny, kz = k >= 1 && k <= g.nz;
  const int c = TPLS_IDX(g, i, j, k);
  const int kk = kz ? k : ((k == 0) ? 1 : g.nz);  // z ghost planes copy k = 1 / nz
  double v;
  if (jy) {
    if (ix) v = dim_upd(g, q, phi, add, phio, addo, src, pin, l, TPLS_IDX(g, i, j, kk));
    else if (!kz) v = pin[c];  // x ghost columns outside k 1..nz: untouched
    else if (i == 0) v = 0.5 + 0.5 * tanh((k * q.dz - 0.5 * q.dz - q.height) / q.zden);
    else v = dim_upd(g, q, phi, add, phio, addo, src, pin, l, TPLS_IDX(g, g.nx, j, k));
  } else {  // periodic y rows, taken before this iteration's x columns
    const int js = (j == 0) ? g.ny : 1;
    if (ix) v = dim_upd(g, q, phi, add, phio, addo, src, pin, l, TPLS_IDX(g, i, js, kk));
    else v = pin[TPLS_IDX(g, i, js, k)];
  }
  pout[c] = v;
}

// :611 phi3 = phiNew - 0.5 (every position), written to the state phi2 and
// to the next step's starting guess
__global__ void __launch_bounds__(DM_BX *DM_BY)
    k_dim_finish(Geo g, const double *__restrict__ pfin, double *__restrict__ phi2, double *__restrict__ phi3) {
  const int i = blockIdx.x * DM_BX + threadIdx.x, j = blockIdx.y * DM_BY + threadIdx.y, k = blockIdx.z;
  if (i > g.nx + 1 || j > g.ny + 1) return;
  const int c = TPLS_IDX(g, i, j, k);
  const double v = pfin[c] - 0.5;
  phi2[c] = v;
  phi3[c] = v;
}

DimK dim_constants(const Phys &ph, double epn, double pe) {
  const double nmda = 0.25, tao = 0.25, alfa1 = 1.1;
  DimK q;
  q.rdx2 = 1.0 / ph.dx / ph.dx;
  q.rdy2 = 1.0 / ph.dy / ph.dy;
  q.rdz2 = 1.0 / ph.dz / ph.dz;
  q.epn2 = epn * epn;
  q.repn = 1.0 / epn;
  q.rpe = 1.0 / pe;
  q.c_nt2 = nmda * tao / 2.0;
  q.c_en2 = q.epn2 * nmda / 2.0;
  q.dt = ph.dt;
  q.kc = ph.dt * nmda / 2.0 / pe;
  q.tao = tao;
  q.alfa1 = alfa1;
  // :236-238 (dx**2.d0 folds to dx*dx; dx**4.d0 is a pow)
  const double a1 = 1.0 / (ph.dx * ph.dx) + 1.0 / (ph.dy * ph.dy) + 1.0 / (ph.dz * ph.dz);
  const double a2 = 2.0 / pow(ph.dx, 4.0) + 2.0 / pow(ph.dy, 4.0) + 2.0 / pow(ph.dz, 4.0);
  const double diagonal = 1.5 + nmda / 2.0 / pe * ph.dt * (2.0 * tao * a1 + q.epn2 * (4.0 * a1 * a1 + a2));
  q.rdiag = 1.0 / diagonal;
  q.dz = ph.dz;
  q.height = ph.height;
  q.zden = 2.0 * sqrt(2.0) * epn;
  return q;
}

static dim3 full_p_grid(const Geo &g) {
  return dim3((g.nx + 2 + DM_BX - 1) / DM_BX, (g.ny + 2 + DM_BY - 1) / DM_BY, g.nz + 2);
}

cudaError_t launch_dim_prep(const Geo &g, const DimK &q, const double *phi, double add, double *e0, double *l0,
                            cudaStream_t st) {
  k_dim_prep<<<full_p_grid(g), dim3(DM_BX, DM_BY), 0, st>>>(g, q, phi, add, e0, l0);
  return cudaGetLastError();
}
cudaError_t launch_dim_source(const Geo &g, const DimK &q, const double *phi, double add, const double *e0,
                              const double *l0, const double *conv2, double *cprev, double *src, cudaStream_t st) {
  dim3 grd((g.nx + DM_BX - 1) / DM_BX, (g.ny + DM_BY - 1) / DM_BY, g.nz);
  k_dim_source<<<grd, dim3(DM_BX, DM_BY), 0, st>>>(g, q, phi, add, e0, l0, conv2, cprev, src);
  return cudaGetLastError();
}
cudaError_t launch_dim_lap(const Geo &g, const DimK &q, const double *pin, double *l, cudaStream_t st) {
  k_dim_lap<<<full_p_grid(g), dim3(DM_BX, DM_BY), 0, st>>>(g, q, pin, l);
  return cudaGetLastError();
}
cudaError_t launch_dim_update(const Geo &g, const DimK &q, const double *phi, double add, const double *phio,
                              double addo, const double *src, const double *pin, const double *l, double *pout,
                              cudaStream_t st) {
  k_dim_update<<<full_p_grid(g), dim3(DM_BX, DM_BY), 0, st>>>(g, q, phi, add, phio, addo, src, pin, l, pout);
  return cudaGetLastError();
}
cudaError_t launch_dim_finish(const Geo &g, const double *pfin, double *phi2, double *phi3, cudaStream_t st) {
  k_dim_finish<<<full_p_grid(g), dim3(DM_BX, DM_BY), 0, st>>>(g, pfin, phi2, phi3);
  return cudaGetLastError();
}

}  // namespace tpls
