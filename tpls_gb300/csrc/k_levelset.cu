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
#include "tpls_kernels.h"

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
__global__ void k_ls_status(Geo g, double h, const double *__restrict__ phi,
                            double *__restrict__ D, signed char *__restrict__ flags) {
  const int i = blockIdx.x * LS_BX + threadIdx.x, j = blockIdx.y * LS_BY + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.nx + 1 || j > g.ny + 1) return;
  const int c = TPLS_IDX(g, i, j, k);
  if (i < 1 || i > g.nx || j < 1 || j > g.ny || k < 1 || k > g.nz) {
    D[c] = 0.0;
    flags[c] = 0;
    return;
  }
  const double p = phi[c];
  const double pxp = phi[c + 1], pxm = phi[c - 1], pyp = phi[c + g.sy], pym = phi[c - g.sy];
  const double pzp = phi[c + g.sz], pzm = phi[c - g.sz];
  const int sgn = (p < 0.0) ? -1 : ((p > 0.0) ? 1 : 0);
  const double mn = fmin(fmin(fmin(p * pxp, p * pxm), fmin(p * pyp, p * pym)), fmin(p * pzp, p * pzm));
  const int st = (mn <= 0.0) ? 1 : 0;
  double d = 0.0;
  if (st) {
    const double gx = pxp - pxm, gy = pyp - pym, gz = pzp - pzm;
    const double b1 = sqrt(gx * gx + gy * gy + gz * gz) * 0.5;
    double mx = fmax(fmax(fabs(pxp - p), fabs(pxm - p)), fmax(fabs(pyp - p), fabs(pym - p)));
    mx = fmax(fmax(mx, fmax(fabs(pzp - p), fabs(pzm - p))), fmax(b1, h));
    d = h * p / mx;
  }
  D[c] = d;
  flags[c] = (signed char)(st | ((sgn + 1) << 1));
}

cudaError_t launch_ls_status(const Geo &g, const Phys &ph, const double *phi3,
                             double *D, signed char *flags, cudaStream_t st) {
  k_ls_status<<<full_grid(g, g.nz + 2), dim3(LS_BX, LS_BY), 0, st>>>(g, ph.dx, phi3, D, flags);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// levelset.f90:97-237 do_levelset_iteration: one Godunov pseudo-time step
// with dtau = 0.3h (h = dx), then the inlet value (with dz = h), the outlet
// copy, linear z extrapolation, periodic y.  err_part (optional) receives
// one partial of sum((pr - pr_new)^2) per block over i 1..nx, j 1..ny,
// k 0..nz+1.
__device__ __forceinline__ double rs_update(const Geo &g, double h, double ktau,
                                            const double *__restrict__ pr,
                                            const double *__restrict__ D,
                                            const signed char *__restrict__ flags, int i, int j,
                                            int k) {
  const int c = TPLS_IDX(g, i, j, k);
  const int f = flags[c];
  const double p = pr[c];
  const double sg = (double)(((f >> 1) & 3) - 1);
  double dc;
  if (f & 1) {
    dc = sg * fabs(p) - D[c];
  } else if (sg > 0.0) {
    // max(aP^2, bM^2) with aP = max(p - p[i-1], 0), bM = min(p[i+1] - p, 0)
    // equals max(p - min(p[i-1], p[i+1]), 0)^2 bit for bit (rounding of a
    // difference and of a square are monotone), likewise in y and z.
    const double ax = fmax(p - fmin(pr[c - 1], pr[c + 1]), 0.0);
    const double ay = fmax(p - fmin(pr[c - g.sy], pr[c + g.sy]), 0.0);
    const double az = fmax(p - fmin(pr[c - g.sz], pr[c + g.sz]), 0.0);
    dc = sg * (sqrt(ax * ax + ay * ay + az * az) - h);
  } else if (sg < 0.0) {
    // max(bP^2, aM^2) = max(max(p[i-1], p[i+1]) - p, 0)^2, likewise y, z
    const double ax = fmax(fmax(pr[c - 1], pr[c + 1]) - p, 0.0);
    const double ay = fmax(fmax(pr[c - g.sy], pr[c + g.sy]) - p, 0.0);
    const double az = fmax(fmax(pr[c - g.sz], pr[c + g.sz]) - p, 0.0);
    // levelset.f90:274-275 sums x, then z, then y
    dc = sg * (sqrt(ax * ax + az * az + ay * ay) - h);
  } else {
    dc = 0.0;
  }
  return p - ktau * dc;
}

__device__ __forceinline__ double rs_val(const Geo &g, const Phys &ph, double h, double ktau,
                                         const double *pr, const double *D,
                                         const signed char *flags, int i, int j, int k) {
  if (i == 0) return (k * h - 0.5 * h) - ph.height;
  return rs_update(g, h, ktau, pr, D, flags, (i == g.nx + 1) ? g.nx : i, j, k);
}

__global__ void __launch_bounds__(LS_BX *LS_BY)
    k_ls_iter(Geo g, Phys ph, double h, double ktau, const double *__restrict__ pr,
              const double *__restrict__ D, const signed char *__restrict__ flags,
              double *__restrict__ out, double *__restrict__ err_part) {
  const int i = blockIdx.x * LS_BX + threadIdx.x, j = blockIdx.y * LS_BY + threadIdx.y;
  const int k = blockIdx.z;
  double e = 0.0;
  if (i <= g.nx + 1 && j <= g.ny + 1) {
    const int jj = wrapy(j, g.ny);
    double v;
    if (k == 0)
      v = 2.0 * rs_val(g, ph, h, ktau, pr, D, flags, i, jj, 1) -
          rs_val(g, ph, h, ktau, pr, D, flags, i, jj, 2);
    else if (k == g.nz + 1)
      v = 2.0 * rs_val(g, ph, h, ktau, pr, D, flags, i, jj, g.nz) -
          rs_val(g, ph, h, ktau, pr, D, flags, i, jj, g.nz - 1);
    else
      v = rs_val(g, ph, h, ktau, pr, D, flags, i, jj, k);
    const int c = TPLS_IDX(g, i, j, k);
    if (err_part && i >= 1 && i <= g.nx && j >= 1 && j <= g.ny) {
      const double d = pr[c] - v;
      e = d * d;
    }
    out[c] = v;
  }
  if (err_part) {
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

int ls_iter_blocks(const Geo &g) {
  dim3 gr = full_grid(g, g.nz + 2);
  return (int)(gr.x * gr.y * gr.z);
}

cudaError_t launch_ls_iter(const Geo &g, const Phys &ph, const double *pr,
                           const double *D, const signed char *flags,
                           double *pr_new, double *err_part, cudaStream_t st) {
  const double h = ph.dx, dtau = 0.3 * h;
  k_ls_iter<<<full_grid(g, g.nz + 2), dim3(LS_BX, LS_BY), 0, st>>>(g, ph, h, dtau / h, pr, D, flags,
                                                                   pr_new, err_part);
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

__device__ __forceinline__ F3 csf_point(const Geo &g, const Phys &ph, double max_kappa,
                                        const double *__restrict__ fi, int i, int j, int k) {
  const int c = TPLS_IDX(g, i, j, k);
  const double p = fi[c];
  F3 r = {0.0, 0.0, 0.0};
  if (p < -ph.sw || p > ph.sw) return r;
  const int sy = g.sy, sz = g.sz;
  const double rdx = 1.0 / ph.dx, rdy = 1.0 / ph.dy, rdz = 1.0 / ph.dz;
  const double r2dx = 0.5 * rdx, r2dy = 0.5 * rdy, r2dz = 0.5 * rdz;
  const double d2x = (fi[c + 1] - 2.0 * p + fi[c - 1]) * (rdx * rdx);
  const double d2y = (fi[c + sy] - 2.0 * p + fi[c - sy]) * (rdy * rdy);
  const double d2z = (fi[c + sz] - 2.0 * p + fi[c - sz]) * (rdz * rdz);
  const double gx = (fi[c + 1] - fi[c - 1]) * r2dx;
  const double gy = (fi[c + sy] - fi[c - sy]) * r2dy;
  const double gz = (fi[c + sz] - fi[c - sz]) * r2dz;
  const double d2xz = ((fi[c + 1 + sz] - fi[c - 1 + sz]) - (fi[c + 1 - sz] - fi[c - 1 - sz])) * (r2dx * r2dz);
  const double d2yz = ((fi[c + sy + sz] - fi[c - sy + sz]) - (fi[c + sy - sz] - fi[c - sy - sz])) * (r2dy * r2dz);
  const double d2xy = ((fi[c + 1 + sy] - fi[c - 1 + sy]) - (fi[c + 1 - sy] - fi[c - 1 - sy])) * (r2dx * r2dy);
  const double nrm = gx * gx + gy * gy + gz * gz;
  double kap;
  if (nrm < 1e-10) {
    kap = 0.0;
  } else {
    const double s = sqrt(nrm);            // nrm**0.5
    const double inv15 = 1.0 / (nrm * s);  // nrm**(-1.5)
    const double term1 = (d2x + d2y + d2z) / s;
    const double term2 = (gx * gx * d2x + gy * gy * d2y + gz * gz * d2z) * inv15;
    const double term3 = 2.0 * (gx * gy * d2xy + gx * gz * d2xz + gy * gz * d2yz) * inv15;
    kap = -(term1 - term2 - term3);
  }
  if (kap > max_kappa) kap = max_kappa;
  const double a = 1.0 / (2.0 * ph.sw);
  const double dirac = a + a * cos(TPLS_PI_SP * p / ph.sw);
  const double m = dirac * ph.scap * kap;
  r.x = m * gx;
  r.y = m * gy;
  r.z = m * gz;
  return r;
}

__device__ __forceinline__ F3 lin2(F3 a, F3 b) {  // 2a - b
  F3 r = {2.0 * a.x - b.x, 2.0 * a.y - b.y, 2.0 * a.z - b.z};
  return r;
}

// value on the i = 1..nx columns including the extrapolated z ghost planes
__device__ __forceinline__ F3 csf_colval(const Geo &g, const Phys &ph, double mk,
                                         const double *fi, int i, int j, int k) {
  if (k == 0) return lin2(csf_point(g, ph, mk, fi, i, j, 1), csf_point(g, ph, mk, fi, i, j, 2));
  if (k == g.nz + 1)
    return lin2(csf_point(g, ph, mk, fi, i, j, g.nz), csf_point(g, ph, mk, fi, i, j, g.nz - 1));
  return csf_point(g, ph, mk, fi, i, j, k);
}

__global__ void k_csf(Geo g, Phys ph, double mk, const double *__restrict__ fi,
                      double *__restrict__ fx, double *__restrict__ fy, double *__restrict__ fz) {
  const int i = blockIdx.x * LS_BX + threadIdx.x, j = blockIdx.y * LS_BY + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.nx + 1 || j > g.ny + 1) return;
  const int jj = wrapy(j, g.ny);
  F3 v;
  if (i == 0)
    v = lin2(csf_colval(g, ph, mk, fi, 1, jj, k), csf_colval(g, ph, mk, fi, 2, jj, k));
  else if (i == g.nx + 1)
    v = lin2(csf_colval(g, ph, mk, fi, g.nx, jj, k), csf_colval(g, ph, mk, fi, g.nx - 1, jj, k));
  else
    v = csf_colval(g, ph, mk, fi, i, jj, k);
  const int c = TPLS_IDX(g, i, j, k);
  fx[c] = v.x;
  fy[c] = v.y;
  fz[c] = v.z;
}

cudaError_t launch_csf(const Geo &g, const Phys &ph, const double *phi3,
                       double *fx, double *fy, double *fz, cudaStream_t st) {
  const double mk = 1.0 / fmin(fmin(ph.dx, ph.dy), ph.dz);
  k_csf<<<full_grid(g, g.nz + 2), dim3(LS_BX, LS_BY), 0, st>>>(g, ph, mk, phi3, fx, fy, fz);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// momentum_allflux.f90:474-521 get_viscosity on x = 0..nx+1 (the ghost
// planes of main_ns_hybrid.F90:653-710 use the same formula and the same
// single-precision pi) and the 2-row periodic-y augmentation.
__global__ void k_visc(Geo g, Phys ph, const double *__restrict__ phi, double *__restrict__ mu) {
  const int i = blockIdx.x * LS_BX + threadIdx.x, j = blockIdx.y * LS_BY + threadIdx.y - 1;
  const int k = blockIdx.z;
  if (i > g.nx + 1 || j > g.ny + 2) return;
  const double p = phi[TPLS_IDX(g, i, wrapy(j, g.ny), k)];
  double hv;
  if (p < -ph.sw)
    hv = 0.0;
  else if (p > ph.sw)
    hv = 1.0;
  else
    hv = 0.5 + (p / (2.0 * ph.sw)) + (1.0 / (2.0 * TPLS_PI_SP)) * sin(TPLS_PI_SP * p / ph.sw);
  mu[TPLS_IDXM(g, i, j, k)] = (ph.mu_plus * hv + ph.mu_minus * (1.0 - hv)) / ph.re;
}

cudaError_t launch_visc(const Geo &g, const Phys &ph, const double *phi2,
                        double *mu, cudaStream_t st) {
  dim3 grd((g.nx + 2 + LS_BX - 1) / LS_BX, (g.ny + 4 + LS_BY - 1) / LS_BY, g.nz + 2);
  k_visc<<<grd, dim3(LS_BX, LS_BY), 0, st>>>(g, ph, phi2, mu);
  return cudaGetLastError();
}

}  // namespace tpls
