// tpls_kernels.h -- host-side launchers of the TPLS kernels (internal).
// Every launcher enqueues on `st` and returns the cudaError_t of the launch.
#pragma once
#include "tpls_common.cuh"

namespace tpls {

// Scalar parameters passed by value to kernels.
struct Phys {
  double dx, dy, dz, dt;
  double re, mu_plus, mu_minus, height, scap, sw;
};

// Deterministic block-partial reduction buffer: kernels write one partial
// per block into part[], finish_sum() adds them in a fixed order.  Above
// FS_ONE_BLOCK partials (nout = 1) it first sums contiguous chunks on many
// SMs into part[nparts ...] (a single SM's FP64 pipe would take ~90 us for
// the 285k partials of a 512x256x256 sweep), so part[] must hold FS_TAIL
// doubles after the partials; finish_sum_kernels() is the launch count.
constexpr int FS_TAIL = 1024, FS_ONE_BLOCK = 8192;
cudaError_t finish_sum(double *part, int nparts, double *out, int nout,
                       cudaStream_t st);
int finish_sum_kernels(int nparts, int nout);

// advect_phi.f90 / weno.f90: conv2_phi from phi2, u2, v2, w2.
cudaError_t launch_advect(const Geo &g, const Phys &ph, const double *phi2,
                          const double *u2, const double *v2,
                          const double *w2, double *conv2_phi,
                          cudaStream_t st);
// exchange2d (mpi.f90:110) on one GPU: periodic copy of rows 0 and ny+1,
// x = 0..nx+1, nzp planes.
cudaError_t launch_exchange(const Geo &g, double *a, int nzp, cudaStream_t st);
cudaError_t launch_exchange(const Geo &g, float *a, int nzp, cudaStream_t st);
// FP32-mixed form: WENO5 faces and flux divergence in FP32 on FP32 copies
// of phi, u, v, w; conv2_phi written in FP64.
cudaError_t launch_advect(const Geo &g, const Phys &ph, const float *phi2,
                          const float *u2, const float *v2, const float *w2,
                          double *conv2_phi, cudaStream_t st);
cudaError_t launch_to_float(const double *a, float *b, size_t n, cudaStream_t st);
// The same FP32 advection with phi staged by TMA: map128 = a 128-byte,
// 64-byte-aligned tensor map made by advect_tma_map for the FP32 phi copy;
// kto counts blocks whose wait for the staged tile ran out (limit polls).
// arm = 0 and one_block = 1: the self-test of that limit (nothing issued).
cudaError_t advect_tma_map(const Geo &g, const float *phi32, void *map128);
cudaError_t launch_advect_tma(const Geo &g, const Phys &ph, const void *map128, const float *u2, const float *v2,
                              const float *w2, double *conv2_phi, double *kto, cudaStream_t st, int arm = 1,
                              int limit = 1 << 22, int one_block = 0);

// cahn_hilliard_solver.f90:41-382 dim (diffuse interface), see k_dim.cu.
// phi + add is the concentration C (the driver's phi2 + 0.5).
struct DimK {
  double rdx2, rdy2, rdz2;  // 1/dx/dx, 1/dy/dy, 1/dz/dz
  double epn2, repn, rpe;   // epn^2, 1/epn, 1/Pe
  double c_nt2, c_en2;      // nmda*tao/2, epn^2*nmda/2
  double dt, kc, tao, alfa1, rdiag;  // kc = dt*nmda/2/Pe, rdiag = 1/diagonal
  double dz, height, zden;  // inlet profile: 0.5+0.5 tanh((z-height)/zden)
};
DimK dim_constants(const Phys &ph, double epn, double pe);
cudaError_t launch_dim_prep(const Geo &g, const DimK &q, const double *phi, double add, double *e0, double *l0,
                            cudaStream_t st);
cudaError_t launch_dim_source(const Geo &g, const DimK &q, const double *phi, double add, const double *e0,
                              const double *l0, const double *conv2, double *cprev, double *src, cudaStream_t st);
cudaError_t launch_dim_lap(const Geo &g, const DimK &q, const double *pin, double *l, cudaStream_t st);
cudaError_t launch_dim_update(const Geo &g, const DimK &q, const double *phi, double add, const double *phio,
                              double addo, const double *src, const double *pin, const double *l, double *pout,
                              cudaStream_t st);
cudaError_t launch_dim_finish(const Geo &g, const double *pfin, double *phi2, double *phi3, cudaStream_t st);

// two_phase_levelset.f90 / levelset.f90
cudaError_t launch_ls_ab3(const Geo &g, const Phys &ph, const double *phi2,
                          const double *c0, const double *c1, const double *c2,
                          double *phi3, cudaStream_t st);
cudaError_t launch_ls_status(const Geo &g, const Phys &ph, const double *phi3,
                             double *D, signed char *flags, cudaStream_t st);
cudaError_t launch_ls_iter(const Geo &g, const Phys &ph, const double *pr,
                           const double *D, const signed char *flags,
                           double *pr_new, double *err_part, cudaStream_t st);
int ls_iter_blocks(const Geo &g);
cudaError_t launch_csf(const Geo &g, const Phys &ph, const double *phi3,
                       double *fx, double *fy, double *fz, cudaStream_t st);
cudaError_t launch_visc(const Geo &g, const Phys &ph, const double *phi2,
                        double *mu, cudaStream_t st, double phi_offset = 0.0);
// FP32-mixed form of the level-set kernels: status decided in FP64 with D
// stored in FP32, the redistancing increments in FP32 on float-pair iterates,
// CSF evaluated in FP64 and stored in FP32, viscosity stored in FP32 (the
// Heaviside evaluated in FP64).
cudaError_t launch_ls_status(const Geo &g, const Phys &ph, const double *phi3,
                             float *D, signed char *flags, cudaStream_t st);
// in64 (FP64 input, first iteration) or the float pair (hi, lo); out64
// (FP64 output, last iteration) or the float pair (ohi, olo).
cudaError_t launch_ls_iter_ff(const Geo &g, const Phys &ph, const double *in64,
                              const float *hi, const float *lo, const float *D,
                              const signed char *flags, double *out64,
                              float *ohi, float *olo, double *err_part,
                              cudaStream_t st);
cudaError_t launch_csf(const Geo &g, const Phys &ph, const double *phi3,
                       float *fx, float *fy, float *fz, cudaStream_t st);
cudaError_t launch_visc(const Geo &g, const Phys &ph, const double *phi2,
                        float *mu, cudaStream_t st);

// momentum_allflux.f90 + main_ns_hybrid.F90:629-641,743-751: per component
// conv2, csf2 (history) and the AB3/CN right-hand side.
cudaError_t launch_mom_rhs(int comp, const Geo &g, const Phys &ph,
                           const double *u2, const double *v2,
                           const double *w2, const double *mu,
                           const double *fcsf, const double *c1,
                           const double *c0, const double *s1,
                           const double *s0, double *conv2, double *csf2,
                           double *rhs, double *diff_out, double *coef,
                           cudaStream_t st);
// FP32-mixed form: FP32 stencils on the FP64 velocity state split into
// FP32 pairs by integer operations and FP32 viscosity, FP64 CSF force and
// AB3 combination; writes the defect-form b of the FP32 sweeps (one float
// per point, rec_slot order) and the AB3 histories.
cudaError_t launch_mom_rhs_pair(int comp, const Geo &g, const Phys &ph,
                                const double *u2, const double *v2,
                                const double *w2, const float *mu,
                                const double *fcsf, const double *c1,
                                const double *c0, const double *s1,
                                const double *s0, double *conv2, double *csf2,
                                float *coef, cudaStream_t st);
// FP64 stencils writing the defect-form b of the FP32 sweeps (FP32-mixed
// form with TPLS_PART_MOM_STENCIL; one float per point, rec_slot order).
cudaError_t launch_mom_rhs64r32(int comp, const Geo &g, const Phys &ph,
                                const double *u2, const double *v2,
                                const double *w2, const double *mu,
                                const double *fcsf, const double *c1,
                                const double *c0, const double *s1,
                                const double *s0, double *conv2,
                                double *csf2, float *bdef, cudaStream_t st);
// Standalone get_conv_all / get_diffusion_all (per-routine entries).
cudaError_t launch_conv_diff(int comp, int want_conv, const Geo &g,
                             const Phys &ph, const double *u2,
                             const double *v2, const double *w2,
                             const double *mu, double *out, cudaStream_t st);
// jacobi_iteration_allflux.f90 / sor_iteration_allflux.f90 with the
// boundary conditions of main_ns_hybrid.F90:756-887 fused in.
//   bc: 0 = plain reference routine (only the routine's own BCs),
//       1 = also the driver's post-sweep BCs (u: inlet copy, pressure outlet,
//           fictitious point; v: inlet/outlet copies; w: walls, inlet,
//           outlet).
cudaError_t launch_jacobi(int comp, const Geo &g, const Phys &ph,
                          const double *xo, const double *rhs,
                          const double *mu, const double *pres, double *x,
                          int bc, int fuse_ghosts, cudaStream_t st);
cudaError_t launch_sor(int comp, const Geo &g, const Phys &ph, double *x,
                       const double *rhs, const double *mu,
                       const double *pres, int flg, int iteration_time,
                       int bc, int fuse_ghosts, cudaStream_t st);
// Tile-shape choice of the sweep kernels (autotuned per grid): jac / even =
// block shape index (0: 32x4, 1: 32x8, 2: 64x4, 3: 16x8); odd is always 0
// (the odd half-sweep has one shape).
struct SweepTiles {
  int jac = 0, even = 0, odd = 0;
};

// State of the segment-chained odd half-sweep of the FP64 form, one per
// context (its launches are ordered on the context's stream): ticket,
// finished-block and epoch counters; per segment (64 levels of 32 columns
// of one row) a ready flag (epoch + 1) and the 32 values entering the
// segment above it.  Zeroed at allocation.
struct OddChain {
  unsigned *ctr = nullptr;   // [0] tickets, [1] blocks done, [2] epoch
  unsigned *flag = nullptr;  // per segment
  double *incl = nullptr;    // per segment, 32 values
  double *kto = nullptr;     // waits that ran out (a context scalar)
  int cap = 0;               // segments the arrays hold
};
// Segments of the largest component's odd half-sweep on grid g.
int odd_chain_segments(const Geo &g);

// Coefficient source of the per-routine sweep entries: the FP64
// viscosity_aug (device mu layout) and right-hand side of host arrays.
struct RefCoef {
  const double *mu;
  const double *rhs;
  double ax2, ay2, az2;
};
// Odd-iteration half-sweep (iteration_time odd) of the per-routine entries
// in the chunk-parallel column form, no boundary rows, no ghost fusing (the
// reference's do_sor_u/v/w leave those to the driver).
cudaError_t launch_sor_ref_odd(int comp, const Geo &g, const Phys &ph, double *x, const double *rhs,
                               const double *mu, int flg, cudaStream_t st, const OddChain *oc);

// Sweeps on the per-point coefficient records written by launch_mom_rhs
// (coef != null there): same updates and boundary rows as launch_jacobi /
// launch_sor with bc = 1.
cudaError_t launch_jacobi_c(int comp, const Geo &g, const Phys &ph,
                            const double *xo, const double *coef,
                            const double *pres, double *x, int fuse_ghosts,
                            cudaStream_t st, const SweepTiles &t = SweepTiles());
// oc: the context's segment-chained odd half-sweep state (null: one block
// walks each column, the same results).
cudaError_t launch_sor_c(int comp, const Geo &g, const Phys &ph, double *x,
                         const double *coef, const double *pres, int flg,
                         int iteration_time, int bc, int fuse_ghosts,
                         cudaStream_t st, const SweepTiles &t = SweepTiles(),
                         const OddChain *oc = nullptr);
// FP32 sweeps in defect form: x holds d = x - X for the FP64 base X (the
// component's state).  Their coefficients are recomputed per point from the
// FP32 viscosity field (face averages and Helmholtz diagonal: a few dozen
// FP32 operations, cheaper than reading a 32-byte record), and only the
// defect right-hand side b (already divided by the diagonal) is stored, one
// float per point in record-slot order.
struct MuCoef {
  const float *mu;     // viscosity on the p-grid with two periodic ghost rows
  const float *b;      // per-point b, rec_slot order
  float ax2, ay2, az2;  // dt/(2 d^2) per axis
  // per (j, k) row (index j + (ny+2) k): the boundary-row offsets of the
  // defect iterate, constant during one momentum solve (launch_bc32_prep):
  // x = inlet copy offset, y = outlet offset, z = u's fictitious-point value
  const float4 *bco;
};
MuCoef mu_coef(const Phys &ph, const float *mu, const float *b, const float4 *bco = nullptr);
// The boundary-row offsets of the FP32 defect sweeps of component comp for
// the base state X (u2, v2 or w2) and pressure P: inlet d(0) = d(1) +
// (X(1) - X(0)); outlet u: d(nx) = d(nx-1) + (X(nx-1) - X(nx)) + dt/dx
// ((P+ - P0) - (P0 - P-)) and d(nx+1) = -X(nx+1); outlet v, w: d(nx+1) =
// d(nx) + (X(nx) - X(nx+1)).  Differences taken from FP32 pairs.
cudaError_t launch_bc32_prep(int comp, const Geo &g, const Phys &ph, const double *X, const double *P,
                             float4 *bco, cudaStream_t st);
cudaError_t launch_jacobi_c(int comp, const Geo &g, const Phys &ph,
                            const float *xo, const MuCoef &coef,
                            const double *pres, const double *X, float *x,
                            int fuse_ghosts, cudaStream_t st,
                            const SweepTiles &t = SweepTiles());
cudaError_t launch_sor_c(int comp, const Geo &g, const Phys &ph, float *x,
                         const MuCoef &coef, const double *pres,
                         const double *X, int flg, int iteration_time, int bc,
                         int fuse_ghosts, cudaStream_t st,
                         const SweepTiles &t = SweepTiles(),
                         const OddChain *oc = nullptr);
// d = -X (n elements) / x = X + d
cudaError_t launch_defect_init(const double *X, float *d, size_t n, cudaStream_t st);
cudaError_t launch_defect_apply(const double *X, const float *d, double *x, size_t n,
                                cudaStream_t st);
// One-time kernel attributes of the sweeps (dynamic shared memory).
cudaError_t sweep_init();
cudaError_t launch_diff2(const Geo &g, const double *a, const double *b,
                         int nzp, double *part, cudaStream_t st);
cudaError_t launch_diff2(const Geo &g, const float *a, const float *b,
                         int nzp, double *part, cudaStream_t st);
int diff2_blocks(const Geo &g, int nzp);

// pressure.f90
cudaError_t launch_source(const Geo &g, const Phys &ph, const double *u3,
                          const double *v3, const double *w3, double *rhs_p,
                          cudaStream_t st);
cudaError_t launch_project(const Geo &g, const Phys &ph, const double *u3,
                           const double *v3, const double *w3,
                           const double *p, const double *u_inlet,
                           double *u_out, double *v_out, double *w_out,
                           cudaStream_t st);

}  // namespace tpls
