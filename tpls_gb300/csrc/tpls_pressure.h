// tpls_pressure.h -- multigrid-preconditioned CG pressure solver (internal).
#pragma once
#include "tpls_kernels.h"

namespace tpls {

struct PoissonSolver;

// cx, cy, cz: coefficients of the x, y, z second differences of the
// reduced operator (1/dy^2, 1/dx^2, 1/dz^2 for the reference's matrix).
// fp32: run the multigrid preconditioner in FP32 (the CG recurrences,
// reductions and the coarsest dense solve stay FP64).
cudaError_t poisson_create(const Geo &g, double cx, double cy, double cz,
                           int fp32, PoissonSolver **out);
void poisson_destroy(PoissonSolver *S);
int poisson_levels(const PoissonSolver *S);
// Device bytes poisson_create allocates for this grid, each allocation
// rounded by rnd (the allocator's granularity).
size_t poisson_footprint(const Geo &g, int fp32, size_t (*rnd)(size_t));
// Solves for pres (full p-grid incl. ghosts) from RHS_p, u3's inlet column
// (u3 is float when u3_fp32), u_inlet and the initial guess pres_old.
// Synchronises the stream once per iteration to test convergence.
cudaError_t poisson_solve(PoissonSolver *S, const Geo &g, const Phys &ph,
                          const double *rhs_p, const void *u3, int u3_fp32,
                          const double *u_inlet, const double *pres_old,
                          double *pres, double rtol, int maxits, int *its,
                          double *rnorm, double *bnorm, int *reason,
                          cudaStream_t st, long *nlaunch);

// The same solve enqueued on `st` while `st` is being captured into a CUDA
// graph: set-up kernels, a WHILE conditional node whose body is one PCG
// iteration (its condition set by the convergence test on the device), and
// the write-back.  nl_static / nl_body count the kernels outside / inside the
// loop body.  The outcome is read afterwards with poisson_read.
cudaError_t poisson_solve_capture(PoissonSolver *S, const Geo &g, const Phys &ph,
                                  const double *rhs_p, const void *u3, int u3_fp32,
                                  const double *u_inlet, const double *pres_old,
                                  double *pres, double rtol, int maxits,
                                  cudaStream_t st, long *nl_static, long *nl_body);
// Last solve's iterations, ||r||, ||b||, reason; the lowest reason since the
// last poisson_reset_worst; iterations of all solves so far.  Synchronises.
cudaError_t poisson_read(PoissonSolver *S, cudaStream_t st, int *its, double *rnorm,
                         double *bnorm, int *reason, int *worst, double *its_total);
cudaError_t poisson_reset_worst(PoissonSolver *S, cudaStream_t st);

}  // namespace tpls
