// tpls_pressure.h -- multigrid-preconditioned CG pressure solver (internal).
#pragma once
#include "tpls_kernels.h"

namespace tpls {

struct PoissonSolver;

// cx, cy, cz: coefficients of the x, y, z second differences of the
// reduced operator (1/dy^2, 1/dx^2, 1/dz^2 for the reference's matrix).
cudaError_t poisson_create(const Geo &g, double cx, double cy, double cz,
                           PoissonSolver **out);
void poisson_destroy(PoissonSolver *S);
int poisson_levels(const PoissonSolver *S);
// Solves for pres (full p-grid incl. ghosts) from RHS_p, u3's inlet column,
// u_inlet and the initial guess pres_old.  Synchronises the stream once per
// iteration to test convergence.
cudaError_t poisson_solve(PoissonSolver *S, const Geo &g, const Phys &ph,
                          const double *rhs_p, const double *u3,
                          const double *u_inlet, const double *pres_old,
                          double *pres, double rtol, int maxits, int *its,
                          double *rnorm, double *bnorm, int *reason,
                          cudaStream_t st, long *nlaunch);

}  // namespace tpls
