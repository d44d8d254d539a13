// tpls_common.cuh -- device layout and helpers shared by every TPLS kernel.
//
// Device layout of a channel nx*ny*nz (one GPU, no sharding):
//   every field keeps the reference's halo'd index space
//   (x 0..nx+1, y 0..ny+1, z from 0) in an x-fastest, pitched array whose
//   rows are PX doubles long (PX a multiple of 4, x=1 on a 32-byte boundary
//   so the interior of every row is sector aligned and double2-vectorisable).
//   Kernels receive pointers already offset to (0,0,0), so element (i,j,k)
//   sits at p[i + SY*j + SZ*k]; the viscosity field has two periodic ghost
//   rows on each side (y -1..ny+2) and its own z stride SZM.
//   y-ghost rows are kept as periodic copies by the kernels that write a
//   field (the single-GPU form of the reference's exchange2d halo swaps).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/tpls_gpu.h"

namespace tpls {

constexpr int XOFF = 3;  // element offset of x=0 inside a row

struct Geo {
  int nx, ny, nz;
  int sy;   // y stride (elements) = PX
  int sz;   // z stride of p/u/v/w fields = PX*(ny+2)
  int szm;  // z stride of the viscosity field = PX*(ny+4)
};

// Single-precision literals of the reference, widened exactly as Fortran does.
#define TPLS_WENO_EPS ((double)1.e-7f)      // weno.f90:184
#define TPLS_PI_SP ((double)3.1415926535f)  // levelset.f90:388, momentum_allflux.f90:489

__host__ __device__ inline int wrapy(int j, int ny) {
  // periodic row index in 1..ny for j in [-ny+1, 2ny]
  return j < 1 ? j + ny : (j > ny ? j - ny : j);
}

// Launch bookkeeping: every launch site calls this so the context can report
// how many of its kernels ran.
struct LaunchCounter {
  long n = 0;
};

}  // namespace tpls

#define TPLS_IDX(g, i, j, k) ((i) + (g).sy * (j) + (g).sz * (k))
#define TPLS_IDXM(g, i, j, k) ((i) + (g).sy * (j) + (g).szm * (k))
