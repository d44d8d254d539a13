// k_noalloc.cu -- get_difference for callers that cannot allocate device
// memory.
//
// Some callers of this library cannot call cudaMalloc.  A time-step loop
// with a latency budget cannot afford it: cudaMalloc and cudaFree may wait
// until the whole device is idle.  A host program whose device memory is
// owned by another runtime's pool, or by a fixed HBM budget that admits
// jobs by their footprint, cannot let a library allocate behind its back
// either: the allocation is not counted and can fail when the budget is
// full.  tpls_get_difference_noalloc computes the same quantity as
// tpls_get_difference (sum of (ua-ub)^2 over i 1..nx, j 1..ny and every z
// plane, jacobi_iteration_allflux.f90:285-311) on arrays the caller already
// has on the device, and writes the sum to a device address the caller
// owns.  Its only scratch is the fixed array below, compiled into the
// library; it calls no allocating routine.
//
// The scratch holds one partial sum per (j, plane) row, so a call accepts at
// most TPLS_NOALLOC_MAX_ROWS = 65536 rows (ny * nzp) -- 512 KB of device
// memory on every GPU that loads the library, held until the process exits.
// Larger calls are rejected with TPLS_ERR_NOALLOC_LIMIT before any launch.
// Every partial is written before it is read in the same call, so nothing
// needs clearing between calls, but all calls share the one array: calls
// that overlap on the GPU (different streams, or different host threads on
// one device) race on it and must be serialised by the caller.
#include <mutex>

#include "tpls_common.cuh"

namespace {

constexpr int kMaxRows = TPLS_NOALLOC_MAX_ROWS;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[kMaxRows];

// Device address of g_noalloc_partials per device ordinal.  In host code the
// array's name is only a host-side stand-in, so the address is looked up
// once per device, with that device current, by the first call made on it,
// and kept until the process exits.  cudaDeviceReset destroys the context
// that holds the array, so the kept address does not survive it: the entry
// is not for use on a device after a reset.
double *g_partials_addr[kMaxDevices] = {nullptr};
std::mutex g_partials_mu;

cudaError_t partials_address(double **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_partials_mu);
  if (!g_partials_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess) return e;
    g_partials_addr[dev] = static_cast<double *>(p);
  }
  *out = g_partials_addr[dev];
  return cudaSuccess;
}

// one warp per (j, k) row of the reference-layout arrays (0:nx+1,0:ny+1,0:nzp-1)
__global__ void k_noalloc_rows(const double *__restrict__ ua, const double *__restrict__ ub, int nx,
                               int ny, int nzp, double *__restrict__ part) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= ny * nzp) return;  // uniform per warp
  const int j = row % ny + 1, k = row / ny;
  const size_t base = (size_t)(nx + 2) * ((size_t)j + (size_t)(ny + 2) * (size_t)k);
  double s = 0.0;
  for (int i = 1 + lane; i <= nx; i += 32) {
    const double d = ua[base + i] - ub[base + i];
    s += d * d;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) part[row] = s;
}

// fixed-order sum of the row partials (one block)
__global__ void k_noalloc_total(const double *__restrict__ part, int rows, double *__restrict__ out) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int r = threadIdx.x; r < rows; r += blockDim.x) s += part[r];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

}  // namespace

extern "C" int tpls_get_difference_noalloc(const double *ua, const double *ub, int nx, int ny, int nzp,
                                           double *diff, void *stream) {
  if (!ua || !ub || !diff || nx < 1 || ny < 1 || nzp < 1) return TPLS_ERR_ARG;
  if ((long long)ny * (long long)nzp > kMaxRows) return TPLS_ERR_NOALLOC_LIMIT;
  double *part = nullptr;
  cudaError_t e = partials_address(&part);
  if (e != cudaSuccess) return TPLS_ERR_CUDA_BASE + (int)e;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int rows = ny * nzp;
  const int threads = 256, blocks = (rows * 32 + threads - 1) / threads;
  k_noalloc_rows<<<blocks, threads, 0, st>>>(ua, ub, nx, ny, nzp, part);
  e = cudaGetLastError();
  if (e != cudaSuccess) return TPLS_ERR_CUDA_BASE + (int)e;
  k_noalloc_total<<<1, 256, 0, st>>>(part, rows, diff);
  e = cudaGetLastError();
  if (e != cudaSuccess) return TPLS_ERR_CUDA_BASE + (int)e;
  return TPLS_OK;
}
