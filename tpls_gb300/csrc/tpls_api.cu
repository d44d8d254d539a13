// tpls_api.cu -- the C ABI (include/tpls_gpu.h): context, device-resident
// state, the timestep driver and the per-routine drop-in entries.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <array>
#include <map>
#include <mutex>
#include <vector>

#include "tpls_pressure.h"
#include "tpls_sweep.cuh"

using namespace tpls;

namespace {

constexpr int kMaxScratch = 8;

// Stream captures and the calls that act on the whole device (allocation,
// release, stream and graph creation) are serialised across host threads,
// so a context can be created or destroyed on one thread while another
// thread captures a step graph: a call of that kind issued during another
// thread's capture can invalidate it.  Recursive: destroy runs inside a
// failed create.
std::recursive_mutex g_dev_mu;
using DevLock = std::lock_guard<std::recursive_mutex>;

}  // namespace

// Batched host transfers.  Downloads are 2-D copies straight from a field's
// pitched rows into the host layout on their own stream (no staging, no
// repack); uploads go through a ring of two contiguous staging buffers (the
// context's own staging buffer and one allocated on first use) on a second
// stream and are repacked into the field on the context's stream (a 2-D
// upload of rows this short runs at a fraction of the link's rate).  A field
// uploaded after a download into the same host array, or from the same
// field, waits for that download on the device, so a download of the state
// followed by an upload of the same arrays uses both copy directions at once.
// Later work on the context's stream waits for pending downloads lazily
// (xfer_fence), so those uploads do not queue behind them.
struct Xfer {
  cudaStream_t h2d = nullptr, d2h = nullptr;
  // upload staging slots: two at first, as many as the largest call's fields
  // once a call has more, so every upload of a call can run before the
  // context's stream reaches its repack
  std::vector<double *> slot;
  std::vector<cudaEvent_t> free_ev;   // the slot may be refilled
  std::vector<cudaEvent_t> ready_ev;  // the slot holds its data
  cudaEvent_t st_ev = nullptr;                   // the context's stream at a download call
  cudaEvent_t up_ev = nullptr;                   // the last repack on the upload stream
  cudaEvent_t d2h_last = nullptr;                // the last download enqueued
  cudaEvent_t field_dl[TPLS_F_COUNT] = {};       // the last download from each field
  bool dl_pending = false;                       // downloads the context's stream has not waited for
  int next = 0;
  std::map<const void *, cudaEvent_t> host_done;  // last download into each host array
};

// A registered host array (tpls_register_host): its device mirror.
struct HostReg {
  double *mirror;
  size_t count;  // doubles
};

struct tpls_ctx {
  int nx, ny, nz;
  tpls_params prm;
  Geo g;
  Phys ph;
  int px;  // row pitch (elements)
  cudaStream_t st = nullptr;
  std::vector<void *> allocs;
  // state
  double *phi2, *u2, *v2, *w2, *pres, *pres_old;
  double *conv_u[3], *conv_v[3], *conv_w[3], *conv_phi[3];
  double *csf_u[3], *csf_v[3], *csf_w[3];
  int phase = 0;  // conv0 = [phase%3], conv1 = [(phase+1)%3], conv2 = [(phase+2)%3]
  // step work arrays
  double *phiA, *phiB, *D;
  signed char *flags;
  double *mu, *fx, *fy, *fz;
  double *rhs_p;
  double *coef[3];  // per-component sweep records (8 doubles per point)
  double *x3[3][2];  // momentum ping-pong per component
  int x3_final[3] = {0, 0, 0};
  double *u_inlet;
  // diffuse-interface method (idm = dim, FP64 form): ConvPrevPhi and the
  // reference's phi3 (the next step's starting guess) are state; bulkE0 and
  // source0 are work arrays, the iterate ping-pongs through phiA / phiB and
  // d2phi lives in D
  int dim = 0;
  double *convprev = nullptr, *phi3d = nullptr, *dimE = nullptr, *dimS = nullptr;
  // FP32-mixed form: FP32 copies of the step inputs and FP32 work arrays
  // (the state above stays FP64)
  int mixed = 0;
  float *phi32, *u32, *v32, *w32, *mu32, *D32;
  float *ffh[2], *ffl[2];  // float-pair redistancing iterates (hi, lo), ping-pong
  float *bdef[3];  // FP32-mixed: defect b of the FP32 sweeps (one float per point)
  float4 *bco32[3];  // FP32-mixed: boundary-row offsets of the FP32 sweeps per (j, k) row
  float *x3f[3][2];
  double *hbuf = nullptr; // interface height (nx*ny)
  double *stage = nullptr; // host-layout staging of one field ((nx+2)(ny+2)(nz+2))
  struct Xfer *xf = nullptr;  // batched host transfers (tpls_set_fields / tpls_get_fields)
  std::map<const double *, HostReg> hreg;  // registered host arrays by base address
  OddChain odd;  // FP64 form: state of the segment-chained odd half-sweep
  alignas(64) unsigned char advmap[128];  // FP32-mixed: tensor map of phi32 for the TMA advection
  bool adv_tma = false;
  size_t n_p, n_uv, n_w;  // elements of each allocation (incl. pitch and padding)
  double *part, *scal, *scal_host;
  size_t part_len;
  PoissonSolver *ps = nullptr;
  tpls_stats stats;
  long launches = 0;
  bool need_exchange = true;
  // CUDA-graph steps: one executable graph per history phase (the AB3 slot
  // pointers differ), captured on first use
  bool use_graphs = true;
  bool capturing = false;
  bool graph_pending = false;  // graph steps launched since the last stats read
  // a step is two graph launches per history phase: the front (viscosity to
  // the momentum right-hand sides) and the back (sweeps, pressure,
  // projection); front_ev is recorded between them
  cudaGraphExec_t gexec[3] = {nullptr, nullptr, nullptr};
  cudaGraphExec_t gexec_back[3] = {nullptr, nullptr, nullptr};
  long g_static[3] = {0, 0, 0};  // kernels per step outside the CG loop body
  cudaEvent_t front_ev = nullptr;
  bool front_ok = false;  // front_ev marks the front of the last work on the stream
  long g_body = 0;               // kernels per CG iteration
  double its_accounted = 0.0;    // pressure iterations already counted in `launches`
  SweepTiles tiles;              // sweep tile shapes (tpls_autotune)
  int tune_version = 0;
  // phase timing (tpls_timing_*)
  bool timing = false;
  int cur_slot = TPLS_T_OTHER;
  std::vector<cudaEvent_t> ev_pool;
  struct TRec {
    int slot;
    cudaEvent_t a, b;
  };
  std::vector<TRec> pending;
  double t_ms[TPLS_T_COUNT] = {0};
  long t_n[TPLS_T_COUNT] = {0};
  // scratch for the per-routine entries (allocated on first use)
  double *scr[kMaxScratch] = {nullptr};
  double *scr_mu = nullptr;
  double *scr_uin = nullptr;
  signed char *scr_flags = nullptr;
};

enum { SC_ERR_PHI = 0, SC_ERR_U, SC_ERR_V, SC_ERR_W, SC_VOL, SC_KTO, SC_N };

#define TCK(x)                                                           \
  do {                                                                   \
    cudaError_t e_ = (x);                                                \
    if (e_ != cudaSuccess) return TPLS_ERR_CUDA_BASE + (int)e_;          \
  } while (0)
// finish_sum launches one or two kernels: count both
#define FSUM(ctx, part, n, out, st)                                      \
  do {                                                                   \
    LCK(ctx, finish_sum(part, n, out, 1, st));                           \
    (ctx)->launches += finish_sum_kernels(n, 1) - 1;                     \
    (ctx)->t_n[(ctx)->cur_slot] += finish_sum_kernels(n, 1) - 1;         \
  } while (0)
#define LCK(ctx, x)                                                      \
  do {                                                                   \
    cudaError_t e_ = (x);                                                \
    (ctx)->launches++;                                                   \
    (ctx)->t_n[(ctx)->cur_slot]++;                                       \
    if (e_ != cudaSuccess) return TPLS_ERR_CUDA_BASE + (int)e_;          \
  } while (0)

// Phase scope: when timing is on, CUDA events on the context stream bracket
// everything enqueued while the scope is alive.
static cudaEvent_t ev_get(tpls_ctx *c);
struct PhaseScope {
  tpls_ctx *c;
  int prev;
  cudaEvent_t a = nullptr;
  int slot;
  PhaseScope(tpls_ctx *c_, int slot_);
  ~PhaseScope();
};

// The odd half-sweep state for launch_sor_c: null walks each column in one
// block (TPLS_FLAG_ODD_COLUMNS; the same results).
static const OddChain *odd_chain(const tpls_ctx *c) {
  return (c->odd.cap > 0 && !(c->prm.flags & TPLS_FLAG_ODD_COLUMNS)) ? &c->odd : nullptr;
}

// State fields a step no longer writes after its front (step_front /
// mixed_front): the level set, its advection histories, the CSF and
// convection histories.  u2, v2, w2, pres, pres_old and the intermediates
// change in the back.
static bool front_final(int f) {
  switch (f) {
    case TPLS_F_PHI2:
    case TPLS_F_CONV0_PHI: case TPLS_F_CONV1_PHI:
    case TPLS_F_CONV0_U: case TPLS_F_CONV1_U: case TPLS_F_CONV0_V: case TPLS_F_CONV1_V:
    case TPLS_F_CONV0_W: case TPLS_F_CONV1_W:
    case TPLS_F_CSF_U0: case TPLS_F_CSF_U1: case TPLS_F_CSF_V0: case TPLS_F_CSF_V1:
    case TPLS_F_CSF_W0: case TPLS_F_CSF_W1:
      return true;
    default:
      return false;
  }
}

static int nz_planes(int kind, int nz) { return kind == 0 ? nz + 2 : (kind == 1 ? nz : nz + 1); }

// device array in the pitched layout; returns the pointer to element (0,0,0)
template <typename T>
static cudaError_t alloc_field(tpls_ctx *c, int rows_before, int rows, int nzp, T **out) {
  void *base = nullptr;
  const size_t n = (size_t)c->px * rows * nzp + 8;
  cudaError_t e = cudaMalloc(&base, n * sizeof(T));
  if (e != cudaSuccess) return e;
  c->allocs.push_back(base);
  e = cudaMemsetAsync(base, 0, n * sizeof(T), c->st);
  if (e != cudaSuccess) return e;
  *out = (T *)base + XOFF + (size_t)c->px * rows_before;
  return cudaSuccess;
}
template <typename T>
static cudaError_t alloc_p(tpls_ctx *c, T **out) { return alloc_field(c, 0, c->ny + 2, c->nz + 2, out); }

static int field_kind(int f) {
  switch (f) {
    case TPLS_F_U2: case TPLS_F_V2: case TPLS_F_CONV0_U: case TPLS_F_CONV1_U:
    case TPLS_F_CONV0_V: case TPLS_F_CONV1_V: case TPLS_F_CSF_U0: case TPLS_F_CSF_U1:
    case TPLS_F_CSF_V0: case TPLS_F_CSF_V1: case TPLS_F_U3: case TPLS_F_V3:
      return 1;
    case TPLS_F_W2: case TPLS_F_CONV0_W: case TPLS_F_CONV1_W: case TPLS_F_CSF_W0:
    case TPLS_F_CSF_W1: case TPLS_F_W3:
      return 2;
    default:
      return 0;
  }
}


static double *field_ptr(tpls_ctx *c, int f) {
  const int s0 = c->phase % 3, s1 = (c->phase + 1) % 3, s2 = (c->phase + 2) % 3;
  switch (f) {
    case TPLS_F_PHI2: return c->phi2;
    case TPLS_F_U2: return c->u2;
    case TPLS_F_V2: return c->v2;
    case TPLS_F_W2: return c->w2;
    case TPLS_F_PRES: return c->pres;
    case TPLS_F_PRES_OLD: return c->pres_old;
    case TPLS_F_CONV0_U: return c->conv_u[s0];
    case TPLS_F_CONV1_U: return c->conv_u[s1];
    case TPLS_F_CONV0_V: return c->conv_v[s0];
    case TPLS_F_CONV1_V: return c->conv_v[s1];
    case TPLS_F_CONV0_W: return c->conv_w[s0];
    case TPLS_F_CONV1_W: return c->conv_w[s1];
    case TPLS_F_CSF_U0: return c->csf_u[s0];
    case TPLS_F_CSF_U1: return c->csf_u[s1];
    case TPLS_F_CSF_V0: return c->csf_v[s0];
    case TPLS_F_CSF_V1: return c->csf_v[s1];
    case TPLS_F_CSF_W0: return c->csf_w[s0];
    case TPLS_F_CSF_W1: return c->csf_w[s1];
    case TPLS_F_CONV0_PHI: return c->conv_phi[s0];
    case TPLS_F_CONV1_PHI: return c->conv_phi[s1];
    // last step's intermediates: after the rotation the step's conv2 sits
    // in the conv1 slot
    case TPLS_F_CONV2_PHI: return c->conv_phi[s1];
    case TPLS_F_PHI3: return c->dim ? c->phi3d : c->phi2;
    case TPLS_F_CONVPREV_PHI: return c->convprev;
    case TPLS_F_RHS_P: return c->rhs_p;
    case TPLS_F_U3: return c->x3[0][c->x3_final[0]];
    case TPLS_F_V3: return c->x3[1][c->x3_final[1]];
    case TPLS_F_W3: return c->x3[2][c->x3_final[2]];
    default: return nullptr;
  }
  (void)s2;
}

// Host fields (Fortran order, rows of nx+2) move through a contiguous
// device staging buffer: one bulk copy at full link bandwidth, and a
// repack kernel between the host row layout and the pitched device rows
// (many short pitched rows copy at a fraction of the link's bandwidth).
__global__ void k_repack(const double *__restrict__ src, int spitch, double *__restrict__ dst, int dpitch, int w,
                         int rows) {
  for (int r = blockIdx.y; r < rows; r += gridDim.y)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w; i += gridDim.x * blockDim.x)
      dst[(size_t)r * dpitch + i] = src[(size_t)r * spitch + i];
}
static cudaError_t repack(const double *src, int spitch, double *dst, int dpitch, int w, int rows,
                          cudaStream_t st) {
  dim3 grd((w + 127) / 128, rows < 32768 ? rows : 32768);
  k_repack<<<grd, 128, 0, st>>>(src, spitch, dst, dpitch, w, rows);
  return cudaGetLastError();
}
// The address the library copies from or to for `count` doubles at a host
// address: inside a registered host array, the same place in its device
// mirror; otherwise the host address itself.  Copies use cudaMemcpyDefault,
// so either kind of address works.
template <typename P>
static P hmap(const tpls_ctx *c, P host, size_t count) {
  if (c->hreg.empty() || !host) return host;
  const double *h = (const double *)host;
  auto it = c->hreg.upper_bound(h);
  if (it == c->hreg.begin()) return host;
  --it;
  const double *b = it->first;
  if (h >= b && (size_t)(h - b) + count <= it->second.count) return (P)(it->second.mirror + (h - b));
  return host;
}

// A registered array's mirror already holds the host layout on the device:
// the repack reads or writes it directly instead of through the staging
// buffer.
static cudaError_t h2d(tpls_ctx *c, double *dev0, const double *host, int nzp) {
  const int w = c->nx + 2, rows = (c->ny + 2) * nzp;
  const size_t n = (size_t)w * rows;
  const double *src = hmap(c, host, n);
  if (src != host) return repack(src, w, dev0, c->px, w, rows, c->st);
  cudaError_t e = cudaMemcpyAsync(c->stage, host, sizeof(double) * n, cudaMemcpyHostToDevice, c->st);
  if (e != cudaSuccess) return e;
  return repack(c->stage, w, dev0, c->px, w, rows, c->st);
}
static cudaError_t d2h(tpls_ctx *c, double *host, const double *dev0, int nzp) {
  const int w = c->nx + 2, rows = (c->ny + 2) * nzp;
  const size_t n = (size_t)w * rows;
  double *dst = hmap(c, host, n);
  if (dst != host) return repack(dev0, c->px, dst, w, w, rows, c->st);
  cudaError_t e = repack(dev0, c->px, c->stage, w, w, rows, c->st);
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(host, c->stage, sizeof(double) * n, cudaMemcpyDeviceToHost, c->st);
}
// viscosity_aug (-1:nx+2,-1:ny+2,0:nz+1) <-> device mu (x 0..nx+1, y -1..ny+2)
static cudaError_t h2d_mu(tpls_ctx *c, double *mu0, const double *host) {
  const size_t w = sizeof(double) * (size_t)(c->nx + 2), n = (size_t)(c->nx + 4) * (c->ny + 4) * (c->nz + 2);
  return cudaMemcpy2DAsync(mu0 - c->px, sizeof(double) * c->px, hmap(c, host, n) + 1, sizeof(double) * (c->nx + 4),
                           w, (size_t)(c->ny + 4) * (c->nz + 2), cudaMemcpyDefault, c->st);
}
static cudaError_t d2h_mu(tpls_ctx *c, double *host, const double *mu0) {
  const size_t w = sizeof(double) * (size_t)(c->nx + 2), n = (size_t)(c->nx + 4) * (c->ny + 4) * (c->nz + 2);
  return cudaMemcpy2DAsync(hmap(c, host, n) + 1, sizeof(double) * (c->nx + 4), mu0 - c->px, sizeof(double) * c->px,
                           w, (size_t)(c->ny + 4) * (c->nz + 2), cudaMemcpyDefault, c->st);
}

static Phys phys_from(const tpls_params &p) {
  Phys ph;
  ph.dx = p.dx;
  ph.dy = p.dy;
  ph.dz = p.dz;
  ph.dt = p.dt;
  ph.re = p.re;
  ph.mu_plus = p.mu_plus;
  ph.mu_minus = p.mu_minus;
  ph.height = p.height;
  ph.scap = p.scap;
  ph.sw = p.smooth_width;
  return ph;
}

static cudaEvent_t ev_get(tpls_ctx *c) {
  if (!c->ev_pool.empty()) {
    cudaEvent_t e = c->ev_pool.back();
    c->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

PhaseScope::PhaseScope(tpls_ctx *c_, int slot_) : c(c_), prev(c_->cur_slot), slot(slot_) {
  c->cur_slot = slot;
  if (c->timing) {
    a = ev_get(c);
    if (a) cudaEventRecord(a, c->st);
  }
}
PhaseScope::~PhaseScope() {
  if (c->timing && a) {
    cudaEvent_t b = ev_get(c);
    if (b) {
      cudaEventRecord(b, c->st);
      c->pending.push_back({slot, a, b});
    } else {
      c->ev_pool.push_back(a);
    }
  }
  c->cur_slot = prev;
}

static void timing_flush(tpls_ctx *c) {
  for (auto &r : c->pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess)
      c->t_ms[r.slot] += ms;
    c->ev_pool.push_back(r.a);
    c->ev_pool.push_back(r.b);
  }
  c->pending.clear();
}

extern "C" {

static int refresh_graph_stats(tpls_ctx *c);

const char *tpls_status_string(int s) {
  if (s == TPLS_OK) return "ok";
  if (s == TPLS_ERR_ARG) return "bad argument or index bounds";
  if (s == TPLS_ERR_ALLOC) return "device allocation failed";
  if (s == TPLS_ERR_STATE) return "call sequence error";
  if (s == TPLS_ERR_NOT_BUILT) return "not available in this build";
  if (s == TPLS_KSP_DIVERGED_ITS) return "pressure solve: KSP_DIVERGED_ITS";
  if (s == TPLS_KSP_DIVERGED_NAN) return "pressure solve: KSP_DIVERGED_NAN";
  if (s >= TPLS_ERR_CUDA_BASE) return cudaGetErrorString((cudaError_t)(s - TPLS_ERR_CUDA_BASE));
  return "unknown status";
}

static void xfer_destroy(Xfer *x) {
  if (!x) return;
  if (x->h2d) cudaStreamSynchronize(x->h2d);
  if (x->d2h) cudaStreamSynchronize(x->d2h);
  for (cudaEvent_t e : x->free_ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : x->ready_ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : x->field_dl)
    if (e) cudaEventDestroy(e);
  for (auto &kv : x->host_done) cudaEventDestroy(kv.second);
  if (x->st_ev) cudaEventDestroy(x->st_ev);
  if (x->up_ev) cudaEventDestroy(x->up_ev);
  if (x->d2h_last) cudaEventDestroy(x->d2h_last);
  if (x->h2d) cudaStreamDestroy(x->h2d);
  if (x->d2h) cudaStreamDestroy(x->d2h);
  delete x;
}

int tpls_gpu_destroy(tpls_ctx *c) {
  if (!c) return TPLS_OK;
  DevLock lk(g_dev_mu);
  xfer_destroy(c->xf);
  c->xf = nullptr;
  if (c->st) cudaStreamSynchronize(c->st);
  timing_flush(c);
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  for (cudaGraphExec_t ge : c->gexec)
    if (ge) cudaGraphExecDestroy(ge);
  for (cudaGraphExec_t ge : c->gexec_back)
    if (ge) cudaGraphExecDestroy(ge);
  if (c->front_ev) cudaEventDestroy(c->front_ev);
  poisson_destroy(c->ps);
  for (auto &kv : c->hreg) cudaFree(kv.second.mirror);
  for (void *p : c->allocs) cudaFree(p);
  if (c->scal_host) cudaFreeHost(c->scal_host);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
  return TPLS_OK;
}

static int create_impl(int nx, int ny, int nz, const tpls_params *prm, const double *u_inlet,
                       tpls_ctx *c) {
  c->nx = nx;
  c->ny = ny;
  c->nz = nz;
  c->prm = *prm;
  c->ph = phys_from(*prm);
  c->px = ((XOFF + nx + 2) + 3) / 4 * 4;
  c->g.nx = nx;
  c->g.ny = ny;
  c->g.nz = nz;
  c->g.sy = c->px;
  c->g.sz = c->px * (ny + 2);
  c->g.szm = c->px * (ny + 4);
  TCK(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
  TCK(cudaEventCreateWithFlags(&c->front_ev, cudaEventDisableTiming));
  TCK(sweep_init());
  c->mixed = (prm->precision == TPLS_PREC_FP32_MIXED);
  c->n_p = (size_t)c->px * (ny + 2) * (nz + 2) + 8;
  c->n_uv = (size_t)c->px * (ny + 2) * nz + 8;
  c->n_w = (size_t)c->px * (ny + 2) * (nz + 1) + 8;
  double **pf[] = {&c->phi2, &c->pres, &c->pres_old, &c->conv_phi[0], &c->conv_phi[1], &c->conv_phi[2],
                   &c->phiA, &c->rhs_p};
  for (double **p : pf) TCK(alloc_p(c, p));
  double **puv[] = {&c->u2, &c->v2, &c->conv_u[0], &c->conv_u[1], &c->conv_u[2], &c->conv_v[0],
                    &c->conv_v[1], &c->conv_v[2], &c->csf_u[0], &c->csf_u[1], &c->csf_u[2],
                    &c->csf_v[0], &c->csf_v[1], &c->csf_v[2]};
  for (double **p : puv) TCK(alloc_field(c, 0, ny + 2, nz, p));
  double **pw[] = {&c->w2, &c->conv_w[0], &c->conv_w[1], &c->conv_w[2], &c->csf_w[0], &c->csf_w[1],
                   &c->csf_w[2]};
  for (double **p : pw) TCK(alloc_field(c, 0, ny + 2, nz + 1, p));
  const int rec = 8;  // record entries per point: 64 B in FP64, 32 B in FP32
  if (!c->mixed) {
    double **pf2[] = {&c->phiB, &c->D, &c->fx, &c->fy, &c->fz};
    for (double **p : pf2) TCK(alloc_p(c, p));
    double **px3[] = {&c->x3[0][0], &c->x3[0][1], &c->x3[1][0], &c->x3[1][1]};
    for (double **p : px3) TCK(alloc_field(c, 0, ny + 2, nz, p));
    TCK(alloc_field(c, 0, ny + 2, nz + 1, &c->x3[2][0]));
    TCK(alloc_field(c, 0, ny + 2, nz + 1, &c->x3[2][1]));
    for (int q = 0; q < 3; q++) {
      void *b = nullptr;
      const size_t n = (size_t)rec * c->px * (ny + 2) * (q == 2 ? nz + 1 : nz);
      TCK(cudaMalloc(&b, n * sizeof(double)));
      c->allocs.push_back(b);
      TCK(cudaMemsetAsync(b, 0, n * sizeof(double), c->st));
      c->coef[q] = (double *)b;
    }
    TCK(alloc_field(c, 1, ny + 4, nz + 2, &c->mu));
    if (prm->idm == TPLS_IDM_DIM) {
      c->dim = 1;
      double **pd[] = {&c->convprev, &c->phi3d, &c->dimE, &c->dimS};
      for (double **p : pd) TCK(alloc_p(c, p));  // zeroed: ConvPrevPhi = 0, phi3 = 0 (:443, :449)
    }
  } else {
    const int parts = prm->fp64_parts;
    if (parts & TPLS_PART_LEVELSET) {
      TCK(alloc_p(c, &c->phiB));
      TCK(alloc_p(c, &c->D));
    }
    {  // FP64 CSF force (every setting); FP64 viscosity for FP64 stencils
      double **pf2[] = {&c->fx, &c->fy, &c->fz};
      for (double **p : pf2) TCK(alloc_p(c, p));
      if (parts & (TPLS_PART_MOMENTUM | TPLS_PART_MOM_STENCIL)) TCK(alloc_field(c, 1, ny + 4, nz + 2, &c->mu));
    }
    // FP64 u3, v3, w3 (the defect-form result, or the FP64 momentum iterates)
    TCK(alloc_field(c, 0, ny + 2, nz, &c->x3[0][0]));
    TCK(alloc_field(c, 0, ny + 2, nz, &c->x3[1][0]));
    TCK(alloc_field(c, 0, ny + 2, nz + 1, &c->x3[2][0]));
    if (parts & TPLS_PART_MOMENTUM) {
      double **px3[] = {&c->x3[0][1], &c->x3[1][1]};
      for (double **p : px3) TCK(alloc_field(c, 0, ny + 2, nz, p));
      TCK(alloc_field(c, 0, ny + 2, nz + 1, &c->x3[2][1]));
      for (int q = 0; q < 3; q++) {
        void *b = nullptr;
        const size_t n = (size_t)rec * c->px * (ny + 2) * (q == 2 ? nz + 1 : nz);
        TCK(cudaMalloc(&b, n * sizeof(double)));
        c->allocs.push_back(b);
        TCK(cudaMemsetAsync(b, 0, n * sizeof(double), c->st));
        c->coef[q] = (double *)b;
      }
    }
    float **qf[] = {&c->phi32, &c->D32, &c->ffh[0], &c->ffl[0], &c->ffh[1], &c->ffl[1]};
    for (float **p : qf) TCK(alloc_p(c, p));
    float **quv[] = {&c->u32, &c->v32, &c->x3f[0][0], &c->x3f[0][1], &c->x3f[1][0], &c->x3f[1][1]};
    for (float **p : quv) TCK(alloc_field(c, 0, ny + 2, nz, p));
    float **qw[] = {&c->w32, &c->x3f[2][0], &c->x3f[2][1]};
    for (float **p : qw) TCK(alloc_field(c, 0, ny + 2, nz + 1, p));
    for (int q = 0; q < 3; q++) {
      void *b = nullptr;
      const size_t n = (size_t)c->px * (ny + 2) * (q == 2 ? nz + 1 : nz);
      TCK(cudaMalloc(&b, n * sizeof(float)));
      c->allocs.push_back(b);
      TCK(cudaMemsetAsync(b, 0, n * sizeof(float), c->st));
      c->bdef[q] = (float *)b;
      void *o = nullptr;
      const size_t no = (size_t)(ny + 2) * (nz + 1);
      TCK(cudaMalloc(&o, no * sizeof(float4)));
      c->allocs.push_back(o);
      TCK(cudaMemsetAsync(o, 0, no * sizeof(float4), c->st));
      c->bco32[q] = (float4 *)o;
    }
    TCK(alloc_field(c, 1, ny + 4, nz + 2, &c->mu32));
    if (!(prm->flags & TPLS_FLAG_NO_TMA) && advect_tma_map(c->g, c->phi32, c->advmap) == cudaSuccess)
      c->adv_tma = true;  // else the advection reads phi through the caches
  }
  {
    void *b = nullptr;
    const size_t n = (size_t)c->px * (ny + 2) * (nz + 2) + 64;
    TCK(cudaMalloc(&b, n));
    c->allocs.push_back(b);
    TCK(cudaMemsetAsync(b, 0, n, c->st));
    c->flags = (signed char *)b + XOFF;
  }
  {
    void *b = nullptr;
    TCK(cudaMalloc(&b, sizeof(double) * nz));
    c->allocs.push_back(b);
    c->u_inlet = (double *)b;
    TCK(cudaMemcpyAsync(c->u_inlet, u_inlet, sizeof(double) * nz, cudaMemcpyHostToDevice, c->st));
  }
  {
    void *b = nullptr;
    TCK(cudaMalloc(&b, sizeof(double) * (size_t)nx * ny));
    c->allocs.push_back(b);
    c->hbuf = (double *)b;
    TCK(cudaMalloc(&b, sizeof(double) * (size_t)(nx + 2) * (ny + 2) * (nz + 2)));
    c->allocs.push_back(b);
    c->stage = (double *)b;
  }
  c->part_len = (size_t)ls_iter_blocks(c->g);
  size_t d2 = (size_t)diff2_blocks(c->g, nz + 1);
  if (d2 > c->part_len) c->part_len = d2;
  {
    void *b = nullptr;
    TCK(cudaMalloc(&b, sizeof(double) * (c->part_len + FS_TAIL)));
    c->allocs.push_back(b);
    c->part = (double *)b;
    TCK(cudaMalloc(&b, sizeof(double) * SC_N));
    c->allocs.push_back(b);
    c->scal = (double *)b;
    TCK(cudaMemsetAsync(c->scal, 0, sizeof(double) * SC_N, c->st));
    TCK(cudaMallocHost(&b, sizeof(double) * SC_N));
    c->scal_host = (double *)b;
  }
  {  // state of the segment-chained odd half-sweep (FP64 coefficient records), zeroed
    const int cap = odd_chain_segments(c->g);
    const size_t nu = 4 + (size_t)cap;
    void *b = nullptr;
    TCK(cudaMalloc(&b, sizeof(unsigned) * nu));
    c->allocs.push_back(b);
    TCK(cudaMemsetAsync(b, 0, sizeof(unsigned) * nu, c->st));
    c->odd.ctr = (unsigned *)b;
    c->odd.flag = (unsigned *)b + 4;
    TCK(cudaMalloc(&b, sizeof(double) * 32 * (size_t)cap));
    c->allocs.push_back(b);
    c->odd.incl = (double *)b;
    c->odd.kto = c->scal + SC_KTO;
    c->odd.cap = cap;
  }
  TCK(poisson_create(c->g, 1.0 / (prm->dy * prm->dy), 1.0 / (prm->dx * prm->dx), 1.0 / (prm->dz * prm->dz),
                     c->mixed ? !(prm->fp64_parts & TPLS_PART_MULTIGRID) : (prm->mg_fp32 != 0), &c->ps));
  memset(&c->stats, 0, sizeof(c->stats));
  // the solver set-up's copies ran on the legacy stream, the zero fills on
  // the context's; no device-wide synchronisation (see g_dev_mu)
  TCK(cudaStreamSynchronize(cudaStreamLegacy));
  TCK(cudaStreamSynchronize(c->st));
  return TPLS_OK;
}

static size_t round_alloc(size_t b) {  // device allocations come in 2 MiB units
  const size_t u = (size_t)2 << 20;
  return (b + u - 1) / u * u;
}

long long tpls_footprint_bytes(int nx, int ny, int nz, int precision) {
  if (nx < 4 || ny < 3 || nz < 4) return -1;
  if (precision != TPLS_PREC_FP64 && precision != TPLS_PREC_FP32_MIXED) return -1;
  const size_t px = (size_t)((XOFF + nx + 2) + 3) / 4 * 4;
  const size_t np = px * (ny + 2) * (nz + 2) + 8, nuv = px * (ny + 2) * nz + 8, nw = px * (ny + 2) * (nz + 1) + 8;
  const size_t nmu = px * (ny + 4) * (nz + 2) + 8;
  const size_t nrec = (size_t)8 * px * (ny + 2);
  const size_t D = sizeof(double), F = sizeof(float);
  size_t t = 8 * round_alloc(D * np) + 14 * round_alloc(D * nuv) + 7 * round_alloc(D * nw);
  if (precision == TPLS_PREC_FP64) {
    // (+4 p-grid arrays of the diffuse-interface method, counted for every FP64 context)
    t += 9 * round_alloc(D * np) + 4 * round_alloc(D * nuv) + 2 * round_alloc(D * nw);
    t += 2 * round_alloc(D * nrec * nz) + round_alloc(D * nrec * (nz + 1)) + round_alloc(D * nmu);
  } else {
    t += 6 * round_alloc(F * np) + 6 * round_alloc(F * nuv) + 3 * round_alloc(F * nw);
    t += 2 * round_alloc(F * (nrec / 8) * nz) + round_alloc(F * (nrec / 8) * (nz + 1)) + round_alloc(F * nmu);
    t += 3 * round_alloc(4 * F * (size_t)(ny + 2) * (nz + 1));  // boundary-row offsets of the FP32 sweeps
    t += 2 * round_alloc(D * nuv) + round_alloc(D * nw);  // FP64 u3, v3, w3
    // FP64 CSF force, the FP64 iterate pair and distance of
    // TPLS_PART_LEVELSET (the setting served and batched jobs use) and the
    // FP64 viscosity of TPLS_PART_MOM_STENCIL, counted for every mixed context
    t += 3 * round_alloc(D * np) + 2 * round_alloc(D * np) + round_alloc(D * nmu);
  }
  t += round_alloc(px * (ny + 2) * (nz + 2) + 64) + round_alloc(D * nz) + round_alloc(D * nx * ny);
  t += round_alloc(D * (size_t)(nx + 2) * (ny + 2) * (nz + 2));  // host-layout staging
  Geo g;
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.sy = (int)px;
  g.sz = (int)(px * (ny + 2));
  g.szm = (int)(px * (ny + 4));
  size_t part = (size_t)ls_iter_blocks(g);
  const size_t d2 = (size_t)diff2_blocks(g, nz + 1);
  if (d2 > part) part = d2;
  t += round_alloc(D * (part + FS_TAIL)) + round_alloc(D * SC_N);
  const size_t oseg = (size_t)odd_chain_segments(g);  // odd half-sweep chain state
  t += round_alloc(sizeof(unsigned) * (4 + oseg)) + round_alloc(D * 32 * oseg);
  t += poisson_footprint(g, precision == TPLS_PREC_FP32_MIXED, round_alloc);
  return (long long)t;
}

int tpls_query(tpls_ctx *c) {
  if (!c) return TPLS_ERR_ARG;
  const cudaError_t e = cudaStreamQuery(c->st);
  if (e == cudaSuccess) return 1;
  if (e == cudaErrorNotReady) return 0;
  return TPLS_ERR_CUDA_BASE + (int)e;
}

int tpls_gpu_create(int nx, int ny, int nz, const tpls_params *prm, const double *u_inlet,
                    tpls_ctx **out) {
  if (!out || !prm || !u_inlet) return TPLS_ERR_ARG;
  *out = nullptr;
  if (nx < 4 || ny < 3 || nz < 4) return TPLS_ERR_ARG;
  const double cells = (double)(nx + 8) * (ny + 4) * (nz + 2);
  if (cells >= 2.0e9) return TPLS_ERR_ARG;  // 32-bit element offsets
  if (!(prm->dx > 0 && prm->dy > 0 && prm->dz > 0 && prm->dt > 0 && prm->re > 0 &&
        prm->smooth_width > 0))
    return TPLS_ERR_ARG;
  if (prm->precision != TPLS_PREC_FP64 && prm->precision != TPLS_PREC_FP32_MIXED) return TPLS_ERR_ARG;
  if (prm->idm != TPLS_IDM_LSM && prm->idm != TPLS_IDM_DIM) return TPLS_ERR_ARG;
  // the diffuse-interface method is built for the FP64 form
  if (prm->idm == TPLS_IDM_DIM &&
      !(prm->precision == TPLS_PREC_FP64 && prm->epn > 0 && prm->pe > 0 && prm->max_iteration_dim >= 0))
    return TPLS_ERR_ARG;
  DevLock lk(g_dev_mu);
  tpls_ctx *c = new tpls_ctx();
  int s = create_impl(nx, ny, nz, prm, u_inlet, c);
  if (s != TPLS_OK) {
    tpls_gpu_destroy(c);
    return s;
  }
  *out = c;
  return TPLS_OK;
}


// Single-field transfers use slot 0 synchronously: wait for batched
// transfers still using it.
static cudaError_t xfer_quiesce(tpls_ctx *c) {
  if (!c->xf) return cudaSuccess;
  cudaError_t e = cudaStreamSynchronize(c->xf->h2d);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->xf->d2h);
  if (e == cudaSuccess) c->xf->dl_pending = false;
  return e;
}

// Work enqueued on the context's stream after tpls_get_fields may overwrite
// the fields those downloads read: it waits for them first.
static cudaError_t xfer_fence(tpls_ctx *c) {
  if (!c->xf || !c->xf->dl_pending) return cudaSuccess;
  c->xf->dl_pending = false;
  return cudaStreamWaitEvent(c->st, c->xf->d2h_last, 0);
}

int tpls_set_field(tpls_ctx *c, int f, const double *host) {
  if (!c || !host || f < 0 || f >= TPLS_F_COUNT) return TPLS_ERR_ARG;
  double *d = field_ptr(c, f);
  if (!d) return TPLS_ERR_ARG;
  TCK(xfer_quiesce(c));
  c->front_ok = false;  // the fields change after the last step's front
  TCK(h2d(c, d, host, nz_planes(field_kind(f), c->nz)));
  TCK(cudaStreamSynchronize(c->st));
  c->need_exchange = true;
  return TPLS_OK;
}

int tpls_get_field(tpls_ctx *c, int f, double *host) {
  if (!c || !host || f < 0 || f >= TPLS_F_COUNT) return TPLS_ERR_ARG;
  double *d = field_ptr(c, f);
  if (!d) return TPLS_ERR_ARG;
  TCK(xfer_quiesce(c));
  TCK(d2h(c, host, d, nz_planes(field_kind(f), c->nz)));
  TCK(cudaStreamSynchronize(c->st));
  return TPLS_OK;
}

// Adds upload staging slots until there are n (the first is the context's
// own staging buffer).
static cudaError_t xfer_slots(tpls_ctx *c, Xfer *x, int n) {
  if ((int)x->slot.size() >= n) return cudaSuccess;
  DevLock lk(g_dev_mu);
  const size_t len = (size_t)(c->nx + 2) * (c->ny + 2) * (c->nz + 2);
  cudaError_t e = cudaSuccess;
  while ((int)x->slot.size() < n && e == cudaSuccess) {
    double *b = nullptr;
    if (x->slot.empty()) {
      b = c->stage;
    } else {
      void *v = nullptr;
      e = cudaMalloc(&v, len * sizeof(double));
      if (e != cudaSuccess) break;
      c->allocs.push_back(v);
      b = (double *)v;
    }
    cudaEvent_t fe = nullptr, re = nullptr;
    e = cudaEventCreateWithFlags(&fe, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&re, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      if (fe) cudaEventDestroy(fe);
      break;
    }
    x->slot.push_back(b);
    x->free_ev.push_back(fe);
    x->ready_ev.push_back(re);
  }
  return e;
}

static cudaError_t xfer_init(tpls_ctx *c) {
  if (c->xf) return cudaSuccess;
  DevLock lk(g_dev_mu);
  Xfer *x = new Xfer();
  cudaError_t e = cudaStreamCreateWithFlags(&x->h2d, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&x->d2h, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&x->d2h_last, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&x->st_ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&x->up_ev, cudaEventDisableTiming);
  for (int f = 0; f < TPLS_F_COUNT && e == cudaSuccess; f++)
    e = cudaEventCreateWithFlags(&x->field_dl[f], cudaEventDisableTiming);
  if (e == cudaSuccess) e = xfer_slots(c, x, 2);
  if (e != cudaSuccess) {
    xfer_destroy(x);
    return e;
  }
  c->xf = x;
  return cudaSuccess;
}

int tpls_set_fields(tpls_ctx *c, int n, const int *fields, const double *const *hosts) {
  if (!c || n < 0 || (n > 0 && (!fields || !hosts))) return TPLS_ERR_ARG;
  for (int i = 0; i < n; i++)
    if (!hosts[i] || fields[i] < 0 || fields[i] >= TPLS_F_COUNT || !field_ptr(c, fields[i])) return TPLS_ERR_ARG;
  TCK(xfer_init(c));
  Xfer *x = c->xf;
  if (n == 0) return TPLS_OK;
  // Right after a graph-launched step, the work still pending on the
  // context's stream (the back of that step) touches none of the fields
  // final after its front: those are uploaded first and repacked on the
  // copy stream as soon as the front is done, the others repacked on the
  // context's stream after the step.
  const bool early = c->front_ok;
  c->front_ok = false;  // the fields change after the last step's front
  TCK(xfer_slots(c, x, n));
  const int K = (int)x->slot.size();
  std::vector<int> order;
  order.reserve(n);
  for (int i = 0; i < n; i++)
    if (early && front_final(fields[i])) order.push_back(i);
  const size_t n_early = order.size();
  for (int i = 0; i < n; i++)
    if (!(early && front_final(fields[i]))) order.push_back(i);
  if (n_early > 0) TCK(cudaStreamWaitEvent(x->h2d, c->front_ev, 0));
  for (size_t o = 0; o < order.size(); o++) {
    const int i = order[o];
    const int f = fields[i], nzp = nz_planes(field_kind(f), c->nz);
    const int w = c->nx + 2, rows = (c->ny + 2) * nzp;
    const int q = x->next % K;
    x->next = (q + 1) % K;
    TCK(cudaStreamWaitEvent(x->h2d, x->free_ev[q], 0));
    auto hd = x->host_done.find(hosts[i]);  // a download into this array still in flight
    if (hd != x->host_done.end()) TCK(cudaStreamWaitEvent(x->h2d, hd->second, 0));
    TCK(cudaMemcpyAsync(x->slot[q], hmap(c, hosts[i], (size_t)w * rows), sizeof(double) * (size_t)w * rows,
                        cudaMemcpyDefault, x->h2d));
    if (o < n_early) {
      TCK(cudaStreamWaitEvent(x->h2d, x->field_dl[f], 0));  // a download from this field still in flight
      LCK(c, repack(x->slot[q], w, field_ptr(c, f), c->px, w, rows, x->h2d));
      TCK(cudaEventRecord(x->free_ev[q], x->h2d));
    } else {
      TCK(cudaEventRecord(x->ready_ev[q], x->h2d));
      TCK(cudaStreamWaitEvent(c->st, x->ready_ev[q], 0));
      TCK(cudaStreamWaitEvent(c->st, x->field_dl[f], 0));  // a download from this field still in flight
      LCK(c, repack(x->slot[q], w, field_ptr(c, f), c->px, w, rows, c->st));
      TCK(cudaEventRecord(x->free_ev[q], c->st));
    }
  }
  if (n_early > 0) {  // later work on the context's stream reads the early fields
    TCK(cudaEventRecord(x->up_ev, x->h2d));
    TCK(cudaStreamWaitEvent(c->st, x->up_ev, 0));
  }
  c->need_exchange = true;
  return TPLS_OK;
}

int tpls_get_fields(tpls_ctx *c, int n, const int *fields, double *const *hosts) {
  if (!c || n < 0 || (n > 0 && (!fields || !hosts))) return TPLS_ERR_ARG;
  for (int i = 0; i < n; i++)
    if (!hosts[i] || fields[i] < 0 || fields[i] >= TPLS_F_COUNT || !field_ptr(c, fields[i])) return TPLS_ERR_ARG;
  TCK(xfer_init(c));
  Xfer *x = c->xf;
  if (x->host_done.size() > 256) {  // bounded bookkeeping: settle and forget
    TCK(cudaStreamSynchronize(x->d2h));
    for (auto &kv : x->host_done) cudaEventDestroy(kv.second);
    x->host_done.clear();
  }
  if (n == 0) return TPLS_OK;
  TCK(cudaEventRecord(x->st_ev, c->st));  // the fields as of this call
  // Right after a graph-launched step, the fields final after its front are
  // copied first, as soon as the front is done (while the back runs); the
  // others after all of the step.
  std::vector<int> order;
  order.reserve(n);
  if (c->front_ok) {
    TCK(cudaStreamWaitEvent(x->d2h, c->front_ev, 0));
    for (int i = 0; i < n; i++)
      if (front_final(fields[i])) order.push_back(i);
  }
  const size_t n_front = order.size();
  for (int i = 0; i < n; i++)
    if (!(c->front_ok && front_final(fields[i]))) order.push_back(i);
  for (size_t o = 0; o < order.size(); o++) {
    const int i = order[o];
    if (o == n_front) TCK(cudaStreamWaitEvent(x->d2h, x->st_ev, 0));
    const int f = fields[i], nzp = nz_planes(field_kind(f), c->nz);
    const size_t w = (size_t)(c->nx + 2), rows = (size_t)(c->ny + 2) * nzp;
    TCK(cudaMemcpy2DAsync(hmap(c, hosts[i], w * rows), sizeof(double) * w, field_ptr(c, f),
                          sizeof(double) * (size_t)c->px, sizeof(double) * w, rows, cudaMemcpyDefault, x->d2h));
    TCK(cudaEventRecord(x->field_dl[f], x->d2h));
    cudaEvent_t &ev = x->host_done[hosts[i]];
    if (!ev) TCK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    TCK(cudaEventRecord(ev, x->d2h));
  }
  TCK(cudaEventRecord(x->d2h_last, x->d2h));
  x->dl_pending = true;
  return TPLS_OK;
}

int tpls_selftest_wait_limit(tpls_ctx *c, int *timeouts, int *nan_out) {
  if (!c || !timeouts || !nan_out) return TPLS_ERR_ARG;
  if (!c->adv_tma) return TPLS_ERR_STATE;
  DevLock lk(g_dev_mu);
  TCK(cudaStreamSynchronize(c->st));
  double *conv = nullptr, *kto = nullptr;
  const size_t n = c->n_p;
  cudaError_t e = cudaMalloc(&conv, sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMalloc(&kto, sizeof(double));
  if (e == cudaSuccess) e = cudaMemsetAsync(conv, 0, sizeof(double) * n, c->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(kto, 0, sizeof(double), c->st);
  if (e == cudaSuccess)  // no load issued: the block's wait runs out after 64 polls
    e = launch_advect_tma(c->g, c->ph, c->advmap, c->u32, c->v32, c->w32, conv + XOFF, kto, c->st, 0, 64, 1);
  double h[2] = {0.0, 0.0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h[0], kto, sizeof(double), cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess)  // the first cell of the block's tile, (1, 1, 1)
    e = cudaMemcpyAsync(&h[1], conv + XOFF + TPLS_IDX(c->g, 1, 1, 1), sizeof(double), cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  if (conv) cudaFree(conv);
  if (kto) cudaFree(kto);
  TCK(e);
  *timeouts = (int)h[0];
  *nan_out = (h[1] != h[1]) ? 1 : 0;
  return TPLS_OK;
}

int tpls_xfer_join(tpls_ctx *c) {
  if (!c) return TPLS_ERR_ARG;
  if (!c->xf) return TPLS_OK;
  TCK(cudaStreamWaitEvent(c->st, c->xf->d2h_last, 0));
  c->xf->dl_pending = false;
  return TPLS_OK;
}

int tpls_sync(tpls_ctx *c) {
  if (!c) return TPLS_ERR_ARG;
  TCK(xfer_quiesce(c));
  TCK(cudaStreamSynchronize(c->st));
  return TPLS_OK;
}

int tpls_register_host(tpls_ctx *c, double *host, long long count) {
  if (!c || !host || count <= 0) return TPLS_ERR_ARG;
  const double *h = host;
  auto it = c->hreg.upper_bound(h);  // no overlap with a registered array
  if (it != c->hreg.end() && it->first < h + count) return TPLS_ERR_ARG;
  if (it != c->hreg.begin()) {
    --it;
    if (h < it->first + it->second.count) return TPLS_ERR_ARG;
  }
  DevLock lk(g_dev_mu);
  TCK(xfer_quiesce(c));
  TCK(cudaStreamSynchronize(c->st));
  void *m = nullptr;
  TCK(cudaMalloc(&m, sizeof(double) * (size_t)count));
  const cudaError_t e = cudaMemcpyAsync(m, host, sizeof(double) * (size_t)count, cudaMemcpyDefault, c->st);
  const cudaError_t e2 = (e == cudaSuccess) ? cudaStreamSynchronize(c->st) : e;
  if (e2 != cudaSuccess) {
    cudaFree(m);
    return TPLS_ERR_CUDA_BASE + (int)e2;
  }
  c->hreg[h] = HostReg{(double *)m, (size_t)count};
  return TPLS_OK;
}

// host == nullptr: every registered array
static int host_refresh(tpls_ctx *c, const double *host, bool down) {
  if (!c) return TPLS_ERR_ARG;
  TCK(xfer_quiesce(c));
  bool found = false;
  for (auto &kv : c->hreg) {
    if (host && kv.first != host) continue;
    found = true;
    double *h = const_cast<double *>(kv.first);
    const size_t bytes = sizeof(double) * kv.second.count;
    if (down) TCK(cudaMemcpyAsync(h, kv.second.mirror, bytes, cudaMemcpyDefault, c->st));
    else TCK(cudaMemcpyAsync(kv.second.mirror, h, bytes, cudaMemcpyDefault, c->st));
  }
  if (host && !found) return TPLS_ERR_ARG;
  TCK(cudaStreamSynchronize(c->st));
  return TPLS_OK;
}

int tpls_download_host(tpls_ctx *c, double *host) { return host_refresh(c, host, true); }
int tpls_upload_host(tpls_ctx *c, const double *host) { return host_refresh(c, host, false); }

int tpls_unregister_host(tpls_ctx *c, double *host) {
  if (!c || !host) return TPLS_ERR_ARG;
  auto it = c->hreg.find(host);
  if (it == c->hreg.end()) return TPLS_ERR_ARG;
  DevLock lk(g_dev_mu);
  TCK(xfer_quiesce(c));
  TCK(cudaStreamSynchronize(c->st));
  cudaFree(it->second.mirror);
  c->hreg.erase(it);
  return TPLS_OK;
}

long tpls_kernel_launches(tpls_ctx *c) {
  if (!c) return -1;
  if (refresh_graph_stats(c) != TPLS_OK) return -1;
  return c->launches;
}

extern "C++" {
// Begin and end of one component's FP32 defect-form momentum solve: d = -X
// and the boundary-row offsets before the sweeps; x = X + d into the FP64
// u3 / v3 / w3 and the logged get_difference of the last two iterates after
// them.  Shared by momentum<float> and the multi-instance sweeps of a batch.
static const double *mom32_base(tpls_ctx *c, int comp) { return comp == 0 ? c->u2 : (comp == 1 ? c->v2 : c->w2); }
static size_t mom32_len(tpls_ctx *c, int comp) {
  return (size_t)c->px * (c->ny + 2) * nz_planes(comp == 2 ? 2 : 1, c->nz) + 8;
}
static int mom32_iters(tpls_ctx *c, int comp) {
  return (comp == 0 ? c->prm.mom_u : (comp == 1 ? c->prm.mom_v : c->prm.mom_w)) / 2;
}
static int mom32_begin(tpls_ctx *c, int comp) {
  const double *base = mom32_base(c, comp);
  LCK(c, launch_defect_init(base - XOFF, c->x3f[comp][0] - XOFF, mom32_len(c, comp), c->st));
  LCK(c, launch_bc32_prep(comp, c->g, c->ph, base, c->pres, c->bco32[comp], c->st));
  return TPLS_OK;
}
static int mom32_end(tpls_ctx *c, int comp, int N) {
  float **X = c->x3f[comp];
  const int nzp = nz_planes(comp == 2 ? 2 : 1, c->nz);
  LCK(c, launch_defect_apply(mom32_base(c, comp) - XOFF, X[N % 2] - XOFF, c->x3[comp][0] - XOFF,
                             mom32_len(c, comp), c->st));
  if (N >= 1) {
    LCK(c, launch_diff2(c->g, X[N % 2], X[(N - 1) % 2], nzp, c->part, c->st));
    FSUM(c, c->part, diff2_blocks(c->g, nzp), c->scal + SC_ERR_U + comp, c->st);
  } else {
    TCK(cudaMemsetAsync(c->scal + SC_ERR_U + comp, 0, sizeof(double), c->st));
  }
  c->x3_final[comp] = 0;
  return TPLS_OK;
}

// One velocity component's Crank-Nicolson solve (main_ns_hybrid.F90:756-887)
// on the iterate pair X: FP64, or in the FP32-mixed form the FP32 defect
// d = x - base (base = the component's FP64 state), iterated from d = -base
// (x = 0, the reference's start) and added back into out64 at the end.
template <typename T, typename CS>
static int momentum(tpls_ctx *c, int comp, CS coef, T **X, int max_iteration, const double *base = nullptr,
                    double *out64 = nullptr) {
  const Geo &g = c->g;
  const int nzp = nz_planes(comp == 2 ? 2 : 1, c->nz);
  const int fuse = (g.ny % 2 == 0);
  const size_t n = (size_t)c->px * (c->ny + 2) * nzp + 8;
  if constexpr (sizeof(T) == sizeof(float)) {
    int s = mom32_begin(c, comp);
    if (s) return s;
  } else {
    TCK(cudaMemsetAsync(X[0] - XOFF, 0, sizeof(T) * n, c->st));
  }
  const SweepTiles tl = c->tiles;
  auto jac = [&](const T *src, T *dst) {
    if constexpr (sizeof(T) == sizeof(float)) return launch_jacobi_c(comp, g, c->ph, src, coef, c->pres, base, dst,
                                                                      fuse, c->st, tl);
    else return launch_jacobi_c(comp, g, c->ph, src, coef, c->pres, dst, fuse, c->st, tl);
  };
  auto sor = [&](T *x, int flg, int it, int bc) {
    if constexpr (sizeof(T) == sizeof(float)) return launch_sor_c(comp, g, c->ph, x, coef, c->pres, base, flg, it,
                                                                   bc, fuse, c->st, tl, odd_chain(c));
    else return launch_sor_c(comp, g, c->ph, x, coef, c->pres, flg, it, bc, fuse, c->st, tl, odd_chain(c));
  };
  const int N = max_iteration / 2;
  for (int it = 1; it <= N; it++) {
    T *src = X[(it - 1) % 2], *dst = X[it % 2];
    {
      PhaseScope ps(c, TPLS_T_JACOBI);
      LCK(c, jac(src, dst));
    }
    if (!fuse) LCK(c, launch_exchange(g, dst, nzp, c->st));
    {
      PhaseScope ps(c, (it % 2) ? TPLS_T_SOR_ODD : TPLS_T_SOR);
      LCK(c, sor(dst, 0, it, 0));
    }
    if (!fuse) LCK(c, launch_exchange(g, dst, nzp, c->st));
    {
      PhaseScope ps(c, (it % 2) ? TPLS_T_SOR_ODD : TPLS_T_SOR);
      LCK(c, sor(dst, 1, it, 1));
    }
    if (!fuse) LCK(c, launch_exchange(g, dst, nzp, c->st));
  }
  if constexpr (sizeof(T) == sizeof(float)) {
    return mom32_end(c, comp, N);
  }
  c->x3_final[comp] = N % 2;
  const int nb = diff2_blocks(g, nzp);
  if (N >= 1) {
    LCK(c, launch_diff2(g, X[N % 2], X[(N - 1) % 2], nzp, c->part, c->st));
    FSUM(c, c->part, nb, c->scal + SC_ERR_U + comp, c->st);
  } else {
    TCK(cudaMemsetAsync(c->scal + SC_ERR_U + comp, 0, sizeof(double), c->st));
  }
  return TPLS_OK;
}
}  // extern "C++"

// Periodic y rows of the velocity state after a host upload
// (advect_phi.f90:317-322 / main_ns_hybrid.F90:728-733); later steps keep
// them current in the kernels that write the state.
static int prologue(tpls_ctx *c) {
  TCK(xfer_fence(c));
  if (c->need_exchange) {
    LCK(c, launch_exchange(c->g, c->u2, c->nz, c->st));
    LCK(c, launch_exchange(c->g, c->v2, c->nz, c->st));
    LCK(c, launch_exchange(c->g, c->w2, c->nz + 1, c->st));
    c->need_exchange = false;
  }
  return TPLS_OK;
}

// Pressure solve of the step (main_ns_hybrid.F90:897-913): host-driven
// iterations when launching eagerly, a WHILE node when capturing.
static int pressure_stage(tpls_ctx *c, const void *u3, int u3_fp32, int *its, double *rn, double *bn,
                          int *reason) {
  *its = 0;
  *rn = *bn = 0.0;
  *reason = 0;
  if (c->capturing) {
    long ns = 0, nb = 0;
    TCK(poisson_solve_capture(c->ps, c->g, c->ph, c->rhs_p, u3, u3_fp32, c->u_inlet, c->pres_old, c->pres,
                              c->prm.p_rtol, c->prm.p_maxits, c->st, &ns, &nb));
    c->launches += ns;
    c->g_body = nb;
    return TPLS_OK;
  }
  const long l0 = c->launches;
  TCK(poisson_solve(c->ps, c->g, c->ph, c->rhs_p, u3, u3_fp32, c->u_inlet, c->pres_old, c->pres, c->prm.p_rtol,
                    c->prm.p_maxits, its, rn, bn, reason, c->st, &c->launches));
  c->t_n[TPLS_T_PRESSURE] += c->launches - l0;
  c->its_accounted += *its;
  return TPLS_OK;
}

// Bookkeeping after an eagerly launched step.
static int finish_eager(tpls_ctx *c, int its, double rn, double bn, int reason) {
  if (c->timing) timing_flush(c);
  c->phase = (c->phase + 1) % 3;
  c->stats.p_its = its;
  c->stats.p_rnorm = rn;
  c->stats.p_bnorm = bn;
  c->stats.p_reason = reason;
  if (reason < c->stats.p_worst) c->stats.p_worst = reason;
  c->stats.steps_done++;
  if (reason < 0) return reason;
  return TPLS_OK;
}

// Diffuse-interface update of one step (main_ns_hybrid.F90:608-611): dim on
// C = phi2 + 0.5 (phi_old equals phi2 at every step, :444 and :2508) from
// the starting guess phi3, then phi3 = phiNew - 0.5 into phi2 and phi3.
// The reference logs no residual for it; err_phi reads 0.
static int dim_stage(tpls_ctx *c, const double *conv2_phi) {
  const Geo &g = c->g;
  cudaStream_t st = c->st;
  const DimK q = dim_constants(c->ph, c->prm.epn, c->prm.pe);
  LCK(c, launch_dim_prep(g, q, c->phi2, 0.5, c->dimE, c->D, st));
  LCK(c, launch_dim_source(g, q, c->phi2, 0.5, c->dimE, c->D, conv2_phi, c->convprev, c->dimS, st));
  const double *pin = c->phi3d;
  double *pp[2] = {c->phiA, c->phiB};
  for (int it = 1; it <= c->prm.max_iteration_dim; it++) {
    double *out = pp[(it - 1) % 2];
    LCK(c, launch_dim_lap(g, q, pin, c->D, st));
    LCK(c, launch_dim_update(g, q, c->phi2, 0.5, c->phi2, 0.5, c->dimS, pin, c->D, out, st));
    pin = out;
  }
  LCK(c, launch_dim_finish(g, pin, c->phi2, c->phi3d, st));
  TCK(cudaMemsetAsync(c->scal + SC_ERR_PHI, 0, sizeof(double), st));
  return TPLS_OK;
}

// The front of a step: viscosity, advection, level set, CSF and the
// momentum right-hand sides.  Every state field but u2, v2, w2, pres and
// pres_old is final after it (front_final).
static int step_front(tpls_ctx *c) {
  const Geo &g = c->g;
  const Phys &ph = c->ph;
  cudaStream_t st = c->st;
  const int s0 = c->phase % 3, s1 = (c->phase + 1) % 3, s2 = (c->phase + 2) % 3;
  // viscosity from the pre-advection level set (main_ns_hybrid.F90:646-724);
  // the diffuse-interface method passes phi2-0.5
  {
    PhaseScope ps(c, TPLS_T_VISC);
    LCK(c, launch_visc(g, ph, c->phi2, c->mu, st, c->dim ? -0.5 : 0.0));
  }
  // advection (:585) and level-set update + redistancing (:596)
  {
    PhaseScope ps(c, TPLS_T_ADVECT);
    LCK(c, launch_advect(g, ph, c->phi2, c->u2, c->v2, c->w2, c->conv_phi[s2], st));
  }
  {
    PhaseScope ls_scope(c, TPLS_T_LEVELSET);
    if (c->dim) {
      int sd;
      if ((sd = dim_stage(c, c->conv_phi[s2]))) return sd;
    } else {
      LCK(c, launch_ls_ab3(g, ph, c->phi2, c->conv_phi[s0], c->conv_phi[s1], c->conv_phi[s2], c->phiA, st));
      LCK(c, launch_ls_status(g, ph, c->phiA, c->D, c->flags, st));
      const int L = c->prm.levelset;
      if (L <= 0) {
        TCK(cudaMemcpyAsync(c->phi2 - XOFF, c->phiA - XOFF,
                            sizeof(double) * ((size_t)c->px * (c->ny + 2) * (c->nz + 2)), cudaMemcpyDeviceToDevice, st));
        TCK(cudaMemsetAsync(c->scal + SC_ERR_PHI, 0, sizeof(double), st));
      }
      for (int it = 1; it <= L; it++) {
        const double *src = (it == 1) ? c->phiA : ((it % 2 == 0) ? c->phiB : c->phiA);
        double *dst = (it == L) ? c->phi2 : ((it % 2 == 1) ? c->phiB : c->phiA);
        LCK(c, launch_ls_iter(g, ph, src, c->D, c->flags, dst, (it == L) ? c->part : nullptr, st));
      }
      if (L > 0) FSUM(c, c->part, ls_iter_blocks(g), c->scal + SC_ERR_PHI, st);
    }
  }
  // CSF from the redistanced phi3 (:618-641)
  {
    PhaseScope ps(c, TPLS_T_CSF);
    LCK(c, launch_csf(g, ph, c->phi2, c->fx, c->fy, c->fz, st));
  }
  {
    PhaseScope rhs_scope(c, TPLS_T_MOM_RHS);
    // convective / diffusive terms and AB3 + CN right-hand sides (:728-751)
    LCK(c, launch_mom_rhs(0, g, ph, c->u2, c->v2, c->w2, c->mu, c->fx, c->conv_u[s1], c->conv_u[s0],
                          c->csf_u[s1], c->csf_u[s0], c->conv_u[s2], c->csf_u[s2], nullptr, nullptr, c->coef[0],
                          st));
    LCK(c, launch_mom_rhs(1, g, ph, c->u2, c->v2, c->w2, c->mu, c->fy, c->conv_v[s1], c->conv_v[s0],
                          c->csf_v[s1], c->csf_v[s0], c->conv_v[s2], c->csf_v[s2], nullptr, nullptr, c->coef[1],
                          st));
    LCK(c, launch_mom_rhs(2, g, ph, c->u2, c->v2, c->w2, c->mu, c->fz, c->conv_w[s1], c->conv_w[s0],
                          c->csf_w[s1], c->csf_w[s0], c->conv_w[s2], c->csf_w[s2], nullptr, nullptr, c->coef[2],
                          st));
  }
  return TPLS_OK;
}

// The back of a step: momentum sweeps, pressure solve, projection.
static int step_back(tpls_ctx *c) {
  const Geo &g = c->g;
  const Phys &ph = c->ph;
  cudaStream_t st = c->st;
  // momentum sweeps (:756-887)
  int s;
  if ((s = momentum<double, const double *>(c, 0, c->coef[0], c->x3[0], c->prm.mom_u))) return s;
  if ((s = momentum<double, const double *>(c, 1, c->coef[1], c->x3[1], c->prm.mom_v))) return s;
  if ((s = momentum<double, const double *>(c, 2, c->coef[2], c->x3[2], c->prm.mom_w))) return s;
  double *u3 = c->x3[0][c->x3_final[0]], *v3 = c->x3[1][c->x3_final[1]], *w3 = c->x3[2][c->x3_final[2]];
  // pressure source (:892) and solve (:897-913)
  int its = 0, reason = 0;
  double rn = 0.0, bn = 0.0;
  {
    PhaseScope ps(c, TPLS_T_PRESSURE);
    LCK(c, launch_source(g, ph, u3, v3, w3, c->rhs_p, st));
    if ((s = pressure_stage(c, u3, 0, &its, &rn, &bn, &reason))) return s;
  }
  // projection into the next state's velocity arrays (:918)
  {
    PhaseScope ps(c, TPLS_T_PROJECT);
    LCK(c, launch_project(g, ph, u3, v3, w3, c->pres, c->u_inlet, c->u2, c->v2, c->w2, st));
    // history rotation (:2480-2509)
    TCK(cudaMemcpyAsync(c->pres_old - XOFF, c->pres - XOFF,
                        sizeof(double) * ((size_t)c->px * (c->ny + 2) * (c->nz + 2)), cudaMemcpyDeviceToDevice, st));
  }
  if (c->capturing) return TPLS_OK;
  return finish_eager(c, its, rn, bn, reason);
}

static int step_once(tpls_ctx *c) {
  const int s = step_front(c);
  return s ? s : step_back(c);
}

// FP32-mixed timestep: the same sequence as step_once with the stencils,
// the redistancing iterations, the momentum sweeps and the multigrid
// preconditioner in FP32.  The state (phi, u, v, w, p, the AB3 histories),
// the AB3 updates, the momentum right-hand sides, the CG recurrences and the
// projection stay FP64; every FP32 array is a rounded copy or an
// intermediate of one step.
// the three FP32 defect-form momentum solves of the FP32-mixed step, the
// FP64 results in x3[q][0]
static int sweeps32(tpls_ctx *c) {
  int s;
  const Phys &ph = c->ph;
  if ((s = momentum<float>(c, 0, mu_coef(ph, c->mu32, c->bdef[0], c->bco32[0]), c->x3f[0], c->prm.mom_u, c->u2, c->x3[0][0])))
    return s;
  if ((s = momentum<float>(c, 1, mu_coef(ph, c->mu32, c->bdef[1], c->bco32[1]), c->x3f[1], c->prm.mom_v, c->v2, c->x3[1][0])))
    return s;
  if ((s = momentum<float>(c, 2, mu_coef(ph, c->mu32, c->bdef[2], c->bco32[2]), c->x3f[2], c->prm.mom_w, c->w2, c->x3[2][0])))
    return s;
  for (int q = 0; q < 3; q++) c->x3_final[q] = 0;
  return TPLS_OK;
}

// The FP32-mixed step in three stages: the front (viscosity, advection,
// level set, CSF and the momentum right-hand sides, and the FP64 sweeps when
// the momentum part is kept in FP64), the FP32 momentum solves (sweeps32, or
// the multi-instance launches of a batch) and the back (pressure solve and
// projection).
static bool mixed_fp32_sweeps(const tpls_ctx *c) { return !(c->prm.fp64_parts & TPLS_PART_MOMENTUM); }

static int mixed_front(tpls_ctx *c) {
  const Geo &g = c->g;
  const Phys &ph = c->ph;
  cudaStream_t st = c->st;
  const int s0 = c->phase % 3, s1 = (c->phase + 1) % 3, s2 = (c->phase + 2) % 3;
  const int parts = c->prm.fp64_parts;
  const bool adv64 = parts & TPLS_PART_ADVECT, ls64 = parts & TPLS_PART_LEVELSET;
  const bool mom64 = parts & TPLS_PART_MOMENTUM;
  const bool sten64 = mom64 || (parts & TPLS_PART_MOM_STENCIL);
  {
    PhaseScope ps(c, TPLS_T_VISC);
    if (sten64) LCK(c, launch_visc(g, ph, c->phi2, c->mu, st));
    // the FP32 sweeps recompute their coefficients from the FP32 viscosity
    if (!mom64) LCK(c, launch_visc(g, ph, c->phi2, c->mu32, st));
  }
  {
    PhaseScope ps(c, TPLS_T_ADVECT);
    if (!adv64) {  // FP32 copies of the velocity state for the FP32 WENO5
      LCK(c, launch_to_float(c->u2 - XOFF, c->u32 - XOFF, c->n_uv, st));
      LCK(c, launch_to_float(c->v2 - XOFF, c->v32 - XOFF, c->n_uv, st));
      LCK(c, launch_to_float(c->w2 - XOFF, c->w32 - XOFF, c->n_w, st));
    }
    if (adv64) {
      LCK(c, launch_advect(g, ph, c->phi2, c->u2, c->v2, c->w2, c->conv_phi[s2], st));
    } else {
      LCK(c, launch_to_float(c->phi2 - XOFF, c->phi32 - XOFF, c->n_p, st));
      if (c->adv_tma)  // phi tiles staged by TMA (same arithmetic, bit-identical)
        LCK(c, launch_advect_tma(g, ph, c->advmap, c->u32, c->v32, c->w32, c->conv_phi[s2], c->scal + SC_KTO, st));
      else
        LCK(c, launch_advect(g, ph, (const float *)c->phi32, c->u32, c->v32, c->w32, c->conv_phi[s2], st));
    }
  }
  {
    PhaseScope ls_scope(c, TPLS_T_LEVELSET);
    LCK(c, launch_ls_ab3(g, ph, c->phi2, c->conv_phi[s0], c->conv_phi[s1], c->conv_phi[s2], c->phiA, st));
    const int L = c->prm.levelset;
    if (ls64) LCK(c, launch_ls_status(g, ph, c->phiA, c->D, c->flags, st));
    else LCK(c, launch_ls_status(g, ph, c->phiA, c->D32, c->flags, st));
    if (L <= 0) {
      TCK(cudaMemcpyAsync(c->phi2 - XOFF, c->phiA - XOFF, sizeof(double) * c->n_p, cudaMemcpyDeviceToDevice, st));
      TCK(cudaMemsetAsync(c->scal + SC_ERR_PHI, 0, sizeof(double), st));
    }
    for (int it = 1; it <= L; it++) {
      double *ep = (it == L) ? c->part : nullptr;
      if (ls64) {
        const double *src = (it == 1) ? c->phiA : ((it % 2 == 0) ? c->phiB : c->phiA);
        double *dst = (it == L) ? c->phi2 : ((it % 2 == 1) ? c->phiB : c->phiA);
        LCK(c, launch_ls_iter(g, ph, src, c->D, c->flags, dst, ep, st));
      } else {  // FP32 increments on float-pair iterates: it reads pair it%2, writes pair (it+1)%2
        const int ri = it % 2, wi = (it + 1) % 2;
        LCK(c, launch_ls_iter_ff(g, ph, (it == 1) ? c->phiA : nullptr, c->ffh[ri], c->ffl[ri], c->D32, c->flags,
                                 (it == L) ? c->phi2 : nullptr, c->ffh[wi], c->ffl[wi], ep, st));
      }
    }
    if (L > 0) FSUM(c, c->part, ls_iter_blocks(g), c->scal + SC_ERR_PHI, st);
  }
  int s;
  if (mom64) {
    {
      PhaseScope ps(c, TPLS_T_CSF);
      LCK(c, launch_csf(g, ph, c->phi2, c->fx, c->fy, c->fz, st));
    }
    {
      PhaseScope ps(c, TPLS_T_MOM_RHS);
      LCK(c, launch_mom_rhs(0, g, ph, c->u2, c->v2, c->w2, c->mu, c->fx, c->conv_u[s1], c->conv_u[s0],
                            c->csf_u[s1], c->csf_u[s0], c->conv_u[s2], c->csf_u[s2], nullptr, nullptr, c->coef[0],
                            st));
      LCK(c, launch_mom_rhs(1, g, ph, c->u2, c->v2, c->w2, c->mu, c->fy, c->conv_v[s1], c->conv_v[s0],
                            c->csf_v[s1], c->csf_v[s0], c->conv_v[s2], c->csf_v[s2], nullptr, nullptr, c->coef[1],
                            st));
      LCK(c, launch_mom_rhs(2, g, ph, c->u2, c->v2, c->w2, c->mu, c->fz, c->conv_w[s1], c->conv_w[s0],
                            c->csf_w[s1], c->csf_w[s0], c->conv_w[s2], c->csf_w[s2], nullptr, nullptr, c->coef[2],
                            st));
    }
    if ((s = momentum<double, const double *>(c, 0, c->coef[0], c->x3[0], c->prm.mom_u))) return s;
    if ((s = momentum<double, const double *>(c, 1, c->coef[1], c->x3[1], c->prm.mom_v))) return s;
    if ((s = momentum<double, const double *>(c, 2, c->coef[2], c->x3[2], c->prm.mom_w))) return s;
  } else if (sten64) {
    {
      PhaseScope ps(c, TPLS_T_CSF);
      LCK(c, launch_csf(g, ph, c->phi2, c->fx, c->fy, c->fz, st));
    }
    {
      PhaseScope ps(c, TPLS_T_MOM_RHS);
      LCK(c, launch_mom_rhs64r32(0, g, ph, c->u2, c->v2, c->w2, c->mu, c->fx, c->conv_u[s1], c->conv_u[s0],
                                 c->csf_u[s1], c->csf_u[s0], c->conv_u[s2], c->csf_u[s2], c->bdef[0], st));
      LCK(c, launch_mom_rhs64r32(1, g, ph, c->u2, c->v2, c->w2, c->mu, c->fy, c->conv_v[s1], c->conv_v[s0],
                                 c->csf_v[s1], c->csf_v[s0], c->conv_v[s2], c->csf_v[s2], c->bdef[1], st));
      LCK(c, launch_mom_rhs64r32(2, g, ph, c->u2, c->v2, c->w2, c->mu, c->fz, c->conv_w[s1], c->conv_w[s0],
                                 c->csf_w[s1], c->csf_w[s0], c->conv_w[s2], c->csf_w[s2], c->bdef[2], st));
    }
  } else {
    {
      PhaseScope ps(c, TPLS_T_CSF);
      LCK(c, launch_csf(g, ph, c->phi2, c->fx, c->fy, c->fz, st));
    }
    {
      PhaseScope ps(c, TPLS_T_MOM_RHS);
      LCK(c, launch_mom_rhs_pair(0, g, ph, c->u2, c->v2, c->w2, c->mu32, c->fx, c->conv_u[s1], c->conv_u[s0],
                                 c->csf_u[s1], c->csf_u[s0], c->conv_u[s2], c->csf_u[s2], c->bdef[0], st));
      LCK(c, launch_mom_rhs_pair(1, g, ph, c->u2, c->v2, c->w2, c->mu32, c->fy, c->conv_v[s1], c->conv_v[s0],
                                 c->csf_v[s1], c->csf_v[s0], c->conv_v[s2], c->csf_v[s2], c->bdef[1], st));
      LCK(c, launch_mom_rhs_pair(2, g, ph, c->u2, c->v2, c->w2, c->mu32, c->fz, c->conv_w[s1], c->conv_w[s0],
                                 c->csf_w[s1], c->csf_w[s0], c->conv_w[s2], c->csf_w[s2], c->bdef[2], st));
    }
  }
  return TPLS_OK;
}

static int mixed_back(tpls_ctx *c) {
  const Geo &g = c->g;
  const Phys &ph = c->ph;
  cudaStream_t st = c->st;
  const void *u3v = c->x3[0][c->x3_final[0]], *v3v = c->x3[1][c->x3_final[1]], *w3v = c->x3[2][c->x3_final[2]];
  int s;
  int its = 0, reason = 0;
  double rn = 0.0, bn = 0.0;
  {
    PhaseScope ps(c, TPLS_T_PRESSURE);
    LCK(c, launch_source(g, ph, (const double *)u3v, (const double *)v3v, (const double *)w3v, c->rhs_p, st));
    if ((s = pressure_stage(c, u3v, 0, &its, &rn, &bn, &reason))) return s;
  }
  {
    PhaseScope ps(c, TPLS_T_PROJECT);
    LCK(c, launch_project(g, ph, (const double *)u3v, (const double *)v3v, (const double *)w3v, c->pres,
                          c->u_inlet, c->u2, c->v2, c->w2, st));
    TCK(cudaMemcpyAsync(c->pres_old - XOFF, c->pres - XOFF, sizeof(double) * c->n_p, cudaMemcpyDeviceToDevice,
                        st));
  }
  if (c->capturing) return TPLS_OK;
  return finish_eager(c, its, rn, bn, reason);
}

static int step_back_mixed(tpls_ctx *c) {
  int s;
  if (mixed_fp32_sweeps(c) && (s = sweeps32(c))) return s;
  return mixed_back(c);
}

static int step_once_mixed(tpls_ctx *c) {
  const int s = mixed_front(c);
  return s ? s : step_back_mixed(c);
}

// Captures one part of a step into an executable graph; *n: the kernels it
// launches outside the CG loop body.
static int capture_part(tpls_ctx *c, int (*part)(tpls_ctx *), cudaGraphExec_t *out, long *n) {
  const long l0 = c->launches;
  TCK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
  c->capturing = true;
  const int s = part(c);
  c->capturing = false;
  cudaGraph_t gr = nullptr;
  const cudaError_t e = cudaStreamEndCapture(c->st, &gr);
  *n = c->launches - l0;
  c->launches = l0;
  if (s != TPLS_OK || e != cudaSuccess) {
    if (gr) cudaGraphDestroy(gr);
    return s != TPLS_OK ? s : TPLS_ERR_CUDA_BASE + (int)e;
  }
  const cudaError_t ei = cudaGraphInstantiate(out, gr, 0);
  cudaGraphDestroy(gr);
  TCK(ei);
  return TPLS_OK;
}

// One step as two CUDA-graph launches (front, back) with front_ev recorded
// between them, so the fields final after the front can be downloaded while
// the back runs; the graphs of this history phase are captured from the
// eager sequence on first use.
static int step_graph(tpls_ctx *c) {
  int s = prologue(c);
  if (s) return s;
  const int ph = c->phase;
  if (!c->gexec[ph] || !c->gexec_back[ph]) {
    DevLock lk(g_dev_mu);
    long nf = 0, nb = 0;
    if (!c->gexec[ph] && (s = capture_part(c, c->mixed ? mixed_front : step_front, &c->gexec[ph], &nf))) return s;
    if ((s = capture_part(c, c->mixed ? step_back_mixed : step_back, &c->gexec_back[ph], &nb))) {
      cudaGraphExecDestroy(c->gexec[ph]);
      c->gexec[ph] = nullptr;
      return s;
    }
    c->g_static[ph] = nf + nb;
  }
  TCK(cudaGraphLaunch(c->gexec[ph], c->st));
  TCK(cudaEventRecord(c->front_ev, c->st));
  TCK(cudaGraphLaunch(c->gexec_back[ph], c->st));
  c->front_ok = true;
  c->launches += c->g_static[ph];
  c->phase = (ph + 1) % 3;
  c->stats.steps_done++;
  c->graph_pending = true;
  return TPLS_OK;
}

// Reads the outcome of graph-launched solves (synchronises): last solve's
// figures, the lowest reason since the previous read, and the CG-loop
// kernels into the launch count.
static int refresh_graph_stats(tpls_ctx *c) {
  if (!c->graph_pending) return TPLS_OK;
  int its, reason, worst;
  double rn, bn, total;
  TCK(poisson_read(c->ps, c->st, &its, &rn, &bn, &reason, &worst, &total));
  TCK(poisson_reset_worst(c->ps, c->st));
  c->stats.p_its = its;
  c->stats.p_rnorm = rn;
  c->stats.p_bnorm = bn;
  c->stats.p_reason = reason;
  if (worst < c->stats.p_worst) c->stats.p_worst = worst;
  c->launches += (long)(total - c->its_accounted) * c->g_body;
  c->its_accounted = total;
  c->graph_pending = false;
  return TPLS_OK;
}

static bool graph_path(const tpls_ctx *c) { return c->use_graphs && !c->timing; }

// A pressure solve that reaches p_maxits (KSP_DIVERGED_ITS) does not stop
// the run, as in the reference's time loop; the status of such a step is
// returned after the remaining steps.  A NaN residual, an argument or a CUDA
// error stops at the failing step (graph launches: at the end of the call).
int tpls_step(tpls_ctx *c, int nsteps) {
  if (!c || nsteps < 0) return TPLS_ERR_ARG;
  if (graph_path(c)) {
    for (int n = 0; n < nsteps; n++) {
      int s = step_graph(c);
      if (s) return s;
    }
    TCK(cudaStreamSynchronize(c->st));
    int s = refresh_graph_stats(c);
    if (s) return s;
    const int worst = c->stats.p_worst;
    c->stats.p_worst = 0;
    return worst < 0 ? worst : TPLS_OK;
  }
  int worst = TPLS_OK;
  c->front_ok = false;
  for (int n = 0; n < nsteps; n++) {
    int s = prologue(c);
    if (s) return s;
    s = c->mixed ? step_once_mixed(c) : step_once(c);
    if (s == TPLS_KSP_DIVERGED_ITS) {
      worst = s;
      continue;
    }
    if (s != TPLS_OK) return s;
  }
  c->stats.p_worst = 0;
  return worst;
}

int tpls_step_async(tpls_ctx *c, int nsteps) {
  if (!c || nsteps < 0) return TPLS_ERR_ARG;
  if (!graph_path(c)) return tpls_step(c, nsteps);
  for (int n = 0; n < nsteps; n++) {
    int s = step_graph(c);
    if (s) return s;
  }
  return TPLS_OK;
}

// ---------------------------------------------------------------------------
// Tile-shape autotuner of the momentum sweeps: each candidate block shape of
// the Jacobi and even half-sweep kernels is timed with CUDA events on the
// context's own records and iterate arrays (reps launches of the u
// component), the fastest kept.  Results are cached per (grid, sweep
// precision) for the process, so batch members of one shape tune once.
}  // extern "C"

static std::mutex g_tune_mu;
static std::map<std::array<int, 4>, SweepTiles> g_tune_cache;

extern "C" {

static void destroy_graphs(tpls_ctx *c) {
  for (cudaGraphExec_t &ge : c->gexec)
    if (ge) {
      cudaGraphExecDestroy(ge);
      ge = nullptr;
    }
  for (cudaGraphExec_t &ge : c->gexec_back)
    if (ge) {
      cudaGraphExecDestroy(ge);
      ge = nullptr;
    }
}

int tpls_autotune(tpls_ctx *c, int reps) {
  if (!c || c->capturing || reps < 1) return TPLS_ERR_ARG;
  TCK(xfer_fence(c));
  c->front_ok = false;
  const bool f32 = c->mixed && !(c->prm.fp64_parts & TPLS_PART_MOMENTUM);
  const std::array<int, 4> key = {c->nx, c->ny, c->nz, f32 ? 1 : 0};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      TCK(cudaStreamSynchronize(c->st));
      c->tiles = it->second;
      c->tune_version++;
      destroy_graphs(c);
      return TPLS_OK;
    }
  }
  TCK(cudaStreamSynchronize(c->st));
  const Geo &g = c->g;
  const int fuse = (g.ny % 2 == 0);
  cudaEvent_t e0, e1;
  TCK(cudaEventCreate(&e0));
  TCK(cudaEventCreate(&e1));
  auto launch = [&](int kind, const SweepTiles &t) -> cudaError_t {
    // kind 0: Jacobi, 1: even half-sweep, 2: odd half-sweep (component u)
    if (f32) {
      float *a = c->x3f[0][0], *b = c->x3f[0][1];
      const MuCoef mc = mu_coef(c->ph, c->mu32, c->bdef[0], c->bco32[0]);
      if (kind == 0) return launch_jacobi_c(0, g, c->ph, a, mc, c->pres, c->u2, b, fuse, c->st, t);
      return launch_sor_c(0, g, c->ph, b, mc, c->pres, c->u2, 0, kind == 1 ? 2 : 1, 1, fuse, c->st, t);
    }
    double *a = c->x3[0][0], *b = c->x3[0][1];
    if (kind == 0) return launch_jacobi_c(0, g, c->ph, a, c->coef[0], c->pres, b, fuse, c->st, t);
    return launch_sor_c(0, g, c->ph, b, c->coef[0], c->pres, 0, kind == 1 ? 2 : 1, 1, fuse, c->st, t, odd_chain(c));
  };
  SweepTiles best = c->tiles;
  // The odd half-sweep's chunking changes its rounding, so it is not tuned:
  // a result must not depend on the tile shapes chosen.
  const int ncand[2] = {4, 4};
  cudaError_t err = cudaSuccess;
  for (int kind = 0; kind < 2 && err == cudaSuccess; kind++) {
    float tbest = 1e30f;
    for (int v = 0; v < ncand[kind] && err == cudaSuccess; v++) {
      SweepTiles t = best;
      if (kind == 0) t.jac = v;
      else if (kind == 1) t.even = v;
      else t.odd = v + 1;
      err = launch(kind, t);  // warm-up
      if (err == cudaSuccess) err = cudaEventRecord(e0, c->st);
      for (int r = 0; r < reps && err == cudaSuccess; r++) err = launch(kind, t);
      if (err == cudaSuccess) err = cudaEventRecord(e1, c->st);
      if (err == cudaSuccess) err = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
      if (err == cudaSuccess && ms < tbest) {
        tbest = ms;
        if (kind == 0) best.jac = t.jac;
        else if (kind == 1) best.even = t.even;
        else best.odd = t.odd;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  TCK(err);
  c->tiles = best;
  c->tune_version++;
  destroy_graphs(c);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = best;
  }
  return TPLS_OK;
}

int tpls_get_tiles(const tpls_ctx *c, int *tiles3) {
  if (!c || !tiles3) return TPLS_ERR_ARG;
  tiles3[0] = c->tiles.jac;
  tiles3[1] = c->tiles.even;
  tiles3[2] = c->tiles.odd;
  return TPLS_OK;
}

int tpls_graphs_enable(tpls_ctx *c, int on) {
  if (!c) return TPLS_ERR_ARG;
  TCK(cudaStreamSynchronize(c->st));
  int s = refresh_graph_stats(c);
  if (s) return s;
  c->use_graphs = (on != 0);
  return TPLS_OK;
}

// ---------------------------------------------------------------------------
// Batches: independent channels advanced in lockstep by one CUDA-graph launch
// per step.  The batch graph is the fork of every member's step (captured
// from each member's own stream, the members' pressure loops as WHILE
// nodes) joined back into the batch stream, so the instances' kernels run
// concurrently under one launch.  One graph per history phase.
}  // extern "C"

struct tpls_batch {
  std::vector<tpls_ctx *> m;
  cudaStream_t st = nullptr;
  cudaEvent_t fork = nullptr, fork2 = nullptr, done = nullptr;
  std::vector<cudaEvent_t> join;
  cudaGraphExec_t gexec[3] = {nullptr, nullptr, nullptr};
  std::vector<long> n_static[3];  // kernels per member outside the CG loop
  std::vector<int> tune_seen;     // members' tune_version when the graphs were captured
  // multi-instance FP32 momentum sweeps: device member descriptors, tile
  // prefixes per (kind, component) (kind 0: Jacobi / checkerboard grid,
  // 1: odd half-sweep grid), the ticket counters, and the launches per step
  int multi = 0;
  SweepMember *dmem = nullptr;
  int *dprefix = nullptr;
  int total[2][3] = {{0, 0, 0}, {0, 0, 0}};
  unsigned *dctr = nullptr;
  int nblocks = 0;
  long n_multi = 0;
};

extern "C" {

int tpls_batch_destroy(tpls_batch *b) {
  if (!b) return TPLS_OK;
  DevLock lk(g_dev_mu);
  if (b->st) cudaStreamSynchronize(b->st);
  for (cudaGraphExec_t ge : b->gexec)
    if (ge) cudaGraphExecDestroy(ge);
  for (cudaEvent_t e : b->join) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->fork2) cudaEventDestroy(b->fork2);
  if (b->dmem) cudaFree(b->dmem);
  if (b->dprefix) cudaFree(b->dprefix);
  if (b->dctr) cudaFree(b->dctr);
  if (b->done) cudaEventDestroy(b->done);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
  return TPLS_OK;
}

int tpls_batch_create(tpls_ctx *const *ctxs, int n, tpls_batch **out) {
  if (!ctxs || n <= 0 || !out) return TPLS_ERR_ARG;
  *out = nullptr;
  for (int q = 0; q < n; q++) {
    if (!ctxs[q]) return TPLS_ERR_ARG;
    for (int r = 0; r < q; r++)
      if (ctxs[r] == ctxs[q]) return TPLS_ERR_ARG;
  }
  DevLock lk(g_dev_mu);
  tpls_batch *b = new tpls_batch();
  b->m.assign(ctxs, ctxs + n);
  cudaError_t e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork2, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
  b->join.assign(n, nullptr);
  for (int q = 0; q < n && e == cudaSuccess; q++) e = cudaEventCreateWithFlags(&b->join[q], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    tpls_batch_destroy(b);
    return TPLS_ERR_CUDA_BASE + (int)e;
  }
  *out = b;
  return TPLS_OK;
}

// The momentum sweeps of every member as multi-instance launches on the
// batch stream (main_ns_hybrid.F90:756-887 per component: Jacobi, then the
// two half-sweeps, mom/2 times), in each member's own launch order.
static int batch_multi_sweeps(tpls_batch *b) {
  const int n = (int)b->m.size();
  for (int comp = 0; comp < 3; comp++) {
    const int N = mom32_iters(b->m[0], comp);
    const int *pf0 = b->dprefix + (0 * 3 + comp) * (n + 1), *pf1 = b->dprefix + (1 * 3 + comp) * (n + 1);
    for (int it = 1; it <= N; it++) {
      const int src = (it - 1) % 2, dst = it % 2;
      TCK(launch_sweep4_multi(0, comp, b->dmem, pf0, n, b->total[0][comp], src, 0, 1, b->dctr, b->nblocks, b->st));
      for (int flg = 0; flg < 2; flg++) {
        if (it % 2 == 0)
          TCK(launch_sweep4_multi(1, comp, b->dmem, pf0, n, b->total[0][comp], dst, flg, flg, b->dctr, b->nblocks,
                                  b->st));
        else
          TCK(launch_odd_multi(comp, b->dmem, pf1, n, b->total[1][comp], dst, flg, flg, b->dctr, b->nblocks, b->st));
      }
      b->n_multi += 3;
    }
  }
  return TPLS_OK;
}

static int batch_capture(tpls_batch *b, int ph) {
  const int n = (int)b->m.size();
  std::vector<long> l0(n);
  for (int q = 0; q < n; q++) l0[q] = b->m[q]->launches;
  b->n_multi = 0;
  DevLock lk(g_dev_mu);
  TCK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
  int s = TPLS_OK;
  cudaError_t e = cudaEventRecord(b->fork, b->st);
  for (int q = 0; q < n && s == TPLS_OK && e == cudaSuccess; q++) {
    tpls_ctx *c = b->m[q];
    e = cudaStreamWaitEvent(c->st, b->fork, 0);
    if (e != cudaSuccess) break;
    c->capturing = true;
    if (b->multi) {  // front stage and the start of the FP32 momentum solves
      s = mixed_front(c);
      for (int comp = 0; comp < 3 && s == TPLS_OK; comp++) s = mom32_begin(c, comp);
    } else {
      s = c->mixed ? step_once_mixed(c) : step_once(c);
    }
    c->capturing = false;
    if (s == TPLS_OK) e = cudaEventRecord(b->join[q], c->st);
    if (s == TPLS_OK && e == cudaSuccess) e = cudaStreamWaitEvent(b->st, b->join[q], 0);
  }
  if (b->multi && s == TPLS_OK && e == cudaSuccess) {
    s = batch_multi_sweeps(b);
    if (s == TPLS_OK) e = cudaEventRecord(b->fork2, b->st);
    for (int q = 0; q < n && s == TPLS_OK && e == cudaSuccess; q++) {
      tpls_ctx *c = b->m[q];
      e = cudaStreamWaitEvent(c->st, b->fork2, 0);
      if (e != cudaSuccess) break;
      c->capturing = true;
      for (int comp = 0; comp < 3 && s == TPLS_OK; comp++) s = mom32_end(c, comp, mom32_iters(c, comp));
      if (s == TPLS_OK) s = mixed_back(c);
      c->capturing = false;
      if (s == TPLS_OK) e = cudaEventRecord(b->join[q], c->st);
      if (s == TPLS_OK && e == cudaSuccess) e = cudaStreamWaitEvent(b->st, b->join[q], 0);
    }
  }
  cudaGraph_t gr = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(b->st, &gr);
  b->n_static[ph].assign(n, 0);
  for (int q = 0; q < n; q++) {
    b->n_static[ph][q] = b->m[q]->launches - l0[q];
    b->m[q]->launches = l0[q];
  }
  if (s != TPLS_OK || e != cudaSuccess || ee != cudaSuccess) {
    if (gr) cudaGraphDestroy(gr);
    if (s != TPLS_OK) return s;
    return TPLS_ERR_CUDA_BASE + (int)(e != cudaSuccess ? e : ee);
  }
  const cudaError_t ei = cudaGraphInstantiate(&b->gexec[ph], gr, 0);
  cudaGraphDestroy(gr);
  TCK(ei);
  return TPLS_OK;
}

int tpls_batch_multi_sweeps(tpls_batch *b, int on) {
  if (!b || (on != 0 && on != 1)) return TPLS_ERR_ARG;
  const int n = (int)b->m.size();
  if (on) {
    int dev0 = -1;
    for (tpls_ctx *c : b->m) {
      if (!c->mixed || !mixed_fp32_sweeps(c) || c->ny % 2 != 0) return TPLS_ERR_ARG;
      for (int comp = 0; comp < 3; comp++)
        if (mom32_iters(c, comp) != mom32_iters(b->m[0], comp)) return TPLS_ERR_ARG;
    }
    TCK(cudaGetDevice(&dev0));
    if (!b->dmem) {
      std::vector<SweepMember> hm(n);
      std::vector<int> pre(6 * (n + 1), 0);
      for (int q = 0; q < n; q++) {
        tpls_ctx *c = b->m[q];
        SweepMember &M = hm[q];
        M.g = c->g;
        M.h = helm_of(c->ph);
        for (int comp = 0; comp < 3; comp++) {
          M.s[comp] = mu_coef(c->ph, c->mu32, c->bdef[comp], c->bco32[comp]);
          M.x[comp][0] = c->x3f[comp][0];
          M.x[comp][1] = c->x3f[comp][1];
          M.X[comp] = mom32_base(c, comp);
        }
        M.P = c->pres;
        M.fuse = 1;
      }
      for (int kind = 0; kind < 2; kind++)
        for (int comp = 0; comp < 3; comp++) {
          int *pf = pre.data() + (kind * 3 + comp) * (n + 1);
          for (int q = 0; q < n; q++)
            pf[q + 1] = pf[q] + (kind == 0 ? sweep4_tiles(comp, b->m[q]->g) : odd_tiles(comp, b->m[q]->g));
          b->total[kind][comp] = pf[n];
        }
      DevLock lk(g_dev_mu);
      TCK(cudaMalloc(&b->dmem, sizeof(SweepMember) * n));
      TCK(cudaMalloc(&b->dprefix, sizeof(int) * pre.size()));
      TCK(cudaMalloc(&b->dctr, 2 * sizeof(unsigned)));
      TCK(cudaMemcpy(b->dmem, hm.data(), sizeof(SweepMember) * n, cudaMemcpyHostToDevice));
      TCK(cudaMemcpy(b->dprefix, pre.data(), sizeof(int) * pre.size(), cudaMemcpyHostToDevice));
      TCK(cudaMemset(b->dctr, 0, 2 * sizeof(unsigned)));
      TCK(cudaStreamSynchronize(cudaStreamLegacy));  // before any stream of the batch reads them
      int sms = 0;
      TCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev0));
      b->nblocks = 8 * sms;
    }
  }
  if (b->multi != on) {
    b->multi = on;
    for (cudaGraphExec_t &ge : b->gexec)
      if (ge) {
        cudaGraphExecDestroy(ge);
        ge = nullptr;
      }
  }
  return TPLS_OK;
}

int tpls_batch_step_async(tpls_batch *b, int nsteps) {
  if (!b || nsteps < 0) return TPLS_ERR_ARG;
  const int n = (int)b->m.size();
  for (int it = 0; it < nsteps; it++) {
    const int ph = b->m[0]->phase;
    for (tpls_ctx *c : b->m)
      if (c->phase != ph || c->timing) return TPLS_ERR_STATE;
    bool stale = b->tune_seen.size() != (size_t)n;
    for (int q = 0; q < n && !stale; q++) stale = (b->tune_seen[q] != b->m[q]->tune_version);
    if (stale) {  // a member was retuned: recapture with its new tile shapes
      for (cudaGraphExec_t &ge : b->gexec)
        if (ge) {
          cudaGraphExecDestroy(ge);
          ge = nullptr;
        }
      b->tune_seen.resize(n);
      for (int q = 0; q < n; q++) b->tune_seen[q] = b->m[q]->tune_version;
    }
    for (int q = 0; q < n; q++) {  // host uploads: ghost rows, then order the member streams before the batch
      tpls_ctx *c = b->m[q];
      c->front_ok = false;
      int s = prologue(c);
      if (s) return s;
      TCK(cudaEventRecord(b->join[q], c->st));
      TCK(cudaStreamWaitEvent(b->st, b->join[q], 0));
    }
    if (!b->gexec[ph]) {
      int s = batch_capture(b, ph);
      if (s) return s;
    }
    TCK(cudaGraphLaunch(b->gexec[ph], b->st));
    TCK(cudaEventRecord(b->done, b->st));
    for (int q = 0; q < n; q++) {
      tpls_ctx *c = b->m[q];
      TCK(cudaStreamWaitEvent(c->st, b->done, 0));  // later work on a member follows the batch step
      // (the multi-instance sweep launches of a step are counted with member 0)
      c->launches += b->n_static[ph][q] + (q == 0 ? b->n_multi : 0);
      c->phase = (ph + 1) % 3;
      c->stats.steps_done++;
      c->graph_pending = true;
    }
  }
  return TPLS_OK;
}

int tpls_batch_step(tpls_batch *b, int nsteps) {
  int s = tpls_batch_step_async(b, nsteps);
  if (s) return s;
  TCK(cudaStreamSynchronize(b->st));
  int worst = TPLS_OK;
  for (tpls_ctx *c : b->m) {
    TCK(cudaStreamSynchronize(c->st));
    s = refresh_graph_stats(c);
    if (s) return s;
    if (c->stats.p_worst < worst) worst = c->stats.p_worst;
    c->stats.p_worst = 0;
  }
  return worst;
}

// interface height per column: first sign change of phi between cell
// centres k and k+1 (k = 1..nz-1), linear interpolation; -1 if none
__global__ void k_iface_height(Geo g, double dz, const double *__restrict__ phi, double *__restrict__ h) {
  const int i = blockIdx.x * 32 + threadIdx.x + 1, j = blockIdx.y * 4 + threadIdx.y + 1;
  if (i > g.nx || j > g.ny) return;
  double out = -1.0;
  double p0 = phi[TPLS_IDX(g, i, j, 1)];
  for (int k = 1; k < g.nz; k++) {
    const double p1 = phi[TPLS_IDX(g, i, j, k + 1)];
    if ((p0 < 0.0 && p1 >= 0.0) || (p0 >= 0.0 && p1 < 0.0)) {
      out = (k - 0.5) * dz + dz * (p0 / (p0 - p1));
      break;
    }
    p0 = p1;
  }
  h[(i - 1) + g.nx * (j - 1)] = out;
}

int tpls_interface_height(tpls_ctx *c, double *h_host) {
  if (!c || !h_host) return TPLS_ERR_ARG;
  const Geo &g = c->g;
  dim3 grd((g.nx + 31) / 32, (g.ny + 3) / 4, 1);
  k_iface_height<<<grd, dim3(32, 4), 0, c->st>>>(g, c->prm.dz, c->phi2, c->hbuf);
  LCK(c, cudaGetLastError());
  TCK(cudaMemcpyAsync(h_host, c->hbuf, sizeof(double) * (size_t)g.nx * g.ny, cudaMemcpyDeviceToHost, c->st));
  TCK(cudaStreamSynchronize(c->st));
  return TPLS_OK;
}

// liquid volume sum over cells of (1 - H(phi)) dV (FP64)
__global__ void k_volume(Geo g, Phys ph, const double *__restrict__ phi, double *part) {
  const int i = blockIdx.x * 32 + threadIdx.x + 1, j = blockIdx.y * 4 + threadIdx.y + 1,
            k = blockIdx.z + 1;
  double e = 0.0;
  if (i <= g.nx && j <= g.ny) {
    const double p = phi[TPLS_IDX(g, i, j, k)];
    double hv;
    if (p < -ph.sw) hv = 0.0;
    else if (p > ph.sw) hv = 1.0;
    else hv = 0.5 + (p / (2.0 * ph.sw)) + (1.0 / (2.0 * TPLS_PI_SP)) * sin(TPLS_PI_SP * p / ph.sw);
    e = 1.0 - hv;
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
  __shared__ double s[4];
  const int t = threadIdx.y * 32 + threadIdx.x;
  if ((t & 31) == 0) s[t >> 5] = e;
  __syncthreads();
  if (t == 0) part[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = s[0] + s[1] + s[2] + s[3];
}

int tpls_timing_enable(tpls_ctx *c, int on) {
  if (!c) return TPLS_ERR_ARG;
  TCK(cudaStreamSynchronize(c->st));
  timing_flush(c);
  c->timing = (on != 0);
  return TPLS_OK;
}

int tpls_timing_read(tpls_ctx *c, double *ms, long *launches, int reset) {
  if (!c) return TPLS_ERR_ARG;
  TCK(cudaStreamSynchronize(c->st));
  timing_flush(c);
  for (int q = 0; q < TPLS_T_COUNT; q++) {
    if (ms) ms[q] = c->t_ms[q];
    if (launches) launches[q] = c->t_n[q];
    if (reset) {
      c->t_ms[q] = 0.0;
      c->t_n[q] = 0;
    }
  }
  return TPLS_OK;
}

void *tpls_stream(tpls_ctx *c) { return c ? (void *)c->st : nullptr; }

int tpls_get_stats(tpls_ctx *c, tpls_stats *out) {
  if (!c || !out) return TPLS_ERR_ARG;
  {
    int s = refresh_graph_stats(c);
    if (s) return s;
  }
  const Geo &g = c->g;
  dim3 grd((g.nx + 31) / 32, (g.ny + 3) / 4, g.nz);
  k_volume<<<grd, dim3(32, 4), 0, c->st>>>(g, c->ph, c->phi2, c->part);
  LCK(c, cudaGetLastError());
  FSUM(c, c->part, (int)(grd.x * grd.y * grd.z), c->scal + SC_VOL, c->st);
  TCK(cudaMemcpyAsync(c->scal_host, c->scal, sizeof(double) * SC_N, cudaMemcpyDeviceToHost, c->st));
  TCK(cudaStreamSynchronize(c->st));
  c->stats.err_phi = c->scal_host[SC_ERR_PHI];
  c->stats.err_u = c->scal_host[SC_ERR_U];
  c->stats.err_v = c->scal_host[SC_ERR_V];
  c->stats.err_w = c->scal_host[SC_ERR_W];
  c->stats.liquid_volume = c->scal_host[SC_VOL] * c->prm.dx * c->prm.dy * c->prm.dz;
  c->stats.kernel_timeouts = (int)c->scal_host[SC_KTO];
  *out = c->stats;
  c->stats.p_worst = 0;
  return TPLS_OK;
}

int tpls_get_dims(const tpls_ctx *c, int *nx, int *ny, int *nz) {
  if (!c || !nx || !ny || !nz) return TPLS_ERR_ARG;
  *nx = c->nx;
  *ny = c->ny;
  *nz = c->nz;
  return TPLS_OK;
}

int tpls_set_steps_done(tpls_ctx *c, long steps_done) {
  if (!c || steps_done < 0) return TPLS_ERR_ARG;
  c->stats.steps_done = steps_done;
  return TPLS_OK;
}

// twophase_initialisation_wave.F90:79-122: viscosity profile of the flat
// interface and 10000 in-place sweeps of the 1-D base-state iteration.
int tpls_base_profile(int nz, double dz, double re, double dpdl, double mu_minus, double mu_plus,
                      double height, double smooth_width, double *u_oned) {
  if (nz < 3 || !u_oned) return TPLS_ERR_ARG;
  const double pi = (double)3.14159265359f;
  const int n = nz + 1;
  std::vector<double> visc(n + 1);
  for (int k = 0; k <= n; k++) {
    const double z_val = dz * k - (dz / 2.0);
    const double phi_val = z_val - height;
    double hv;
    if (phi_val < -smooth_width) hv = 0.0;
    else if (phi_val > smooth_width) hv = 1.0;
    else hv = 0.5 + (phi_val / (2.0 * smooth_width)) + (1.0 / (2.0 * pi)) * sin(pi * phi_val / smooth_width);
    const double temp = mu_plus * hv + mu_minus * (1.0 - hv);
    visc[k] = temp / re;
  }
  std::vector<double> u(n - 1, 0.0);
  for (int it = 0; it < 10000; it++) {
    for (int k = 0; k <= n - 2; k++) {
      const double umz = (k == 0) ? -2.0 * u[0] + u[1] / 3.0 : u[k - 1];
      const double upz = (k == n - 2) ? -2.0 * u[n - 2] + u[n - 3] / 3.0 : u[k + 1];
      const double mm = (visc[k] + visc[k + 1]) / 2.0;
      const double mp = (visc[k + 2] + visc[k + 1]) / 2.0;
      const double diag = (mp + mm) / (dz * dz);
      u[k] = (1.0 / diag) * (((mp * upz + mm * umz) / (dz * dz)) - dpdl);
    }
  }
  for (int k = 0; k < nz; k++) u_oned[k] = u[k];
  return TPLS_OK;
}

// ---------------------------------------------------------------------------
// per-routine drop-in entries (host arrays)

static int check_bounds(const tpls_ctx *c, const int *sx, const int *ex, const int *sy, const int *ey) {
  if ((sx && *sx != 1) || (ex && *ex != c->nx) || (sy && *sy != 1) || (ey && *ey != c->ny)) return TPLS_ERR_ARG;
  return TPLS_OK;
}
#define CHECKB(c, a, b, d, e)                  \
  do {                                         \
    if (!(c)) return TPLS_ERR_ARG;             \
    int s_ = check_bounds((c), a, b, d, e);    \
    if (s_) return s_;                         \
  } while (0)
#define REQ(cond)                        \
  do {                                   \
    if (!(cond)) return TPLS_ERR_ARG;    \
  } while (0)

static int scratch(tpls_ctx *c) {
  if (c->scr[0]) return TPLS_OK;
  DevLock lk(g_dev_mu);
  for (int q = 0; q < kMaxScratch; q++) TCK(alloc_p(c, &c->scr[q]));
  TCK(alloc_field(c, 1, c->ny + 4, c->nz + 2, &c->scr_mu));
  void *b = nullptr;
  TCK(cudaMalloc(&b, sizeof(double) * c->nz));
  c->allocs.push_back(b);
  c->scr_uin = (double *)b;
  TCK(cudaMalloc(&b, (size_t)c->px * (c->ny + 2) * (c->nz + 2) + 64));
  c->allocs.push_back(b);
  c->scr_flags = (signed char *)b + XOFF;
  return TPLS_OK;
}

static Phys phys_with(const tpls_ctx *c, const double *dx, const double *dy, const double *dz,
                      const double *dt) {
  Phys ph = c->ph;
  if (dx) ph.dx = *dx;
  if (dy) ph.dy = *dy;
  if (dz) ph.dz = *dz;
  if (dt) ph.dt = *dt;
  return ph;
}

int tpls_exchange2d(tpls_ctx *c, double *uu, const int *ex, const int *ey, const int *ez, const int *sx,
                    const int *sy, const int *sz) {
  CHECKB(c, sx, ex, sy, ey);
  REQ(uu && ez && sz && *sz == 0 && *ez >= 0 && *ez <= c->nz + 1);
  int s;
  if ((s = scratch(c))) return s;
  const int nzp = *ez + 1;
  TCK(h2d(c, c->scr[0], uu, nzp));
  LCK(c, launch_exchange(c->g, c->scr[0], nzp, c->st));
  TCK(d2h(c, uu, c->scr[0], nzp));
  TCK(cudaStreamSynchronize(c->st));
  return TPLS_OK;
}

int tpls_do_advect_phi(tpls_ctx *c, const double *phi2, double *u2, double *v2, double *w2, double *conv2_phi,
                       const int *sx, const int *ex, const int *sy, const int *ey, const int *sz_p,
                       const int *ez_p, const int *sz_uv, const int *sz_w, const int *ez_uv, const int *ez_w,
                       const int *maxl, const int *maxn, const int *ex_max, const int *neighbours,
                       const int *comm2d_quasiperiodic, const double *dx, const double *dy, const double *dz,
                       const int *, const int *, const int *, const int *, const int *, const int *,
                       const int *, const int *, const int *, const int *) {
  CHECKB(c, sx, ex, sy, ey);
  const int nz = c->nz;
  REQ(phi2 && u2 && v2 && w2 && conv2_phi && dx && dy && dz);
  REQ(!sz_p || *sz_p == 0);
  REQ(!ez_p || *ez_p == nz + 1);
  REQ(!sz_uv || *sz_uv == 0);
  REQ(!sz_w || *sz_w == 0);
  REQ(!ez_uv || *ez_uv == nz - 1);
  REQ(!ez_w || *ez_w == nz);
  REQ(!maxl || *maxl == c->nx + 1);
  REQ(!maxn || *maxn == nz + 1);
  REQ(!ex_max || *ex_max == c->nx);
  (void)neighbours;
  (void)comm2d_quasiperiodic;
  int s;
  if ((s = scratch(c))) return s;
  const Phys ph = phys_with(c, dx, dy, dz, nullptr);
  double *P = c->scr[0], *U = c->scr[1], *V = c->scr[2], *W = c->scr[3], *C = c->scr[4];
  TCK(h2d(c, P, phi2, nz + 2));
  TCK(h2d(c, U, u2, nz));
  TCK(h2d(c, V, v2, nz));
  TCK(h2d(c, W, w2, nz + 1));
  TCK(cudaMemsetAsync(C - XOFF, 0, sizeof(double) * ((size_t)c->px * (c->ny + 2) * (nz + 2)), c->st));
  LCK(c, launch_advect(c->g, ph, P, U, V, W, C, c->st));
  LCK(c, launch_exchange(c->g, U, nz, c->st));
  LCK(c, launch_exchange(c->g, V, nz, c->st));
  LCK(c, launch_exchange(c->g, W, nz + 1, c->st));
  TCK(d2h(c, conv2_phi, C, nz + 2));
  TCK(d2h(c, u2, U, nz));
  TCK(d2h(c, v2, V, nz));
  TCK(d2h(c, w2, W, nz + 1));
  TCK(cudaStreamSynchronize(c->st));
  return TPLS_OK;
}

int tpls_do_tpls(tpls_ctx *c, double *phi2, double *phi3, double *conv0_phi, double *conv1_phi,
                 double *conv2_phi, const int *sx, const int *ex, const int *sy, const int *ey,
                 const int *sz_p, const int *ez_p, const int *maxn, const int *ex_max, const int *,
                 const int *, const int *max_iteration_levelset, const int *, const int *,
                 const double *height, double *err2, const double *dx, const double *dz, const double *dt) {
  CHECKB(c, sx, ex, sy, ey);
  const int nz = c->nz;
  REQ(phi2 && phi3 && conv0_phi && conv1_phi && conv2_phi && max_iteration_levelset && height && err2 && dx &&
      dz && dt);
  REQ(!sz_p || *sz_p == 0);
  REQ(!ez_p || *ez_p == nz + 1);
  REQ(!maxn || *maxn == nz + 1);
  REQ(!ex_max || *ex_max == c->nx);
  int s;
  if ((s = scratch(c))) return s;
  Phys ph = phys_with(c, dx, nullptr, dz, dt);
  ph.height = *height;
  double *P2 = c->scr[0], *C0 = c->scr[1], *C1 = c->scr[2], *C2 = c->scr[3], *A = c->scr[4], *B = c->scr[5],
         *OUT = c->scr[6], *Dd = c->scr[7];
  TCK(h2d(c, P2, phi2, nz + 2));
  TCK(h2d(c, C0, conv0_phi, nz + 2));
  TCK(h2d(c, C1, conv1_phi, nz + 2));
  TCK(h2d(c, C2, conv2_phi, nz + 2));
  LCK(c, launch_ls_ab3(c->g, ph, P2, C0, C1, C2, A, c->st));
  LCK(c, launch_ls_status(c->g, ph, A, Dd, c->scr_flags, c->st));
  const int L = *max_iteration_levelset;
  const double *src = A;
  if (L <= 0) {
    TCK(cudaMemsetAsync(c->scal + SC_ERR_PHI, 0, sizeof(double), c->st));
  }
  for (int it = 1; it <= L; it++) {
    double *dst = (it == L) ? OUT : ((it % 2 == 1) ? B : A);
    if (it == 1 && L > 1) dst = B;
    LCK(c, launch_ls_iter(c->g, ph, src, Dd, c->scr_flags, dst, (it == L) ? c->part : nullptr, c->st));
    src = dst;
  }
  if (L > 0) FSUM(c, c->part, ls_iter_blocks(c->g), c->scal + SC_ERR_PHI, c->st);
  TCK(d2h(c, phi3, src, nz + 2));
  TCK(cudaMemcpyAsync(c->scal_host, c->scal, sizeof(double) * SC_N, cudaMemcpyDeviceToHost, c->st));
  TCK(cudaStreamSynchronize(c->st));
  *err2 = c->scal_host[SC_ERR_PHI];
  return TPLS_OK;
}

int tpls_dim(tpls_ctx *c, const int *maxl, const int *maxn, const double *dx, const double *dy, const double *dz,
             const double *dt, const double *epn, const double *pe, const double *phi, const double *phi_old,
             const double *conv2_phi, double *conv_prev_phi, double *phi_new, const int *sx, const int *ex,
             const int *sy, const int *ey, const int *sz_p, const int *ez_p, const double *height, const int *,
             const int *, const int *, const int *, const int *max_iteration_dim) {
  CHECKB(c, sx, ex, sy, ey);
  const int nz = c->nz;
  REQ(dx && dy && dz && dt && epn && pe && phi && phi_old && conv2_phi && conv_prev_phi && phi_new && height &&
      max_iteration_dim);
  REQ(*epn > 0 && *pe > 0 && *max_iteration_dim >= 0);
  REQ(!maxl || *maxl == c->nx + 1);
  REQ(!maxn || *maxn == nz + 1);
  REQ(!sz_p || *sz_p == 0);
  REQ(!ez_p || *ez_p == nz + 1);
  int s;
  if ((s = scratch(c))) return s;
  Phys ph = phys_with(c, dx, dy, dz, dt);
  ph.height = *height;
  const DimK q = dim_constants(ph, *epn, *pe);
  // scr[5] holds bulkE0 until the source term is formed, then the iterate's
  // second buffer
  double *P = c->scr[0], *O = c->scr[1], *C2 = c->scr[2], *CP = c->scr[3], *N0 = c->scr[4], *N1 = c->scr[5],
         *L = c->scr[6], *S = c->scr[7];
  TCK(h2d(c, P, phi, nz + 2));
  TCK(h2d(c, O, phi_old, nz + 2));
  TCK(h2d(c, C2, conv2_phi, nz + 2));
  TCK(h2d(c, CP, conv_prev_phi, nz + 2));
  TCK(h2d(c, N0, phi_new, nz + 2));
  LCK(c, launch_dim_prep(c->g, q, P, 0.0, N1, L, c->st));
  LCK(c, launch_dim_source(c->g, q, P, 0.0, N1, L, C2, CP, S, c->st));
  const double *pin = N0;
  double *pp[2] = {N1, N0};
  for (int it = 1; it <= *max_iteration_dim; it++) {
    double *out = pp[(it - 1) % 2];
    LCK(c, launch_dim_lap(c->g, q, pin, L, c->st));
    LCK(c, launch_dim_update(c->g, q, P, 0.0, O, 0.0, S, pin, L, out, c->st));
    pin = out;
  }
  TCK(d2h(c, phi_new, pin, nz + 2));
  TCK(d2h(c, conv_prev_phi, CP, nz + 2));
  TCK(cudaStreamSynchronize(c->st));
  return TPLS_OK;
}

int tpls_get_csf(tpls_ctx *c, double *fx_csf, double *fy_csf, double *fz_csf, const double *fi, const int *sx,
                 const int *ex, const int *sy, const int *ey, const int *n, const int *ex_max, const double *dx,
                 const double *dy, const double *dz, const double *scap, const double *smooth_width) {
  CHECKB(c, sx, ex, sy, ey);
  REQ(fx_csf && fy_csf && fz_csf && fi && dx && dy && dz && scap && smooth_width);
  REQ(!n || *n == c->nz + 1);
  REQ(!ex_max || *ex_max == c->nx);
  int s;
  if ((s = scratch(c))) return s;
  Phys ph = phys_with(c, dx, dy, dz, nullptr);
  ph.scap = *scap;
  ph.sw = *smooth_width;
  const int nz = c->nz;
  TCK(h2d(c, c->scr[0], fi, nz + 2));
  LCK(c, launch_csf(c->g, ph, c->scr[0], c->scr[1], c->scr[2], c->scr[3], c->st));
  TCK(d2h(c, fx_csf, c->scr[1], nz + 2));
  TCK(d2h(c, fy_csf, c->scr[2], nz + 2));
  TCK(d2h(c, fz_csf, c->scr[3], nz + 2));
  TCK(cudaStreamSynchronize(c->st));
  return TPLS_OK;
}

int tpls_get_viscosity(tpls_ctx *c, double *viscosity_aug, const double *phi, const int *ex, const int *ey,
                       const int *sx, const int *sy, const int *maxn, const double *smooth_width,
                       const double *re, const double *mu_minus, const double *mu_plus) {
  CHECKB(c, sx, ex, sy, ey);
  REQ(viscosity_aug && phi && smooth_width && re && mu_minus && mu_plus);
  REQ(!maxn || *maxn == c->nz + 1);
  int s;
  if ((s = scratch(c))) return s;
  Phys ph = c->ph;
  ph.sw = *smooth_width;
  ph.re = *re;
  ph.mu_minus = *mu_minus;
  ph.mu_plus = *mu_plus;
  TCK(h2d(c, c->scr[0], phi, c->nz + 2));
  LCK(c, launch_visc(c->g, ph, c->scr[0], c->scr_mu, c->st));
  TCK(d2h_mu(c, viscosity_aug, c->scr_mu));
  TCK(cudaStreamSynchronize(c->st));
  return TPLS_OK;
}

static int conv_diff_entry(tpls_ctx *c, int want_conv, double *o_u, double *o_v, double *o_w,
                           const double *va, const double *u2, const double *v2, const double *w2,
                           const double *dx, const double *dy, const double *dz) {
  REQ(o_u && o_v && o_w && va && u2 && v2 && w2 && dx && dy && dz);
  int s;
  if ((s = scratch(c))) return s;
  const Phys ph = phys_with(c, dx, dy, dz, nullptr);
  const int nz = c->nz;
  double *U = c->scr[0], *V = c->scr[1], *W = c->scr[2], *OU = c->scr[3], *OV = c->scr[4], *OW = c->scr[5];
  TCK(h2d(c, U, u2, nz));
  TCK(h2d(c, V, v2, nz));
  TCK(h2d(c, W, w2, nz + 1));
  TCK(h2d_mu(c, c->scr_mu, va));
  const size_t bytes = sizeof(double) * ((size_t)c->px * (c->ny + 2) * (nz + 2));
  TCK(cudaMemsetAsync(OU - XOFF, 0, bytes, c->st));
  TCK(cudaMemsetAsync(OV - XOFF, 0, bytes, c->st));
  TCK(cudaMemsetAsync(OW - XOFF, 0, bytes, c->st));
  LCK(c, launch_conv_diff(0, want_conv, c->g, ph, U, V, W, c->scr_mu, OU, c->st));
  LCK(c, launch_conv_diff(1, want_conv, c->g, ph, U, V, W, c->scr_mu, OV, c->st));
  LCK(c, launch_conv_diff(2, want_conv, c->g, ph, U, V, W, c->scr_mu, OW, c->st));
  TCK(d2h(c, o_u, OU, nz));
  TCK(d2h(c, o_v, OV, nz));
  TCK(d2h(c, o_w, OW, nz + 1));
  TCK(cudaStreamSynchronize(c->st));
  return TPLS_OK;
}

int tpls_get_conv_all(tpls_ctx *c, double *conv_u2, double *conv_v2, double *conv_w2, const double *va,
                      const double *u2, const double *v2, const double *w2, const int *sx, const int *sy,
                      const int *ex, const int *ey, const int *maxn, const int *ex_max, const double *dx,
                      const double *dy, const double *dz) {
  CHECKB(c, sx, ex, sy, ey);
  REQ(!maxn || *maxn == c->nz + 1);
  REQ(!ex_max || *ex_max == c->nx);
  return conv_diff_entry(c, 1, conv_u2, conv_v2, conv_w2, va, u2, v2, w2, dx, dy, dz);
}

int tpls_get_diffusion_all(tpls_ctx *c, double *diff_u, double *diff_v, double *diff_w, const double *va,
                           const double *u2, const double *v2, const double *w2, const int *sx, const int *sy,
                           const int *ex, const int *ey, const int *maxn, const int *ex_max, const double *dx,
                           const double *dy, const double *dz) {
  CHECKB(c, sx, ex, sy, ey);
  REQ(!maxn || *maxn == c->nz + 1);
  REQ(!ex_max || *ex_max == c->nx);
  return conv_diff_entry(c, 0, diff_u, diff_v, diff_w, va, u2, v2, w2, dx, dy, dz);
}

static int jacobi_entry(tpls_ctx *c, int comp, double *x3, const double *x3_old, const double *rhs,
                        const double *va, const double *dx, const double *dy, const double *dz,
                        const double *dt) {
  REQ(x3 && x3_old && rhs && va && dx && dy && dz && dt);
  int s;
  if ((s = scratch(c))) return s;
  const Phys ph = phys_with(c, dx, dy, dz, dt);
  const int nzp = nz_planes(comp == 2 ? 2 : 1, c->nz);
  double *X = c->scr[0], *XO = c->scr[1], *R = c->scr[2];
  TCK(h2d(c, X, x3, nzp));
  TCK(h2d(c, XO, x3_old, nzp));
  TCK(h2d(c, R, rhs, nzp));
  TCK(h2d_mu(c, c->scr_mu, va));
  LCK(c, launch_jacobi(comp, c->g, ph, XO, R, c->scr_mu, nullptr, X, 0, 0, c->st));
  TCK(d2h(c, x3, X, nzp));
  TCK(cudaStreamSynchronize(c->st));
  return TPLS_OK;
}

#define JAC_ENTRY(NAME, COMP)                                                                                   \
  int NAME(tpls_ctx *c, double *x3, const double *x3_old, const double *rhs, const double *viscosity,          \
           const double *dx, const double *dy, const double *dz, const double *dt, const int *ex, const int *ey, \
           const int *sx, const int *sy, const int *maxn, const int *ex_max) {                                  \
    CHECKB(c, sx, ex, sy, ey);                                                                                  \
    REQ(!maxn || *maxn == c->nz + 1);                                                                           \
    REQ(!ex_max || *ex_max == c->nx);                                                                           \
    return jacobi_entry(c, COMP, x3, x3_old, rhs, viscosity, dx, dy, dz, dt);                                   \
  }
JAC_ENTRY(tpls_do_jacobi_u, 0)
JAC_ENTRY(tpls_do_jacobi_v, 1)
JAC_ENTRY(tpls_do_jacobi_w, 2)

static int sor_entry(tpls_ctx *c, int comp, double *x3, const double *rhs, const double *va, const double *dx,
                     const double *dy, const double *dz, const double *dt, const int *flg,
                     const int *iteration_time) {
  REQ(x3 && rhs && va && dx && dy && dz && dt && flg && iteration_time);
  REQ(*flg == 0 || *flg == 1);
  int s;
  if ((s = scratch(c))) return s;
  const Phys ph = phys_with(c, dx, dy, dz, dt);
  const int nzp = nz_planes(comp == 2 ? 2 : 1, c->nz);
  double *X = c->scr[0], *R = c->scr[1];
  TCK(h2d(c, X, x3, nzp));
  TCK(h2d(c, R, rhs, nzp));
  TCK(h2d_mu(c, c->scr_mu, va));
  if (*iteration_time % 2 == 0)
    LCK(c, launch_sor(comp, c->g, ph, X, R, c->scr_mu, nullptr, *flg, *iteration_time, 0, 0, c->st));
  else  // the column recurrence in chunks (as the step's sweeps), not one thread per column
    LCK(c, launch_sor_ref_odd(comp, c->g, ph, X, R, c->scr_mu, *flg, c->st, odd_chain(c)));
  TCK(d2h(c, x3, X, nzp));
  TCK(cudaStreamSynchronize(c->st));
  return TPLS_OK;
}

int tpls_do_sor_u(tpls_ctx *c, double *u3, const double *rhs, const double *viscosity, const double *dx,
                  const double *dy, const double *dz, const double *dt, const int *ex, const int *ey,
                  const int *sx, const int *sy, const int *maxn, const int *ex_max, const int *flg,
                  const int *iteration_time) {
  CHECKB(c, sx, ex, sy, ey);
  REQ(!maxn || *maxn == c->nz + 1);
  REQ(!ex_max || *ex_max == c->nx);
  return sor_entry(c, 0, u3, rhs, viscosity, dx, dy, dz, dt, flg, iteration_time);
}
int tpls_do_sor_v(tpls_ctx *c, double *v3, const double *rhs, const double *viscosity, const double *dx,
                  const double *dy, const double *dz, const double *dt, const int *ex, const int *ey,
                  const int *sx, const int *sy, const int *maxn, const int *flg, const int *iteration_time) {
  CHECKB(c, sx, ex, sy, ey);
  REQ(!maxn || *maxn == c->nz + 1);
  return sor_entry(c, 1, v3, rhs, viscosity, dx, dy, dz, dt, flg, iteration_time);
}
int tpls_do_sor_w(tpls_ctx *c, double *w3, const double *rhs, const double *viscosity, const double *dx,
                  const double *dy, const double *dz, const double *dt, const int *ex, const int *ey,
                  const int *sx, const int *sy, const int *maxn, const int *flg, const int *iteration_time) {
  CHECKB(c, sx, ex, sy, ey);
  REQ(!maxn || *maxn == c->nz + 1);
  return sor_entry(c, 2, w3, rhs, viscosity, dx, dy, dz, dt, flg, iteration_time);
}

int tpls_get_difference(tpls_ctx *c, const double *ua, const double *ub, const int *ex, const int *ey,
                        const int *ez, const int *sx, const int *sy, const int *sz, double *diff) {
  CHECKB(c, sx, ex, sy, ey);
  REQ(ua && ub && ez && sz && diff && *sz == 0 && *ez >= 0 && *ez <= c->nz + 1);
  int s;
  if ((s = scratch(c))) return s;
  const int nzp = *ez + 1;
  TCK(h2d(c, c->scr[0], ua, nzp));
  TCK(h2d(c, c->scr[1], ub, nzp));
  LCK(c, launch_diff2(c->g, c->scr[0], c->scr[1], nzp, c->part, c->st));
  FSUM(c, c->part, diff2_blocks(c->g, nzp), c->scal + SC_ERR_U, c->st);
  TCK(cudaMemcpyAsync(c->scal_host, c->scal, sizeof(double) * SC_N, cudaMemcpyDeviceToHost, c->st));
  TCK(cudaStreamSynchronize(c->st));
  *diff = c->scal_host[SC_ERR_U];
  return TPLS_OK;
}

int tpls_get_source_pres(tpls_ctx *c, double *rhs, const double *u3, const double *v3, const double *w3,
                         const int *ex, const int *ey, const int *sx, const int *sy, const int *maxn,
                         const double *dx, const double *dy, const double *dz, const double *dt) {
  CHECKB(c, sx, ex, sy, ey);
  REQ(rhs && u3 && v3 && w3 && dx && dy && dz && dt);
  REQ(!maxn || *maxn == c->nz + 1);
  int s;
  if ((s = scratch(c))) return s;
  const Phys ph = phys_with(c, dx, dy, dz, dt);
  const int nz = c->nz;
  TCK(h2d(c, c->scr[0], u3, nz));
  TCK(h2d(c, c->scr[1], v3, nz));
  TCK(h2d(c, c->scr[2], w3, nz + 1));
  LCK(c, launch_source(c->g, ph, c->scr[0], c->scr[1], c->scr[2], c->scr[3], c->st));
  TCK(d2h(c, rhs, c->scr[3], nz + 2));
  TCK(cudaStreamSynchronize(c->st));
  return TPLS_OK;
}

int tpls_get_uvw_pres(tpls_ctx *c, double *u3, double *v3, double *w3, const double *p, const int *ex,
                      const int *ey, const int *sx, const int *sy, const int *maxn, const int *ex_max,
                      const double *dx, const double *dy, const double *dz, const double *dt,
                      const double *u_inlet) {
  CHECKB(c, sx, ex, sy, ey);
  REQ(u3 && v3 && w3 && p && dx && dy && dz && dt && u_inlet);
  REQ(!maxn || *maxn == c->nz + 1);
  REQ(!ex_max || *ex_max == c->nx);
  int s;
  if ((s = scratch(c))) return s;
  const Phys ph = phys_with(c, dx, dy, dz, dt);
  const int nz = c->nz;
  double *U = c->scr[0], *V = c->scr[1], *W = c->scr[2], *P = c->scr[3], *UO = c->scr[4], *VO = c->scr[5],
         *WO = c->scr[6];
  TCK(h2d(c, U, u3, nz));
  TCK(h2d(c, V, v3, nz));
  TCK(h2d(c, W, w3, nz + 1));
  TCK(h2d(c, P, p, nz + 2));
  TCK(cudaMemcpyAsync(c->scr_uin, hmap(c, u_inlet, nz), sizeof(double) * nz, cudaMemcpyDefault, c->st));
  LCK(c, launch_project(c->g, ph, U, V, W, P, c->scr_uin, UO, VO, WO, c->st));
  // the reference updates rows 1..ny only; its ghost rows keep their values
  const size_t w = sizeof(double) * (size_t)(c->nx + 2);
  for (int k = 0; k <= nz; k++) {
    double *dsts[3] = {u3, v3, w3};
    double *srcs[3] = {UO, VO, WO};
    for (int q = 0; q < 3; q++) {
      if (q < 2 && k == nz) continue;
      double *d = hmap(c, dsts[q] + (size_t)(c->nx + 2) * ((size_t)(c->ny + 2) * k + 1), (size_t)(c->nx + 2) * c->ny);
      TCK(cudaMemcpy2DAsync(d, w,
                            srcs[q] + (size_t)c->g.sz * k + c->g.sy, sizeof(double) * c->px, w, c->ny,
                            cudaMemcpyDefault, c->st));
    }
  }
  TCK(cudaStreamSynchronize(c->st));
  return TPLS_OK;
}

int tpls_pressure_solve(tpls_ctx *c, double *pres, const double *pres_old, const double *rhs_p, const double *u3,
                        const double *u_inlet, const double *dx, const double *dy, const double *dz,
                        const double *dt, const double *rtol, const int *maxits, int *its, double *rnorm,
                        int *reason) {
  if (!c) return TPLS_ERR_ARG;
  REQ(pres && pres_old && rhs_p && u3 && u_inlet && dx && dy && dz && dt && its && rnorm && reason);
  REQ(*dx == c->prm.dx && *dy == c->prm.dy && *dz == c->prm.dz);  // operator is set up at create
  int s;
  if ((s = scratch(c))) return s;
  const Phys ph = phys_with(c, dx, dy, dz, dt);
  const int nz = c->nz;
  double *P = c->scr[0], *PO = c->scr[1], *R = c->scr[2], *U = c->scr[3];
  TCK(h2d(c, PO, pres_old, nz + 2));
  TCK(h2d(c, R, rhs_p, nz + 2));
  TCK(h2d(c, U, u3, nz));
  TCK(cudaMemcpyAsync(c->scr_uin, hmap(c, u_inlet, nz), sizeof(double) * nz, cudaMemcpyDefault, c->st));
  const double rt = (rtol && *rtol > 0) ? *rtol : c->prm.p_rtol;
  const int mi = (maxits && *maxits > 0) ? *maxits : c->prm.p_maxits;
  double bn = 0.0;
  TCK(poisson_solve(c->ps, c->g, ph, R, U, 0, c->scr_uin, PO, P, rt, mi, its, rnorm, &bn, reason, c->st,
                    &c->launches));
  c->its_accounted += *its;
  TCK(d2h(c, pres, P, nz + 2));
  TCK(cudaStreamSynchronize(c->st));
  return (*reason < 0) ? *reason : TPLS_OK;
}

}  // extern "C"
