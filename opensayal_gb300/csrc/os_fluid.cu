// os_fluid.cu — host side of the GB300 wind tunnel: handle lifecycle, the
// captured per-step CUDA graph, and the C ABI declared in
// include/opensayal_gb300.h.
//
// One handle = one grid = the reference's Fluid object (inc/fluid.cuh:15-116).
// Its fields live in device memory in the reference's layout for the whole
// life of the handle; a step is one replay of a CUDA graph captured at the
// first update (the reference launches ~157 kernels per step on the legacy
// stream and synchronises, src/fluid.cu:770-795). Per-step inputs (dt and the
// Source) sit in a device-side StepParams block that is refreshed only when
// they change, so one graph serves every step.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <tuple>
#include <type_traits>
#include <vector>

#include "../../include/opensayal_gb300.h"
#include "../../include/opensayal_gb300/config_parser.hpp"
#include "os_kernels.cuh"

using namespace osg;

namespace {

thread_local char g_err[512] = "";

int set_err(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return code;
}

#define CUDA_OR_RETURN(expr)                                                    \
  do {                                                                          \
    cudaError_t e_ = (expr);                                                    \
    if (e_ != cudaSuccess)                                                      \
      return set_err(OS_ERR_CUDA, "%s failed: %s", #expr, cudaGetErrorString(e_)); \
  } while (0)

size_t storage_bytes(int storage) {
  switch (storage) {
    case OS_STORAGE_F32: return 4;
    case OS_STORAGE_F16: return 2;
    case OS_STORAGE_BF16: return 2;
    case OS_STORAGE_F64: return 8;
    default: return 0;
  }
}

// Device memory with a byte budget: one cudaMalloc up front, carved into
// 256-byte-aligned blocks, best fit, neighbouring free blocks merged on
// release. Admission against the budget is then a host-side decision that
// never touches the driver.
class Arena {
 public:
  int init(size_t bytes) {
    capacity_ = (bytes + kAlign - 1) / kAlign * kAlign;
    cudaError_t e = cudaMalloc(&base_, capacity_);
    if (e != cudaSuccess) {
      base_ = nullptr;
      return OS_ERR_NOMEM;
    }
    free_[0] = capacity_;
    return OS_OK;
  }
  ~Arena() {
    if (base_) cudaFree(base_);
  }
  void* alloc(size_t bytes) {
    std::lock_guard<std::mutex> lock(mu_);
    const size_t n = std::max<size_t>(kAlign, (bytes + kAlign - 1) / kAlign * kAlign);
    auto best = free_.end();
    for (auto it = free_.begin(); it != free_.end(); ++it)
      if (it->second >= n && (best == free_.end() || it->second < best->second)) best = it;
    if (best == free_.end()) return nullptr;
    const size_t off = best->first, size = best->second;
    free_.erase(best);
    if (size > n) free_[off + n] = size - n;
    live_[off] = n;
    used_ += n;
    return base_ + off;
  }
  void release(void* p) {
    std::lock_guard<std::mutex> lock(mu_);
    const size_t off = static_cast<char*>(p) - base_;
    auto it = live_.find(off);
    if (it == live_.end()) return;
    size_t start = off, size = it->second;
    used_ -= size;
    live_.erase(it);
    auto next = free_.lower_bound(start);
    if (next != free_.end() && start + size == next->first) {
      size += next->second;
      next = free_.erase(next);
    }
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == start) {
        start = prev->first;
        size += prev->second;
        free_.erase(prev);
      }
    }
    free_[start] = size;
  }
  bool owns(const void* p) const {
    return base_ && p >= base_ && static_cast<const char*>(p) < base_ + capacity_;
  }
  size_t used() const { return used_; }
  size_t capacity() const { return capacity_; }

 private:
  static constexpr size_t kAlign = 256;
  char* base_ = nullptr;
  size_t capacity_ = 0, used_ = 0;
  std::map<size_t, size_t> free_;  // offset -> size
  std::map<size_t, size_t> live_;  // offset -> size
  std::mutex mu_;
};

}  // namespace

struct os_handle {
  os_config cfg;
  Consts c;
  int W = 0, H = 0;
  size_t N = 0;
  int storage = OS_STORAGE_F32;
  size_t esize = 4;
  int smoke_period = 1;
  int block_k = 0;  // red/black sweeps per blocked pass; -1: plain form
  int diff_k = 0;   // Jacobi sweeps per blocked diffusion pass; 0: block_k
  cudaStream_t stream = nullptr;
  // fields (reference layout); u, v, s in storage precision
  void *u = nullptr, *v = nullptr, *s = nullptr;
  void *ub = nullptr, *vb = nullptr, *sb = nullptr;
  float* p = nullptr;
  int32_t *is_solid = nullptr, *total_s = nullptr;
  uint8_t* flags = nullptr;
  uint16_t* nbr = nullptr;  // fluid neighbourhoods of [-1, W] x [-1, H] (samplers)
  StepParams* d_params = nullptr;
  StepParams* h_params = nullptr;        // pinned staging slot
  cudaEvent_t params_event = nullptr;    // completion of the last copy out of it
  int64_t params_bytes = 0;              // host->device parameter bytes so far
  StepParams last_params;
  bool params_valid = false;
  int* d_pkeys = nullptr;   // pressure extrema as ordered integer keys
  int* h_pkeys = nullptr;   // pinned copy
  float* conv = nullptr;    // FP32 staging for non-FP32 storage transfers
  double* diag = nullptr;   // diagnostics partials and result (first use)
  // Resident projection (one cooperative launch per phase): tile flags, the
  // device error word, and a mapped host word the kernel sets on a failed wait.
  // Diffusion passes staged by the tensor memory accelerator: maps of u, ub.
  CUtensorMap diff_maps[2];
  bool tma_diffusion = false;
  // Step kernels launched with programmatic dependent launch.
  bool pdl = true;
  int resident = 0;       // projection
  int resident_diff = 0;  // diffusion
  unsigned* rflags = nullptr;
  unsigned* dflags = nullptr;
  int* rerr = nullptr;
  int* host_rerr = nullptr;
  int* d_host_rerr = nullptr;
  cudaGraphExec_t graph = nullptr;
  int kernels_per_step = 0;
  int64_t launches = 0;
  float min_pressure = 0.0f, max_pressure = 0.0f;
  // Device memory: one arena block carved in order, or one cudaMalloc each.
  Arena* arena = nullptr;
  char* arena_block = nullptr;
  size_t arena_size = 0, arena_used = 0;
  size_t device_bytes = 0;  // device memory this handle holds
};

namespace {

// Diagnostics scratch: 256 block partials and the result, 7 doubles each.
constexpr size_t kDiagBytes = (256 + 1) * 7 * sizeof(double);

// Device bytes a handle of this configuration takes from an arena: fields and
// their buffers, pressure, mask, counts, flags, neighbourhoods, the parameter
// block, the pressure keys and, for 16-bit storage, the FP32 transfer staging.
size_t handle_footprint(const os_config& c) {
  const size_t N = (size_t)c.width * c.height;
  const size_t e = storage_bytes(c.storage);
  auto r = [](size_t b) { return (b + 255) / 256 * 256; };
  size_t bytes = 6 * r(N * e) + 3 * r(N * 4) + r(N) + r(sizeof(StepParams)) + r(2 * sizeof(int));
  bytes += r((size_t)(c.width + 2) * (c.height + 2) * sizeof(uint16_t));
  if (c.storage != OS_STORAGE_F32) bytes += r(N * 4);
  bytes += r(kDiagBytes);
  return bytes;
}

cudaError_t dev_alloc(os_handle* h, void** p, size_t bytes) {
  if (h->arena_block) {
    const size_t off = (h->arena_used + 255) / 256 * 256;
    if (off + bytes > h->arena_size) return cudaErrorMemoryAllocation;
    *p = h->arena_block + off;
    h->arena_used = off + bytes;
  } else {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return e;
    h->device_bytes += bytes;
  }
  return cudaSuccess;
}

void dev_free(os_handle* h, void* p) {
  if (p && !h->arena_block) cudaFree(p);
}

}  // namespace

// The temporally blocked projection/diffusion engine works on the handle.
#include "os_blocked.cuh"
// The projection phase with tiles resident in shared memory across passes.
#include "os_resident.cuh"
// FP64 divergence-residual and conservation sums.
#include "os_diag.cuh"
// Pixel colours, velocity arrows and path lines as device buffers.
#include "os_visual.cuh"

namespace {

// ---------------------------------------------------------------------------
// Step enqueue (captured into the graph).
// ---------------------------------------------------------------------------

struct Enq {
  cudaStream_t st;
  int count = 0;
  bool failed = false;  // a launch that reports its refusal by return value
  // Recorded on `st` after a diffusion or projection phase's own kernels,
  // before the copy back that a phase called on its own may add.
  cudaEvent_t kernels_done = nullptr;
};

// Where the live velocity sits while a step is enqueued: 0 = the public
// fields u/v, 1 = the buffers ub/vb. Blocked passes and advection alternate
// between the two instead of copying back.
template <class S>
struct Vel {
  S* U[2];
  S* V[2];
  int cu = 0, cv = 0;
  S* u() const { return U[cu]; }
  S* v() const { return V[cv]; }
};

template <class S>
Vel<S> vel_of(os_handle* h) {
  Vel<S> w;
  w.U[0] = static_cast<S*>(h->u);
  w.U[1] = static_cast<S*>(h->ub);
  w.V[0] = static_cast<S*>(h->v);
  w.V[1] = static_cast<S*>(h->vb);
  return w;
}

template <class S, class A>
bool use_blocked(const os_handle* h) {
  return h->block_k > 0 && blocked_supported<S, A>(h);
}

template <class S, class A>
constexpr bool kBlockedTypes = std::is_same<A, float>::value &&
                               (std::is_same<S, float>::value || std::is_same<S, __half>::value ||
                                std::is_same<S, __nv_bfloat16>::value);

template <class S, class A>
void enqueue_diffusion(os_handle* h, Vel<S>& w, Enq& q) {
  if constexpr (kBlockedTypes<S, A>) {
    if (use_blocked<S, A>(h) && h->resident_diff) {
      const int n = enqueue_resident_diffusion<S>(h, q.st, &w.cu);
      if (n > 0) {
        q.count += n;
        return;
      }
      q.failed = true;
      return;
    }
    if (use_blocked<S, A>(h)) {
      q.count += enqueue_blocked_diffusion<S>(h, q.st, &w.cu);
      return;
    }
  }
  const dim3 g2((h->W + 127) / 128, h->H);
  for (int t = 0; t < h->c.n; t++) {
    launch_pdl(h->pdl, k_diffuse<S, A>, g2, 128, 0, q.st, w.U[w.cu], w.U[1 - w.cu], h->c, h->d_params);
    w.cu = 1 - w.cu;
    q.count++;
  }
}

// With `extrapolated` non-null, the resident form may apply the extrapolation
// that follows in a step to its last pass's regions; *extrapolated says
// whether it did.
template <class S, class A>
void enqueue_projection(os_handle* h, Vel<S>& w, Enq& q, bool zero_pressure_first,
                        bool* extrapolated = nullptr) {
  if (extrapolated) *extrapolated = false;
  if constexpr (kBlockedTypes<S, A>) {
    if (use_blocked<S, A>(h) && h->resident) {
      const int n = enqueue_resident_projection<S>(h, q.st, &w.cu, &w.cv, zero_pressure_first,
                                                   extrapolated);
      if (n > 0) {
        q.count += n;
        return;
      }
      q.failed = true;
      return;
    }
    if (use_blocked<S, A>(h)) {
      q.count += enqueue_blocked_projection<S>(h, q.st, &w.cu, &w.cv, zero_pressure_first);
      return;
    }
  }
  const dim3 gp(((h->W + 1) / 2 + 127) / 128, h->H);
  for (int t = 0; t < h->c.n; t++) {
    launch_pdl(h->pdl, k_project_half<S, A, 0>, gp, 128, 0, q.st, w.u(), w.v(), h->p, h->flags, h->c, h->d_params);
    launch_pdl(h->pdl, k_project_half<S, A, 1>, gp, 128, 0, q.st, w.u(), w.v(), h->p, h->flags, h->c, h->d_params);
    q.count += 2;
  }
}

// Copies a field that ended in its buffer back to the public array.
template <class S>
void settle(os_handle* h, Vel<S>& w, Enq& q) {
  const int64_t N = (int64_t)h->N;
  const unsigned g1 = (unsigned)((N + 255) / 256);
  if (w.cu) {
    launch_pdl(h->pdl, k_copy1<S>, g1, 256, 0, q.st, w.U[1], w.U[0], N);
    q.count++;
    w.cu = 0;
  }
  if (w.cv) {
    launch_pdl(h->pdl, k_copy1<S>, g1, 256, 0, q.st, w.V[1], w.V[0], N);
    q.count++;
    w.cv = 0;
  }
}

// Advection launches: the unit cell size (sim.cell_size 1, the default) has
// its own instantiation, in which the divisions by the cell size fold away.
template <class S, class A>
void launch_velocity_advection(os_handle* h, cudaStream_t st, S* u, S* v, S* ub, S* vb) {
  const dim3 g2((h->W + 127) / 128, (h->H + kAdvRows - 1) / kAdvRows);
  if (h->c.h == 1)
    launch_pdl(h->pdl, k_advect_velocity<S, A, 1>, g2, 128, 0, st, u, v, ub, vb, h->nbr, h->c, h->d_params);
  else
    launch_pdl(h->pdl, k_advect_velocity<S, A, 0>, g2, 128, 0, st, u, v, ub, vb, h->nbr, h->c, h->d_params);
}

template <class S, class A, bool COPY_U, bool COPY_V>
void launch_smoke_advection(os_handle* h, cudaStream_t st, S* ub, S* vb, S* s, S* sb, S* u0, S* v0) {
  const dim3 g2((h->W + 127) / 128, (h->H + kAdvRows - 1) / kAdvRows);
  if (h->c.h == 1)
    launch_pdl(h->pdl, k_advect_smoke<S, A, COPY_U, COPY_V, 1>, g2, 128, 0, st, ub, vb, s, sb, u0, v0, h->nbr, h->c, h->d_params);
  else
    launch_pdl(h->pdl, k_advect_smoke<S, A, COPY_U, COPY_V, 0>, g2, 128, 0, st, ub, vb, s, sb, u0, v0, h->nbr, h->c, h->d_params);
}

template <class S, class A>
void enqueue_smoke_advection(os_handle* h, Vel<S>& w, Enq& q) {
  S* s = static_cast<S*>(h->s);
  S* sb = static_cast<S*>(h->sb);
  S* u0 = w.U[0];
  S* v0 = w.V[0];
  // smoke advection on the live velocities, copying them back as it goes
  if (w.cu && w.cv)
    launch_smoke_advection<S, A, true, true>(h, q.st, w.u(), w.v(), s, sb, u0, v0);
  else if (w.cu)
    launch_smoke_advection<S, A, true, false>(h, q.st, w.u(), w.v(), s, sb, u0, v0);
  else if (w.cv)
    launch_smoke_advection<S, A, false, true>(h, q.st, w.u(), w.v(), s, sb, u0, v0);
  else
    launch_smoke_advection<S, A, false, false>(h, q.st, w.u(), w.v(), s, sb, u0, v0);
  w.cu = w.cv = 0;
  q.count++;
}

template <class S, class A>
int enqueue_phase(os_handle* h, int phase, Enq& q) {
  const Consts& c = h->c;
  Vel<S> w = vel_of<S>(h);
  S* s = static_cast<S*>(h->s);
  S* sb = static_cast<S*>(h->sb);
  const int64_t N = (int64_t)h->N;
  const unsigned g1 = (unsigned)((N + 255) / 256);
  cudaStream_t st = q.st;
  switch (phase) {
    case OS_PHASE_FORCES:
      launch_pdl(h->pdl, k_forces<S, A>, cell_grid(h->W, h->H), kCellThreads, 0, st, w.u(), w.v(), s, c, h->smoke_period, h->d_params);
      q.count++;
      break;
    case OS_PHASE_ZERO_PRESSURE:
      launch_pdl(h->pdl, k_zero, g1, 256, 0, st, h->p, N);
      q.count++;
      break;
    case OS_PHASE_DIFFUSION:
      enqueue_diffusion<S, A>(h, w, q);
      if (q.kernels_done) cudaEventRecord(q.kernels_done, st);
      settle(h, w, q);
      break;
    case OS_PHASE_PROJECTION:
      enqueue_projection<S, A>(h, w, q, false);
      if (q.kernels_done) cudaEventRecord(q.kernels_done, st);
      settle(h, w, q);
      break;
    case OS_PHASE_PRESSURE_RANGE:
      launch_pdl(h->pdl, k_prange_init, 1, 32, 0, st, h->d_pkeys);
      launch_pdl(h->pdl, k_prange, 152 * 4, 256, 0, st, h->p, N, h->d_pkeys);
      q.count += 2;
      break;
    case OS_PHASE_EXTRAPOLATION:
      launch_pdl(h->pdl, k_extrapolate<S>, 1, 1024, 0, st, w.u(), w.v(), c);
      q.count++;
      break;
    case OS_PHASE_VEL_ADVECTION:
      launch_velocity_advection<S, A>(h, st, w.U[0], w.V[0], w.U[1], w.V[1]);
      w.cu = w.cv = 1;
      q.count++;
      settle(h, w, q);
      break;
    case OS_PHASE_SMOKE_ADVECTION:
      enqueue_smoke_advection<S, A>(h, w, q);
      launch_pdl(h->pdl, k_copy1<S>, g1, 256, 0, st, sb, s, N);
      q.count++;
      break;
    case OS_PHASE_DECAY:
      launch_pdl(h->pdl, k_finish_smoke<S, A>, (unsigned)((h->N + 256 * kCellsPerThread - 1) / (256 * kCellsPerThread)), 256, 0, st, s, s, c, h->d_params, N);
      q.count++;
      break;
    default:
      return set_err(OS_ERR_INVALID, "unknown phase %d", phase);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_err(OS_ERR_CUDA, "launch failed: %s", cudaGetErrorString(e));
  if (q.failed) return set_err(OS_ERR_CUDA, "resident projection launch refused");
  return OS_OK;
}

// Fluid::update (src/fluid.cu:770-795) as one launch sequence. The order of
// the phases is the reference's; copies between phases are avoided by
// letting the live velocity alternate between the fields and their buffers.
template <class S, class A>
int enqueue_step(os_handle* h, Enq& q) {
  const os_config& cfg = h->cfg;
  Vel<S> w = vel_of<S>(h);
  S* s = static_cast<S*>(h->s);
  S* sb = static_cast<S*>(h->sb);
  const Consts& c = h->c;
  const int64_t N = (int64_t)h->N;
  const unsigned g1 = (unsigned)((N + 255) / 256);
  launch_pdl(h->pdl, k_forces<S, A>, cell_grid(h->W, h->H), kCellThreads, 0, q.st, w.u(), w.v(), s, c, h->smoke_period, h->d_params);
  q.count++;
  // The blocked projection zeroes the pressure in its first pass.
  if (cfg.enable_pressure && !(use_blocked<S, A>(h) && c.n > 0)) {
    launch_pdl(h->pdl, k_zero, g1, 256, 0, q.st, h->p, N);
    q.count++;
  }
  if (cfg.viscosity != 0.0f) enqueue_diffusion<S, A>(h, w, q);
  bool extrapolated = false;
  enqueue_projection<S, A>(h, w, q, cfg.enable_pressure != 0, &extrapolated);
  if (cfg.enable_pressure) {
    launch_pdl(h->pdl, k_prange_init, 1, 32, 0, q.st, h->d_pkeys);
    launch_pdl(h->pdl, k_prange, 152 * 4, 256, 0, q.st, h->p, N, h->d_pkeys);
    q.count += 2;
  }
  if (!extrapolated) {
    launch_pdl(h->pdl, k_extrapolate<S>, 1, 1024, 0, q.st, w.u(), w.v(), c);
    q.count++;
  }
  launch_velocity_advection<S, A>(h, q.st, w.u(), w.v(), w.U[1 - w.cu], w.V[1 - w.cv]);
  w.cu = 1 - w.cu;
  w.cv = 1 - w.cv;
  q.count++;
  if (cfg.enable_smoke && cfg.tunnel_smoke != 0.0f) {
    enqueue_smoke_advection<S, A>(h, w, q);
    launch_pdl(h->pdl, k_finish_smoke<S, A>, (unsigned)((h->N + 256 * kCellsPerThread - 1) / (256 * kCellsPerThread)), 256, 0, q.st, sb, s, c, h->d_params, N);
    q.count++;
  } else {
    settle(h, w, q);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_err(OS_ERR_CUDA, "launch failed: %s", cudaGetErrorString(e));
  if (q.failed) return set_err(OS_ERR_CUDA, "resident projection launch refused");
  return OS_OK;
}

int dispatch_step(os_handle* h, Enq& q) {
  switch (h->storage) {
    case OS_STORAGE_F32: return enqueue_step<float, float>(h, q);
    case OS_STORAGE_F16: return enqueue_step<__half, float>(h, q);
    case OS_STORAGE_BF16: return enqueue_step<__nv_bfloat16, float>(h, q);
    case OS_STORAGE_F64: return enqueue_step<double, double>(h, q);
  }
  return set_err(OS_ERR_INVALID, "bad storage");
}

int dispatch_phase(os_handle* h, int phase, Enq& q) {
  switch (h->storage) {
    case OS_STORAGE_F32: return enqueue_phase<float, float>(h, phase, q);
    case OS_STORAGE_F16: return enqueue_phase<__half, float>(h, phase, q);
    case OS_STORAGE_BF16: return enqueue_phase<__nv_bfloat16, float>(h, phase, q);
    case OS_STORAGE_F64: return enqueue_phase<double, double>(h, phase, q);
  }
  return set_err(OS_ERR_INVALID, "bad storage");
}

int build_graph(os_handle* h) {
  if (h->graph) return OS_OK;
  Enq q{h->stream};
  CUDA_OR_RETURN(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  int rc = dispatch_step(h, q);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return set_err(OS_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&h->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return set_err(OS_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
  h->kernels_per_step = q.count;
  return OS_OK;
}

int push_params(os_handle* h, const os_source* src, float dt, cudaStream_t st) {
  StepParams p;
  memset(&p, 0, sizeof p);
  p.dt = dt;
  if (src && src->active) {
    p.src_active = 1;
    p.src_smoke = src->smoke;
    p.src_velocity = src->velocity;
    p.src_x = src->position_x;
    p.src_y = src->position_y;
  }
  if (h->params_valid && memcmp(&p, &h->last_params, sizeof p) == 0) return OS_OK;
  if (h->h_params) {
    // Pinned staging slot; the previous copy out of it must have completed
    // before it is rewritten.
    CUDA_OR_RETURN(cudaEventSynchronize(h->params_event));
    *h->h_params = p;
    CUDA_OR_RETURN(cudaMemcpyAsync(h->d_params, h->h_params, sizeof p, cudaMemcpyHostToDevice, st));
    CUDA_OR_RETURN(cudaEventRecord(h->params_event, st));
  } else {
    // Handles without a pinned slot (scenarios of a batch): a pageable copy,
    // staged by the driver before the call returns.
    CUDA_OR_RETURN(cudaMemcpyAsync(h->d_params, &p, sizeof p, cudaMemcpyHostToDevice, st));
  }
  h->params_bytes += sizeof p;
  h->last_params = p;
  h->params_valid = true;
  return OS_OK;
}

int validate(const os_config* c) {
  if (c->width < 3 || c->height < 3)
    return set_err(OS_ERR_INVALID, "grid must be at least 3x3 (got %dx%d)", c->width, c->height);
  // The reference indexes cells with int (Fluid::indx, src/fluid.cu:163-165),
  // so its grids stay below 2^31 cells; the library's gathers use 32-bit
  // indices over the grid and its one-cell ring.
  if ((int64_t)(c->width + 2) * (c->height + 2) > INT32_MAX)
    return set_err(OS_ERR_INVALID, "grid too large: (width + 2) * (height + 2) must be below 2^31");
  if ((int)c->cell_size < 1)
    return set_err(OS_ERR_INVALID, "sim.cell_size must be >= 1 (Fluid truncates it to int)");
  if (c->projection_n < 0) return set_err(OS_ERR_INVALID, "sim.projection.n must be >= 0");
  if (c->block_size_x < 1 || c->block_size_y < 1)
    return set_err(OS_ERR_INVALID, "thread.cuda.block_size_* must be >= 1");
  if (storage_bytes(c->storage) == 0) return set_err(OS_ERR_INVALID, "unknown storage %d", c->storage);
  if (c->idw_mode < 0 || c->idw_mode > 2) return set_err(OS_ERR_INVALID, "idw_mode must be 0, 1 or 2");
  if (c->projection_resident < -1 || c->projection_resident > 3)
    return set_err(OS_ERR_INVALID, "projection_resident must be -1, 0, 1, 2 or 3");
  if (c->diffusion_block < 0) return set_err(OS_ERR_INVALID, "diffusion_block must be >= 0");
  if (c->smoke_count != 1) {
    if (c->smoke_count - 1 == 0) return set_err(OS_ERR_INVALID, "smoke_count");
    const int spacing = (c->pipe_height - c->smoke_count * c->smoke_height) / (c->smoke_count - 1);
    if (spacing + c->smoke_height == 0)
      return set_err(OS_ERR_INVALID,
                     "sim.wind_tunnel.smoke_count/smoke_height give a zero smoke period");
  }
  return OS_OK;
}

// Blocking depth and projection form chosen by timing, per configuration
// shape, and the diffusion's own pass depth where it runs pass by pass.
struct TuneChoice {
  int K;
  int resident;
  int diff_k;  // 0: K
};
TuneChoice autotune_projection(const os_config& base);

int ensure_error_words(os_handle* h);

// Sets up the resident projection (mask bit 0) and diffusion (bit 1) that
// the grid fits (flags, error words).
int enable_resident(os_handle* h, int mask) {
  if (h->block_k <= 0 || h->storage == OS_STORAGE_F64 || h->arena) return OS_OK;
  const bool pressure = h->cfg.enable_pressure != 0;
  const int sms = sm_count(h->cfg.device);
  TileGeom g, gd;
  bool proj = (mask & 1) && resident_geom(h->W, h->H, h->block_k, pressure, sms, &g);
  bool diff = (mask & 2) && resident_diffusion_geom(h->W, h->H, h->block_k, sms, &gd);
  switch (h->storage) {
    case OS_STORAGE_F32:
      proj = proj && (pressure ? resident_launchable<true, float>(g, sms)
                               : resident_launchable<false, float>(g, sms));
      diff = diff && resident_diffusion_launchable<float>(gd, sms);
      break;
    case OS_STORAGE_F16:
      proj = proj && (pressure ? resident_launchable<true, __half>(g, sms)
                               : resident_launchable<false, __half>(g, sms));
      diff = diff && resident_diffusion_launchable<__half>(gd, sms);
      break;
    case OS_STORAGE_BF16:
      proj = proj && (pressure ? resident_launchable<true, __nv_bfloat16>(g, sms)
                               : resident_launchable<false, __nv_bfloat16>(g, sms));
      diff = diff && resident_diffusion_launchable<__nv_bfloat16>(gd, sms);
      break;
  }
  cudaGetLastError();
  if (!proj && !diff) return OS_OK;
  const size_t fb = (size_t)sms * sizeof(unsigned);
  CUDA_OR_RETURN(cudaMalloc(&h->rflags, fb));
  CUDA_OR_RETURN(cudaMemset(h->rflags, 0, fb));
  CUDA_OR_RETURN(cudaMalloc(&h->dflags, fb));
  CUDA_OR_RETURN(cudaMemset(h->dflags, 0, fb));
  int rc = ensure_error_words(h);
  if (rc) return rc;
  h->resident = proj;
  h->resident_diff = diff;
  return OS_OK;
}

// Device error word and the mapped host word a kernel sets on a failed
// bounded wait (allocated once).
int ensure_error_words(os_handle* h) {
  if (h->rerr) return OS_OK;
  CUDA_OR_RETURN(cudaMalloc(&h->rerr, sizeof(int)));
  CUDA_OR_RETURN(cudaMemset(h->rerr, 0, sizeof(int)));
  CUDA_OR_RETURN(cudaHostAlloc(&h->host_rerr, sizeof(int), cudaHostAllocMapped));
  *h->host_rerr = 0;
  CUDA_OR_RETURN(cudaHostGetDevicePointer((void**)&h->d_host_rerr, h->host_rerr, 0));
  return OS_OK;
}

// After the handle's stream has drained: a resident projection whose waits
// gave up left its fields undefined and its flags out of step; report it and
// reset the flags so the next launch starts clean.
int check_resident(os_handle* h) {
  if (!h->host_rerr || *(volatile int*)h->host_rerr == 0) return OS_OK;
  *(volatile int*)h->host_rerr = 0;
  const int sms = sm_count(h->cfg.device);
  if (h->rflags) cudaMemsetAsync(h->rflags, 0, (size_t)sms * sizeof(unsigned), h->stream);
  if (h->dflags) cudaMemsetAsync(h->dflags, 0, (size_t)sms * sizeof(unsigned), h->stream);
  cudaMemsetAsync(h->rerr, 0, sizeof(int), h->stream);
  cudaStreamSynchronize(h->stream);
  return set_err(OS_ERR_TIMEOUT,
                 "a bounded device wait gave up (resident projection or diffusion "
                 "neighbours, or a tensor copy); the fields are undefined");
}

void free_handle(os_handle* h) {
  if (!h) return;
  if (h->graph) cudaGraphExecDestroy(h->graph);
  void* ptrs[] = {h->u, h->v, h->s, h->ub, h->vb, h->sb, h->p, h->is_solid,
                  h->total_s, h->flags, h->nbr, h->d_params, h->d_pkeys, h->conv, h->diag};
  for (void* q : ptrs) dev_free(h, q);
  if (h->arena_block) h->arena->release(h->arena_block);
  if (h->h_pkeys) cudaFreeHost(h->h_pkeys);
  if (h->h_params) cudaFreeHost(h->h_params);
  if (h->rflags) cudaFree(h->rflags);
  if (h->dflags) cudaFree(h->dflags);
  if (h->rerr) cudaFree(h->rerr);
  if (h->host_rerr) cudaFreeHost(h->host_rerr);
  if (h->params_event) cudaEventDestroy(h->params_event);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int select_device(const os_handle* h) {
  int cur = -1;
  CUDA_OR_RETURN(cudaGetDevice(&cur));
  if (cur != h->cfg.device) CUDA_OR_RETURN(cudaSetDevice(h->cfg.device));
  return OS_OK;
}

// Host-side float <-> storage conversions for os_upload/os_download.
template <class S>
__global__ void k_from_f32(const float* __restrict__ a, S* __restrict__ x, int64_t n) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) st(x + k, a[k]);
}
template <>
__global__ void k_from_f32<double>(const float* __restrict__ a, double* __restrict__ x, int64_t n) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) x[k] = (double)a[k];
}
template <class S>
__global__ void k_to_f32(const S* __restrict__ x, float* __restrict__ a, int64_t n) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) a[k] = (float)ld<float, S>(x + k);
}
template <>
__global__ void k_to_f32<double>(const double* __restrict__ x, float* __restrict__ a, int64_t n) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) a[k] = (float)x[k];
}

int convert(os_handle* h, void* field, bool to_storage) {
  const int64_t N = (int64_t)h->N;
  const unsigned g = (unsigned)((N + 255) / 256);
  switch (h->storage) {
    case OS_STORAGE_F16:
      if (to_storage) k_from_f32<__half><<<g, 256, 0, h->stream>>>(h->conv, (__half*)field, N);
      else k_to_f32<__half><<<g, 256, 0, h->stream>>>((const __half*)field, h->conv, N);
      break;
    case OS_STORAGE_BF16:
      if (to_storage) k_from_f32<__nv_bfloat16><<<g, 256, 0, h->stream>>>(h->conv, (__nv_bfloat16*)field, N);
      else k_to_f32<__nv_bfloat16><<<g, 256, 0, h->stream>>>((const __nv_bfloat16*)field, h->conv, N);
      break;
    case OS_STORAGE_F64:
      if (to_storage) k_from_f32<double><<<g, 256, 0, h->stream>>>(h->conv, (double*)field, N);
      else k_to_f32<double><<<g, 256, 0, h->stream>>>((const double*)field, h->conv, N);
      break;
    default:
      return set_err(OS_ERR_INVALID, "bad storage");
  }
  h->launches++;
  CUDA_OR_RETURN(cudaGetLastError());
  return OS_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================

extern "C" {

int32_t os_abi_version(void) { return OS_ABI_VERSION; }

const char* os_last_error(void) { return g_err; }

int os_config_defaults(int32_t width, int32_t height, os_config* out) {
  if (!out) return set_err(OS_ERR_INVALID, "null config");
  if (width < 1 || height < 1) return set_err(OS_ERR_INVALID, "bad size");
  memset(out, 0, sizeof *out);
  // src/config_parser.cpp:21-179, in order.
  out->block_size_x = 64;
  out->block_size_y = 1;
  out->height = height;
  out->width = width;
  out->cell_pixel_size = 1;
  out->cell_size = 1.0f;
  out->enable_drain = 1;
  out->enable_pressure = 0;
  out->enable_smoke = 1;
  out->enable_interactive = 0;
  out->projection_n = 50;
  out->projection_o = 1.9f;
  out->pipe_height = height / 4;
  out->pipe_length = 0;  // hard-coded by the parser (config_parser.cpp:64)
  out->smoke_length = 1;
  out->smoke_height = height / 4;
  out->smoke_count = 1;
  out->tunnel_speed = 0.0f;
  out->tunnel_smoke = 1.0f;
  out->g = 0.0f;
  out->d_t = 0.05f;
  out->enable_real_time = 0;
  out->real_time_multiplier = 1.0f;
  out->smoke_enable_decay = 0;
  out->smoke_decay_rate = 0.05f;
  out->obstacle_enable = 1;
  out->obstacle_center_x = width / 2;
  out->obstacle_center_y = height / 2;
  out->obstacle_radius = std::min(height, width) / 30.0f;
  out->density = 1.0f;
  out->drag_coeff = 0.0f;
  out->viscosity = 0.001f;
  out->storage = OS_STORAGE_F32;
  out->device = 0;
  out->projection_block = 0;
  out->idw_mode = 0;
  return OS_OK;
}

// A validated configuration becomes a handle. With an arena, the device
// memory is one block of it (carved by dev_alloc) and the handle gets no
// pinned host slots: such handles are the scenarios of a batch, whose
// creation and release must not stall the device.
static int create_handle(const os_config* cfg, Arena* arena, os_handle** out) {
  os_handle* h = new (std::nothrow) os_handle();
  if (!h) return set_err(OS_ERR_NOMEM, "host allocation failed");
  h->cfg = *cfg;
  h->W = cfg->width;
  h->H = cfg->height;
  h->N = (size_t)cfg->width * cfg->height;
  h->storage = cfg->storage;
  h->esize = storage_bytes(cfg->storage);
  Consts& c = h->c;
  c.W = cfg->width;
  c.H = cfg->height;
  c.h = (int)cfg->cell_size;
  c.n = cfg->projection_n;
  c.g = cfg->g;
  c.density = cfg->density;
  c.viscosity = cfg->viscosity;
  c.o = cfg->projection_o;
  c.drag = cfg->drag_coeff;
  c.speed = cfg->tunnel_speed;
  c.tunnel_smoke = cfg->tunnel_smoke;
  c.decay_rate = cfg->smoke_decay_rate;
  c.smoke_length = cfg->smoke_length;
  c.smoke_count = cfg->smoke_count;
  c.smoke_height = cfg->smoke_height;
  c.pipe_height = cfg->pipe_height;
  c.enable_decay = cfg->smoke_enable_decay != 0;
  c.enable_pressure = cfg->enable_pressure != 0;
  c.idw_mode = cfg->idw_mode;
  if (cfg->smoke_count != 1) {
    const int spacing = (cfg->pipe_height - cfg->smoke_count * cfg->smoke_height) /
                        (cfg->smoke_count - 1);
    h->smoke_period = spacing + cfg->smoke_height;
  }
  h->block_k = choose_block_k(h);
  h->diff_k = cfg->diffusion_block > 0 ? std::min(cfg->diffusion_block, 32) : 0;

  auto fail = [&](int code) {
    free_handle(h);
    return code;
  };
  cudaError_t e = cudaSetDevice(cfg->device);
  if (e != cudaSuccess)
    return fail(set_err(OS_ERR_CUDA, "cudaSetDevice(%d): %s", cfg->device, cudaGetErrorString(e)));
  // The depth and form are chosen before this handle allocates anything, so
  // that the trial handles never share the device with it.
  int resident = cfg->projection_resident > 0 ? cfg->projection_resident : 0;
  if (h->block_k == 0) {
    if (h->storage == OS_STORAGE_F64) {
      h->block_k = -1;
    } else {
      const TuneChoice t = autotune_projection(*cfg);
      h->block_k = t.K;
      if (t.diff_k > 0) h->diff_k = t.diff_k;
      resident = t.resident;
    }
  }
  if (arena) {
    h->arena = arena;
    h->arena_size = handle_footprint(*cfg);
    h->arena_block = static_cast<char*>(arena->alloc(h->arena_size));
    if (!h->arena_block)
      return fail(set_err(OS_ERR_NOMEM, "device budget: %zu bytes needed, %zu of %zu in use",
                          h->arena_size, arena->used(), arena->capacity()));
    h->device_bytes = h->arena_size;
  }
  if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return fail(set_err(OS_ERR_CUDA, "stream: %s", cudaGetErrorString(e)));
  const size_t fb = h->N * h->esize;
  void** fields[] = {&h->u, &h->v, &h->s, &h->ub, &h->vb, &h->sb};
  for (void** f : fields) {
    if ((e = dev_alloc(h, f, fb)) != cudaSuccess)
      return fail(set_err(OS_ERR_NOMEM, "cudaMalloc(%zu): %s", fb, cudaGetErrorString(e)));
    cudaMemsetAsync(*f, 0, fb, h->stream);
  }
  if ((e = dev_alloc(h, (void**)&h->p, h->N * 4)) != cudaSuccess ||
      (e = dev_alloc(h, (void**)&h->is_solid, h->N * 4)) != cudaSuccess ||
      (e = dev_alloc(h, (void**)&h->total_s, h->N * 4)) != cudaSuccess ||
      (e = dev_alloc(h, (void**)&h->flags, h->N)) != cudaSuccess ||
      (e = dev_alloc(h, (void**)&h->nbr, (size_t)(h->W + 2) * (h->H + 2) * sizeof(uint16_t))) !=
          cudaSuccess ||
      (e = dev_alloc(h, (void**)&h->d_params, sizeof(StepParams))) != cudaSuccess ||
      (e = dev_alloc(h, (void**)&h->d_pkeys, 2 * sizeof(int))) != cudaSuccess)
    return fail(set_err(OS_ERR_NOMEM, "cudaMalloc: %s", cudaGetErrorString(e)));
  if (!arena) {
    if ((e = cudaMallocHost(&h->h_pkeys, 2 * sizeof(int))) != cudaSuccess ||
        (e = cudaMallocHost(&h->h_params, sizeof(StepParams))) != cudaSuccess)
      return fail(set_err(OS_ERR_NOMEM, "cudaMallocHost: %s", cudaGetErrorString(e)));
    if ((e = cudaEventCreateWithFlags(&h->params_event, cudaEventDisableTiming)) != cudaSuccess)
      return fail(set_err(OS_ERR_CUDA, "event: %s", cudaGetErrorString(e)));
  }
  cudaMemsetAsync(h->p, 0, h->N * 4, h->stream);
  MaskParams m;
  m.enable_drain = cfg->enable_drain != 0;
  m.obstacle_enable = cfg->obstacle_enable != 0;
  m.cx = cfg->obstacle_center_x;
  m.cy = cfg->obstacle_center_y;
  m.pipe_length = cfg->pipe_length;
  m.pipe_height = cfg->pipe_height;
  m.radius = cfg->obstacle_radius;
  const dim3 g2((h->W + 127) / 128, h->H);
  k_init_solid<<<g2, 128, 0, h->stream>>>(h->is_solid, c, m);
  k_init_flags<<<g2, 128, 0, h->stream>>>(h->is_solid, h->total_s, h->flags, c);
  k_init_neighbourhoods<<<dim3((h->W + 2 + 127) / 128, h->H + 2), 128, 0, h->stream>>>(
      h->is_solid, h->nbr, c);
  h->launches += 3;
  if ((e = cudaGetLastError()) != cudaSuccess ||
      (e = cudaStreamSynchronize(h->stream)) != cudaSuccess)
    return fail(set_err(OS_ERR_CUDA, "init: %s", cudaGetErrorString(e)));
  if (resident) {
    const int rc = enable_resident(h, resident);
    if (rc) return fail(rc);
  }
  const char* pdl_env = std::getenv("OPENSAYAL_GB300_PDL");
  h->pdl = !(pdl_env && pdl_env[0] == '0');
  // Tensor-copy staging of the diffusion passes is opt-in: inside a step it
  // measured 2% slower than the vector loads (with programmatic launch both
  // overlap the previous kernel, the vector loads more so).
  const char* tma_env = std::getenv("OPENSAYAL_GB300_TMA");
  if (!arena && tma_env && tma_env[0] == '1' && prepare_tma_diffusion(h)) {
    const int rc = ensure_error_words(h);
    if (rc) return fail(rc);
    h->tma_diffusion = true;
  }
  *out = h;
  return OS_OK;
}

int os_create(const os_config* cfg, os_handle** out) {
  if (!cfg || !out) return set_err(OS_ERR_INVALID, "null argument");
  *out = nullptr;
  int rc = validate(cfg);
  if (rc) return rc;
  return create_handle(cfg, nullptr, out);
}

int os_destroy(os_handle* h) {
  if (!h) return OS_OK;
  cudaSetDevice(h->cfg.device);
  cudaStreamSynchronize(h->stream);
  free_handle(h);
  return OS_OK;
}

int os_update_async(os_handle* h, const os_source* src, float dt, int32_t steps, void* stream) {
  if (!h) return set_err(OS_ERR_INVALID, "null handle");
  if (steps < 0) return set_err(OS_ERR_INVALID, "steps < 0");
  int rc = select_device(h);
  if (rc) return rc;
  if ((rc = build_graph(h))) return rc;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : h->stream;
  if ((rc = push_params(h, src, dt, st))) return rc;
  for (int t = 0; t < steps; t++) CUDA_OR_RETURN(cudaGraphLaunch(h->graph, st));
  h->launches += (int64_t)steps * h->kernels_per_step;
  return OS_OK;
}

int os_synchronize(os_handle* h) {
  if (!h) return set_err(OS_ERR_INVALID, "null handle");
  CUDA_OR_RETURN(cudaStreamSynchronize(h->stream));
  return check_resident(h);
}

int os_query(os_handle* h, int32_t* idle) {
  if (!h || !idle) return set_err(OS_ERR_INVALID, "null argument");
  *idle = 0;
  int rc = select_device(h);
  if (rc) return rc;
  const cudaError_t e = cudaStreamQuery(h->stream);
  if (e == cudaErrorNotReady) return OS_OK;
  if (e != cudaSuccess) return set_err(OS_ERR_CUDA, "stream query: %s", cudaGetErrorString(e));
  if ((rc = check_resident(h))) return rc;
  *idle = 1;
  return OS_OK;
}

int os_update(os_handle* h, const os_source* src, float dt) {
  int rc = os_update_async(h, src, dt, 1, nullptr);
  if (rc) return rc;
  if (h->cfg.enable_pressure)
    CUDA_OR_RETURN(cudaMemcpyAsync(h->h_pkeys, h->d_pkeys, 2 * sizeof(int),
                                   cudaMemcpyDeviceToHost, h->stream));
  CUDA_OR_RETURN(cudaStreamSynchronize(h->stream));
  if ((rc = check_resident(h))) return rc;
  if (h->cfg.enable_pressure) {
    h->min_pressure = key_to_float(h->h_pkeys[0]);
    h->max_pressure = key_to_float(h->h_pkeys[1]);
  }
  return OS_OK;
}

int os_fields(os_handle* h, os_fields_view* out) {
  if (!h || !out) return set_err(OS_ERR_INVALID, "null argument");
  memset(out, 0, sizeof *out);
  out->width = h->W;
  out->height = h->H;
  out->storage = h->storage;
  out->projection_block = h->block_k;
  out->vel_x = h->u;
  out->vel_y = h->v;
  out->smoke = h->s;
  out->pressure = h->p;
  out->is_solid = h->is_solid;
  out->total_s = h->total_s;
  out->projection_resident = (h->resident ? 1 : 0) | (h->resident_diff ? 2 : 0);
  out->tma_staging = h->tma_diffusion ? 1 : 0;
  return OS_OK;
}

static int field_target(os_handle* h, int32_t field, void** ptr, bool* is_float_field) {
  *is_float_field = true;
  switch (field) {
    case OS_FIELD_VEL_X: *ptr = h->u; return OS_OK;
    case OS_FIELD_VEL_Y: *ptr = h->v; return OS_OK;
    case OS_FIELD_SMOKE: *ptr = h->s; return OS_OK;
    case OS_FIELD_PRESSURE: *ptr = h->p; *is_float_field = false; return OS_OK;
    case OS_FIELD_IS_SOLID: *ptr = h->is_solid; *is_float_field = false; return OS_OK;
    case OS_FIELD_TOTAL_S: *ptr = h->total_s; *is_float_field = false; return OS_OK;
  }
  return set_err(OS_ERR_INVALID, "unknown field %d", field);
}

int os_upload(os_handle* h, int32_t field, const void* host, size_t count) {
  if (!h || !host) return set_err(OS_ERR_INVALID, "null argument");
  if (count != h->N) return set_err(OS_ERR_INVALID, "count %zu != width*height %zu", count, h->N);
  if (field == OS_FIELD_IS_SOLID || field == OS_FIELD_TOTAL_S)
    return set_err(OS_ERR_INVALID, "the solid mask and neighbour counts are fixed at creation");
  void* dst;
  bool storage_field;
  int rc = field_target(h, field, &dst, &storage_field);
  if (rc) return rc;
  if ((rc = select_device(h))) return rc;
  if (!storage_field || h->storage == OS_STORAGE_F32) {
    CUDA_OR_RETURN(cudaMemcpyAsync(dst, host, h->N * 4, cudaMemcpyHostToDevice, h->stream));
  } else {
    if (!h->conv) CUDA_OR_RETURN(dev_alloc(h, (void**)&h->conv, h->N * 4));
    CUDA_OR_RETURN(cudaMemcpyAsync(h->conv, host, h->N * 4, cudaMemcpyHostToDevice, h->stream));
    if ((rc = convert(h, dst, true))) return rc;
  }
  CUDA_OR_RETURN(cudaStreamSynchronize(h->stream));
  return OS_OK;
}

int os_download(os_handle* h, int32_t field, void* host, size_t count) {
  if (!h || !host) return set_err(OS_ERR_INVALID, "null argument");
  if (count != h->N) return set_err(OS_ERR_INVALID, "count %zu != width*height %zu", count, h->N);
  void* src;
  bool storage_field;
  int rc = field_target(h, field, &src, &storage_field);
  if (rc) return rc;
  if ((rc = select_device(h))) return rc;
  if (!storage_field || h->storage == OS_STORAGE_F32) {
    CUDA_OR_RETURN(cudaMemcpyAsync(host, src, h->N * 4, cudaMemcpyDeviceToHost, h->stream));
  } else {
    if (!h->conv) CUDA_OR_RETURN(dev_alloc(h, (void**)&h->conv, h->N * 4));
    if ((rc = convert(h, src, false))) return rc;
    CUDA_OR_RETURN(cudaMemcpyAsync(host, h->conv, h->N * 4, cudaMemcpyDeviceToHost, h->stream));
  }
  CUDA_OR_RETURN(cudaStreamSynchronize(h->stream));
  return OS_OK;
}

int os_snapshot_async(os_handle* h, int32_t field, void* device_dst, size_t count,
                      void* stream) {
  if (!h || !device_dst) return set_err(OS_ERR_INVALID, "null argument");
  if (count != h->N) return set_err(OS_ERR_INVALID, "count %zu != width*height %zu", count, h->N);
  void* src;
  bool storage_field;
  int rc = field_target(h, field, &src, &storage_field);
  if (rc) return rc;
  if ((rc = select_device(h))) return rc;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : h->stream;
  if (!storage_field || h->storage == OS_STORAGE_F32) {
    CUDA_OR_RETURN(cudaMemcpyAsync(device_dst, src, h->N * 4, cudaMemcpyDeviceToDevice, st));
    return OS_OK;
  }
  const int64_t N = (int64_t)h->N;
  const unsigned g = (unsigned)((N + 255) / 256);
  float* dst = static_cast<float*>(device_dst);
  switch (h->storage) {
    case OS_STORAGE_F16: k_to_f32<__half><<<g, 256, 0, st>>>((const __half*)src, dst, N); break;
    case OS_STORAGE_BF16:
      k_to_f32<__nv_bfloat16><<<g, 256, 0, st>>>((const __nv_bfloat16*)src, dst, N);
      break;
    case OS_STORAGE_F64: k_to_f32<double><<<g, 256, 0, st>>>((const double*)src, dst, N); break;
    default: return set_err(OS_ERR_INVALID, "bad storage");
  }
  h->launches++;
  CUDA_OR_RETURN(cudaGetLastError());
  return OS_OK;
}

int os_diagnose(os_handle* h, os_diag* out) {
  if (!h || !out) return set_err(OS_ERR_INVALID, "null argument");
  static_assert(kDiagBytes == (kDiagBlocks + 1) * kDiagSlots * sizeof(double),
                "diagnostics scratch size");
  int rc = select_device(h);
  if (rc) return rc;
  if (!h->diag) CUDA_OR_RETURN(dev_alloc(h, (void**)&h->diag, kDiagBytes));
  double* partials = h->diag;
  double* res = h->diag + (size_t)kDiagBlocks * kDiagSlots;
  const int64_t need = ((int64_t)h->N + kDiagThreads - 1) / kDiagThreads;
  const int blocks = (int)std::min<int64_t>(kDiagBlocks, std::max<int64_t>(1, need));
  const uint8_t* fl = h->flags;
  switch (h->storage) {
    case OS_STORAGE_F32:
      k_diag_partial<float><<<blocks, kDiagThreads, 0, h->stream>>>(
          (const float*)h->u, (const float*)h->v, (const float*)h->s, fl, h->c, partials);
      break;
    case OS_STORAGE_F16:
      k_diag_partial<__half><<<blocks, kDiagThreads, 0, h->stream>>>(
          (const __half*)h->u, (const __half*)h->v, (const __half*)h->s, fl, h->c, partials);
      break;
    case OS_STORAGE_BF16:
      k_diag_partial<__nv_bfloat16><<<blocks, kDiagThreads, 0, h->stream>>>(
          (const __nv_bfloat16*)h->u, (const __nv_bfloat16*)h->v, (const __nv_bfloat16*)h->s,
          fl, h->c, partials);
      break;
    default:
      k_diag_partial<double><<<blocks, kDiagThreads, 0, h->stream>>>(
          (const double*)h->u, (const double*)h->v, (const double*)h->s, fl, h->c, partials);
      break;
  }
  k_diag_final<<<1, kDiagThreads, 0, h->stream>>>(partials, blocks, res);
  h->launches += 2;
  CUDA_OR_RETURN(cudaGetLastError());
  double v[kDiagSlots];
  CUDA_OR_RETURN(cudaMemcpyAsync(v, res, sizeof v, cudaMemcpyDeviceToHost, h->stream));
  CUDA_OR_RETURN(cudaStreamSynchronize(h->stream));
  const double cs = (double)h->c.h;
  memset(out, 0, sizeof *out);
  out->divergence_l2 = sqrt(v[0]);
  out->divergence_sum = v[1];
  out->divergence_max = v[kDiagSums];
  out->smoke_mass = v[2] * cs * cs;
  out->inflow_flux = v[3] * cs;
  out->outflow_flux = v[4] * cs;
  out->active_cells = (int64_t)v[5];
  return OS_OK;
}

int os_visual_defaults(os_visual_config* out) {
  if (!out) return set_err(OS_ERR_INVALID, "null argument");
  memset(out, 0, sizeof *out);
  out->cell_pixel_size = 1;
  out->arrow_distance = 20;
  out->arrow_length_multiplier = 0.1f;
  out->arrow_disable_threshold = 0.0f;
  out->arrow_head_length = 5;
  out->trace_distance = 20;
  out->trace_length = 20;
  return OS_OK;
}

int os_config_parse(const char* json_text, size_t length, os_config* cfg,
                    os_visual_config* visual) {
  if (!json_text || !cfg) return set_err(OS_ERR_INVALID, "null argument");
  try {
    const Config c =
        opensayal::config_from_json(opensayal::json::parse(std::string(json_text, length)));
    int rc = opensayal::to_os_config(c, cfg);
    if (rc != OS_OK) return rc;
    if (visual) opensayal::to_os_visual_config(c, visual);
  } catch (const std::exception& e) {
    return set_err(OS_ERR_INVALID, "config: %s", e.what());
  }
  return OS_OK;
}

static int visual_params(const os_handle* h, const os_visual_config* v, VisualParams* vp) {
  if (!v) return set_err(OS_ERR_INVALID, "null visual config");
  if (v->cell_pixel_size < 1 || v->arrow_distance < 1 || v->trace_distance < 1 ||
      v->trace_length < 1)
    return set_err(OS_ERR_INVALID, "visual distances, lengths and pixel size must be >= 1");
  memset(vp, 0, sizeof *vp);
  vp->cell_px = v->cell_pixel_size;
  vp->arrow_distance = v->arrow_distance;
  vp->arrow_length_multiplier = v->arrow_length_multiplier;
  vp->arrow_disable_threshold = v->arrow_disable_threshold;
  vp->arrow_head_length = (float)v->arrow_head_length;
  vp->arrow_head_angle = (float)(M_PI / 8);  // ARROW_HEAD_ANGLE, inc/config.hpp:6
  vp->arrows_w = h->W / v->arrow_distance;
  vp->arrows_h = h->H / v->arrow_distance;
  vp->trace_distance = v->trace_distance;
  vp->trace_length = v->trace_length;
  vp->traces_w = h->W / v->trace_distance;
  vp->traces_h = h->H / v->trace_distance;
  return OS_OK;
}

int os_render_pixels(os_handle* h, int32_t* d_pixels, void* stream) {
  if (!h || !d_pixels) return set_err(OS_ERR_INVALID, "null argument");
  int rc = select_device(h);
  if (rc) return rc;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : h->stream;
  const int64_t n = (int64_t)h->N;
  const unsigned g = (unsigned)((n + 4 * 128 - 1) / (4 * 128));
  const int ep = h->cfg.enable_pressure != 0, es = h->cfg.enable_smoke != 0;
  // Field arrays come from cudaMalloc or the arena (256-byte aligned).
  const int vec = (reinterpret_cast<uintptr_t>(d_pixels) % 16) == 0;
  switch (h->storage) {
    case OS_STORAGE_F32:
      k_render_pixels<float><<<g, 128, 0, st>>>((const float*)h->s, h->p, h->flags, n, ep, es,
                                                h->min_pressure, h->max_pressure, d_pixels, vec);
      break;
    case OS_STORAGE_F16:
      k_render_pixels<__half><<<g, 128, 0, st>>>((const __half*)h->s, h->p, h->flags, n, ep, es,
                                                 h->min_pressure, h->max_pressure, d_pixels, vec);
      break;
    case OS_STORAGE_BF16:
      k_render_pixels<__nv_bfloat16><<<g, 128, 0, st>>>((const __nv_bfloat16*)h->s, h->p,
                                                        h->flags, n, ep, es, h->min_pressure,
                                                        h->max_pressure, d_pixels, vec);
      break;
    default:
      return set_err(OS_ERR_UNSUPPORTED, "visuals need FP32, FP16 or BF16 storage");
  }
  h->launches++;
  CUDA_OR_RETURN(cudaGetLastError());
  return OS_OK;
}

int os_render_arrows(os_handle* h, const os_visual_config* v, os_arrow* d_arrows, void* stream) {
  if (!h || !d_arrows) return set_err(OS_ERR_INVALID, "null argument");
  VisualParams vp;
  int rc = visual_params(h, v, &vp);
  if (rc || (rc = select_device(h))) return rc;
  if (vp.arrows_w < 1 || vp.arrows_h < 1) return OS_OK;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : h->stream;
  const dim3 b(16, 16), g((vp.arrows_w + 15) / 16, (vp.arrows_h + 15) / 16);
  switch (h->storage) {
    case OS_STORAGE_F32:
      k_render_arrows<float><<<g, b, 0, st>>>((const float*)h->u, (const float*)h->v, h->flags,
                                              h->nbr, h->c, vp, d_arrows);
      break;
    case OS_STORAGE_F16:
      k_render_arrows<__half><<<g, b, 0, st>>>((const __half*)h->u, (const __half*)h->v,
                                               h->flags, h->nbr, h->c, vp, d_arrows);
      break;
    case OS_STORAGE_BF16:
      k_render_arrows<__nv_bfloat16><<<g, b, 0, st>>>(
          (const __nv_bfloat16*)h->u, (const __nv_bfloat16*)h->v, h->flags, h->nbr, h->c, vp, d_arrows);
      break;
    default:
      return set_err(OS_ERR_UNSUPPORTED, "visuals need FP32, FP16 or BF16 storage");
  }
  h->launches++;
  CUDA_OR_RETURN(cudaGetLastError());
  return OS_OK;
}

int os_render_traces(os_handle* h, const os_visual_config* v, float dt, int32_t* d_x,
                     int32_t* d_y, void* stream) {
  if (!h || !d_x || !d_y) return set_err(OS_ERR_INVALID, "null argument");
  VisualParams vp;
  int rc = visual_params(h, v, &vp);
  if (rc || (rc = select_device(h))) return rc;
  if (vp.traces_w < 1 || vp.traces_h < 1) return OS_OK;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : h->stream;
  const dim3 b(16, 16), g((vp.traces_w + 15) / 16, (vp.traces_h + 15) / 16);
  switch (h->storage) {
    case OS_STORAGE_F32:
      k_render_traces<float><<<g, b, 0, st>>>((const float*)h->u, (const float*)h->v, h->flags,
                                              h->nbr, h->c, vp, dt, d_x, d_y);
      break;
    case OS_STORAGE_F16:
      k_render_traces<__half><<<g, b, 0, st>>>((const __half*)h->u, (const __half*)h->v,
                                               h->flags, h->nbr, h->c, vp, dt, d_x, d_y);
      break;
    case OS_STORAGE_BF16:
      k_render_traces<__nv_bfloat16><<<g, b, 0, st>>>((const __nv_bfloat16*)h->u,
                                                      (const __nv_bfloat16*)h->v, h->flags, h->nbr,
                                                      h->c, vp, dt, d_x, d_y);
      break;
    default:
      return set_err(OS_ERR_UNSUPPORTED, "visuals need FP32, FP16 or BF16 storage");
  }
  h->launches++;
  CUDA_OR_RETURN(cudaGetLastError());
  return OS_OK;
}

int os_selftest_bounded_wait(int32_t device, int32_t* status) {
  if (!status) return set_err(OS_ERR_INVALID, "null argument");
  *status = OS_OK;
  CUDA_OR_RETURN(cudaSetDevice(device));
  unsigned* flags = nullptr;
  int* dev_err = nullptr;
  int* host_err = nullptr;
  int* d_host_err = nullptr;
  cudaError_t e = cudaMalloc(&flags, 2 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(flags, 0, 2 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&dev_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(dev_err, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaHostAlloc(&host_err, sizeof(int), cudaHostAllocMapped);
  if (e == cudaSuccess) {
    *host_err = 0;
    e = cudaHostGetDevicePointer((void**)&d_host_err, host_err, 0);
  }
  if (e == cudaSuccess) {
    k_wait_selftest<<<1, 32>>>(ResidentSync{flags, dev_err, d_host_err});
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) *status = *(volatile int*)host_err ? OS_ERR_TIMEOUT : OS_OK;
  if (flags) cudaFree(flags);
  if (dev_err) cudaFree(dev_err);
  if (host_err) cudaFreeHost(host_err);
  if (e != cudaSuccess) return set_err(OS_ERR_CUDA, "self-test: %s", cudaGetErrorString(e));
  return OS_OK;
}

namespace {

// One pass of the bandwidth probe: every thread copies its float4 elements
// of the buffer `reps` times, alternating direction (a -> b, then b -> a),
// with cache-at-L2 loads and stores in volatile inline PTX, so that no copy
// is elided or served from L1. Grid-stride over n4 elements.
__global__ void k_probe_copy(float4* a, float4* b, int64_t n4, int reps) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int r = 0; r < reps; r++) {
    float4* src = (r & 1) ? b : a;
    float4* dst = (r & 1) ? a : b;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += stride) {
      float4 x;
      asm volatile("ld.global.cg.v4.f32 {%0, %1, %2, %3}, [%4];"
                   : "=f"(x.x), "=f"(x.y), "=f"(x.z), "=f"(x.w)
                   : "l"(src + k));
      asm volatile("st.global.cg.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst + k), "f"(x.x),
                   "f"(x.y), "f"(x.z), "f"(x.w)
                   : "memory");
    }
  }
}

}  // namespace

int os_probe_copy_bandwidth(int32_t device, uint64_t bytes, int32_t reps, float* gbs) {
  if (!gbs || reps < 1 || bytes < 16 || (bytes & 15))
    return set_err(OS_ERR_INVALID, "probe: bytes must be a positive multiple of 16, reps >= 1");
  *gbs = 0.0f;
  CUDA_OR_RETURN(cudaSetDevice(device));
  float4* a = nullptr;
  float4* b = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaStream_t st = nullptr;
  cudaError_t e = cudaMalloc(&a, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&b, bytes);
  if (e == cudaSuccess) e = cudaMemset(a, 0, bytes);
  if (e == cudaSuccess) e = cudaMemset(b, 0, bytes);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  const int64_t n4 = (int64_t)(bytes / 16);
  const int blocks = sm_count(device) * 4;
  if (e == cudaSuccess) {
    k_probe_copy<<<blocks, 512, 0, st>>>(a, b, n4, 2);  // first touch
    cudaEventRecord(e0, st);
    k_probe_copy<<<blocks, 512, 0, st>>>(a, b, n4, reps);
    cudaEventRecord(e1, st);
    e = cudaEventSynchronize(e1);
  }
  float ms = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e == cudaSuccess && ms > 0.0f) *gbs = (float)(2.0 * (double)bytes * reps / (ms * 1e-3) / 1e9);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (a) cudaFree(a);
  if (b) cudaFree(b);
  if (e != cudaSuccess) return set_err(OS_ERR_CUDA, "probe: %s", cudaGetErrorString(e));
  return OS_OK;
}

int os_pressure_range(os_handle* h, float* min_out, float* max_out) {
  if (!h || !min_out || !max_out) return set_err(OS_ERR_INVALID, "null argument");
  *min_out = h->min_pressure;
  *max_out = h->max_pressure;
  return OS_OK;
}

int os_run_phase(os_handle* h, int32_t phase, const os_source* src, float dt) {
  if (!h) return set_err(OS_ERR_INVALID, "null handle");
  int rc = select_device(h);
  if (rc) return rc;
  if ((rc = push_params(h, src, dt, h->stream))) return rc;
  Enq q{h->stream};
  if ((rc = dispatch_phase(h, phase, q))) return rc;
  h->launches += q.count;
  if (phase == OS_PHASE_PRESSURE_RANGE)
    CUDA_OR_RETURN(cudaMemcpyAsync(h->h_pkeys, h->d_pkeys, 2 * sizeof(int),
                                   cudaMemcpyDeviceToHost, h->stream));
  CUDA_OR_RETURN(cudaStreamSynchronize(h->stream));
  if ((rc = check_resident(h))) return rc;
  if (phase == OS_PHASE_PRESSURE_RANGE) {
    h->min_pressure = key_to_float(h->h_pkeys[0]);
    h->max_pressure = key_to_float(h->h_pkeys[1]);
  }
  return OS_OK;
}

int os_kernel_launches(os_handle* h, int64_t* out) {
  if (!h || !out) return set_err(OS_ERR_INVALID, "null argument");
  *out = h->launches;
  return OS_OK;
}

int os_profile_phase_kernels(os_handle* h, int32_t phase, const os_source* src, float dt,
                             int32_t reps, void* stream, float* kernel_ms_out, float* ms_out,
                             int32_t* kernels_out) {
  if (!h || !kernel_ms_out || !ms_out || reps < 1) return set_err(OS_ERR_INVALID, "bad argument");
  int rc = select_device(h);
  if (rc) return rc;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : h->stream;
  if ((rc = push_params(h, src, dt, st))) return rc;
  std::vector<cudaEvent_t> ev(2 * (size_t)reps + 1, nullptr);
  for (auto& x : ev)
    if (cudaEventCreate(&x) != cudaSuccess) {
      for (auto& y : ev)
        if (y) cudaEventDestroy(y);
      return set_err(OS_ERR_CUDA, "profile: event creation failed");
    }
  // ev[2r]: repetition r starts; ev[2r+1]: its own kernels done; ev[2reps]: end.
  Enq q{st};
  for (int r = 0; r < reps && rc == OS_OK; r++) {
    cudaEventRecord(ev[2 * r], st);
    q.kernels_done = ev[2 * r + 1];
    rc = dispatch_phase(h, phase, q);
    // Phases without a copy back leave the mark unrecorded: their kernels
    // are the whole repetition.
    if (phase != OS_PHASE_DIFFUSION && phase != OS_PHASE_PROJECTION)
      cudaEventRecord(ev[2 * r + 1], st);
  }
  cudaEventRecord(ev[2 * reps], st);
  cudaError_t e = cudaEventSynchronize(ev[2 * reps]);
  float kernels_ms = 0.0f, total = 0.0f;
  for (int r = 0; r < reps && e == cudaSuccess; r++) {
    float x = 0.0f;
    e = cudaEventElapsedTime(&x, ev[2 * r], ev[2 * r + 1]);
    kernels_ms += x;
  }
  if (e == cudaSuccess) e = cudaEventElapsedTime(&total, ev[0], ev[2 * reps]);
  for (auto& x : ev) cudaEventDestroy(x);
  if (rc) return rc;
  if (e != cudaSuccess) return set_err(OS_ERR_CUDA, "profile: %s", cudaGetErrorString(e));
  if ((rc = check_resident(h))) return rc;
  h->launches += q.count;
  *kernel_ms_out = kernels_ms;
  *ms_out = total;
  if (kernels_out) *kernels_out = q.count;
  return OS_OK;
}

int os_profile_phase(os_handle* h, int32_t phase, const os_source* src, float dt, int32_t reps,
                     void* stream, float* ms_out, int32_t* kernels_out) {
  if (!h || !ms_out || reps < 1) return set_err(OS_ERR_INVALID, "bad argument");
  int rc = select_device(h);
  if (rc) return rc;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : h->stream;
  if ((rc = push_params(h, src, dt, st))) return rc;
  cudaEvent_t a = nullptr, b = nullptr;
  CUDA_OR_RETURN(cudaEventCreate(&a));
  CUDA_OR_RETURN(cudaEventCreate(&b));
  Enq q{st};
  cudaEventRecord(a, st);
  for (int r = 0; r < reps && rc == OS_OK; r++) rc = dispatch_phase(h, phase, q);
  cudaEventRecord(b, st);
  cudaError_t e = cudaEventSynchronize(b);
  float ms = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  if (e != cudaSuccess) return set_err(OS_ERR_CUDA, "profile: %s", cudaGetErrorString(e));
  if ((rc = check_resident(h))) return rc;
  h->launches += q.count;
  *ms_out = ms;
  if (kernels_out) *kernels_out = q.count;
  return OS_OK;
}

}  // extern "C"

// ===========================================================================
// Autotuner for the blocking depth
//
// The best number of sweeps per blocked pass depends on the grid: a deeper
// pass stages the field fewer times but recomputes a wider halo and, at some
// depth, no longer fits one tile per SM. os_create with projection_block == 0
// times each candidate depth on a scratch grid of the same configuration
// (2 warm-up steps, then 3 timed with CUDA events) and keeps the fastest. The
// answer is cached per process for the configuration's shape, so later
// handles of the same shape pay nothing. OPENSAYAL_GB300_AUTOTUNE=0 skips the
// timing and uses 4.
// ===========================================================================

namespace {

struct TuneKey {
  int W, H, n, viscous, pressure, storage, device, resident, diffusion_block;
  bool operator<(const TuneKey& o) const {
    return std::tie(W, H, n, viscous, pressure, storage, device, resident, diffusion_block) <
           std::tie(o.W, o.H, o.n, o.viscous, o.pressure, o.storage, o.device, o.resident,
                    o.diffusion_block);
  }
};
std::map<TuneKey, TuneChoice> g_tuned;
std::mutex g_tune_mu;

float time_steps(os_handle* t, float dt, int warm, int reps) {
  if (os_update_async(t, nullptr, dt, warm, nullptr) != OS_OK) return -1.0f;
  cudaEvent_t a = nullptr, b = nullptr;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return -1.0f;
  float ms = -1.0f;
  cudaEventRecord(a, t->stream);
  if (os_update_async(t, nullptr, dt, reps, nullptr) == OS_OK) {
    cudaEventRecord(b, t->stream);
    if (cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&ms, a, b) != cudaSuccess)
      ms = -1.0f;
  }
  cudaStreamSynchronize(t->stream);
  if (check_resident(t) != OS_OK) ms = -1.0f;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms;
}

// Candidates: depths {2, 4, 6, 8, 12} pass by pass and, unless
// projection_resident is -1, the resident forms the depth allows (projection
// for even depths, diffusion for multiples of 4, alone or together) where
// the grid fits them; a positive projection_resident fixes the forms and
// leaves only the depth to choose.
TuneChoice autotune_projection(const os_config& base) {
  constexpr TuneChoice kDefault{4, 0, 0};
  const char* env = std::getenv("OPENSAYAL_GB300_AUTOTUNE");
  if (env && env[0] == '0')
    return TuneChoice{kDefault.K, base.projection_resident > 0 ? base.projection_resident : 0, 0};
  const TuneKey key{base.width, base.height, base.projection_n, base.viscosity != 0.0f,
                    base.enable_pressure != 0, base.storage, base.device,
                    base.projection_resident, base.diffusion_block};
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) return it->second;
  }
  std::vector<TuneChoice> cands;
  for (int K : {2, 4, 6, 8, 12}) {
    if (base.projection_resident > 0) {
      cands.push_back({K, base.projection_resident, 0});
      continue;
    }
    cands.push_back({K, 0, 0});
    if (base.projection_resident == -1) continue;
    if (K % 2 == 0 && K <= 8) cands.push_back({K, 1, 0});
    if (K % 4 == 0 && base.viscosity != 0.0f) {
      cands.push_back({K, 2, 0});
      if (K <= 8) cands.push_back({K, 3, 0});
    }
  }
  const float dt = base.d_t > 0.0f ? base.d_t : 0.05f;
  // ms per step of a candidate over `steps` steps, or 0 when the grid does
  // not take that form.
  auto time_choice = [&](const TuneChoice& cand, int steps) -> float {
    os_config c = base;
    c.projection_block = cand.K;
    c.projection_resident = cand.resident ? cand.resident : -1;
    os_handle* t = nullptr;
    if (os_create(&c, &t) != OS_OK) return 0.0f;  // e.g. out of memory: skip
    const int got = (t->resident ? 1 : 0) | (t->resident_diff ? 2 : 0);
    if (got != cand.resident) {  // the grid does not fit that form
      os_destroy(t);
      return 0.0f;
    }
    if (cand.diff_k > 0) t->diff_k = cand.diff_k;  // before the first step captures the graph
    const float ms = time_steps(t, dt, 3, steps);
    os_destroy(t);
    return ms;
  };
  // Two rounds: 12 steps of every candidate, then 60 steps of the three
  // fastest, since forms within a percent of each other are told apart only
  // by longer timings.
  std::vector<std::pair<float, TuneChoice>> timed;
  for (const TuneChoice& cand : cands)
    if (cand.K <= std::max(1, base.projection_n)) {
      const float ms = time_choice(cand, 12);
      if (ms > 0.0f) timed.push_back({ms, cand});
    }
  std::sort(timed.begin(), timed.end(),
            [](const auto& a, const auto& b) { return a.first < b.first; });
  TuneChoice best = kDefault;
  float best_ms = 0.0f;
  for (size_t r = 0; r < timed.size() && r < 3; r++) {
    const float ms = time_choice(timed[r].second, 60);
    if (ms > 0.0f && (best_ms == 0.0f || ms < best_ms)) {
      best_ms = ms;
      best = timed[r].second;
    }
  }
  // Deeper diffusion passes than the projection's (the Jacobi halo is half
  // the red/black one), when the diffusion runs pass by pass.
  if (base.viscosity != 0.0f && base.diffusion_block == 0 && best_ms > 0.0f &&
      !(best.resident & 2)) {
    const TuneChoice chosen = best;
    for (int dk : {12, 16, 20})
      if (dk > chosen.K && dk <= base.projection_n) {
        const TuneChoice cand{chosen.K, chosen.resident, dk};
        const float ms = time_choice(cand, 60);
        if (ms > 0.0f && ms < best_ms) {
          best_ms = ms;
          best = cand;
        }
      }
  }
  g_err[0] = '\0';  // a candidate that failed is not the caller's error
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tuned[key] = best;
  return best;
}

}  // namespace

// ===========================================================================
// Allocation-free diffusion
//
// Some callers cannot allocate device memory at the moment they want to run
// a step: code whose memory is owned by another allocator (a framework pool
// or a renderer that forbids stray cudaMalloc/cudaFree calls), code on a
// real-time frame path where an allocation's implicit synchronisation would
// stall the frame, and code that must keep a fixed device footprint. For them
// the diffusion phase runs on a caller-owned field with the Jacobi ping-pong
// buffer taken from a fixed array in the library's own device memory instead
// of from a handle's buffers.
// ===========================================================================

namespace {

// Largest grid (width * height) os_diffuse_noalloc accepts: 1 Mi cells, e.g.
// 1024 x 1024. The array costs 4 MiB on every GPU that loads the library, for
// as long as the library stays loaded.
constexpr size_t kNoAllocMaxCells = size_t(1) << 20;

static __device__ __align__(256) float g_noalloc_scratch[kNoAllocMaxCells];

// Device address of g_noalloc_scratch on each device, looked up once per
// device with that device current. In host code the symbol itself only names
// a host-side shadow and must never be passed to a kernel.
constexpr int kNoAllocMaxDevices = 64;
float* g_noalloc_ptr[kNoAllocMaxDevices] = {};
std::mutex g_noalloc_mu;

int noalloc_scratch(int device, float** out) {
  if (device < 0 || device >= kNoAllocMaxDevices)
    return set_err(OS_ERR_INVALID, "device %d out of range", device);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return set_err(OS_ERR_CUDA, "cudaGetSymbolAddress(noalloc scratch): %s",
                     cudaGetErrorString(e));
    g_noalloc_ptr[device] = static_cast<float*>(p);
  }
  *out = g_noalloc_ptr[device];
  return OS_OK;
}

// k_diffuse's sweep (the same diffuse_cell) with dt passed by value, so no
// device parameter block is needed.
__global__ void k_diffuse_noalloc(const float* __restrict__ uin, float* __restrict__ uout,
                                  Consts c, float d_t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= c.W) return;
  const int W = c.W;
  const int64_t k = cell_index(W, c.H, i, j);
  if (i >= W - 1 || j >= c.H - 1 || i <= 0 || j <= 0) {
    uout[k] = uin[k];
    return;
  }
  diffuse_cell<float, float>(uin, uout, k, W, diffusion_coeff<float>(c, d_t));
}

}  // namespace

extern "C" int os_diffuse_noalloc(const os_config* cfg, float* u, float dt, void* stream) {
  if (!cfg || !u) return set_err(OS_ERR_INVALID, "null argument");
  if (cfg->width < 3 || cfg->height < 3)
    return set_err(OS_ERR_INVALID, "grid must be at least 3x3 (got %dx%d)", cfg->width,
                   cfg->height);
  if ((int)cfg->cell_size < 1)
    return set_err(OS_ERR_INVALID, "sim.cell_size must be >= 1 (Fluid truncates it to int)");
  if (cfg->projection_n < 0) return set_err(OS_ERR_INVALID, "sim.projection.n must be >= 0");
  const size_t N = (size_t)cfg->width * (size_t)cfg->height;
  if (N > kNoAllocMaxCells)
    return set_err(OS_ERR_INVALID,
                   "os_diffuse_noalloc: %dx%d = %zu cells exceeds its fixed scratch of %zu cells",
                   cfg->width, cfg->height, N, kNoAllocMaxCells);
  int device = 0;
  CUDA_OR_RETURN(cudaGetDevice(&device));
  float* scratch = nullptr;
  int rc = noalloc_scratch(device, &scratch);
  if (rc) return rc;
  if (cfg->viscosity == 0.0f || cfg->projection_n == 0) return OS_OK;
  Consts c{};
  c.W = cfg->width;
  c.H = cfg->height;
  c.h = (int)cfg->cell_size;
  c.n = cfg->projection_n;
  c.viscosity = cfg->viscosity;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const dim3 g2((c.W + 127) / 128, c.H);
  // Every sweep writes every cell of its output, so the scratch needs no
  // clearing: nothing is read from it before this call has written it.
  for (int t = 0; t < c.n; t++) {
    const float* in = (t & 1) ? scratch : u;
    float* out = (t & 1) ? u : scratch;
    k_diffuse_noalloc<<<g2, 128, 0, st>>>(in, out, c, dt);
  }
  if (c.n & 1) {
    const int64_t n = (int64_t)N;
    k_copy1<float><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(scratch, u, n);
  }
  CUDA_OR_RETURN(cudaGetLastError());
  return OS_OK;
}

// Batched and served scenarios: os_batch_*, built on the handles above.
#include "os_batch_host.cuh"
