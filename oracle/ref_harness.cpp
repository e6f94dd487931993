// ref_harness.cpp — runs the reference's own CUDA kernels on a GPU.
//
// TEST INFRASTRUCTURE ONLY (the parity tests and bench.py's reference arm).
//
// oracle/_ref/fluid_ref.cubin is the device code of the reference's
// src/fluid.cu, compiled unmodified for sm_103a with the reference's Release
// flags (-O3 --use_fast_math -rdc=true) by oracle/Makefile. This file loads it
// with cudaLibraryLoadFromFile and drives its eleven kernels exactly as the
// reference's host code does:
//   * a byte-for-byte replica of `class Fluid` (inc/fluid.cuh:39-76) is copied
//     to the device, because every reference kernel reads its parameters and
//     field pointers through that object (`Fluid* d_fluid`);
//   * the constructor's host work (src/fluid.cu:62-68, 99-161) and the launch
//     sequence of Fluid::update (src/fluid.cu:770-795) are restated here with
//     the same grid and block shapes, the same legacy default stream and the
//     same synchronisation at the end of every step.
// The reference's host code cannot run as-is without SDL and nlohmann::json;
// its device code — every arithmetic operation of the path — is what runs.
//
// Deliberate differences, all on the host side:
//   * d_total_s is counted from zero (the reference mallocs it uncleared,
//     src/fluid.cu:102-103).
//   * the diffusion loop runs `diffusion_sweeps` launches (the reference's
//     loop counter is uninitialised, src/fluid.cu:186; its x86-64 g++ 13 -O3
//     build starts it at zero, i.e. n launches).
//   * pressure extrema are reduced on the host from a device copy instead of
//     by thrust::reduce (src/fluid.cu:778-787); min and max are exact.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../include/opensayal_gb300.h"

namespace {

// Layout of the reference's Source (inc/fluid.cuh:8-13).
struct RefSource {
  bool active;
  float smoke;
  float velocity;
  int position_x;
  int position_y;
};
static_assert(sizeof(RefSource) == 20, "Source layout");

// Layout of the reference's class Fluid (inc/fluid.cuh:39-76): public data
// members in declaration order, no virtual functions, no base class.
struct RefFluid {
  int width;
  int height;
  float g;
  float density;
  float viscosity;
  float o;
  int cell_size;
  int n;
  float drag_coeff;
  int wind_tunnel_smoke_length;
  int wind_tunnel_smoke_count;
  int wind_tunnel_smoke_height;
  float wind_tunnel_speed;
  int wind_tunnel_height;
  float wind_tunnel_smoke;
  bool enable_smoke_decay;
  bool enable_pressure;
  bool enable_smoke;
  bool enable_interactive;
  float smoke_decay_rate;
  float min_pressure;
  float max_pressure;
  float* d_pressure;
  float* d_vel_x;
  float* d_vel_y;
  float* d_smoke;
  float* d_vel_x_buffer;
  float* d_vel_y_buffer;
  float* d_smoke_buffer;
  int* d_is_solid;
  int* d_total_s;
  RefFluid* d_this;
  dim3 kernel_grid_dim;
  dim3 kernel_block_dim;
};
static_assert(sizeof(RefFluid) == 184, "Fluid layout");
static_assert(offsetof(RefFluid, n) == 28, "Fluid::n offset");
static_assert(offsetof(RefFluid, d_pressure) == 80, "Fluid::d_pressure offset");
static_assert(offsetof(RefFluid, d_this) == 152, "Fluid::d_this offset");
static_assert(offsetof(RefFluid, kernel_grid_dim) == 160, "grid dim offset");

// Mangled names of the reference kernels (src/fluid.cu).
const char* const kNames[] = {
    "_Z28apply_external_forces_kernel6SourceP5Fluidf",   // 0
    "_Z20zero_pressure_kernelP5Fluid",                    // 1
    "_Z22apply_diffusion_kernelP5Fluidf",                 // 2
    "_Z28apply_projection_even_kernelP5Fluidf",           // 3
    "_Z27apply_projection_odd_kernelP5Fluidf",            // 4
    "_Z26apply_extrapolation_kernelP5Fluid",              // 5
    "_Z31apply_velocity_advection_kernelP5Fluidf",        // 6
    "_Z32update_velocity_advection_kernelP5Fluidf",       // 7
    "_Z28apply_smoke_advection_kernelP5Fluidf",           // 8
    "_Z29update_smoke_advection_kernelP5Fluidf",          // 9
    "_Z18decay_smoke_kernelP5Fluidf",                     // 10
};
constexpr int kNumKernels = 11;

cudaLibrary_t g_lib = nullptr;
cudaKernel_t g_kernels[kNumKernels];
char g_err[512];

int fail(const char* what, cudaError_t e) {
  snprintf(g_err, sizeof g_err, "%s: %s", what, cudaGetErrorString(e));
  return -1;
}

struct Ref {
  RefFluid f;          // host copy
  RefFluid* d_this;    // device copy
  size_t cells;
  dim3 grid, block, proj_grid;
};

int launch(int k, dim3 grid, dim3 block, void** args) {
  cudaError_t e = cudaLaunchKernel((const void*)g_kernels[k], grid, block,
                                   args, 0, (cudaStream_t)0);
  if (e != cudaSuccess) return fail(kNames[k], e);
  return 0;
}

float* field_ptr(Ref* r, int field) {
  switch (field) {
    case OS_FIELD_VEL_X: return r->f.d_vel_x;
    case OS_FIELD_VEL_Y: return r->f.d_vel_y;
    case OS_FIELD_SMOKE: return r->f.d_smoke;
    case OS_FIELD_PRESSURE: return r->f.d_pressure;
    case OS_FIELD_IS_SOLID: return reinterpret_cast<float*>(r->f.d_is_solid);
    case OS_FIELD_TOTAL_S: return reinterpret_cast<float*>(r->f.d_total_s);
    default: return nullptr;
  }
}

}  // namespace

extern "C" {

const char* ref_last_error(void) { return g_err; }

// Loads the cubin and resolves the eleven kernels. Returns 0 on success.
int ref_open(const char* cubin_path) {
  if (g_lib) return 0;
  cudaError_t e = cudaLibraryLoadFromFile(&g_lib, cubin_path, nullptr, nullptr,
                                          0, nullptr, nullptr, 0);
  if (e != cudaSuccess) return fail("cudaLibraryLoadFromFile", e);
  for (int k = 0; k < kNumKernels; k++) {
    e = cudaLibraryGetKernel(&g_kernels[k], g_lib, kNames[k]);
    if (e != cudaSuccess) return fail(kNames[k], e);
  }
  return 0;
}

// Fluid::Fluid(Config) (src/fluid.cu:41-161). Returns an opaque handle or NULL.
void* ref_create(const os_config* c, const int32_t* is_solid,
                 const int32_t* total_s) {
  Ref* r = new Ref();
  RefFluid& f = r->f;
  memset(&f, 0, sizeof f);
  f.width = c->width;
  f.height = c->height;
  f.g = c->g;
  f.density = c->density;
  f.viscosity = c->viscosity;
  f.o = c->projection_o;
  f.cell_size = static_cast<int>(c->cell_size);
  f.n = c->projection_n;
  f.drag_coeff = c->drag_coeff;
  f.wind_tunnel_smoke_length = c->smoke_length;
  f.wind_tunnel_smoke_count = c->smoke_count;
  f.wind_tunnel_smoke_height = c->smoke_height;
  f.wind_tunnel_speed = c->tunnel_speed;
  f.wind_tunnel_height = c->pipe_height;
  f.wind_tunnel_smoke = c->tunnel_smoke;
  f.enable_smoke_decay = c->smoke_enable_decay != 0;
  f.enable_pressure = c->enable_pressure != 0;
  f.enable_smoke = c->enable_smoke != 0;
  f.enable_interactive = c->enable_interactive != 0;
  f.smoke_decay_rate = c->smoke_decay_rate;
  const int bx = c->block_size_x, by = c->block_size_y;
  const int gx = static_cast<int>(std::ceil(static_cast<float>(f.width) / bx));
  const int gy = static_cast<int>(std::ceil(static_cast<float>(f.height) / by));
  f.kernel_grid_dim = dim3(gx, gy, 1);
  f.kernel_block_dim = dim3(bx, by, 1);
  r->grid = f.kernel_grid_dim;
  r->block = f.kernel_block_dim;
  // src/fluid.cu:283-287
  r->proj_grid = dim3(
      static_cast<int>(std::ceil(static_cast<float>(f.width) / r->block.x / 2)),
      static_cast<int>(std::ceil(static_cast<float>(f.height) / r->block.y)));
  r->cells = static_cast<size_t>(f.width) * f.height;
  const size_t fb = r->cells * sizeof(float);
  float** fields[] = {&f.d_pressure,     &f.d_vel_x,        &f.d_vel_y,
                      &f.d_smoke,        &f.d_vel_x_buffer, &f.d_vel_y_buffer,
                      &f.d_smoke_buffer};
  for (float** p : fields) {
    if (cudaMalloc(p, fb) != cudaSuccess || cudaMemset(*p, 0, fb) != cudaSuccess) {
      snprintf(g_err, sizeof g_err, "cudaMalloc of a field failed");
      return nullptr;
    }
  }
  if (cudaMalloc(&f.d_is_solid, r->cells * 4) != cudaSuccess ||
      cudaMalloc(&f.d_total_s, r->cells * 4) != cudaSuccess ||
      cudaMalloc(&r->d_this, sizeof(RefFluid)) != cudaSuccess) {
    snprintf(g_err, sizeof g_err, "cudaMalloc failed");
    return nullptr;
  }
  f.d_this = r->d_this;
  cudaMemcpy(f.d_is_solid, is_solid, r->cells * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(f.d_total_s, total_s, r->cells * 4, cudaMemcpyHostToDevice);
  cudaError_t e = cudaMemcpy(r->d_this, &f, sizeof f, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    fail("upload Fluid", e);
    return nullptr;
  }
  return r;
}

int ref_destroy(void* h) {
  Ref* r = static_cast<Ref*>(h);
  if (!r) return 0;
  RefFluid& f = r->f;
  void* ptrs[] = {f.d_pressure,     f.d_vel_x,      f.d_vel_y,
                  f.d_smoke,        f.d_vel_x_buffer, f.d_vel_y_buffer,
                  f.d_smoke_buffer, f.d_is_solid,   f.d_total_s,
                  r->d_this};
  for (void* p : ptrs) cudaFree(p);
  delete r;
  return 0;
}

int ref_upload(void* h, int field, const void* host) {
  Ref* r = static_cast<Ref*>(h);
  float* d = field_ptr(r, field);
  if (!d) return -1;
  cudaError_t e = cudaMemcpy(d, host, r->cells * 4, cudaMemcpyHostToDevice);
  return e == cudaSuccess ? 0 : fail("upload", e);
}

int ref_download(void* h, int field, void* host) {
  Ref* r = static_cast<Ref*>(h);
  float* d = field_ptr(r, field);
  if (!d) return -1;
  cudaError_t e = cudaMemcpy(host, d, r->cells * 4, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? 0 : fail("download", e);
}

// One phase of Fluid::update, launched like the reference's phase methods.
int ref_phase(void* h, int phase, const os_source* src, float dt,
              int diffusion_sweeps) {
  Ref* r = static_cast<Ref*>(h);
  RefFluid* d = r->d_this;
  void* a_fd[] = {&d, &dt};
  void* a_f[] = {&d};
  switch (phase) {
    case OS_PHASE_FORCES: {  // src/fluid.cu:351-354
      RefSource s;
      memset(&s, 0, sizeof s);
      if (src) {
        s.active = src->active != 0;
        s.smoke = src->smoke;
        s.velocity = src->velocity;
        s.position_x = src->position_x;
        s.position_y = src->position_y;
      }
      void* a[] = {&s, &d, &dt};
      return launch(0, r->grid, r->block, a);
    }
    case OS_PHASE_ZERO_PRESSURE:  // src/fluid.cu:216-219
      return launch(1, r->grid, r->block, a_f);
    case OS_PHASE_DIFFUSION:  // src/fluid.cu:185-190
      for (int t = 0; t < diffusion_sweeps; t++)
        if (launch(2, r->grid, r->block, a_fd)) return -1;
      return 0;
    case OS_PHASE_PROJECTION:  // src/fluid.cu:282-295
      for (int t = 0; t < r->f.n; t++) {
        if (launch(3, r->proj_grid, r->block, a_fd)) return -1;
        if (launch(4, r->proj_grid, r->block, a_fd)) return -1;
      }
      return 0;
    case OS_PHASE_PRESSURE_RANGE: {  // src/fluid.cu:778-787
      std::vector<float> p(r->cells);
      cudaError_t e = cudaMemcpy(p.data(), r->f.d_pressure, r->cells * 4,
                                 cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return fail("pressure copy", e);
      float lo = INFINITY, hi = -INFINITY;
      for (float x : p) {
        lo = std::fmin(lo, x);
        hi = std::fmax(hi, x);
      }
      r->f.min_pressure = lo;
      r->f.max_pressure = hi;
      return 0;
    }
    case OS_PHASE_EXTRAPOLATION:  // src/fluid.cu:744-747
      return launch(5, r->grid, r->block, a_f);
    case OS_PHASE_VEL_ADVECTION:  // src/fluid.cu:637-642
      if (launch(6, r->grid, r->block, a_fd)) return -1;
      return launch(7, r->grid, r->block, a_fd);
    case OS_PHASE_SMOKE_ADVECTION:  // src/fluid.cu:591-596
      if (launch(8, r->grid, r->block, a_fd)) return -1;
      return launch(9, r->grid, r->block, a_fd);
    case OS_PHASE_DECAY:  // src/fluid.cu:764-767
      return launch(10, r->grid, r->block, a_fd);
    default:
      snprintf(g_err, sizeof g_err, "unknown phase %d", phase);
      return -1;
  }
}

// Fluid::update (src/fluid.cu:770-795), ending with cudaDeviceSynchronize.
int ref_update(void* h, const os_source* src, float dt, int diffusion_sweeps) {
  Ref* r = static_cast<Ref*>(h);
  const RefFluid& f = r->f;
  if (ref_phase(h, OS_PHASE_FORCES, src, dt, 0)) return -1;
  if (f.enable_pressure && ref_phase(h, OS_PHASE_ZERO_PRESSURE, src, dt, 0))
    return -1;
  if (f.viscosity != 0 &&
      ref_phase(h, OS_PHASE_DIFFUSION, src, dt, diffusion_sweeps))
    return -1;
  if (ref_phase(h, OS_PHASE_PROJECTION, src, dt, 0)) return -1;
  if (f.enable_pressure && ref_phase(h, OS_PHASE_PRESSURE_RANGE, src, dt, 0))
    return -1;
  if (ref_phase(h, OS_PHASE_EXTRAPOLATION, src, dt, 0)) return -1;
  if (ref_phase(h, OS_PHASE_VEL_ADVECTION, src, dt, 0)) return -1;
  if (f.enable_smoke && f.wind_tunnel_smoke != 0) {
    if (ref_phase(h, OS_PHASE_SMOKE_ADVECTION, src, dt, 0)) return -1;
    if (ref_phase(h, OS_PHASE_DECAY, src, dt, 0)) return -1;
  }
  cudaError_t e = cudaDeviceSynchronize();
  return e == cudaSuccess ? 0 : fail("cudaDeviceSynchronize", e);
}

int ref_pressure_range(void* h, float* mn, float* mx) {
  Ref* r = static_cast<Ref*>(h);
  *mn = r->f.min_pressure;
  *mx = r->f.max_pressure;
  return 0;
}

// ---------------------------------------------------------------------------
// Visuals: oracle/_ref/visual_ref.cubin (ref_visual.cu linked with the
// reference's fluid.cu and helper.cu). Each call copies `inout` to a device
// buffer, runs the kernel on the handle's Fluid and copies the buffer back,
// so entries a kernel leaves alone keep the caller's values.
// ---------------------------------------------------------------------------

cudaLibrary_t g_vlib = nullptr;
cudaKernel_t g_vpixels, g_vtraces, g_varrows, g_vsample;

int ref_visual_open(const char* cubin_path) {
  if (g_vlib) return 0;
  cudaError_t e = cudaLibraryLoadFromFile(&g_vlib, cubin_path, nullptr, nullptr, 0, nullptr,
                                          nullptr, 0);
  if (e != cudaSuccess) return fail("cudaLibraryLoadFromFile(visual)", e);
  if ((e = cudaLibraryGetKernel(&g_vpixels, g_vlib, "ref_pixels")) != cudaSuccess ||
      (e = cudaLibraryGetKernel(&g_vtraces, g_vlib, "ref_traces")) != cudaSuccess ||
      (e = cudaLibraryGetKernel(&g_varrows, g_vlib, "ref_arrows")) != cudaSuccess ||
      (e = cudaLibraryGetKernel(&g_vsample, g_vlib, "ref_sample")) != cudaSuccess)
    return fail("visual kernels", e);
  return 0;
}

static int run_inout(const void* kernel, dim3 grid, dim3 block, void** args, void* dbuf,
                     void* inout, size_t bytes) {
  cudaError_t e = cudaMemcpy(dbuf, inout, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaLaunchKernel(kernel, grid, block, args, 0, (cudaStream_t)0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(inout, dbuf, bytes, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? 0 : fail("visual kernel", e);
}

int ref_render_pixels(void* h, float min_pressure, float max_pressure, int32_t* inout) {
  Ref* r = static_cast<Ref*>(h);
  const size_t bytes = r->cells * sizeof(int32_t);
  int32_t* d = nullptr;
  if (cudaMalloc(&d, bytes) != cudaSuccess) return fail("cudaMalloc", cudaErrorMemoryAllocation);
  void* args[] = {&r->d_this, &d, &min_pressure, &max_pressure};
  const dim3 block(16, 16), grid((r->f.width + 15) / 16, (r->f.height + 15) / 16);
  const int rc = run_inout((const void*)g_vpixels, grid, block, args, d, inout, bytes);
  cudaFree(d);
  return rc;
}

int ref_render_traces(void* h, float dt, int distance, int length, int32_t* xs, int32_t* ys) {
  Ref* r = static_cast<Ref*>(h);
  int tw = r->f.width / distance, th = r->f.height / distance;
  if (tw < 1 || th < 1) return 0;
  const size_t bytes = (size_t)tw * th * length * sizeof(int32_t);
  int32_t *dx = nullptr, *dy = nullptr;
  if (cudaMalloc(&dx, bytes) != cudaSuccess || cudaMalloc(&dy, bytes) != cudaSuccess)
    return fail("cudaMalloc", cudaErrorMemoryAllocation);
  cudaMemcpy(dy, ys, bytes, cudaMemcpyHostToDevice);
  void* args[] = {&r->d_this, &dt, &dx, &dy, &distance, &length, &tw, &th};
  const dim3 block(16, 16), grid((tw + 15) / 16, (th + 15) / 16);
  int rc = run_inout((const void*)g_vtraces, grid, block, args, dx, xs, bytes);
  if (!rc && cudaMemcpy(ys, dy, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = fail("copy traces", cudaErrorUnknown);
  cudaFree(dx);
  cudaFree(dy);
  return rc;
}

// `inout`: (W / d) * (H / d) ArrowData records of 36 bytes.
int ref_render_arrows(void* h, int cell_size, float length_multiplier, float disable_threshold,
                      float head_length, float head_angle, int distance, void* inout) {
  Ref* r = static_cast<Ref*>(h);
  int aw = r->f.width / distance, ah = r->f.height / distance;
  if (aw < 1 || ah < 1) return 0;
  const size_t bytes = (size_t)aw * ah * 36;
  void* d = nullptr;
  if (cudaMalloc(&d, bytes) != cudaSuccess) return fail("cudaMalloc", cudaErrorMemoryAllocation);
  void* args[] = {&r->d_this, &d, &cell_size, &length_multiplier, &disable_threshold,
                  &head_length, &head_angle, &distance, &aw, &ah};
  const dim3 block(16, 16), grid((aw + 15) / 16, (ah + 15) / 16);
  const int rc = run_inout((const void*)g_varrows, grid, block, args, d, inout, bytes);
  cudaFree(d);
  return rc;
}

// The reference's get_general_velocity at n points (px, py) -> (u, v).
int ref_sample_velocity(void* h, int n, const float* px, const float* py, float* ou, float* ov) {
  Ref* r = static_cast<Ref*>(h);
  if (n < 1) return 0;
  const size_t bytes = (size_t)n * sizeof(float);
  float* d = nullptr;
  if (cudaMalloc(&d, 4 * bytes) != cudaSuccess) return fail("cudaMalloc", cudaErrorMemoryAllocation);
  float *dx = d, *dy = d + n, *du = d + 2 * (size_t)n, *dv = d + 3 * (size_t)n;
  cudaError_t e = cudaMemcpy(dx, px, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dy, py, bytes, cudaMemcpyHostToDevice);
  void* args[] = {&r->d_this, &dx, &dy, &n, &du, &dv};
  if (e == cudaSuccess)
    e = cudaLaunchKernel((const void*)g_vsample, dim3((n + 127) / 128), dim3(128), args, 0,
                         (cudaStream_t)0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(ou, du, bytes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(ov, dv, bytes, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? 0 : fail("sample kernel", e);
}

}  // extern "C"
