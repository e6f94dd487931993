// os_common.cuh — shared device-side definitions of the GB300 wind tunnel.
//
// Conventions (the reference's, src/fluid.cu:163-165 and 547-558): a W x H
// grid of cells; every field is a W*H array indexed by
//   indx(i, j) = (H - 1 - j) * W + i
// so j = 0 (the bottom row) is stored last and "up" (j + 1) is -W in memory.
// u(i, j) is the x-velocity on the left face of cell (i, j), v(i, j) the
// y-velocity on its bottom face; smoke and pressure sit at the centre.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace osg {

// Per-cell flag byte, built once from the solid mask (src/fluid.cu:111-142).
// "fluid" means in-bounds and not solid (Fluid::is_valid_fluid,
// src/fluid.cu:360-362).
enum : uint8_t {
  F_FLUID = 1u << 0,   // the cell itself
  F_LEFT = 1u << 1,    // (i-1, j)
  F_RIGHT = 1u << 2,   // (i+1, j)
  F_BOTTOM = 1u << 3,  // (i, j-1)
  F_TOP = 1u << 4,     // (i, j+1)
  F_ACTIVE = 1u << 5,  // interior and not solid: the projection updates it
  F_NBR_MASK = F_LEFT | F_RIGHT | F_BOTTOM | F_TOP,
};

// Fluid's constants as its constructor copies them (src/fluid.cu:41-61).
struct Consts {
  int W, H;
  int h;               // cell_size, truncated to int (inc/fluid.cuh:46)
  int n;               // projection sweeps
  float g, density, viscosity, o, drag;
  float speed, tunnel_smoke, decay_rate;
  int smoke_length, smoke_count, smoke_height, pipe_height;
  int enable_decay, enable_pressure;
  int idw_mode;        // smoke inverse distances: 0 FP32 pair, 1 FP64, 2 FP32
};

// Per-step inputs, kept in device memory so that one captured graph serves
// every step: Fluid::update's `Source` and `d_t` (inc/fluid.cuh:8-13,115).
struct StepParams {
  float dt;
  int src_active;
  float src_smoke;
  float src_velocity;
  int src_x;
  int src_y;
  int pad[2];
};

// Storage <-> arithmetic conversions. FP32 storage with FP32 arithmetic is the
// reference's; FP16/BF16 storage keeps FP32 arithmetic; FP64 is the error
// yardstick for the reduced-precision variants.
template <class A, class S> __device__ __forceinline__ A ld(const S* p);
template <> __device__ __forceinline__ float ld<float, float>(const float* p) { return *p; }
template <> __device__ __forceinline__ float ld<float, __half>(const __half* p) { return __half2float(*p); }
template <> __device__ __forceinline__ float ld<float, __nv_bfloat16>(const __nv_bfloat16* p) { return __bfloat162float(*p); }
template <> __device__ __forceinline__ double ld<double, double>(const double* p) { return *p; }

__device__ __forceinline__ void st(float* p, float x) { *p = x; }
__device__ __forceinline__ void st(__half* p, float x) { *p = __float2half_rn(x); }
__device__ __forceinline__ void st(__nv_bfloat16* p, float x) { *p = __float2bfloat16_rn(x); }
__device__ __forceinline__ void st(double* p, double x) { *p = x; }

// Read-only-path loads for the advection gathers.
template <class A, class S> __device__ __forceinline__ A ldg(const S* p);
template <> __device__ __forceinline__ float ldg<float, float>(const float* p) { return __ldg(p); }
template <> __device__ __forceinline__ float ldg<float, __half>(const __half* p) { return __half2float(__ldg(p)); }
template <> __device__ __forceinline__ float ldg<float, __nv_bfloat16>(const __nv_bfloat16* p) { return __bfloat162float(__ldg(p)); }
template <> __device__ __forceinline__ double ldg<double, double>(const double* p) { return __ldg(p); }

__host__ __device__ __forceinline__ int64_t cell_index(int W, int H, int i, int j) {
  return (int64_t)(H - 1 - j) * W + i;
}

// The same index in 32 bits, for the gathers of the advection kernels: a
// grid, with its one-cell ring, has fewer than 2^31 cells (the reference's
// own indices are int, and os_create refuses larger grids), so every index
// and offset fits, and each address is one 32 x 64-bit multiply-add.
__host__ __device__ __forceinline__ int cell_index32(int W, int H, int i, int j) {
  return (H - 1 - j) * W + i;
}

}  // namespace osg
