// ref_visual.cu — kernels that run the reference's own visual arithmetic.
//
// TEST INFRASTRUCTURE ONLY (the visual parity tests). Compiled by
// oracle/Makefile with the reference's Release flags and linked with its
// src/fluid.cu and src/helper.cu, both unmodified, into
// oracle/_ref/visual_ref.cubin. The reference's visual kernels live in
// src/graphics_handler.cu next to its SDL window code, which has no place on a
// machine without a graphics stack, so their control flow is restated here
// around the reference's own device functions:
//   * ref_pixels: update_fluid_pixels_kernel (src/graphics_handler.cu:262-287)
//     and its three colourings (:214-260), calling the reference's
//     hsv_to_rgb, map_rgba and clamp (src/helper.cu:3-50);
//   * ref_traces: update_traces_kernel / update_trace_at (:361-393), calling
//     the reference's Fluid::trace (src/fluid.cu:16-36);
//   * ref_arrows: update_center_velocity_arrow_kernel / _at (:304-335) and
//     make_arrow_data (:168-200), restated, calling the reference's
//     Fluid::get_general_velocity (src/fluid.cu:541-545);
//   * ref_sample: the reference's Fluid::get_general_velocity at given
//     points, as consumer kernels call it (src/graphics_handler.cu:269-283).
// The Fluid object is the harness's byte-for-byte replica (ref_harness.cpp).
// One deliberate difference: the reference's trace and arrow kernels bound
// only the cell (i < width, j < height), so the threads of a grid that
// overhangs width / d or height / d write outside their buffers; both kernels
// here bound the line or arrow index, as the library does.
#include <cstdint>

#include "fluid.cuh"
#include "helper.cuh"

// ArrowData (inc/graphics_handler.cuh:17-27).
struct RefArrowData {
  int start_x;
  int start_y;
  int end_x;
  int end_y;
  int right_head_end_x;
  int right_head_end_y;
  int left_head_end_x;
  int left_head_end_y;
  bool valid;
};

extern "C" __global__ void ref_pixels(Fluid* d_fluid, int* pixels, float min_pressure,
                                      float max_pressure) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= d_fluid->width or j >= d_fluid->height) return;
  const int x = i;
  const int y = d_fluid->height - j - 1;
  int* out = pixels + y * d_fluid->width + x;
  if (d_fluid->d_is_solid[d_fluid->indx(i, j)]) {
    *out = map_rgba(80, 80, 80, 255);
  } else if (d_fluid->enable_pressure && d_fluid->enable_smoke) {
    const float smoke = d_fluid->d_smoke[d_fluid->indx(i, j)];
    const float pressure = d_fluid->d_pressure[d_fluid->indx(i, j)];
    float norm_p = 0;
    if (pressure < 0 and min_pressure != 0) {
      norm_p = -pressure / min_pressure;
    } else if (max_pressure != 0) {
      norm_p = pressure / max_pressure;
    }
    norm_p = clamp(norm_p, -1.0f, 1.0f);
    float hue = (1.0f - norm_p) * 120.0f;
    uint8_t r, g, b;
    hsv_to_rgb(hue, 1.0f, smoke, r, g, b);
    *out = map_rgba(r, g, b, 255);
  } else if (d_fluid->enable_pressure) {
    const float pressure = d_fluid->d_pressure[d_fluid->indx(i, j)];
    float norm_p;
    if (pressure < 0) {
      norm_p = -pressure / min_pressure;
    } else {
      norm_p = pressure / max_pressure;
    }
    norm_p = clamp(norm_p, -1.0f, 1.0f);
    float hue = (1.0f - norm_p) * 120.0f;
    uint8_t r, g, b;
    hsv_to_rgb(hue, 1.0f, 1.0f, r, g, b);
    *out = map_rgba(r, g, b, 255);
  } else if (d_fluid->enable_smoke) {
    const float smoke = d_fluid->d_smoke[d_fluid->indx(i, j)];
    uint8_t color = 255 - static_cast<uint8_t>(smoke * 255);
    *out = map_rgba(255, color, color, 255);
  }
}

extern "C" __global__ void ref_traces(Fluid* d_fluid, float d_t, int* xs, int* ys, int distance,
                                      int length, int traces_w, int traces_h) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= traces_w || j >= traces_h) return;
  i *= distance;
  j *= distance;
  if (i >= d_fluid->width || j >= d_fluid->height) return;
  const int ti = i / distance, tj = j / distance;
  const int base = (traces_h - tj - 1) * traces_w * length + ti * length;
  if (d_fluid->d_is_solid[d_fluid->indx(i, j)]) {
    xs[base] = -1;
    ys[base] = -1;
  } else {
    d_fluid->trace(i, j, d_t, &xs[base], &ys[base], length);
  }
}

extern "C" __global__ void ref_arrows(Fluid* d_fluid, RefArrowData* out, int cell_size,
                                      float length_multiplier, float disable_threshold,
                                      float head_length, float head_angle, int distance,
                                      int arrows_w, int arrows_h) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= arrows_w || j >= arrows_h) return;
  i *= distance;
  j *= distance;
  if (i >= d_fluid->width or j >= d_fluid->height) return;
  if (d_fluid->d_is_solid[d_fluid->indx(i, j)]) return;
  const int height = d_fluid->height;
  float x = (i + 0.5) * cell_size;
  float y = (height - j - 1 + 0.5) * cell_size;
  Vector2d<float> velocity = d_fluid->get_general_velocity(x, height * cell_size - y);
  auto vel_x = velocity.get_x();
  auto vel_y = velocity.get_y();
  auto angle = atan2(vel_y, vel_x);
  auto length = sqrt(vel_x * vel_x + vel_y * vel_y);
  // make_arrow_data(int x, int y, float length, float angle)
  const int ax = x, ay = y;
  RefArrowData a;
  if (length < disable_threshold) {
    a.valid = false;
  } else {
    a.valid = true;
    a.start_x = ax;
    a.start_y = ay;
    length *= length_multiplier;
    int x_offset = length * cos(angle);
    int y_offset = -length * sin(angle);
    a.end_x = ax + x_offset;
    a.end_y = ay + y_offset;
    int arrow_x_offset = -head_length * cos(angle + head_angle);
    int arrow_y_offset = head_length * sin(angle + head_angle);
    a.left_head_end_x = a.end_x + arrow_x_offset;
    a.left_head_end_y = a.end_y + arrow_y_offset;
    arrow_x_offset = -head_length * cos(head_angle - angle);
    arrow_y_offset = -head_length * sin(head_angle - angle);
    a.right_head_end_x = a.end_x + arrow_x_offset;
    a.right_head_end_y = a.end_y + arrow_y_offset;
  }
  out[(arrows_h - j / distance - 1) * arrows_w + i / distance] = a;
}

extern "C" __global__ void ref_sample(Fluid* d_fluid, const float* px, const float* py, int n,
                                      float* out_u, float* out_v) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  Vector2d<float> vel = d_fluid->get_general_velocity(px[k], py[k]);
  out_u[k] = vel.get_x();
  out_v[k] = vel.get_y();
}
