// os_visual.cuh — the reference's per-frame visual arithmetic as headless
// device buffers: the fluid pixel colours, the velocity arrows and the path
// lines (src/graphics_handler.cu:214-396, src/helper.cu:3-50,
// src/fluid.cu:16-36). No window, renderer or graphics library is involved:
// each kernel writes integers the caller can copy out or draw itself.
#pragma once

namespace osg {

// map_rgba (src/helper.cu:44-46).
__device__ __forceinline__ int vis_rgba(int r, int g, int b, int a) {
  return r << 24 | g << 16 | b << 8 | a;
}

// clamp (src/helper.cu:48-50).
__device__ __forceinline__ float vis_clamp(float x, float lower, float upper) {
  return (x < lower) ? lower : (x > upper) ? upper : x;
}

// hsv_to_rgb (src/helper.cu:3-42): hue in degrees, six 60-degree sectors,
// channels truncated to 8 bits.
__device__ __forceinline__ void vis_hsv_to_rgb(float h, float s, float v, uint8_t& r,
                                               uint8_t& g, uint8_t& b) {
  const float c = v * s;
  const float x = c * (1 - fabsf(fmodf(h / 60.0f, 2) - 1));
  const float m = v - c;
  float rr, gg, bb;
  if (h < 60) {
    rr = c, gg = x, bb = 0;
  } else if (h < 120) {
    rr = x, gg = c, bb = 0;
  } else if (h < 180) {
    rr = 0, gg = c, bb = x;
  } else if (h < 240) {
    rr = 0, gg = x, bb = c;
  } else if (h < 300) {
    rr = x, gg = 0, bb = c;
  } else {
    rr = c, gg = 0, bb = x;
  }
  r = static_cast<uint8_t>((rr + m) * 255);
  g = static_cast<uint8_t>((gg + m) * 255);
  b = static_cast<uint8_t>((bb + m) * 255);
}

// The colour of one cell (update_fluid_pixels_kernel, src/graphics_handler.cu:
// 262-287, with its three colourings, :214-260); `keep` = the pixel's current
// value, returned when neither smoke nor pressure colours it.
__device__ __forceinline__ int pixel_colour(uint32_t flag, float smoke, float p, int keep,
                                            int enable_pressure, int enable_smoke,
                                            float min_pressure, float max_pressure) {
  if (!(flag & F_FLUID)) return vis_rgba(80, 80, 80, 255);
  if (enable_pressure && enable_smoke) {
    float norm_p = 0;
    if (p < 0 && min_pressure != 0) {
      norm_p = -p / min_pressure;
    } else if (max_pressure != 0) {
      norm_p = p / max_pressure;
    }
    norm_p = vis_clamp(norm_p, -1.0f, 1.0f);
    const float hue = (1.0f - norm_p) * 120.0f;
    uint8_t r, g, b;
    vis_hsv_to_rgb(hue, 1.0f, smoke, r, g, b);
    return vis_rgba(r, g, b, 255);
  }
  if (enable_pressure) {
    float norm_p;
    if (p < 0) {
      norm_p = -p / min_pressure;
    } else {
      norm_p = p / max_pressure;
    }
    norm_p = vis_clamp(norm_p, -1.0f, 1.0f);
    const float hue = (1.0f - norm_p) * 120.0f;
    uint8_t r, g, b;
    vis_hsv_to_rgb(hue, 1.0f, 1.0f, r, g, b);
    return vis_rgba(r, g, b, 255);
  }
  if (enable_smoke) {
    const uint8_t col = 255 - static_cast<uint8_t>(smoke * 255);
    return vis_rgba(255, col, col, 255);
  }
  return keep;
}

// Pixel (x, y) = (i, H - 1 - j) is stored at y * W + x, the cell's own index,
// so the pass is flat over the W*H cells, four per thread with vector loads
// and stores where the arrays allow (the pixel buffer 16-byte aligned).
template <class S>
__global__ void k_render_pixels(const S* __restrict__ smoke, const float* __restrict__ pressure,
                                const uint8_t* __restrict__ fl, int64_t n, int enable_pressure,
                                int enable_smoke, float min_pressure, float max_pressure,
                                int* __restrict__ pixels, int vec) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k0 = 4 * q;
  if (k0 >= n) return;
  if (vec && k0 + 3 < n) {
    const uint32_t f4 = __ldg(reinterpret_cast<const uint32_t*>(fl + k0));
    const float4 s4 = enable_smoke ? vec4_to_f32(smoke + k0) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 p4 = enable_pressure ? __ldg(reinterpret_cast<const float4*>(pressure + k0))
                                      : make_float4(0.f, 0.f, 0.f, 0.f);
    int4 keep = make_int4(0, 0, 0, 0);
    if (!enable_pressure && !enable_smoke) keep = *reinterpret_cast<const int4*>(pixels + k0);
    int4 out;
    out.x = pixel_colour(f4 & 0xffu, s4.x, p4.x, keep.x, enable_pressure, enable_smoke,
                         min_pressure, max_pressure);
    out.y = pixel_colour((f4 >> 8) & 0xffu, s4.y, p4.y, keep.y, enable_pressure, enable_smoke,
                         min_pressure, max_pressure);
    out.z = pixel_colour((f4 >> 16) & 0xffu, s4.z, p4.z, keep.z, enable_pressure, enable_smoke,
                         min_pressure, max_pressure);
    out.w = pixel_colour(f4 >> 24, s4.w, p4.w, keep.w, enable_pressure, enable_smoke,
                         min_pressure, max_pressure);
    *reinterpret_cast<int4*>(pixels + k0) = out;
    return;
  }
  for (int64_t k = k0; k < n && k < k0 + 4; k++)
    pixels[k] = pixel_colour(fl[k], enable_smoke ? ld<float>(smoke + k) : 0.0f,
                             enable_pressure ? pressure[k] : 0.0f, pixels[k], enable_pressure,
                             enable_smoke, min_pressure, max_pressure);
}

struct VisualParams {
  int cell_px;              // sim.cell_pixel_size
  int arrow_distance;
  float arrow_length_multiplier;
  float arrow_disable_threshold;
  float arrow_head_length;  // the reference keeps it as a float member
  float arrow_head_angle;   // ARROW_HEAD_ANGLE = M_PI / 8, as a float member
  int arrows_w, arrows_h;   // W / distance, H / distance
  int trace_distance, trace_length, traces_w, traces_h;
};

// update_center_velocity_arrow_kernel and update_center_velocity_arrow_at
// (src/graphics_handler.cu:304-335) with make_arrow_data (:168-200). Entries of
// solid cells are left as they are. The reference bounds only i < W and
// j < H, so threads of a grid that overhangs W / d or H / d write outside its
// buffer (before it, for the rows); here the entry index itself is bounded.
template <class S>
__global__ void k_render_arrows(const S* __restrict__ u, const S* __restrict__ v,
                                const uint8_t* __restrict__ fl, const uint16_t* __restrict__ nb,
                                Consts c, VisualParams vp, os_arrow* __restrict__ arrows) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= vp.arrows_w || j >= vp.arrows_h) return;
  i *= vp.arrow_distance;
  j *= vp.arrow_distance;
  if (i >= c.W || j >= c.H) return;
  if (!(fl[cell_index(c.W, c.H, i, j)] & F_FLUID)) return;
  // (i + 0.5) * cell_px and (H - j - 1 + 0.5) * cell_px, rounded once to float.
  const float x = centre(0.0f, i, vp.cell_px);
  const float y = centre(0.0f, c.H - j - 1, vp.cell_px);
  const float sy = c.H * vp.cell_px - y;
  const float vel_x = sample_u<S, float>(c, nb, u, x, sy);
  const float vel_y = sample_v<S, float>(c, nb, v, x, sy);
  const float angle = atan2f(vel_y, vel_x);
  float length = sqrtf(vel_x * vel_x + vel_y * vel_y);
  os_arrow a;
  memset(&a, 0, sizeof a);
  const int ax = (int)x, ay = (int)y;  // make_arrow_data takes int coordinates
  if (length < vp.arrow_disable_threshold) {
    a.valid = 0;
  } else {
    a.valid = 1;
    a.start_x = ax;
    a.start_y = ay;
    length *= vp.arrow_length_multiplier;
    const int x_offset = length * cosf(angle);
    const int y_offset = -length * sinf(angle);
    a.end_x = ax + x_offset;
    a.end_y = ay + y_offset;
    int hx = -vp.arrow_head_length * cosf(angle + vp.arrow_head_angle);
    int hy = vp.arrow_head_length * sinf(angle + vp.arrow_head_angle);
    a.left_head_end_x = a.end_x + hx;
    a.left_head_end_y = a.end_y + hy;
    hx = -vp.arrow_head_length * cosf(vp.arrow_head_angle - angle);
    hy = -vp.arrow_head_length * sinf(vp.arrow_head_angle - angle);
    a.right_head_end_x = a.end_x + hx;
    a.right_head_end_y = a.end_y + hy;
  }
  arrows[(vp.arrows_h - j / vp.arrow_distance - 1) * vp.arrows_w + i / vp.arrow_distance] = a;
}

// update_traces_kernel and update_trace_at (src/graphics_handler.cu:361-393)
// with Fluid::trace (src/fluid.cu:16-36): a path line of `trace_length`
// points from the cell centre, stepped with the sampled velocity; solid cells
// get (-1, -1) as their first point only. The line index is bounded as the
// arrows' is (the reference bounds only the cell).
template <class S>
__global__ void k_render_traces(const S* __restrict__ u, const S* __restrict__ v,
                                const uint8_t* __restrict__ fl, const uint16_t* __restrict__ nb,
                                Consts c, VisualParams vp, float d_t, int* __restrict__ xs,
                                int* __restrict__ ys) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= vp.traces_w || j >= vp.traces_h) return;
  i *= vp.trace_distance;
  j *= vp.trace_distance;
  if (i >= c.W || j >= c.H) return;
  const int ti = i / vp.trace_distance, tj = j / vp.trace_distance;
  const int64_t base = ((int64_t)(vp.traces_h - tj - 1) * vp.traces_w + ti) * vp.trace_length;
  if (!(fl[cell_index(c.W, c.H, i, j)] & F_FLUID)) {
    xs[base] = -1;
    ys[base] = -1;
    return;
  }
  float px = centre(0.0f, i, c.h), py = centre(0.0f, j, c.h);
  xs[base] = static_cast<int>(roundf(px));
  ys[base] = c.H - 1 - static_cast<int>(roundf(py));
  for (int k = 1; k < vp.trace_length; k++) {
    const float vx = sample_u<S, float>(c, nb, u, px, py);
    const float vy = sample_v<S, float>(c, nb, v, px, py);
    px = px + vx * d_t;
    py = py + vy * d_t;
    xs[base + k] = static_cast<int>(roundf(px));
    ys[base + k] = c.H - 1 - static_cast<int>(roundf(py));
  }
}

}  // namespace osg
