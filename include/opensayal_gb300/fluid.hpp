// fluid.hpp — the reference's C++ interface (inc/fluid.cuh:8-116,
// inc/config_parser.hpp:9-116, inc/helper.cuh:7-75) rebuilt on the C ABI of
// libopensayal_gb300.so, so that code written against OpenSayal's `Fluid`
// (its main loop, src/main.cu:42-107) compiles unchanged:
//
//   Config config = ...;            // same nested structs and field names
//   Fluid fluid(config);            // allocates, rasterises the mask
//   fluid.update(source, d_t);      // one synchronous step
//   float* smoke = fluid.d_smoke;   // device fields in the reference layout
//
// d_this is a device copy of the object taken in the constructor, as in the
// reference, and the class carries the reference's device helpers
// (get_general_velocity, trace, is_valid_fluid, indx) for the caller's own
// kernels when the including file is compiled by nvcc.
//
// Differences a caller can observe:
//   * errors throw opensayal::Error (the reference ignores CUDA errors);
//   * kernel_grid_dim/kernel_block_dim are computed as the reference does but
//     only informative: the library picks its own launch shapes;
//   * the reference's private phase methods (apply_projection_at, ...) are
//     not members: the library runs the step.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>

#include "../opensayal_gb300.h"
#include "config_parser.hpp"

// Host and device qualifiers for code that nvcc compiles; a plain C++
// compiler sees host functions only (the device helpers below are left out).
#ifdef __CUDACC__
#define OPENSAYAL_HD __host__ __device__
#else
#define OPENSAYAL_HD
#endif

// --- inc/helper.cuh:7-75 ---------------------------------------------------
template <typename T>
class Vector2d {
 public:
  OPENSAYAL_HD Vector2d() : x_(0), y_(0) {}
  OPENSAYAL_HD Vector2d(T x, T y) : x_(x), y_(y) {}
  OPENSAYAL_HD T get_x() const { return x_; }
  OPENSAYAL_HD T get_y() const { return y_; }
  OPENSAYAL_HD void set_x(T x) { x_ = x; }
  OPENSAYAL_HD void set_y(T y) { y_ = y; }

  OPENSAYAL_HD Vector2d<T> operator+(const Vector2d<T>& other) {
    return Vector2d<T>(x_ + other.x_, y_ + other.y_);
  }
  OPENSAYAL_HD Vector2d<T> operator-(const Vector2d<T>& other) {
    return Vector2d<T>(x_ - other.x_, y_ - other.y_);
  }
  template <typename G>
  OPENSAYAL_HD friend Vector2d<T> operator*(const Vector2d<T>& vector, G scalar) {
    return Vector2d<T>(vector.x_ * scalar, vector.y_ * scalar);
  }
  template <typename G>
  OPENSAYAL_HD friend Vector2d<T> operator/(const Vector2d<T>& vector, G scalar) {
    return Vector2d<T>(vector.x_ / scalar, vector.y_ / scalar);
  }

 private:
  T x_;
  T y_;
};

template <typename T>
OPENSAYAL_HD inline T square(T a) {
  return a * a;
}

// --- inc/fluid.cuh:8-13 -----------------------------------------------------
struct Source {
  bool active;
  float smoke;
  float velocity;
  Vector2d<int> position;
};

namespace opensayal {

inline os_handle* create(const Config& c) {
  os_config o;
  check(to_os_config(c, &o));
  os_handle* h = nullptr;
  check(os_create(&o, &h));
  return h;
}

}  // namespace opensayal

// --- inc/fluid.cuh:15-116 ---------------------------------------------------
class Fluid {
 private:
  os_handle* handle_;

  os_fields_view view() const {
    os_fields_view v;
    opensayal::check(os_fields(handle_, &v));
    return v;
  }

 public:
  const int width;
  const int height;
  const float g;
  const float density;
  const float viscosity;
  const float o;
  const int cell_size;
  const int n;
  const float drag_coeff;
  const int wind_tunnel_smoke_length;
  const int wind_tunnel_smoke_count;
  const int wind_tunnel_smoke_height;
  const float wind_tunnel_speed;
  const int wind_tunnel_height;
  const float wind_tunnel_smoke;
  const bool enable_smoke_decay;
  const bool enable_pressure;
  const bool enable_smoke;
  const bool enable_interactive;
  const float smoke_decay_rate;

  float min_pressure = 0.0f;
  float max_pressure = 0.0f;

  float* d_pressure;
  float* d_vel_x;
  float* d_vel_y;
  float* d_smoke;
  float* d_vel_x_buffer = nullptr;
  float* d_vel_y_buffer = nullptr;
  float* d_smoke_buffer = nullptr;
  int* d_is_solid;
  int* d_total_s;

  Fluid* d_this = nullptr;
  dim3 kernel_grid_dim;
  dim3 kernel_block_dim;

  explicit Fluid(Config config)
      : handle_(opensayal::create(config)),
        width(config.sim.width),
        height(config.sim.height),
        g(config.sim.physics.g),
        density(config.fluid.density),
        viscosity(config.fluid.viscosity),
        o(config.sim.projection.o),
        cell_size(static_cast<int>(config.sim.cell_size)),
        n(config.sim.projection.n),
        drag_coeff(config.fluid.drag_coeff),
        wind_tunnel_smoke_length(config.sim.wind_tunnel.smoke_length),
        wind_tunnel_smoke_count(config.sim.wind_tunnel.smoke_count),
        wind_tunnel_smoke_height(config.sim.wind_tunnel.smoke_height),
        wind_tunnel_speed(config.sim.wind_tunnel.speed),
        wind_tunnel_height(config.sim.wind_tunnel.pipe_height),
        wind_tunnel_smoke(config.sim.wind_tunnel.smoke),
        enable_smoke_decay(config.sim.smoke.enable_decay),
        enable_pressure(config.sim.enable_pressure),
        enable_smoke(config.sim.enable_smoke),
        enable_interactive(config.sim.enable_interactive),
        smoke_decay_rate(config.sim.smoke.decay_rate) {
    const os_fields_view v = view();
    d_pressure = v.pressure;
    d_vel_x = static_cast<float*>(v.vel_x);
    d_vel_y = static_cast<float*>(v.vel_y);
    d_smoke = static_cast<float*>(v.smoke);
    d_is_solid = v.is_solid;
    d_total_s = v.total_s;
    // src/fluid.cu:62-68
    const int bx = config.thread.cuda.block_size_x, by = config.thread.cuda.block_size_y;
    kernel_grid_dim = dim3(static_cast<int>(std::ceil(static_cast<float>(width) / bx)),
                           static_cast<int>(std::ceil(static_cast<float>(height) / by)), 1);
    kernel_block_dim = dim3(bx, by, 1);
    // A device copy of this object for the caller's kernels, taken once here
    // as the reference takes it (src/fluid.cu:87,154): later host-side changes
    // to the members are not seen through it.
    if (cudaMalloc(reinterpret_cast<void**>(&d_this), sizeof(Fluid)) != cudaSuccess ||
        cudaMemcpy(d_this, this, sizeof(Fluid), cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaFree(d_this);
      os_destroy(handle_);
      throw opensayal::Error(OS_ERR_CUDA, "device copy of Fluid (d_this) failed");
    }
  }

  Fluid(const Fluid&) = delete;
  Fluid& operator=(const Fluid&) = delete;

  ~Fluid() {
    cudaFree(d_this);
    os_destroy(handle_);
  }

  // Fluid::indx (src/fluid.cu:163-165).
  OPENSAYAL_HD int indx(int i, int j) const { return (height - j - 1) * width + i; }

  // Fluid::is_edge (src/fluid.cu:38-40).
  OPENSAYAL_HD bool is_edge(int i, int j) const {
    return i == 0 || j == 0 || i == width - 1 || j == height - 1;
  }

  // Fluid::index_is_valid (src/fluid.cu:356-358).
  OPENSAYAL_HD bool index_is_valid(int i, int j) const {
    return i < width && j < height && i >= 0 && j >= 0;
  }

#ifdef __CUDACC__
  // Device helpers for kernels of the caller that read the fields, as the
  // reference's renderer does (src/graphics_handler.cu:269-283,327,378):
  // call them through d_this, e.g. d_fluid->get_general_velocity(x, y).
  // Same taps, weights and operation order as the reference's
  // (src/fluid.cu:16-36,360-362,418-558), so a caller compiled with the same
  // flags gets the same bits.

  // Fluid::is_valid_fluid (src/fluid.cu:360-362).
  __device__ bool is_valid_fluid(int i, int j) const {
    return index_is_valid(i, j) && !d_is_solid[indx(i, j)];
  }

  // Fluid::get_center_position (src/fluid.cu:547-550): (i + 1/2) h in double.
  __device__ Vector2d<float> get_center_position(int i, int j) const {
    return Vector2d<float>((i + 0.5) * cell_size, (j + 0.5) * cell_size);
  }

  // Fluid::get_general_velocity_x (src/fluid.cu:479-539): u at (x, y) from
  // the four faces around it, each only if its cell is fluid.
  __device__ float get_general_velocity_x(float x, float y) const {
    int i = x / cell_size;
    int j = y / cell_size;
    if (!is_valid_fluid(i, j)) return 0;
    float in_x = x - i * cell_size;
    float in_y = y - j * cell_size;
    float avg_u = 0;
    if (in_y <= cell_size / 2.0) {  // with the row below
      float d_y = cell_size / 2.0 - in_y;
      float w_x = 1 - in_x / cell_size;
      float w_y = 1 - d_y / cell_size;
      if (is_valid_fluid(i, j)) avg_u += w_y * w_x * d_vel_x[indx(i, j)];
      if (is_valid_fluid(i + 1, j)) avg_u += w_y * (1 - w_x) * d_vel_x[indx(i + 1, j)];
      if (is_valid_fluid(i, j - 1)) avg_u += (1 - w_y) * w_x * d_vel_x[indx(i, j - 1)];
      if (is_valid_fluid(i + 1, j - 1))
        avg_u += (1 - w_y) * (1 - w_x) * d_vel_x[indx(i + 1, j - 1)];
    } else {  // with the row above
      float d_y = in_y - cell_size / 2.0;
      float w_x = 1 - in_x / cell_size;
      float w_y = 1 - d_y / cell_size;
      if (is_valid_fluid(i, j)) avg_u += w_y * w_x * d_vel_x[indx(i, j)];
      if (is_valid_fluid(i, j + 1)) avg_u += (1 - w_y) * w_x * d_vel_x[indx(i, j + 1)];
      if (is_valid_fluid(i + 1, j)) avg_u += w_y * (1 - w_x) * d_vel_x[indx(i + 1, j)];
      if (is_valid_fluid(i + 1, j + 1))
        avg_u += (1 - w_y) * (1 - w_x) * d_vel_x[indx(i + 1, j + 1)];
    }
    return avg_u;
  }

  // Fluid::get_general_velocity_y (src/fluid.cu:418-477): the mirror of the
  // above, choosing the left columns on a strict in_x < h/2.
  __device__ float get_general_velocity_y(float x, float y) const {
    int i = x / cell_size;
    int j = y / cell_size;
    if (!is_valid_fluid(i, j)) return 0;
    float in_x = x - i * cell_size;
    float in_y = y - j * cell_size;
    float avg_v = 0;
    if (in_x < cell_size / 2.0) {  // with the column to the left
      float d_x = cell_size / 2.0 - in_x;
      float w_x = 1 - d_x / cell_size;
      float w_y = 1 - in_y / cell_size;
      if (is_valid_fluid(i, j)) avg_v += w_y * w_x * d_vel_y[indx(i, j)];
      if (is_valid_fluid(i - 1, j)) avg_v += w_y * (1 - w_x) * d_vel_y[indx(i - 1, j)];
      if (is_valid_fluid(i - 1, j + 1))
        avg_v += (1 - w_y) * (1 - w_x) * d_vel_y[indx(i - 1, j + 1)];
      if (is_valid_fluid(i, j + 1)) avg_v += (1 - w_y) * w_x * d_vel_y[indx(i, j + 1)];
    } else {  // with the column to the right
      float d_x = in_x - cell_size / 2.0;
      float w_x = 1 - d_x / cell_size;
      float w_y = 1 - in_y / cell_size;
      if (is_valid_fluid(i, j)) avg_v += w_y * w_x * d_vel_y[indx(i, j)];
      if (is_valid_fluid(i, j + 1)) avg_v += (1 - w_y) * w_x * d_vel_y[indx(i, j + 1)];
      if (is_valid_fluid(i + 1, j + 1))
        avg_v += (1 - w_y) * (1 - w_x) * d_vel_y[indx(i + 1, j + 1)];
      if (is_valid_fluid(i + 1, j)) avg_v += w_y * (1 - w_x) * d_vel_y[indx(i + 1, j)];
    }
    return avg_v;
  }

  // Fluid::get_general_velocity (src/fluid.cu:541-545).
  __device__ Vector2d<float> get_general_velocity(float x, float y) const {
    float u = get_general_velocity_x(x, y);
    float v = get_general_velocity_y(x, y);
    return Vector2d<float>(u, v);
  }

  // Fluid::trace (src/fluid.cu:16-36): a path line of trace_length points
  // from the centre of cell (i, j), stepped by d_t with the sampled
  // velocity, in pixel rows (height - 1 - y).
  __device__ void trace(int i, int j, float d_t, int* trace_line_x, int* trace_line_y,
                        int trace_length) const {
    Vector2d<float> position = get_center_position(i, j);
    trace_line_x[0] = static_cast<int>(round(position.get_x()));
    trace_line_y[0] = height - 1 - static_cast<int>(round(position.get_y()));
    for (int k = 1; k < trace_length; k++) {
      auto x = position.get_x();
      auto y = position.get_y();
      Vector2d<float> velocity = get_general_velocity(x, y);
      position = position + velocity * d_t;
      trace_line_x[k] = static_cast<int>(round(position.get_x()));
      trace_line_y[k] = height - 1 - static_cast<int>(round(position.get_y()));
    }
  }
#endif  // __CUDACC__

  // Fluid::update (src/fluid.cu:770-795): one synchronous step.
  void update(Source source, float d_t) {
    os_source s{source.active ? 1 : 0, source.smoke, source.velocity,
                source.position.get_x(), source.position.get_y()};
    opensayal::check(os_update(handle_, &s, d_t));
    if (enable_pressure) opensayal::check(os_pressure_range(handle_, &min_pressure, &max_pressure));
  }

  os_handle* handle() const { return handle_; }
};
