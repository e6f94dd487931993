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
// Differences a caller can observe:
//   * errors throw opensayal::Error (the reference ignores CUDA errors);
//   * d_this is nullptr: the library has no device copy of the object, and the
//     device helpers of the reference class (get_general_velocity, trace) are
//     not part of this header;
//   * kernel_grid_dim/kernel_block_dim are computed as the reference does but
//     only informative: the library picks its own launch shapes.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>

#include "../opensayal_gb300.h"
#include "config_parser.hpp"

// --- inc/helper.cuh:7-75 ---------------------------------------------------
template <typename T>
class Vector2d {
 public:
  Vector2d() : x_(0), y_(0) {}
  Vector2d(T x, T y) : x_(x), y_(y) {}
  T get_x() const { return x_; }
  T get_y() const { return y_; }
  void set_x(T x) { x_ = x; }
  void set_y(T y) { y_ = y; }

 private:
  T x_;
  T y_;
};

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
  }

  Fluid(const Fluid&) = delete;
  Fluid& operator=(const Fluid&) = delete;

  ~Fluid() { os_destroy(handle_); }

  // Fluid::indx (src/fluid.cu:163-165).
  int indx(int i, int j) const { return (height - j - 1) * width + i; }

  // Fluid::is_edge (src/fluid.cu:38-40).
  bool is_edge(int i, int j) const {
    return i == 0 || j == 0 || i == width - 1 || j == height - 1;
  }

  // Fluid::update (src/fluid.cu:770-795): one synchronous step.
  void update(Source source, float d_t) {
    os_source s{source.active ? 1 : 0, source.smoke, source.velocity,
                source.position.get_x(), source.position.get_y()};
    opensayal::check(os_update(handle_, &s, d_t));
    if (enable_pressure) opensayal::check(os_pressure_range(handle_, &min_pressure, &max_pressure));
  }

  os_handle* handle() const { return handle_; }
};
