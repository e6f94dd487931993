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

// --- inc/config_parser.hpp:9-116 -------------------------------------------
struct ColorConfig { int r; int g; int b; int a; };
struct OpenMPConfig { int thread_count; };
struct CudaConfig { int block_size_x; int block_size_y; };
struct ThreadConfig { OpenMPConfig openMP; CudaConfig cuda; };
struct ProjectionConfig { int n; float o; };
struct PhysicsConfig { float g; };
struct WindTunnelConfig {
  int pipe_height; int pipe_length; int smoke_length; int smoke_height; int smoke_count;
  float speed; float smoke;
};
struct ObstacleConfig { bool enable; int center_x; int center_y; float radius; };
struct TimeConfig { float d_t; bool enable_real_time; float real_time_multiplier; };
struct SmokeConfig { bool enable_decay; float decay_rate; };
struct PathLineConfig { bool enable; int length; ColorConfig color; int distance; };
struct FluidConfig { float density; float drag_coeff; float viscosity; };
struct SimConfig {
  int height; int width; int cell_pixel_size; float cell_size;
  bool enable_drain; bool enable_pressure; bool enable_smoke; bool enable_interactive;
  ProjectionConfig projection; WindTunnelConfig wind_tunnel; PhysicsConfig physics;
  TimeConfig time; SmokeConfig smoke; ObstacleConfig obstacle;
};
struct ArrowConfig {
  ColorConfig color; bool enable; int distance; float length_multiplier;
  float disable_threshold; int head_length;
};
struct VisualConfig { ArrowConfig arrows; PathLineConfig path_line; };
struct Config { ThreadConfig thread; SimConfig sim; FluidConfig fluid; VisualConfig visual; };

// --- inc/fluid.cuh:8-13 -----------------------------------------------------
struct Source {
  bool active;
  float smoke;
  float velocity;
  Vector2d<int> position;
};

namespace opensayal {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& what) : std::runtime_error(what), code(c) {}
};

inline void check(int rc) {
  if (rc != OS_OK) throw Error(rc, os_last_error());
}

// Config -> os_config (every key the simulation reads).
inline os_config to_os_config(const Config& c) {
  os_config o;
  check(os_config_defaults(c.sim.width, c.sim.height, &o));
  o.block_size_x = c.thread.cuda.block_size_x;
  o.block_size_y = c.thread.cuda.block_size_y;
  o.cell_pixel_size = c.sim.cell_pixel_size;
  o.cell_size = c.sim.cell_size;
  o.enable_drain = c.sim.enable_drain;
  o.enable_pressure = c.sim.enable_pressure;
  o.enable_smoke = c.sim.enable_smoke;
  o.enable_interactive = c.sim.enable_interactive;
  o.projection_n = c.sim.projection.n;
  o.projection_o = c.sim.projection.o;
  o.pipe_height = c.sim.wind_tunnel.pipe_height;
  o.pipe_length = c.sim.wind_tunnel.pipe_length;
  o.smoke_length = c.sim.wind_tunnel.smoke_length;
  o.smoke_height = c.sim.wind_tunnel.smoke_height;
  o.smoke_count = c.sim.wind_tunnel.smoke_count;
  o.tunnel_speed = c.sim.wind_tunnel.speed;
  o.tunnel_smoke = c.sim.wind_tunnel.smoke;
  o.g = c.sim.physics.g;
  o.d_t = c.sim.time.d_t;
  o.enable_real_time = c.sim.time.enable_real_time;
  o.real_time_multiplier = c.sim.time.real_time_multiplier;
  o.smoke_enable_decay = c.sim.smoke.enable_decay;
  o.smoke_decay_rate = c.sim.smoke.decay_rate;
  o.obstacle_enable = c.sim.obstacle.enable;
  o.obstacle_center_x = c.sim.obstacle.center_x;
  o.obstacle_center_y = c.sim.obstacle.center_y;
  o.obstacle_radius = c.sim.obstacle.radius;
  o.density = c.fluid.density;
  o.drag_coeff = c.fluid.drag_coeff;
  o.viscosity = c.fluid.viscosity;
  return o;
}

inline os_handle* create(const Config& c) {
  os_config o = to_os_config(c);
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
