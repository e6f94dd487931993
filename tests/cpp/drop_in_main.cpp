// A program written against the reference's C++ interface (ConfigParser,
// Config, Source, Fluid, fluid.update, fluid.d_smoke, fluid.indx — as
// src/main.cu uses them), built on include/opensayal_gb300/fluid.hpp.
//
//   drop_in_main W H STEPS         runs STEPS steps of a W x H tunnel and
//                                  prints the FP64 sums of u, v and smoke
//   drop_in_main --config FILE     parses FILE with ConfigParser and prints
//                                  every Config field, one "key value" a line
//   drop_in_main --run FILE STEPS  the simulation of the first form, with its
//                                  Config read from FILE by ConfigParser
//
// The tests compare each output with the Python binding and loader.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "opensayal_gb300/fluid.hpp"

static Config make_config(int width, int height) {
  Config c{};
  c.thread.cuda = {64, 1};
  c.sim.width = width;
  c.sim.height = height;
  c.sim.cell_pixel_size = 1;
  c.sim.cell_size = 1.0f;
  c.sim.enable_drain = false;
  c.sim.enable_pressure = true;
  c.sim.enable_smoke = true;
  c.sim.projection = {50, 1.9f};
  c.sim.wind_tunnel = {height / 4, 0, 1, height / 4, 1, 2.0f, 1.0f};
  c.sim.physics.g = -5.0f;
  c.sim.time = {0.05f, false, 1.0f};
  c.sim.smoke = {false, 0.05f};
  c.sim.obstacle = {true, width / 2, height / 2, 9.5f};
  c.fluid = {1.0f, 0.0f, 0.001f};
  return c;
}

static void print_config(const Config& c) {
#define I(name, v) std::printf("%s %d\n", name, static_cast<int>(v))
#define F(name, v) std::printf("%s %.9g\n", name, static_cast<double>(v))
  I("thread.openMP.thread_count", c.thread.openMP.thread_count);
  I("thread.cuda.block_size_x", c.thread.cuda.block_size_x);
  I("thread.cuda.block_size_y", c.thread.cuda.block_size_y);
  I("sim.height", c.sim.height);
  I("sim.width", c.sim.width);
  I("sim.cell_pixel_size", c.sim.cell_pixel_size);
  F("sim.cell_size", c.sim.cell_size);
  I("sim.enable_drain", c.sim.enable_drain);
  I("sim.enable_pressure", c.sim.enable_pressure);
  I("sim.enable_smoke", c.sim.enable_smoke);
  I("sim.enable_interactive", c.sim.enable_interactive);
  I("sim.projection.n", c.sim.projection.n);
  F("sim.projection.o", c.sim.projection.o);
  I("sim.wind_tunnel.pipe_height", c.sim.wind_tunnel.pipe_height);
  I("sim.wind_tunnel.pipe_length", c.sim.wind_tunnel.pipe_length);
  I("sim.wind_tunnel.smoke_length", c.sim.wind_tunnel.smoke_length);
  I("sim.wind_tunnel.smoke_height", c.sim.wind_tunnel.smoke_height);
  I("sim.wind_tunnel.smoke_count", c.sim.wind_tunnel.smoke_count);
  F("sim.wind_tunnel.speed", c.sim.wind_tunnel.speed);
  F("sim.wind_tunnel.smoke", c.sim.wind_tunnel.smoke);
  F("sim.physics.g", c.sim.physics.g);
  F("sim.time.d_t", c.sim.time.d_t);
  I("sim.time.enable_real_time", c.sim.time.enable_real_time);
  F("sim.time.real_time_multiplier", c.sim.time.real_time_multiplier);
  I("sim.smoke.enable_decay", c.sim.smoke.enable_decay);
  F("sim.smoke.decay_rate", c.sim.smoke.decay_rate);
  I("sim.obstacle.enable", c.sim.obstacle.enable);
  I("sim.obstacle.center_x", c.sim.obstacle.center_x);
  I("sim.obstacle.center_y", c.sim.obstacle.center_y);
  F("sim.obstacle.radius", c.sim.obstacle.radius);
  F("fluid.density", c.fluid.density);
  F("fluid.drag_coeff", c.fluid.drag_coeff);
  F("fluid.viscosity", c.fluid.viscosity);
  I("visual.arrows.color.r", c.visual.arrows.color.r);
  I("visual.arrows.color.g", c.visual.arrows.color.g);
  I("visual.arrows.color.b", c.visual.arrows.color.b);
  I("visual.arrows.color.a", c.visual.arrows.color.a);
  I("visual.arrows.enable", c.visual.arrows.enable);
  I("visual.arrows.distance", c.visual.arrows.distance);
  F("visual.arrows.length_multiplier", c.visual.arrows.length_multiplier);
  F("visual.arrows.disable_threshold", c.visual.arrows.disable_threshold);
  I("visual.arrows.head_length", c.visual.arrows.head_length);
  I("visual.path_line.enable", c.visual.path_line.enable);
  I("visual.path_line.length", c.visual.path_line.length);
  I("visual.path_line.color.r", c.visual.path_line.color.r);
  I("visual.path_line.color.g", c.visual.path_line.color.g);
  I("visual.path_line.color.b", c.visual.path_line.color.b);
  I("visual.path_line.color.a", c.visual.path_line.color.a);
  I("visual.path_line.distance", c.visual.path_line.distance);
#undef I
#undef F
}

static int simulate(const Config& config, int steps) {
  Fluid fluid(config);
  Source source{false, 0.0f, 0.0f, Vector2d<int>(0, 0)};
  for (int t = 0; t < steps; t++) fluid.update(source, config.sim.time.d_t);
  const size_t n = static_cast<size_t>(fluid.width) * fluid.height;
  std::vector<float> u(n), v(n), s(n);
  cudaMemcpy(u.data(), fluid.d_vel_x, n * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(v.data(), fluid.d_vel_y, n * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(s.data(), fluid.d_smoke, n * 4, cudaMemcpyDeviceToHost);
  double su = 0, sv = 0, ss = 0;
  for (size_t k = 0; k < n; k++) {
    su += u[k];
    sv += v[k];
    ss += s[k];
  }
  std::printf("%.17g %.17g %.17g %.9g %.9g %d\n", su, sv, ss, fluid.min_pressure,
              fluid.max_pressure, fluid.indx(3, 0));
  return 0;
}

int main(int argc, char** argv) {
  try {
    if (argc > 2 && std::strcmp(argv[1], "--config") == 0) {
      print_config(ConfigParser(argv[2]).parse());
      return 0;
    }
    if (argc > 3 && std::strcmp(argv[1], "--run") == 0)
      return simulate(ConfigParser(argv[2]).parse(), std::atoi(argv[3]));
    const int width = argc > 1 ? std::atoi(argv[1]) : 256;
    const int height = argc > 2 ? std::atoi(argv[2]) : 128;
    const int steps = argc > 3 ? std::atoi(argv[3]) : 10;
    return simulate(make_config(width, height), steps);
  } catch (const opensayal::Error& e) {
    std::fprintf(stderr, "error %d: %s\n", e.code, e.what());
    return 2;
  }
}
