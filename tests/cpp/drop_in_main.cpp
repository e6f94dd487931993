// A program written against the reference's C++ interface (Config, Source,
// Fluid, fluid.update, fluid.d_smoke, fluid.indx — as src/main.cu uses them),
// built on include/opensayal_gb300/fluid.hpp. It runs `steps` steps of a
// width x height tunnel and prints the FP64 sums of u, v and smoke, which the
// test compares with the same run made through the Python binding.
#include <cstdio>
#include <cstdlib>
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

int main(int argc, char** argv) {
  const int width = argc > 1 ? std::atoi(argv[1]) : 256;
  const int height = argc > 2 ? std::atoi(argv[2]) : 128;
  const int steps = argc > 3 ? std::atoi(argv[3]) : 10;
  try {
    Fluid fluid(make_config(width, height));
    Source source{false, 0.0f, 0.0f, Vector2d<int>(0, 0)};
    for (int t = 0; t < steps; t++) fluid.update(source, 0.05f);
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
  } catch (const opensayal::Error& e) {
    std::fprintf(stderr, "error %d: %s\n", e.code, e.what());
    return 2;
  }
  return 0;
}
