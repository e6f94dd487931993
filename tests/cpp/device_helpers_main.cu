// A caller's own kernels on the drop-in's device helpers, as the reference's
// renderer uses them (src/graphics_handler.cu:269-283,327,378): a Fluid is
// read from a JSON configuration through ConfigParser, stepped, and then
//   * sample_kernel calls d_fluid->get_general_velocity(x, y) at given points;
//   * trace_kernel calls d_fluid->trace from every d-th cell, laid out as the
//     reference's update_traces_kernel lays its lines out.
// Compiled by nvcc with the reference's Release flags. Usage:
//   device_helpers_main CONFIG STEPS POINTS_IN OUT
// POINTS_IN holds int32 n then n float x and n float y; OUT receives u and v
// (W*H floats each), the n sampled (u, v) pairs as two arrays, and the trace
// points (x then y, tw*th*length int32 each) for d = 8, length = 12.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "opensayal_gb300/fluid.hpp"

__global__ void sample_kernel(Fluid* d_fluid, const float* px, const float* py, int n,
                              float* out_u, float* out_v) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  Vector2d<float> vel = d_fluid->get_general_velocity(px[k], py[k]);
  out_u[k] = vel.get_x();
  out_v[k] = vel.get_y();
}

__global__ void trace_kernel(Fluid* d_fluid, float d_t, int* xs, int* ys, int distance,
                             int length, int traces_w, int traces_h) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= traces_w || j >= traces_h) return;
  i *= distance;
  j *= distance;
  const int base = (traces_h - j / distance - 1) * traces_w * length + (i / distance) * length;
  if (d_fluid->d_is_solid[d_fluid->indx(i, j)]) {
    xs[base] = -1;
    ys[base] = -1;
  } else {
    d_fluid->trace(i, j, d_t, &xs[base], &ys[base], length);
  }
}

static void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    std::fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
    std::exit(3);
  }
}

int main(int argc, char** argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: %s CONFIG STEPS POINTS_IN OUT\n", argv[0]);
    return 1;
  }
  try {
    const Config config = ConfigParser(argv[1]).parse();
    const int steps = std::atoi(argv[2]);
    Fluid fluid(config);
    Source source{false, 0.0f, 0.0f, Vector2d<int>(0, 0)};
    for (int t = 0; t < steps; t++) fluid.update(source, config.sim.time.d_t);

    FILE* fin = std::fopen(argv[3], "rb");
    if (!fin) return 1;
    int n = 0;
    if (std::fread(&n, 4, 1, fin) != 1 || n < 1) return 1;
    std::vector<float> px(n), py(n), ou(n), ov(n);
    if (std::fread(px.data(), 4, n, fin) != (size_t)n || std::fread(py.data(), 4, n, fin) != (size_t)n)
      return 1;
    std::fclose(fin);

    const int W = fluid.width, H = fluid.height, d = 8, length = 12;
    const int tw = W / d, th = H / d;
    const size_t cells = (size_t)W * H, tn = (size_t)tw * th * length;
    float* dp = nullptr;
    int* dt = nullptr;
    check_cuda(cudaMalloc(&dp, 4 * (size_t)n * sizeof(float)), "cudaMalloc");
    check_cuda(cudaMalloc(&dt, 2 * tn * sizeof(int)), "cudaMalloc");
    check_cuda(cudaMemcpy(dp, px.data(), n * 4, cudaMemcpyHostToDevice), "copy");
    check_cuda(cudaMemcpy(dp + n, py.data(), n * 4, cudaMemcpyHostToDevice), "copy");
    check_cuda(cudaMemset(dt, 0, 2 * tn * sizeof(int)), "memset");
    sample_kernel<<<(n + 127) / 128, 128>>>(fluid.d_this, dp, dp + n, n, dp + 2 * n, dp + 3 * n);
    trace_kernel<<<dim3((tw + 15) / 16, (th + 15) / 16), dim3(16, 16)>>>(
        fluid.d_this, config.sim.time.d_t, dt, dt + tn, d, length, tw, th);
    check_cuda(cudaDeviceSynchronize(), "kernels");

    std::vector<float> u(cells), v(cells);
    std::vector<int> xs(tn), ys(tn);
    check_cuda(cudaMemcpy(u.data(), fluid.d_vel_x, cells * 4, cudaMemcpyDeviceToHost), "copy");
    check_cuda(cudaMemcpy(v.data(), fluid.d_vel_y, cells * 4, cudaMemcpyDeviceToHost), "copy");
    check_cuda(cudaMemcpy(ou.data(), dp + 2 * n, n * 4, cudaMemcpyDeviceToHost), "copy");
    check_cuda(cudaMemcpy(ov.data(), dp + 3 * n, n * 4, cudaMemcpyDeviceToHost), "copy");
    check_cuda(cudaMemcpy(xs.data(), dt, tn * 4, cudaMemcpyDeviceToHost), "copy");
    check_cuda(cudaMemcpy(ys.data(), dt + tn, tn * 4, cudaMemcpyDeviceToHost), "copy");
    cudaFree(dp);
    cudaFree(dt);

    FILE* fout = std::fopen(argv[4], "wb");
    if (!fout) return 1;
    std::fwrite(u.data(), 4, cells, fout);
    std::fwrite(v.data(), 4, cells, fout);
    std::fwrite(ou.data(), 4, n, fout);
    std::fwrite(ov.data(), 4, n, fout);
    std::fwrite(xs.data(), 4, tn, fout);
    std::fwrite(ys.data(), 4, tn, fout);
    std::fclose(fout);
  } catch (const opensayal::Error& e) {
    std::fprintf(stderr, "error %d: %s\n", e.code, e.what());
    return 2;
  }
  return 0;
}
