// Every float bit pattern x, for each divisor den = 1 + 4a of the diffusion
// (a = viscosity * dt / h^2, formed as the library's sweeps form it) over a
// spread of viscosities, steps and cell sizes, and for further divisors up to
// 1e6: the fast-math division x / den (run-time den, src/fluid.cu:178-182)
// against the product x * __fdividef(1, den) that the library's diffusion
// passes on column-parity planes use below den = 2^20. Built with the
// reference's Release flags (--use_fast_math), as the library is.
//
// Prints one line per divisor: "<den> <inputs whose results differ> <first such
// input, hex>"; a NaN from both counts as the same result.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <vector>

__global__ void k_den(const float* visc, const float* dt, const int* h, int n, float* den) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float a = visc[t] * dt[t] / (float)(h[t] * h[t]);
  den[t] = __fmaf_rn(4.0f, a, 1.0f);
}

__global__ void k_compare(const float* __restrict__ den_ptr, unsigned long long* mismatches,
                          unsigned int* first) {
  const float den = *den_ptr;
  const float rden = __fdividef(1.0f, den);
  unsigned long long local = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (1ull << 32);
       t += stride) {
    const float x = __uint_as_float((unsigned int)t);
    const float q = x / den;
    const float p = __fmul_rn(x, rden);
    if (!(__float_as_uint(q) == __float_as_uint(p) || (q != q && p != p))) {
      local++;
      atomicMin(first, (unsigned int)t);
    }
  }
  if (local) atomicAdd(mismatches, local);
}

int main() {
  std::vector<float> visc, dt;
  std::vector<int> h;
  for (float v : {1e-6f, 0.001f, 0.02f, 0.05f, 0.5f, 2.0f, 7.0f, 100.0f})
    for (float d : {0.05f, 0.02f, 1.0f / 60.0f, 0.1f, 0.016f})
      for (int c : {1, 2}) {
        visc.push_back(v);
        dt.push_back(d);
        h.push_back(c);
      }
  const int n = (int)visc.size();
  float *d_visc, *d_dt, *d_den;
  int* d_h;
  cudaMalloc(&d_visc, n * sizeof(float));
  cudaMalloc(&d_dt, n * sizeof(float));
  cudaMalloc(&d_h, n * sizeof(int));
  cudaMalloc(&d_den, (n + 16) * sizeof(float));
  cudaMemcpy(d_visc, visc.data(), n * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(d_dt, dt.data(), n * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(d_h, h.data(), n * sizeof(int), cudaMemcpyHostToDevice);
  k_den<<<(n + 127) / 128, 128>>>(d_visc, d_dt, d_h, n, d_den);
  std::vector<float> dens(n);
  cudaMemcpy(dens.data(), d_den, n * sizeof(float), cudaMemcpyDeviceToHost);
  for (float d : {1.0f, 1.5f, 2.6f, 3.7f, 10.0f, 100.0f, 1000.0f, 65536.0f, 999999.0f})
    dens.push_back(d);
  unsigned long long* d_count;
  unsigned int* d_first;
  cudaMalloc(&d_count, sizeof(unsigned long long));
  cudaMalloc(&d_first, sizeof(unsigned int));
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  for (float den : dens) {
    const unsigned long long zero = 0;
    const unsigned int none = 0xffffffffu;
    cudaMemcpy(d_den, &den, sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(d_count, &zero, sizeof(zero), cudaMemcpyHostToDevice);
    cudaMemcpy(d_first, &none, sizeof(none), cudaMemcpyHostToDevice);
    k_compare<<<sms * 8, 256>>>(d_den, d_count, d_first);
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      fprintf(stderr, "kernel: %s\n", cudaGetErrorString(e));
      return 1;
    }
    unsigned long long count = 0;
    unsigned int first = 0;
    cudaMemcpy(&count, d_count, sizeof(count), cudaMemcpyDeviceToHost);
    cudaMemcpy(&first, d_first, sizeof(first), cudaMemcpyDeviceToHost);
    printf("%.9g %llu %08x\n", den, count, first);
  }
  return 0;
}
