// Every float bit pattern x: the division x / s by s = 4 read at run time,
// as apply_projection_at divides the divergence of a cell with four fluid
// neighbours (src/fluid.cu:240, s from d_total_s), against the product
// x * 0.25 that the library's all-fluid sweep path computes. Built with the
// reference's Release flags (--use_fast_math), as the library is.
//
// Prints "<inputs whose results differ in any bit> <first such input, hex>";
// a NaN from both counts as the same result.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

__global__ void k_compare(const float* __restrict__ s_ptr, unsigned long long* mismatches,
                          unsigned int* first) {
  const float s = *s_ptr;
  unsigned long long local = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (1ull << 32);
       t += stride) {
    const float x = __uint_as_float((unsigned int)t);
    const float a = x / s;
    const float b = __fmul_rn(x, 0.25f);
    const bool same = __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b);
    if (!same) {
      local++;
      atomicMin(first, (unsigned int)t);
    }
  }
  if (local) atomicAdd(mismatches, local);
}

int main() {
  float* d_s = nullptr;
  unsigned long long* d_count = nullptr;
  unsigned int* d_first = nullptr;
  const float four = 4.0f;
  const unsigned long long zero = 0;
  const unsigned int none = 0xffffffffu;
  if (cudaMalloc(&d_s, sizeof(float)) != cudaSuccess ||
      cudaMalloc(&d_count, sizeof(zero)) != cudaSuccess ||
      cudaMalloc(&d_first, sizeof(none)) != cudaSuccess) {
    fprintf(stderr, "cudaMalloc failed\n");
    return 1;
  }
  cudaMemcpy(d_s, &four, sizeof(four), cudaMemcpyHostToDevice);
  cudaMemcpy(d_count, &zero, sizeof(zero), cudaMemcpyHostToDevice);
  cudaMemcpy(d_first, &none, sizeof(none), cudaMemcpyHostToDevice);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  k_compare<<<sms * 8, 256>>>(d_s, d_count, d_first);
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    fprintf(stderr, "kernel: %s\n", cudaGetErrorString(e));
    return 1;
  }
  unsigned long long count = 0;
  unsigned int first = 0;
  cudaMemcpy(&count, d_count, sizeof(count), cudaMemcpyDeviceToHost);
  cudaMemcpy(&first, d_first, sizeof(first), cudaMemcpyDeviceToHost);
  printf("%llu %08x\n", count, first);
  cudaFree(d_s);
  cudaFree(d_count);
  cudaFree(d_first);
  return 0;
}
