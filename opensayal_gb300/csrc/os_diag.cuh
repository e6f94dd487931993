// os_diag.cuh — FP64 diagnostics of a grid: the divergence residual the
// projection drives down, and the smoke-mass and boundary-flux sums.
//
// No reference counterpart (the reference computes only the pressure extrema).
// The residual of cell (i, j) is the projection's divergence
// ((u(i+1,j) - u(i,j)) + v(i,j+1)) - v(i,j) (src/fluid.cu:229-262), evaluated
// in FP64 on the stored values for every cell the projection updates. Sums
// are reduced with warp shuffles inside a block, block partials are written to
// a fixed array, and one block folds them in a fixed order, so a result does
// not depend on scheduling and repeats bit for bit.
#pragma once

namespace osg {

constexpr int kDiagBlocks = 256;
constexpr int kDiagThreads = 256;
constexpr int kDiagSums = 6;  // div^2, div, smoke, inflow, outflow, active cells
constexpr int kDiagSlots = kDiagSums + 1;  // + max |div|

template <class S>
__device__ __forceinline__ double as_f64(const S* p) {
  return (double)ld<float, S>(p);
}
template <>
__device__ __forceinline__ double as_f64<double>(const double* p) {
  return *p;
}

__device__ __forceinline__ double warp_sum(double x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}
__device__ __forceinline__ double warp_max(double x) {
  for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_down_sync(0xffffffffu, x, o));
  return x;
}

// Folds v[kDiagSlots] over the block (sums, then the max in the last slot);
// thread 0 ends up with the block's values in out.
__device__ __forceinline__ void block_fold(double (&v)[kDiagSlots], double* out) {
  __shared__ double part[kDiagThreads / 32][kDiagSlots];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kDiagSums; q++) v[q] = warp_sum(v[q]);
  v[kDiagSums] = warp_max(v[kDiagSums]);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < kDiagSlots; q++) part[warp][q] = v[q];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < kDiagSlots; q++) v[q] = lane < kDiagThreads / 32 ? part[lane][q] : 0.0;
#pragma unroll
    for (int q = 0; q < kDiagSums; q++) v[q] = warp_sum(v[q]);
    v[kDiagSums] = warp_max(v[kDiagSums]);
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < kDiagSlots; q++) out[q] = v[q];
  }
}

template <class S>
__global__ void __launch_bounds__(kDiagThreads)
k_diag_partial(const S* __restrict__ u, const S* __restrict__ v, const S* __restrict__ s,
               const uint8_t* __restrict__ fl, Consts c, double* __restrict__ partials) {
  const int W = c.W, H = c.H;
  const int64_t N = (int64_t)W * H;
  double acc[kDiagSlots] = {0, 0, 0, 0, 0, 0, 0};
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < N;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(k / W), i = (int)(k - (int64_t)r * W), j = H - 1 - r;
    const uint32_t f = fl[k];
    if (f & F_ACTIVE) {
      const double d = ((as_f64(u + cell_index(W, H, i + 1, j)) - as_f64(u + k)) +
                        as_f64(v + cell_index(W, H, i, j + 1))) - as_f64(v + k);
      acc[0] += d * d;
      acc[1] += d;
      acc[5] += 1.0;
      acc[kDiagSums] = fmax(acc[kDiagSums], fabs(d));
    }
    if (f & F_FLUID) {
      acc[2] += as_f64(s + k);
      // Volume flux through the first and the last column of faces with
      // fluid on both sides: u(2, j) just inside the inlet (the step leaves
      // the inlet face u(1, j) at 0, src/fluid.cu:720-747) and u(W-1, j)
      // into the drain column.
      if (i == 2 && (fl[cell_index(W, H, 1, j)] & F_FLUID)) acc[3] += as_f64(u + k);
      if (i == W - 1 && (fl[cell_index(W, H, W - 2, j)] & F_FLUID)) acc[4] += as_f64(u + k);
    }
  }
  block_fold(acc, partials + (size_t)blockIdx.x * kDiagSlots);
}

// One block folds the kDiagBlocks partials in a fixed order.
__global__ void __launch_bounds__(kDiagThreads)
k_diag_final(const double* __restrict__ partials, int blocks, double* __restrict__ out) {
  double acc[kDiagSlots] = {0, 0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < blocks; b += blockDim.x) {
#pragma unroll
    for (int q = 0; q < kDiagSums; q++) acc[q] += partials[(size_t)b * kDiagSlots + q];
    acc[kDiagSums] = fmax(acc[kDiagSums], partials[(size_t)b * kDiagSlots + kDiagSums]);
  }
  block_fold(acc, out);
}

}  // namespace osg
