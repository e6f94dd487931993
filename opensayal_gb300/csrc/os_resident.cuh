// os_resident.cuh — the whole projection (or diffusion) phase in one
// cooperative launch, with every tile resident in shared memory from the
// first sweep to the last.
//
// The pass-by-pass engine (os_blocked.cuh) restages each tile and its halo
// from L2/HBM and relaunches for every K sweeps. Here each CTA stages its
// region once, and between passes exchanges only what its neighbours need:
//   1. after the K sweeps of pass q the owned cells are exact and the halo is
//      stale (validity shrinks one cell per half-sweep);
//   2. the CTA writes the band of owned cells within `halo` of its edges —
//      exactly the cells that lie in its neighbours' halos — to copy X_q of
//      (u, v), then publishes "pass q done" on its flag (release);
//   3. it waits (acquire, bounded) for its up to 8 neighbours to publish
//      pass q and reloads its halo ring from X_q, part by part: each of the
//      ring's four parts (the bands above and below, the two sides) as soon
//      as the tiles that own it have published (ring_part_wait).
// After the last pass it writes its whole owned tile to X_last. Every update
// is the pass engine's, in the same order, so the result is bit-identical to
// ceil(n/K) blocked passes, and to n per-sweep launches.
//
// X_q alternates between the two copies, starting with the one the input is
// not in. A CTA writes X_q only after its neighbours have published pass q-1,
// which they do after reloading from X_{q-2} (the same copy) and after
// staging their input, so no CTA overwrites data a neighbour still reads.
// All CTAs must be resident together (one per SM), which the cooperative
// launch guarantees or refuses. Waits are bounded: a CTA that gives up (or
// sees another give up) records the failure and returns; the host reports
// OS_ERR_TIMEOUT and resets the flags.
#pragma once

namespace osg {

constexpr int kSpinLimit = 1 << 20;  // polls per wait (tens of ms with the back-off)

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Publishes this CTA's pass: the barrier orders every thread's band stores
// before thread 0's fence, whose release ordering (cumulative over what the
// barrier made visible to it) precedes the flag store.
__device__ __forceinline__ void publish_flag(unsigned* flag, unsigned v) {
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
    st_release_gpu(flag, v);
  }
}

// Owned cells in region rows [y0, y1) x quads [q0, q1) from the planes to
// global u and v. Every quad lies wholly inside the owned tile (halo and TX
// are multiples of 4 here); cells off the grid are skipped.
template <bool PRESSURE, class S>
__device__ __forceinline__ void publish_rect(const float* smem, int RH, S* __restrict__ u,
                                             S* __restrict__ v, int W, int H, int gx0, int gy0,
                                             int y0, int y1, int q0, int q1, bool vec) {
  const ProjPlanes P = proj_planes<PRESSURE>(const_cast<float*>(smem), RH);
  const int nq = q1 - q0;
  const int items = (y1 - y0) * nq;
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    const int y = y0 + it / nq, x = 4 * (q0 + it % nq);
    const int i = gx0 + x, j = gy0 + y;
    if (j >= H || i >= W) continue;
    const int s = y * kHalfW + (x >> 1);
    const float2 ue = *reinterpret_cast<const float2*>(P.ue + s);
    const float2 uo = *reinterpret_cast<const float2*>(P.uo + s);
    const float2 ve = *reinterpret_cast<const float2*>(P.ve + s);
    const float2 vo = *reinterpret_cast<const float2*>(P.vo + s);
    store_quad(u, W, H, i, j, vec, make_float4(ue.x, uo.x, ue.y, uo.y));
    store_quad(v, W, H, i, j, vec, make_float4(ve.x, vo.x, ve.y, vo.y));
  }
}

// With 16-bit storage the pass engine rounds every owned value to storage at
// the end of each pass and stages the rounded values for the next one; the
// owned cells kept in shared memory get the same rounding here, so the two
// forms agree bit for bit.
__device__ __forceinline__ float to_storage_and_back(float x, const float*) { return x; }
__device__ __forceinline__ float to_storage_and_back(float x, const __half*) {
  return __half2float(__float2half_rn(x));
}
__device__ __forceinline__ float to_storage_and_back(float x, const __nv_bfloat16*) {
  return __bfloat162float(__float2bfloat16_rn(x));
}

template <bool PRESSURE, class S>
__device__ __forceinline__ void round_owned(float* smem, int RH, int halo, int TX, int TY) {
  if (std::is_same<S, float>::value) return;
  const ProjPlanes P = proj_planes<PRESSURE>(smem, RH);
  const int hw = TX / 2;  // owned cells per parity plane and row
  const int items = TY * hw;
  const S* tag = nullptr;
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    const int s = (halo + it / hw) * kHalfW + halo / 2 + it % hw;
    P.ue[s] = to_storage_and_back(P.ue[s], tag);
    P.uo[s] = to_storage_and_back(P.uo[s], tag);
    P.ve[s] = to_storage_and_back(P.ve[s], tag);
    P.vo[s] = to_storage_and_back(P.vo[s], tag);
  }
}

struct ResidentSync {
  unsigned* flags;      // one per tile: passes published so far (monotonic)
  int* dev_err;         // set by a CTA that gave up; polled by the others
  int* host_err;        // mapped host word the host reads after synchronising
};

// Part `part` of the halo ring: 0 the region rows [0, halo) (owned by the
// tiles one row down, ty - 1), 1 the rows [halo + TY, RH) (the tiles one row
// up), 2 the left quads [0, hq) of the owned rows (the tile on the left),
// 3 the right quads (the tile on the right). Cell `it` of the part.
__device__ __forceinline__ int ring_part_items(int part, int halo, int TY, int hq) {
  return part < 2 ? halo * kQuads : TY * hq;
}
__device__ __forceinline__ void ring_part_cell(int part, int it, int halo, int TY, int hq, int* y,
                                               int* q) {
  if (part < 2) {
    *y = (part ? halo + TY : 0) + it / kQuads;
    *q = it % kQuads;
  } else {
    *y = halo + it / hq;
    *q = (part == 3 ? kQuads - hq : 0) + it % hq;
  }
}

// The wait of a halo exchange, part by part: each part of the ring is
// reloaded as soon as the tiles that own it have published, instead of the
// whole ring after all eight neighbours have. The warps are split among the
// four parts about in proportion to their sizes (3/8 to each band, 1/8 to
// each side); each part's first warp polls its neighbours' flags (three for
// a band, one for a side, with the same bounded wait as wait_neighbours)
// and the part's warps meet at a named barrier of their own, so the acquire
// loads order the reloads that follow. On return *part is this thread's
// part, and the thread reloads the part's cells t0, t0 + stride, ...; the
// result is the CTA's give-up word, which the caller reads after the
// barrier that ends the reload (non-zero: a wait gave up, here or in
// another CTA, and the ring is not to be used).
__device__ __forceinline__ volatile int* ring_part_wait(const ResidentSync& sync, int tx, int ty,
                                                        int tiles_x, int tiles_y, unsigned want,
                                                        int* part_out, int* t0, int* stride) {
  __shared__ int give_up;
  if (threadIdx.x == 0) give_up = 0;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int n_band = nw * 3 / 8, n_side = nw / 8;  // 12 and 4 of 32 warps
  int part, w0, wn;
  if (warp < n_band) {
    part = 0, w0 = 0, wn = n_band;
  } else if (warp < 2 * n_band) {
    part = 1, w0 = n_band, wn = n_band;
  } else if (warp < 2 * n_band + n_side) {
    part = 2, w0 = 2 * n_band, wn = n_side;
  } else {
    part = 3, w0 = 2 * n_band + n_side, wn = nw - w0;
  }
  if (warp == w0 && lane < (part < 2 ? 3 : 1)) {
    const int nx = part < 2 ? tx + lane - 1 : tx + (part == 2 ? -1 : 1);
    const int ny = part < 2 ? ty + (part == 0 ? -1 : 1) : ty;
    if (nx >= 0 && nx < tiles_x && ny >= 0 && ny < tiles_y) {
      const unsigned* f = sync.flags + ny * tiles_x + nx;
      for (int it = 0; (int)(ld_acquire_gpu(f) - want) < 0; it++) {
        if (it >= kSpinLimit || (it % 64 == 63 && *(volatile int*)sync.dev_err)) {
          if (atomicCAS(sync.dev_err, 0, 1) == 0) {
            *(volatile int*)sync.host_err = 1;
            __threadfence_system();
          }
          *(volatile int*)&give_up = 1;
          break;
        }
        __nanosleep(32);
      }
    }
  }
  __syncwarp();
  asm volatile("bar.sync %0, %1;" ::"r"(1 + part), "r"(wn * 32) : "memory");
  *part_out = part;
  *t0 = threadIdx.x - w0 * 32;
  *stride = wn * 32;
  return &give_up;
}

// The projection's exchange: the ring of u and v into the parity planes,
// part by part (ring_part_wait). Ends with a barrier of the whole CTA;
// returns false, in every thread, when a wait gave up.
template <bool PRESSURE, class S>
__device__ __forceinline__ bool exchange_ring(const ResidentSync& sync, float* smem, int RH,
                                              const S* __restrict__ u, const S* __restrict__ v,
                                              int W, int H, int gx0, int gy0, int halo, int TY,
                                              bool vec, int tx, int ty, int tiles_x, int tiles_y,
                                              unsigned want) {
  int part, t0, stride;
  volatile int* give_up = ring_part_wait(sync, tx, ty, tiles_x, tiles_y, want, &part, &t0, &stride);
  if (!*give_up) {
    const ProjPlanes P = proj_planes<PRESSURE>(smem, RH);
    const int hq = halo / 4;
    const int items = ring_part_items(part, halo, TY, hq);
    for (int base = t0; base < items; base += stride * kInFlight) {
      float4 uq[kInFlight], vq[kInFlight];
#pragma unroll
      for (int r = 0; r < kInFlight; r++) {
        const int it = base + r * stride;
        uq[r] = vq[r] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (it < items) {
          int y, q;
          ring_part_cell(part, it, halo, TY, hq, &y, &q);
          uq[r] = load_quad_cg(u, W, H, gx0 + 4 * q, gy0 + y, vec);
          vq[r] = load_quad_cg(v, W, H, gx0 + 4 * q, gy0 + y, vec);
        }
      }
#pragma unroll
      for (int r = 0; r < kInFlight; r++) {
        const int it = base + r * stride;
        if (it >= items) break;
        int y, q;
        ring_part_cell(part, it, halo, TY, hq, &y, &q);
        const int s = y * kHalfW + 2 * q;
        *reinterpret_cast<float2*>(P.ue + s) = make_float2(uq[r].x, uq[r].z);
        *reinterpret_cast<float2*>(P.uo + s) = make_float2(uq[r].y, uq[r].w);
        *reinterpret_cast<float2*>(P.ve + s) = make_float2(vq[r].x, vq[r].z);
        *reinterpret_cast<float2*>(P.vo + s) = make_float2(vq[r].y, vq[r].w);
      }
    }
  }
  __syncthreads();
  return *give_up == 0;
}

// The diffusion's exchange: the ring of u into the dense region A, part by
// part (ring_part_wait). Ends with a barrier; returns false, in every
// thread, when a wait gave up.
template <class S>
__device__ __forceinline__ bool exchange_ring_dense(const ResidentSync& sync, float* A,
                                                    const S* __restrict__ u, int W, int H,
                                                    int gx0, int gy0, int halo, int TY, bool vec,
                                                    int tx, int ty, int tiles_x, int tiles_y,
                                                    unsigned want) {
  int part, t0, stride;
  volatile int* give_up = ring_part_wait(sync, tx, ty, tiles_x, tiles_y, want, &part, &t0, &stride);
  if (!*give_up) {
    const int hq = halo / 4;
    const int items = ring_part_items(part, halo, TY, hq);
    for (int base = t0; base < items; base += stride * kInFlight) {
      float4 uq[kInFlight];
#pragma unroll
      for (int r = 0; r < kInFlight; r++) {
        const int it = base + r * stride;
        uq[r] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (it < items) {
          int y, q;
          ring_part_cell(part, it, halo, TY, hq, &y, &q);
          uq[r] = load_quad_cg(u, W, H, gx0 + 4 * q, gy0 + y, vec);
        }
      }
#pragma unroll
      for (int r = 0; r < kInFlight; r++) {
        const int it = base + r * stride;
        if (it >= items) break;
        int y, q;
        ring_part_cell(part, it, halo, TY, hq, &y, &q);
        *reinterpret_cast<float4*>(A + y * kRegionW + 4 * q) = uq[r];
      }
    }
  }
  __syncthreads();
  return *give_up == 0;
}

template <bool PRESSURE, class S>
__global__ void __launch_bounds__(kBlockThreads, 1)
k_project_resident(S* U0, S* U1, S* V0, S* V1, int cu, int cv, float* __restrict__ p,
                   const uint8_t* __restrict__ fl, Consts c, const StepParams* __restrict__ prm,
                   int K, int halo, int TX, int TY, int tiles_x, int tiles_y, ResidentSync sync,
                   int zero_pressure, int extrapolate) {
  extern __shared__ __align__(16) float smem[];
  const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
  const int RH = TY + 2 * halo;
  const int W = c.W, H = c.H;
  const int gx0 = tx * TX - halo, gy0 = ty * TY - halo;
  const bool vec = ((W & 3) == 0) && ((gx0 & 3) == 0);
  const unsigned epoch = ld_acquire_gpu(sync.flags + blockIdx.x);
  // Through L2: this launch later writes the input copy (X_1).
  proj_stage_in<PRESSURE, S, true>(smem, tx, ty, cu ? U1 : U0, cv ? V1 : V0, p, fl, c, halo,
                                   TX, TY, zero_pressure);
  __syncthreads();
  const int passes = (c.n + K - 1) / K;
  const int hq = halo / 4, oq0 = hq, oq1 = hq + TX / 4;  // owned quads
  for (int q = 0; q < passes; q++) {
    proj_sweeps_fast<PRESSURE>(smem, c, prm, min(K, c.n - q * K), halo, TY);
    S* uo = ((cu + q + 1) & 1) ? U1 : U0;
    S* vo = ((cv + q + 1) & 1) ? V1 : V0;
    if (q == passes - 1) {
      if (extrapolate) extrapolate_region<PRESSURE>(smem, RH, gx0, gy0, halo, TX, TY, W, H);
      proj_stage_out<PRESSURE, S>(smem, tx, ty, uo, vo, p, c, halo, TX, TY);
      return;
    }
    // The band of owned cells within `halo` of the tile's edges.
    publish_rect<PRESSURE, S>(smem, RH, uo, vo, W, H, gx0, gy0, halo, 2 * halo, oq0, oq1, vec);
    publish_rect<PRESSURE, S>(smem, RH, uo, vo, W, H, gx0, gy0, TY, TY + halo, oq0, oq1, vec);
    publish_rect<PRESSURE, S>(smem, RH, uo, vo, W, H, gx0, gy0, 2 * halo, TY, oq0, oq0 + hq, vec);
    publish_rect<PRESSURE, S>(smem, RH, uo, vo, W, H, gx0, gy0, 2 * halo, TY, oq1 - hq, oq1, vec);
    publish_flag(sync.flags + blockIdx.x, epoch + q + 1);
    // Owned cells rounded as the pass engine's write-back would round them
    // (the owned cells and the ring are disjoint, so this may precede the
    // reload), then the halo ring from the neighbours' bands, part by part.
    round_owned<PRESSURE, S>(smem, RH, halo, TX, TY);
    if (!exchange_ring<PRESSURE, S>(sync, smem, RH, uo, vo, W, H, gx0, gy0, halo, TY, vec, tx,
                                    ty, tiles_x, tiles_y, epoch + q + 1))
      return;
  }
}

// ---------------------------------------------------------------------------
// Resident Jacobi diffusion: the same scheme for apply_diffusion_at
// (src/fluid.cu:176-183), halo K for K sweeps, on the dense two-buffer region
// of the pass engine (diff_stage_in / diff_sweeps / diff_store_owned). Only
// the buffer holding the current sweep's input needs the fresh ring: cells no
// sweep updates (domain boundary, off the grid) are constant and staged into
// both buffers at the start.
// ---------------------------------------------------------------------------

// Owned cells within `halo` of the tile's edges, from A to global.
template <class S>
__device__ __forceinline__ void publish_band_dense(const float* A, S* __restrict__ u, int W, int H,
                                                   int gx0, int gy0, int halo, int TX, int TY,
                                                   bool vec) {
  const int hq = halo / 4, oq = TX / 4;  // owned quads per row: [hq, hq + oq)
  const int band = halo * oq, side = (TY - 2 * halo > 0 ? TY - 2 * halo : 0) * hq;
  const int items = 2 * band + 2 * side;
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    int y, q;
    if (it < band) {
      y = halo + it / oq;
      q = hq + it % oq;
    } else if (it < 2 * band) {
      y = TY + (it - band) / oq;
      q = hq + (it - band) % oq;
    } else {
      const int r = it - 2 * band;
      const int sd = r / side, k = r - sd * side;
      y = 2 * halo + k / hq;
      q = (sd ? hq + oq - hq : hq) + k % hq;
    }
    const int i = gx0 + 4 * q, j = gy0 + y;
    if (j >= H || i >= W) continue;
    store_quad(u, W, H, i, j, vec, *reinterpret_cast<const float4*>(A + y * kRegionW + 4 * q));
  }
}

template <class S>
__device__ __forceinline__ void round_owned_dense(float* A, int halo, int TX, int TY) {
  if (std::is_same<S, float>::value) return;
  const S* tag = nullptr;
  for (int it = threadIdx.x; it < TY * TX; it += blockDim.x) {
    const int e = (halo + it / TX) * kRegionW + halo + it % TX;
    A[e] = to_storage_and_back(A[e], tag);
  }
}

template <class S>
__global__ void __launch_bounds__(kBlockThreads, 1)
k_diffuse_resident(S* U0, S* U1, int cu, Consts c, const StepParams* __restrict__ prm, int K,
                   int halo, int TX, int TY, int tiles_x, int tiles_y, ResidentSync sync) {
  extern __shared__ __align__(16) float smem[];
  const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
  const int RH = TY + 2 * halo;
  const int W = c.W, H = c.H;
  const int gx0 = tx * TX - halo, gy0 = ty * TY - halo;
  const bool vec = ((W & 3) == 0) && ((gx0 & 3) == 0);
  float* A = smem;
  float* B = smem + RH * kRegionW + kArrPad;
  const unsigned epoch = ld_acquire_gpu(sync.flags + blockIdx.x);
  // Through L2: this launch later writes the input copy (X_1).
  diff_stage_in<S, true>(A, B, tx, ty, cu ? U1 : U0, c, halo, TX, TY);
  __syncthreads();
  const int passes = (c.n + K - 1) / K;
  for (int q = 0; q < passes; q++) {
    diff_sweeps(A, B, tx, ty, c, prm, min(K, c.n - q * K), halo, TX, TY);
    S* uo = ((cu + q + 1) & 1) ? U1 : U0;
    if (q == passes - 1) {
      diff_store_owned<S>(A, tx, ty, uo, c, halo, TX, TY);
      return;
    }
    publish_band_dense<S>(A, uo, W, H, gx0, gy0, halo, TX, TY, vec);
    publish_flag(sync.flags + blockIdx.x, epoch + q + 1);
    // Owned cells rounded as the pass engine's write-back would round them
    // (disjoint from the ring), then the ring, part by part.
    round_owned_dense<S>(A, halo, TX, TY);
    if (!exchange_ring_dense<S>(sync, A, uo, W, H, gx0, gy0, halo, TY, vec, tx, ty, tiles_x,
                                tiles_y, epoch + q + 1))
      return;
  }
}

// Failure-detection self-test: tile 0 of a 2 x 1 grid waits for tile 1,
// which no CTA runs, so the wait must give up and report.
__global__ void k_wait_selftest(ResidentSync sync) {
  int part, t0, stride;
  ring_part_wait(sync, 0, 0, 2, 1, 1u, &part, &t0, &stride);
  __syncthreads();
}

// Host: tile geometry for K sweeps per exchange (halo 2K), with at most one
// tile per SM. False when the grid does not fit that way: halo and tile widths
// must be multiples of 4 (K even), tiles at least two halos wide and high,
// and the region within shared memory.
inline bool resident_geom(int W, int H, int K, bool pressure, int sms, TileGeom* out) {
  if (K < 2 || (K & 1)) return false;
  TileGeom g;
  g.halo = 2 * K;
  g.TX = kRegionW - 2 * g.halo;
  if (g.TX < 2 * g.halo) return false;
  g.tiles_x = (W + g.TX - 1) / g.TX;
  const int rows_of_tiles = sms / g.tiles_x;
  if (rows_of_tiles < 1) return false;
  int TY = (H + rows_of_tiles - 1) / rows_of_tiles;
  TY = std::max(2 * g.halo, (TY + 1) & ~1);
  g.TY = TY;
  g.RH = TY + 2 * g.halo;
  g.tiles_y = (H + TY - 1) / TY;
  g.smem = projection_smem(g.RH, pressure);
  // Static shared memory of the kernel (the wait flag) sits beside the region.
  if (g.smem + kStaticSmem > kMaxSmem || g.tiles_x * g.tiles_y > sms) return false;
  *out = g;
  return true;
}

// The same for the resident diffusion: halo K, K a multiple of 4.
inline bool resident_diffusion_geom(int W, int H, int K, int sms, TileGeom* out) {
  if (K < 4 || (K & 3)) return false;
  TileGeom g;
  g.halo = K;
  g.TX = kRegionW - 2 * g.halo;
  if (g.TX < 2 * g.halo) return false;
  g.tiles_x = (W + g.TX - 1) / g.TX;
  const int rows_of_tiles = sms / g.tiles_x;
  if (rows_of_tiles < 1) return false;
  int TY = (H + rows_of_tiles - 1) / rows_of_tiles;
  TY = std::max(2 * g.halo, (TY + 1) & ~1);
  g.TY = TY;
  g.RH = TY + 2 * g.halo;
  g.tiles_y = (H + TY - 1) / TY;
  g.smem = diffusion_smem(g.RH);
  if (g.smem + kStaticSmem > kMaxSmem || g.tiles_x * g.tiles_y > sms) return false;
  *out = g;
  return true;
}

template <class S>
inline bool resident_diffusion_launchable(const TileGeom& g, int sms) {
  auto fn = k_diffuse_resident<S>;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem) !=
      cudaSuccess)
    return false;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kBlockThreads, g.smem) !=
      cudaSuccess)
    return false;
  return per_sm >= 1 && g.tiles_x * g.tiles_y <= per_sm * sms;
}

template <class S>
inline int enqueue_resident_diffusion(os_handle* h, cudaStream_t st, int* cur_u) {
  const int K = h->block_k;
  TileGeom g;
  if (!resident_diffusion_geom(h->W, h->H, K, sm_count(h->cfg.device), &g)) return -1;
  const ResidentSync rs{h->dflags, h->rerr, h->d_host_rerr};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(g.tiles_x * g.tiles_y);
  cfg.blockDim = dim3(kBlockThreads);
  cfg.dynamicSmemBytes = g.smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaFuncSetAttribute(k_diffuse_resident<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)g.smem);
  const cudaError_t e = cudaLaunchKernelEx(
      &cfg, k_diffuse_resident<S>, static_cast<S*>(h->u), static_cast<S*>(h->ub), *cur_u, h->c,
      (const StepParams*)h->d_params, K, g.halo, g.TX, g.TY, g.tiles_x, g.tiles_y, rs);
  if (e != cudaSuccess) return -1;
  if (((h->c.n + K - 1) / K) & 1) *cur_u = 1 - *cur_u;
  return 1;
}

template <bool PRESSURE, class S>
inline bool resident_launchable(const TileGeom& g, int sms) {
  auto fn = k_project_resident<PRESSURE, S>;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem) !=
      cudaSuccess)
    return false;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kBlockThreads, g.smem) !=
      cudaSuccess)
    return false;
  return per_sm >= 1 && g.tiles_x * g.tiles_y <= per_sm * sms;
}

// The whole projection phase as one cooperative launch; `cur_u`/`cur_v`
// advance as after ceil(n/K) passes of the pass engine.
template <class S>
inline int enqueue_resident_projection(os_handle* h, cudaStream_t st, int* cur_u, int* cur_v,
                                       bool zero_first, bool* extrapolated) {
  const int K = h->block_k;
  const bool pressure = h->cfg.enable_pressure != 0;
  TileGeom g;
  if (!resident_geom(h->W, h->H, K, pressure, sm_count(h->cfg.device), &g)) return -1;
  // The extrapolation that follows the projection in a step, on the staged
  // regions of the last pass.
  const int extrapolate =
      (extrapolated && h->c.n > 0 && extrapolation_tile_local(h->W, h->H, g.TX, g.TY)) ? 1 : 0;
  S* U0 = static_cast<S*>(h->u);
  S* U1 = static_cast<S*>(h->ub);
  S* V0 = static_cast<S*>(h->v);
  S* V1 = static_cast<S*>(h->vb);
  const ResidentSync rs{h->rflags, h->rerr, h->d_host_rerr};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(g.tiles_x * g.tiles_y);
  cfg.blockDim = dim3(kBlockThreads);
  cfg.dynamicSmemBytes = g.smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e;
  if (pressure) {
    cudaFuncSetAttribute(k_project_resident<true, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)g.smem);
    e = cudaLaunchKernelEx(&cfg, k_project_resident<true, S>, U0, U1, V0, V1, *cur_u, *cur_v,
                           h->p, (const uint8_t*)h->flags, h->c,
                           (const StepParams*)h->d_params, K, g.halo, g.TX, g.TY, g.tiles_x,
                           g.tiles_y, rs, zero_first ? 1 : 0, extrapolate);
  } else {
    cudaFuncSetAttribute(k_project_resident<false, S>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem);
    e = cudaLaunchKernelEx(&cfg, k_project_resident<false, S>, U0, U1, V0, V1, *cur_u, *cur_v,
                           h->p, (const uint8_t*)h->flags, h->c,
                           (const StepParams*)h->d_params, K, g.halo, g.TX, g.TY, g.tiles_x,
                           g.tiles_y, rs, 0, extrapolate);
  }
  if (e != cudaSuccess) return -1;
  if (extrapolated) *extrapolated = extrapolate != 0;
  const int passes = (h->c.n + K - 1) / K;
  if (passes & 1) {
    *cur_u = 1 - *cur_u;
    *cur_v = 1 - *cur_v;
  }
  return 1;
}

}  // namespace osg
