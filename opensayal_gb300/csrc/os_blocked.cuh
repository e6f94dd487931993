// os_blocked.cuh — temporally blocked Jacobi diffusion and red/black
// projection: several sweeps per trip through L2/HBM.
//
// A CTA owns a TX x TY tile of cells. It stages the tile plus a halo into
// shared memory, runs `sweeps` sweeps there, and writes back only the cells it
// owns. Validity shrinks by one cell per dependent update, so:
//   * Jacobi diffusion (apply_diffusion_at, src/fluid.cu:176-183) needs a halo
//     of K cells for K sweeps;
//   * red/black SOR (apply_projection_at, src/fluid.cu:229-262) needs 2K
//     cells for K full sweeps, because each colour half-sweep extends the
//     dependency by one cell.
// Every update is the plain kernels' (and the reference's) expression in the
// same order, so a blocked pass gives the same bits as K per-sweep launches.
//
// The region is 256 cells wide (fixed; TX = 256 - 2*halo) and RH = TY +
// 2*halo rows high. The projection region is stored split by column parity
// (even and odd columns in separate arrays), so that the 32 active cells of a
// warp in one colour read and write 32 consecutive words: no bank conflicts
// despite the stride-2 colour pattern. Tiles and passes read one global copy
// and write the other (fields <-> buffers), so no CTA reads a neighbour's
// half-updated halo.
#pragma once

#include <algorithm>
#include <type_traits>

namespace osg {

constexpr int kRegionW = 256;            // region width in cells
constexpr int kHalfW = kRegionW / 2;     // cells per parity per row
constexpr int kArrPad = 16;              // words between parity arrays (bank shift)
constexpr int kBlockThreads = 1024;

struct TileGeom {
  int halo;     // halo in cells on every side
  int TX, TY;   // owned tile
  int RH;       // region rows
  int tiles_x, tiles_y;
  size_t smem;  // dynamic shared memory per CTA
};

__host__ __device__ inline size_t projection_smem(int RH, bool pressure) {
  const size_t plane = (size_t)RH * kHalfW + kArrPad;  // words per parity plane
  const size_t words = plane * (pressure ? 6 : 4);
  return words * 4 + 2 * ((size_t)RH * kHalfW + 64);
}

__host__ __device__ inline size_t diffusion_smem(int RH) {
  return 2 * ((size_t)RH * kRegionW + kArrPad) * 4;
}

// ---------------------------------------------------------------------------
// Blocked red/black projection.
// ---------------------------------------------------------------------------

struct ProjPlanes {
  float *ue, *uo, *ve, *vo, *pe, *po;
  uint8_t *fe, *fo;
};

template <bool PRESSURE>
__device__ __forceinline__ ProjPlanes proj_planes(float* smem, int RH) {
  ProjPlanes P;
  const int plane = RH * kHalfW + kArrPad;
  P.ue = smem;
  P.uo = P.ue + plane;
  P.ve = P.uo + plane;
  P.vo = P.ve + plane;
  float* next = P.vo + plane;
  if (PRESSURE) {
    P.pe = next;
    P.po = P.pe + plane;
    next = P.po + plane;
  } else {
    P.pe = P.po = nullptr;
  }
  P.fe = reinterpret_cast<uint8_t*>(next);
  P.fo = P.fe + RH * kHalfW + 64;
  return P;
}

// One colour half-sweep over the region. Active cells of row y sit at
// x = 2k + par with par = (y + COLOUR) & 1 (region origin has even global
// coordinates, so local parity is global parity).
template <int COLOUR, bool PRESSURE>
__device__ __forceinline__ void proj_half_sweep(const ProjPlanes& P, int RH, const Consts& c,
                                                float d_t) {
  const int k = threadIdx.x & (kHalfW - 1);
  const int rows_per_iter = blockDim.x / kHalfW;
  for (int y = threadIdx.x / kHalfW; y < RH - 1; y += rows_per_iter) {
    const int par = (y + COLOUR) & 1;
    if (par && k == kHalfW - 1) continue;  // its right face lies outside the region
    const int s = y * kHalfW + k;
    const uint8_t f = (par ? P.fo : P.fe)[s];
    if (!(f & F_ACTIVE)) continue;
    float* uL = par ? P.uo : P.ue;   // left face u(x)     at s
    float* uR = par ? P.ue : P.uo;   // right face u(x+1)  at sr
    float* vv = par ? P.vo : P.ve;   // v(x, y) at s, v(x, y+1) at s + kHalfW
    const int sr = s + par;
    const float uc = uL[s];
    const float vc = vv[s];
    const float top_v = vv[s + kHalfW];
    const float right_u = uR[sr];
    const float divergence = right_u - uc + top_v - vc;
    const int sn = __popc(f & F_NBR_MASK);
    // A rounded product: the reference keeps it (its later use sits behind a
    // runtime branch) rather than fusing it into the four face updates.
    const float velocity_diff = mul_rn(c.o, divergence / (float)sn);
    if (PRESSURE) {
      float* pp = par ? P.po : P.pe;
      pp[s] += velocity_diff * c.density * (float)c.h / d_t;  // src/fluid.cu:225-226
    }
    if (f & F_LEFT) uL[s] = uc + velocity_diff;
    if (f & F_RIGHT) uR[sr] = right_u - velocity_diff;
    if (f & F_BOTTOM) vv[s] = vc + velocity_diff;
    if (f & F_TOP) vv[s + kHalfW] = top_v - velocity_diff;
  }
}

// With PRESSURE the first pass of a step zeroes p (zero_pressure,
// src/fluid.cu:203-219) as it loads; later passes continue the accumulation.
template <bool PRESSURE>
__global__ void __launch_bounds__(kBlockThreads, 1)
k_project_blocked(const float* __restrict__ u_in, const float* __restrict__ v_in,
                  float* __restrict__ u_out, float* __restrict__ v_out, float* __restrict__ p,
                  const uint8_t* __restrict__ fl, Consts c, const StepParams* __restrict__ prm,
                  int sweeps, int halo, int TX, int TY, int tiles_x, int zero_pressure) {
  extern __shared__ __align__(16) float smem[];
  const int RH = TY + 2 * halo;
  const ProjPlanes P = proj_planes<PRESSURE>(smem, RH);
  const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
  const int gx0 = tx * TX - halo, gy0 = ty * TY - halo;
  const int W = c.W, H = c.H;
  for (int e = threadIdx.x; e < RH * kRegionW; e += blockDim.x) {
    const int y = e / kRegionW, x = e % kRegionW;
    const int i = gx0 + x, j = gy0 + y;
    float uu = 0.0f, vv = 0.0f, pp = 0.0f;
    uint8_t ff = 0;
    if (i >= 0 && i < W && j >= 0 && j < H) {
      const int64_t gk = cell_index(W, H, i, j);
      uu = u_in[gk];
      vv = v_in[gk];
      ff = fl[gk];
      if (PRESSURE && !zero_pressure && x >= halo && x < halo + TX && y >= halo && y < halo + TY)
        pp = p[gk];
    }
    const int s = y * kHalfW + (x >> 1);
    if (x & 1) {
      P.uo[s] = uu; P.vo[s] = vv; P.fo[s] = ff;
      if (PRESSURE) P.po[s] = pp;
    } else {
      P.ue[s] = uu; P.ve[s] = vv; P.fe[s] = ff;
      if (PRESSURE) P.pe[s] = pp;
    }
  }
  __syncthreads();
  const float d_t = prm->dt;
  for (int t = 0; t < sweeps; t++) {
    proj_half_sweep<0, PRESSURE>(P, RH, c, d_t);
    __syncthreads();
    proj_half_sweep<1, PRESSURE>(P, RH, c, d_t);
    __syncthreads();
  }
  for (int e = threadIdx.x; e < TY * kRegionW; e += blockDim.x) {
    const int y = halo + e / kRegionW, x = e % kRegionW;
    if (x < halo || x >= halo + TX) continue;
    const int i = gx0 + x, j = gy0 + y;
    if (i >= W || j >= H) continue;
    const int64_t gk = cell_index(W, H, i, j);
    const int s = y * kHalfW + (x >> 1);
    u_out[gk] = (x & 1) ? P.uo[s] : P.ue[s];
    v_out[gk] = (x & 1) ? P.vo[s] : P.ve[s];
    if (PRESSURE) p[gk] = (x & 1) ? P.po[s] : P.pe[s];
  }
}

// ---------------------------------------------------------------------------
// Blocked Jacobi diffusion of u.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlockThreads, 1)
k_diffuse_blocked(const float* __restrict__ u_in, float* __restrict__ u_out, Consts c,
                  const StepParams* __restrict__ prm, int sweeps, int halo, int TX, int TY,
                  int tiles_x) {
  extern __shared__ __align__(16) float smem[];
  const int RH = TY + 2 * halo;
  float* A = smem;
  float* B = smem + RH * kRegionW + kArrPad;
  const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
  const int gx0 = tx * TX - halo, gy0 = ty * TY - halo;
  const int W = c.W, H = c.H;
  for (int e = threadIdx.x; e < RH * kRegionW; e += blockDim.x) {
    const int y = e / kRegionW, x = e % kRegionW;
    const int i = gx0 + x, j = gy0 + y;
    A[e] = (i >= 0 && i < W && j >= 0 && j < H) ? u_in[cell_index(W, H, i, j)] : 0.0f;
  }
  __syncthreads();
  const float d_t = prm->dt;
  const float a = c.viscosity * d_t / (float)(c.h * c.h);
  for (int t = 0; t < sweeps; t++) {
    for (int e = threadIdx.x; e < RH * kRegionW; e += blockDim.x) {
      const int y = e / kRegionW, x = e % kRegionW;
      const int i = gx0 + x, j = gy0 + y;
      const bool interior = i > 0 && j > 0 && i < W - 1 && j < H - 1 && x > 0 &&
                            x < kRegionW - 1 && y > 0 && y < RH - 1;
      if (interior) {
        // src/fluid.cu:178-182: neighbours (i-1, j), (i+1, j), (i, j-1), (i, j+1)
        B[e] = (A[e] + a * (A[e - 1] + A[e + 1] + A[e - kRegionW] + A[e + kRegionW])) /
               (1 + 4 * a);
      } else {
        B[e] = A[e];
      }
    }
    __syncthreads();
    float* T = A;
    A = B;
    B = T;
  }
  for (int e = threadIdx.x; e < TY * kRegionW; e += blockDim.x) {
    const int y = halo + e / kRegionW, x = e % kRegionW;
    if (x < halo || x >= halo + TX) continue;
    const int i = gx0 + x, j = gy0 + y;
    if (i >= W || j >= H) continue;
    u_out[cell_index(W, H, i, j)] = A[y * kRegionW + x];
  }
}

// ---------------------------------------------------------------------------
// Host: tile geometry and pass enqueue.
// ---------------------------------------------------------------------------

constexpr size_t kMaxSmem = 227 * 1024;

// Owned tile height for a given halo: aim for one CTA per SM per wave
// (152 SMs), keep TY even (region origin parity), and fit shared memory.
inline TileGeom make_geom(int W, int H, int halo, bool projection, bool pressure, int sms) {
  TileGeom g;
  g.halo = halo;
  g.TX = kRegionW - 2 * halo;
  g.tiles_x = (W + g.TX - 1) / g.TX;
  const int want_tiles_y = std::max(1, sms / g.tiles_x);
  int TY = (H + want_tiles_y - 1) / want_tiles_y;
  TY = std::max(2, (TY + 1) & ~1);
  auto smem_of = [&](int ty) {
    const int rh = ty + 2 * halo;
    return projection ? projection_smem(rh, pressure) : diffusion_smem(rh);
  };
  while (TY > 2 && smem_of(TY) > kMaxSmem) TY -= 2;
  g.TY = TY;
  g.RH = TY + 2 * halo;
  g.tiles_y = (H + TY - 1) / TY;
  g.smem = smem_of(TY);
  return g;
}

inline int choose_block_k(const os_handle* h) {
  if (h->cfg.projection_block < 0) return -1;
  if (h->cfg.projection_block > 0) return std::min(h->cfg.projection_block, 32);
  return 4;
}

template <class S, class A>
inline bool blocked_supported(const os_handle*) {
  return std::is_same<S, float>::value && std::is_same<A, float>::value;
}

inline int sm_count(int device) {
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || n < 1)
    n = 152;
  return n;
}

// Projection: ceil(n / K) passes of up to K sweeps; each pass reads one copy of
// (u, v) and writes the other. `cur` tracks which copy holds the live field
// (0: u/v, 1: ub/vb) and is updated for the caller.
// `zero_first`: the first pass also performs zero_pressure (inside a step).
inline int enqueue_blocked_projection_f32(os_handle* h, cudaStream_t st, int* cur_u, int* cur_v,
                                          bool zero_first) {
  const int K = h->block_k;
  const bool pressure = h->cfg.enable_pressure != 0;
  const TileGeom g = make_geom(h->W, h->H, 2 * K, true, pressure, sm_count(h->cfg.device));
  float* U[2] = {static_cast<float*>(h->u), static_cast<float*>(h->ub)};
  float* V[2] = {static_cast<float*>(h->v), static_cast<float*>(h->vb)};
  const int tiles = g.tiles_x * g.tiles_y;
  int launches = 0;
  for (int done = 0, pass = 0; done < h->c.n; pass++) {
    const int sweeps = std::min(K, h->c.n - done);
    const float* uin = U[*cur_u];
    const float* vin = V[*cur_v];
    float* uout = U[1 - *cur_u];
    float* vout = V[1 - *cur_v];
    if (pressure) {
      cudaFuncSetAttribute(k_project_blocked<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)g.smem);
      k_project_blocked<true><<<tiles, kBlockThreads, g.smem, st>>>(
          uin, vin, uout, vout, h->p, h->flags, h->c, h->d_params, sweeps, g.halo, g.TX, g.TY,
          g.tiles_x, (zero_first && pass == 0) ? 1 : 0);
    } else {
      cudaFuncSetAttribute(k_project_blocked<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)g.smem);
      k_project_blocked<false><<<tiles, kBlockThreads, g.smem, st>>>(
          uin, vin, uout, vout, h->p, h->flags, h->c, h->d_params, sweeps, g.halo, g.TX, g.TY,
          g.tiles_x, 0);
    }
    launches++;
    *cur_u = 1 - *cur_u;
    *cur_v = 1 - *cur_v;
    done += sweeps;
  }
  return launches;
}

inline int enqueue_blocked_diffusion_f32(os_handle* h, cudaStream_t st, int* cur_u) {
  const int K = h->block_k;
  const TileGeom g = make_geom(h->W, h->H, K, false, false, sm_count(h->cfg.device));
  float* U[2] = {static_cast<float*>(h->u), static_cast<float*>(h->ub)};
  const int tiles = g.tiles_x * g.tiles_y;
  cudaFuncSetAttribute(k_diffuse_blocked, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)g.smem);
  int launches = 0;
  for (int done = 0; done < h->c.n;) {
    const int sweeps = std::min(K, h->c.n - done);
    k_diffuse_blocked<<<tiles, kBlockThreads, g.smem, st>>>(
        U[*cur_u], U[1 - *cur_u], h->c, h->d_params, sweeps, g.halo, g.TX, g.TY, g.tiles_x);
    launches++;
    *cur_u = 1 - *cur_u;
    done += sweeps;
  }
  return launches;
}

}  // namespace osg
