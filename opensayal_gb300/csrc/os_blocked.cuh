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
//
// Staging moves 4 consecutive cells per access (float4 / 32-bit flag words)
// with several independent loads in flight per thread; cells off the grid
// read as zero (they are never active and never feed an active cell).
#pragma once

#include <cuda.h>  // CUtensorMap and its enums (types only; no driver-library link)

#include <algorithm>
#include <mutex>
#include <type_traits>

namespace osg {

constexpr int kRegionW = 256;            // region width in cells
constexpr int kHalfW = kRegionW / 2;     // cells per parity per row
constexpr int kQuads = kRegionW / 4;     // 4-cell groups per region row
constexpr int kArrPad = 16;              // words between arrays (bank shift, alignment)
constexpr int kBlockThreads = 1024;
constexpr int kInFlight = 4;             // staging groups per thread per batch

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

// Four consecutive stored values as FP32 (one vector load).
__device__ __forceinline__ float4 vec4_to_f32(const float* p) {
  return __ldg(reinterpret_cast<const float4*>(p));
}
__device__ __forceinline__ float4 vec4_to_f32(const __half* p) {
  const uint2 r = __ldg(reinterpret_cast<const uint2*>(p));
  const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&r.x));
  const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&r.y));
  return make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ float4 vec4_to_f32(const __nv_bfloat16* p) {
  const uint2 r = __ldg(reinterpret_cast<const uint2*>(p));
  const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&r.x));
  const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&r.y));
  return make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ void f32_to_vec4(float* p, float4 q) {
  *reinterpret_cast<float4*>(p) = q;
}
__device__ __forceinline__ void f32_to_vec4(__half* p, float4 q) {
  __half2 a = __floats2half2_rn(q.x, q.y), b = __floats2half2_rn(q.z, q.w);
  uint2 r;
  r.x = *reinterpret_cast<uint32_t*>(&a);
  r.y = *reinterpret_cast<uint32_t*>(&b);
  *reinterpret_cast<uint2*>(p) = r;
}
__device__ __forceinline__ void f32_to_vec4(__nv_bfloat16* p, float4 q) {
  __nv_bfloat162 a = __floats2bfloat162_rn(q.x, q.y), b = __floats2bfloat162_rn(q.z, q.w);
  uint2 r;
  r.x = *reinterpret_cast<uint32_t*>(&a);
  r.y = *reinterpret_cast<uint32_t*>(&b);
  *reinterpret_cast<uint2*>(p) = r;
}

// Four consecutive cells (i..i+3) of logical row j as FP32, zero off the
// grid. `vec` = rows start aligned to 4 elements and i is a multiple of 4.
template <class S>
__device__ __forceinline__ float4 load_quad(const S* __restrict__ f, int W, int H, int i, int j,
                                            bool vec) {
  float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
  if (j < 0 || j >= H) return q;
  const int64_t row = (int64_t)(H - 1 - j) * W;
  if (vec && i >= 0 && i + 3 < W) return vec4_to_f32(f + row + i);
  if (i >= 0 && i < W) q.x = ldg<float>(f + row + i);
  if (i + 1 >= 0 && i + 1 < W) q.y = ldg<float>(f + row + i + 1);
  if (i + 2 >= 0 && i + 2 < W) q.z = ldg<float>(f + row + i + 2);
  if (i + 3 >= 0 && i + 3 < W) q.w = ldg<float>(f + row + i + 3);
  return q;
}

// Loads of data that other CTAs of the same launch wrote: through L2 only,
// so a line this SM cached earlier is never returned.
__device__ __forceinline__ float4 vec4_cg(const float* p) {
  return __ldcg(reinterpret_cast<const float4*>(p));
}
__device__ __forceinline__ float4 vec4_cg(const __half* p) {
  const uint2 r = __ldcg(reinterpret_cast<const uint2*>(p));
  const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&r.x));
  const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&r.y));
  return make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ float4 vec4_cg(const __nv_bfloat16* p) {
  const uint2 r = __ldcg(reinterpret_cast<const uint2*>(p));
  const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&r.x));
  const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&r.y));
  return make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ float scalar_cg(const float* p) { return __ldcg(p); }
__device__ __forceinline__ float scalar_cg(const __half* p) { return __half2float(__ldcg(p)); }
__device__ __forceinline__ float scalar_cg(const __nv_bfloat16* p) {
  return __bfloat162float(__ldcg(p));
}

template <class S>
__device__ __forceinline__ float4 load_quad_cg(const S* __restrict__ f, int W, int H, int i, int j,
                                               bool vec) {
  float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
  if (j < 0 || j >= H) return q;
  const int64_t row = (int64_t)(H - 1 - j) * W;
  if (vec && i >= 0 && i + 3 < W) return vec4_cg(f + row + i);
  if (i >= 0 && i < W) q.x = scalar_cg(f + row + i);
  if (i + 1 >= 0 && i + 1 < W) q.y = scalar_cg(f + row + i + 1);
  if (i + 2 >= 0 && i + 2 < W) q.z = scalar_cg(f + row + i + 2);
  if (i + 3 >= 0 && i + 3 < W) q.w = scalar_cg(f + row + i + 3);
  return q;
}

__device__ __forceinline__ uint32_t load_quad_u8(const uint8_t* __restrict__ f, int W, int H,
                                                 int i, int j, bool vec) {
  if (j < 0 || j >= H) return 0;
  const int64_t row = (int64_t)(H - 1 - j) * W;
  if (vec && i >= 0 && i + 3 < W) return __ldg(reinterpret_cast<const uint32_t*>(f + row + i));
  uint32_t q = 0;
#pragma unroll
  for (int d = 0; d < 4; d++)
    if (i + d >= 0 && i + d < W) q |= (uint32_t)__ldg(f + row + i + d) << (8 * d);
  return q;
}

template <class S>
__device__ __forceinline__ void store_quad(S* __restrict__ f, int W, int H, int i, int j,
                                           bool vec, float4 q) {
  const int64_t row = (int64_t)(H - 1 - j) * W;
  if (vec && i + 3 < W) {
    f32_to_vec4(f + row + i, q);
    return;
  }
  if (i < W) st(f + row + i, q.x);
  if (i + 1 < W) st(f + row + i + 1, q.y);
  if (i + 2 < W) st(f + row + i + 2, q.z);
  if (i + 3 < W) st(f + row + i + 3, q.w);
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

// Colours: the active cells of region row y in half-sweep COLOUR sit at
// x = 2k + ((y + COLOUR) & 1) (the region origin has even global coordinates,
// so local parity is global parity).
//
// A cell's flag byte as the blocked sweeps keep it in shared memory: 0 for a
// cell the projection does not update (not F_ACTIVE); otherwise bit 0 set, the
// neighbour bits F_LEFT .. F_TOP in place, and in bits 5-7 the number of
// fluid neighbours, s of apply_projection_at (0 to 4). The per-cell test and
// count are then one compare and one shift.
constexpr int kSweepCountShift = 5;
__device__ __forceinline__ uint32_t sweep_flag(uint32_t f) {
  return (f & F_ACTIVE) ? 1u | (f & F_NBR_MASK) |
                              ((uint32_t)__popc(f & F_NBR_MASK) << kSweepCountShift)
                        : 0u;
}
__device__ __forceinline__ uint32_t sweep_flags4(uint32_t q) {
  return sweep_flag(q & 0xffu) | sweep_flag((q >> 8) & 0xffu) << 8 |
         sweep_flag((q >> 16) & 0xffu) << 16 | sweep_flag(q >> 24) << 24;
}

// apply_projection_at (src/fluid.cu:229-262) for one cell given its four faces
// and sweep flag byte; faces it may not touch come back unchanged. (A table of
// the reciprocals of s in shared memory gives the same bits as the fast-math
// division, but measured slower: shared-memory traffic, not the reciprocal,
// binds these sweeps.)
template <bool PRESSURE>
__device__ __forceinline__ void project_faces(uint32_t f, const Consts& c, float d_t, float& uc,
                                              float& right_u, float& vc, float& top_v,
                                              float& pc) {
  if (!f) return;
  const float divergence = right_u - uc + top_v - vc;
  const int sn = (int)(f >> kSweepCountShift);
  // A rounded product: the reference keeps it (its later use sits behind a
  // runtime branch) rather than fusing it into the four face updates.
  const float velocity_diff = mul_rn(c.o, divergence / (float)sn);
  if (PRESSURE) pc += velocity_diff * c.density * (float)c.h / d_t;  // src/fluid.cu:225-226
  if (f & F_LEFT) uc = uc + velocity_diff;
  if (f & F_RIGHT) right_u = right_u - velocity_diff;
  if (f & F_BOTTOM) vc = vc + velocity_diff;
  if (f & F_TOP) top_v = top_v - velocity_diff;
}

// A thread takes two neighbouring cells of the colour in one row (k, k+1:
// x = 2k + par and 2k + 2 + par) and steps through rows 2*(blockDim/64)
// apart, so its parity, and with it every plane offset, is fixed for the
// whole loop. Faces move as 64-bit pairs; every face of a cell of this colour
// belongs to that cell alone, so writing back unchanged faces is safe.
// Planes are word offsets from the __shared__ base: ue 0, uo 1, ve 2, vo 3,
// pe 4, po 5 (x plane).
template <int PAR, bool PRESSURE>
__device__ __forceinline__ void proj_rows(float* __restrict__ S, const uint8_t* __restrict__ F,
                                          int plane, int fo_off, const Consts& c, float d_t,
                                          int k, int y_begin, int y_end, int rows_per_iter) {
  // With PAR = 1 the cell at k = 127 has its right face outside the region.
  const bool second = !(PAR && k == kHalfW - 2);
  const int oL = PAR ? plane : 0;      // plane of the left face u(x)
  const int oR = plane - oL;           // plane of the right face u(x+1)
  const int oV = 2 * plane + oL;       // plane of v(x, .)
  const int oP = 4 * plane + oL;       // plane of p(x, .)
  const int oF = PAR ? fo_off : 0;
  for (int y = y_begin; y < y_end; y += rows_per_iter) {
    const int s = y * kHalfW + k;
    const uint32_t f2 = *reinterpret_cast<const uint16_t*>(F + oF + s);
    if (!f2) continue;
    float2 uL = *reinterpret_cast<const float2*>(S + oL + s);
    float2 vB = *reinterpret_cast<const float2*>(S + oV + s);
    float2 vT = *reinterpret_cast<const float2*>(S + oV + s + kHalfW);
    float2 uR;
    if (PAR) {
      uR.x = S[oR + s + 1];
      uR.y = second ? S[oR + s + 2] : 0.0f;
    } else {
      uR = *reinterpret_cast<const float2*>(S + oR + s);
    }
    float2 pp = make_float2(0.0f, 0.0f);
    if (PRESSURE) pp = *reinterpret_cast<const float2*>(S + oP + s);
    project_faces<PRESSURE>(f2 & 0xffu, c, d_t, uL.x, uR.x, vB.x, vT.x, pp.x);
    if (second) project_faces<PRESSURE>(f2 >> 8, c, d_t, uL.y, uR.y, vB.y, vT.y, pp.y);
    *reinterpret_cast<float2*>(S + oL + s) = uL;
    *reinterpret_cast<float2*>(S + oV + s) = vB;
    *reinterpret_cast<float2*>(S + oV + s + kHalfW) = vT;
    if (PAR) {
      S[oR + s + 1] = uR.x;
      if (second) S[oR + s + 2] = uR.y;
    } else {
      *reinterpret_cast<float2*>(S + oR + s) = uR;
    }
    if (PRESSURE) *reinterpret_cast<float2*>(S + oP + s) = pp;
  }
}

// `reach`: the half-sweeps still to come in this pass. A face stored in an
// owned cell is last written by that cell or by its left / lower neighbour,
// and every earlier half-sweep widens that set by one cell per side, so only
// cells in [halo - 1 - reach, size - halo + reach) on each axis are computed;
// the rest of the region is stale and never reaches an owned face.
template <int COLOUR, bool PRESSURE>
__device__ __forceinline__ void proj_half_sweep(float* __restrict__ S,
                                                const uint8_t* __restrict__ F, int plane,
                                                int fo_off, int RH, int halo, int reach,
                                                const Consts& c, float d_t) {
  constexpr int kPairs = kHalfW / 2;
  const int k = 2 * (threadIdx.x % kPairs);
  const int rows_per_iter = blockDim.x / kPairs;  // even
  const int y0 = threadIdx.x / kPairs;
  const int par = (y0 + COLOUR) & 1;
  const int lo = max(0, halo - 1 - reach);        // first needed cell, both axes
  const int x = 2 * k + par;                      // the pair covers x .. x + 2
  if (x + 2 < lo || x >= kRegionW - halo + reach) return;
  const int y_end = min(RH - 1, RH - halo + reach);
  const int skip = lo > y0 ? (lo - y0 + rows_per_iter - 1) / rows_per_iter : 0;
  const int y_begin = y0 + skip * rows_per_iter;
  if (par)
    proj_rows<1, PRESSURE>(S, F, plane, fo_off, c, d_t, k, y_begin, y_end, rows_per_iter);
  else
    proj_rows<0, PRESSURE>(S, F, plane, fo_off, c, d_t, k, y_begin, y_end, rows_per_iter);
}

// With PRESSURE the first pass of a step zeroes p (zero_pressure,
// src/fluid.cu:203-219) as it loads; later passes continue the accumulation.
// p is staged for owned cells only (halo pressure is never needed), so no CTA
// reads pressure that another CTA writes in the same pass.
// One tile (tx, ty) of one grid: stage, `sweeps` red/black sweeps, write back.
// The three parts are separate so that a caller holding several storage types
// instantiates the sweeps once.
template <bool PRESSURE, class S, bool CG = false>
__device__ __forceinline__ void proj_stage_in(float* smem, int tx, int ty,
                                              const S* __restrict__ u_in,
                                              const S* __restrict__ v_in,
                                              const float* __restrict__ p,
                                              const uint8_t* __restrict__ fl, const Consts& c,
                                              int halo, int TX, int TY, int zero_pressure) {
  const int RH = TY + 2 * halo;
  const ProjPlanes P = proj_planes<PRESSURE>(smem, RH);
  const int gx0 = tx * TX - halo, gy0 = ty * TY - halo;
  const int W = c.W, H = c.H;
  const bool vec = ((W & 3) == 0) && ((gx0 & 3) == 0);
  const int items = RH * kQuads;
  for (int base = threadIdx.x; base < items; base += blockDim.x * kInFlight) {
    float4 uq[kInFlight], vq[kInFlight];
    uint32_t fq[kInFlight];
#pragma unroll
    for (int r = 0; r < kInFlight; r++) {
      const int it = base + r * blockDim.x;
      const int y = it / kQuads, x = 4 * (it % kQuads);
      const bool ok = it < items;
      const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
      if (CG) {
        uq[r] = ok ? load_quad_cg(u_in, W, H, gx0 + x, gy0 + y, vec) : z;
        vq[r] = ok ? load_quad_cg(v_in, W, H, gx0 + x, gy0 + y, vec) : z;
      } else {
        uq[r] = ok ? load_quad(u_in, W, H, gx0 + x, gy0 + y, vec) : z;
        vq[r] = ok ? load_quad(v_in, W, H, gx0 + x, gy0 + y, vec) : z;
      }
      fq[r] = ok ? load_quad_u8(fl, W, H, gx0 + x, gy0 + y, vec) : 0u;
    }
#pragma unroll
    for (int r = 0; r < kInFlight; r++) {
      const int it = base + r * blockDim.x;
      if (it >= items) break;
      const int y = it / kQuads, q = it % kQuads;
      const int s = y * kHalfW + 2 * q;  // cells 4q, 4q+2 -> even plane; 4q+1, 4q+3 -> odd
      *reinterpret_cast<float2*>(P.ue + s) = make_float2(uq[r].x, uq[r].z);
      *reinterpret_cast<float2*>(P.uo + s) = make_float2(uq[r].y, uq[r].w);
      *reinterpret_cast<float2*>(P.ve + s) = make_float2(vq[r].x, vq[r].z);
      *reinterpret_cast<float2*>(P.vo + s) = make_float2(vq[r].y, vq[r].w);
      const uint32_t f = sweep_flags4(fq[r]);
      *reinterpret_cast<uint16_t*>(P.fe + s) = (uint16_t)((f & 0xffu) | ((f >> 8) & 0xff00u));
      *reinterpret_cast<uint16_t*>(P.fo + s) = (uint16_t)(((f >> 8) & 0xffu) | ((f >> 16) & 0xff00u));
    }
  }
  if (PRESSURE) {
    for (int e = threadIdx.x; e < RH * kRegionW; e += blockDim.x) {
      const int y = e / kRegionW, x = e % kRegionW;
      const int i = gx0 + x, j = gy0 + y;
      float pp = 0.0f;
      if (!zero_pressure && x >= halo && x < halo + TX && y >= halo && y < halo + TY && i < W &&
          j < H)
        pp = p[cell_index(W, H, i, j)];
      ((x & 1) ? P.po : P.pe)[y * kHalfW + (x >> 1)] = pp;
    }
  }
}

// `sweeps` red/black sweeps on the staged tile; ends with a barrier.
template <bool PRESSURE>
__device__ __forceinline__ void proj_sweeps(float* smem, const Consts& c,
                                            const StepParams* __restrict__ prm, int sweeps,
                                            int halo, int TY) {
  const int RH = TY + 2 * halo;
  const ProjPlanes P = proj_planes<PRESSURE>(smem, RH);
  const float d_t = prm->dt;
  const int plane = RH * kHalfW + kArrPad;
  const int fo_off = RH * kHalfW + 64;
  for (int t = 0; t < sweeps; t++) {
    const int reach = 2 * (sweeps - t) - 1;  // half-sweeps after the even one
    proj_half_sweep<0, PRESSURE>(smem, P.fe, plane, fo_off, RH, halo, reach, c, d_t);
    __syncthreads();
    proj_half_sweep<1, PRESSURE>(smem, P.fe, plane, fo_off, RH, halo, reach - 1, c, d_t);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// The same sweeps with the vertical faces in registers.
//
// Thread t owns the column pair (2p, 2p + 1) over the R rows [y0, y0 + R) of
// strip s = t / 128, y0 = s * R; the 128 threads of a strip cover p = 0 .. 127
// (in column blocks of 32 rotated by the strip, see proj_sweeps_vreg). R is
// even, so every strip
// starts on an even row and the active column of the pair in row y0 + r is
// (r + colour) & 1 for every thread: fixed once the row loop is unrolled. The
// thread's faces v(x, y0 .. y0 + R - 1) stay in registers for all the sweeps of
// a pass (one load from and one store to the v planes per pass); only u, the
// flags and p are read and written in shared memory, and lanes take
// consecutive words, so there are no bank conflicts. Per cell update that is
// 2 loads and 2 stores of u and a flag byte, against 4 face loads, 4 face
// stores and the flags when all faces live in shared memory.
//
// The face v(x, Y) on the boundary Y = y0 + R between a strip and the one
// above belongs to a cell of each: both keep a copy. A half-sweep changes at
// most one of the two copies of each such face (the lower strip's where its
// top-row cell is active, the upper strip's where its bottom-row cell is), and
// that side then writes the new value to the face's own word in the v plane;
// after the barrier the other side reads it. The word is next written by the
// side that just read it, so one barrier per half-sweep suffices.
//
// Most cells have four fluid neighbours. A warp whose cells the half-sweep
// needs are all such cells runs a loop of its own without flag loads, flag
// tests or the division by the neighbour count (vreg_half_sweep); measured on
// the 1920 x 1080 tunnel, that took a pass of 8 sweeps from 22.9 to 17.0 us
// on the tiles without walls, the obstacle or cells off the grid, and to
// 20.2-20.8 us on the others, where a quarter of the warps still test flags.
// ---------------------------------------------------------------------------
// project_faces without branches and without the pressure, for cells taken
// two rows at a time: `f` is the sweep flag byte, 0 for any cell not updated
// (inactive, off the cone or off the region), whose faces then keep their
// values. The expressions are project_faces' own.
__device__ __forceinline__ void project_faces_sel(uint32_t f, const Consts& c, float& uc,
                                                  float& right_u, float& vc, float& top_v) {
  const float divergence = right_u - uc + top_v - vc;
  const int sn = (int)(f >> kSweepCountShift);
  const float velocity_diff = mul_rn(c.o, divergence / (float)sn);
  if (f & F_LEFT) uc = uc + velocity_diff;
  if (f & F_RIGHT) right_u = right_u - velocity_diff;
  if (f & F_BOTTOM) vc = vc + velocity_diff;
  if (f & F_TOP) top_v = top_v - velocity_diff;
}

// The sweep flag of an active cell whose four neighbours are all fluid.
constexpr uint32_t kFullFlag = 1u | F_NBR_MASK | (4u << kSweepCountShift);

// project_faces_sel for a cell with flag kFullFlag: every face is updated,
// and s = 4. The division by 4 is the product by 0.25, which gives the bits
// of the fast-math division by a runtime 4 for every float input (all 2^32
// patterns compared by tests/cpp/quarter_division.cu).
__device__ __forceinline__ void project_faces_full(const Consts& c, float& uc, float& right_u,
                                                   float& vc, float& top_v) {
  const float divergence = right_u - uc + top_v - vc;
  const float velocity_diff = mul_rn(c.o, mul_rn(divergence, 0.25f));
  uc = uc + velocity_diff;
  right_u = right_u - velocity_diff;
  vc = vc + velocity_diff;
  top_v = top_v - velocity_diff;
}

// One row of a half-sweep, with branches (the accumulated pressure needs the
// registers that the paired, branch-free rows below would use): the active
// cell in column CC of row r.
template <int CC, bool PRESSURE, int R>
__device__ __forceinline__ void vreg_row(const ProjPlanes& P, float (&v)[2][R], float (&vt)[2],
                                         int p, int y0, int r, bool in, const Consts& c,
                                         float d_t) {
  if (!in) return;
  const int e = (y0 + r) * kHalfW + p;
  const uint32_t f = (CC ? P.fo : P.fe)[e];
  if (!f) return;
  float* uL = (CC ? P.uo : P.ue) + e;
  float* uR = CC ? P.ue + e + 1 : P.uo + e;
  float a0 = *uL, a1 = *uR, pp = 0.0f;
  if (PRESSURE) pp = (CC ? P.po : P.pe)[e];
  float& top = (r + 1 < R) ? v[CC][r + 1] : vt[CC];
  project_faces<PRESSURE>(f, c, d_t, a0, a1, v[CC][r], top, pp);
  *uL = a0;
  *uR = a1;
  if (PRESSURE) (CC ? P.po : P.pe)[e] = pp;
}

// One colour half-sweep over the thread's strip. Rows go two at a time (the
// two active cells sit in different columns and share no face): both rows'
// loads first, then both updates, then both stores, with no branches, so the
// two dependency chains overlap (with the pressure on, each row on its own,
// vreg_row). A pair of rows wholly outside the cone or the region is skipped
// (a branch that is the same for the whole warp). An inactive cell stores
// its faces unchanged (no other cell of the colour touches them).
//
// Within a pair that is not skipped, a cell off the cone is updated like the
// others. That is harmless, since the cone shrinks by one cell per side each
// half-sweep: the faces of a cell off the cone belong to it and to its
// neighbours, which are off the cone from the next half-sweep on, so what it
// writes never reaches a cell in the cone or an owned face. Only the cell in
// column kRegionW - 1 (the odd column of the last thread) has a face in
// shared memory outside the region, u(kRegionW), and that face is never
// stored; the top face of row RH - 1 is a register that is never stored or
// passed to another strip. With the pressure on the cone is kept per cell.
//
// Bit r of `full` (the same in every lane of the warp) says that the active
// cell of row r has flag kFullFlag in every lane. When both rows of every
// pair the half-sweep needs are full, the warp takes project_faces_full
// without reading or testing flags.
template <int COLOUR, bool PRESSURE, int R>
__device__ __forceinline__ void vreg_half_sweep(const ProjPlanes& P, float (&v)[2][R],
                                                float (&vt)[2], int p, int y0, int RH, int halo,
                                                int reach, const Consts& c, float d_t,
                                                uint32_t full) {
  const int lo = max(0, halo - 1 - reach);      // first needed cell, both axes
  const int y_end = min(RH - 1, RH - halo + reach);
  const int x_end = kRegionW - halo + reach;    // at most 255: u(x + 1) stays in the row
  const int rlo = min(max(lo - y0, 0), R), rhi = min(max(y_end - y0, 0), R);
  const uint32_t rows = ((1u << rhi) - 1u) & ~((1u << rlo) - 1u);
  const bool col_ok[2] = {2 * p >= lo && 2 * p < x_end, 2 * p + 1 >= lo && 2 * p + 1 < x_end};
  constexpr int ca = COLOUR & 1, cb = ca ^ 1;   // active columns of even and odd rows
  // Row pairs with a row in the cone, and row pairs whose two rows are full
  // (bit r of each, r even); both masks are the same in every lane.
  const uint32_t pairs = (rows | (rows >> 1)) & 0x55555555u;
  const uint32_t pairs_full = full & (full >> 1) & 0x55555555u;
  if (!PRESSURE && (pairs & ~pairs_full) == 0u) {
    // Every pair the half-sweep needs is full: a loop of its own, so that
    // the warps on it run a short stretch of code.
    const bool edge = p == kHalfW - 1;
#pragma unroll
    for (int r = 0; r < R; r += 2) {
      if (((pairs >> r) & 1u) == 0u) continue;
      // Both rows lie below the region's top row (the flags say so), so
      // every load is inside the region.
      const int ea = (y0 + r) * kHalfW + p, eb = ea + kHalfW;
      float* uLa = (ca ? P.uo : P.ue) + ea;
      float* uRa = ca ? P.ue + ea + 1 : P.uo + ea;
      float* uLb = (cb ? P.uo : P.ue) + eb;
      float* uRb = cb ? P.ue + eb + 1 : P.uo + eb;
      float a0 = *uLa, a1 = *uRa;
      float b0 = *uLb, b1 = *uRb;
      float& top_b = (r + 2 < R) ? v[cb][r + 2] : vt[cb];
      project_faces_full(c, a0, a1, v[ca][r], v[ca][r + 1]);
      project_faces_full(c, b0, b1, v[cb][r + 1], top_b);
      *uLa = a0;
      if (!(ca && edge)) *uRa = a1;
      *uLb = b0;
      if (!(cb && edge)) *uRb = b1;
    }
  } else {
    const bool edge = p == kHalfW - 1;
#pragma unroll
    for (int r = 0; r < R; r += 2) {
      if (((rows >> r) & 3u) == 0u) continue;  // both rows off the cone: the same for the warp
      if constexpr (PRESSURE) {
        const uint32_t live =
            rows & ((col_ok[ca] ? 0x55555555u : 0u) | (col_ok[cb] ? 0xaaaaaaaau : 0u));
        vreg_row<ca, PRESSURE, R>(P, v, vt, p, y0, r, (live >> r) & 1u, c, d_t);
        vreg_row<cb, PRESSURE, R>(P, v, vt, p, y0, r + 1, (live >> (r + 1)) & 1u, c, d_t);
        continue;
      }
      const int ea = (y0 + r) * kHalfW + p, eb = ea + kHalfW;
      float* uLa = (ca ? P.uo : P.ue) + ea;
      float* uRa = ca ? P.ue + ea + 1 : P.uo + ea;
      float* uLb = (cb ? P.uo : P.ue) + eb;
      float* uRb = cb ? P.ue + eb + 1 : P.uo + eb;
      const uint32_t fa = (ca ? P.fo : P.fe)[ea];
      const uint32_t fb = (cb ? P.fo : P.fe)[eb];
      float a0 = *uLa, a1 = *uRa;
      float b0 = *uLb, b1 = *uRb;
      float& top_b = (r + 2 < R) ? v[cb][r + 2] : vt[cb];
      project_faces_sel(fa, c, a0, a1, v[ca][r], v[ca][r + 1]);
      project_faces_sel(fb, c, b0, b1, v[cb][r + 1], top_b);
      *uLa = a0;
      if (!(ca && edge)) *uRa = a1;
      *uLb = b0;
      if (!(cb && edge)) *uRb = b1;
    }
  }
  // Boundary faces this half-sweep may have changed, for the neighbouring strip.
  const int cT = (R - 1 + COLOUR) & 1;  // active column of the top row
  const int cB = COLOUR & 1;            // active column of the bottom row
  if (y0 + R < RH) (cT ? P.vo : P.ve)[(y0 + R) * kHalfW + p] = vt[cT];
  if (y0 > 0 && y0 < RH) (cB ? P.vo : P.ve)[y0 * kHalfW + p] = v[cB][0];
}

// After the barrier that ends a half-sweep: the neighbours' changed copies.
template <int COLOUR, int R>
__device__ __forceinline__ void vreg_receive(const ProjPlanes& P, float (&v)[2][R], float (&vt)[2],
                                             int p, int y0, int RH) {
  const int cT = (R - 1 + COLOUR) & 1;
  const int cB = COLOUR & 1;
  if (y0 + R < RH) vt[cB] = (cB ? P.vo : P.ve)[(y0 + R) * kHalfW + p];
  if (y0 > 0 && y0 < RH) v[cT][0] = (cT ? P.vo : P.ve)[y0 * kHalfW + p];
}

// `sweeps` red/black sweeps on the staged tile (RH <= R * blockDim.x / 128),
// whose planes start at the base of the dynamic shared memory; the v planes
// hold the result on return. Ends with a barrier. Not inlined: every storage
// type's kernels call the one copy (the constants come by value).
template <bool PRESSURE, int R>
__device__ __noinline__ void proj_sweeps_vreg(const Consts c, float d_t, int sweeps, int halo,
                                              int TY) {
  static_assert(R % 2 == 0, "strips must start on even rows");
  extern __shared__ __align__(16) float dyn_smem[];
  const int RH = TY + 2 * halo;
  const ProjPlanes P = proj_planes<PRESSURE>(dyn_smem, RH);
  // Strip s's four warps take the column blocks (w + s) mod 4, so that the
  // warps each scheduler partition holds (warp w of every strip) cover every
  // block: the rows that need the flag-driven path (walls, the obstacle,
  // cells off the grid) do not all fall to one partition.
  const int strip = threadIdx.x / kHalfW;
  const int p = ((((threadIdx.x >> 5) + strip) & (kHalfW / 32 - 1)) << 5) | (threadIdx.x & 31);
  const int y0 = strip * R;
  float v[2][R], vt[2];
#pragma unroll
  for (int r = 0; r < R; r++) {
    const int e = (y0 + r) * kHalfW + p;
    const bool in = y0 + r < RH;
    v[0][r] = in ? P.ve[e] : 0.0f;
    v[1][r] = in ? P.vo[e] : 0.0f;
  }
  const bool top_in = y0 + R < RH;
  vt[0] = top_in ? P.ve[(y0 + R) * kHalfW + p] : 0.0f;
  vt[1] = top_in ? P.vo[(y0 + R) * kHalfW + p] : 0.0f;
  // Per colour, the rows whose active cell has flag kFullFlag in every lane
  // of the warp (rows from the region's top row on never do; the warp's
  // lanes share y0). The flags do not change during the sweeps.
  uint32_t full[2] = {0u, 0u};
  if (!PRESSURE) {
#pragma unroll
    for (int colour = 0; colour < 2; colour++) {
      uint32_t m = 0u;
#pragma unroll
      for (int r = 0; r < R; r++) {
        const int y = y0 + r;
        const uint8_t* F = ((r + colour) & 1) ? P.fo : P.fe;
        if (y < RH - 1 && F[y * kHalfW + p] == kFullFlag) m |= 1u << r;
      }
      full[colour] = __reduce_and_sync(0xffffffffu, m);
    }
  }
  // Every thread has its copies before any boundary word is rewritten.
  __syncthreads();
  for (int t = 0; t < sweeps; t++) {
    const int reach = 2 * (sweeps - t) - 1;  // half-sweeps after the even one
    vreg_half_sweep<0, PRESSURE, R>(P, v, vt, p, y0, RH, halo, reach, c, d_t, full[0]);
    __syncthreads();
    vreg_receive<0, R>(P, v, vt, p, y0, RH);
    vreg_half_sweep<1, PRESSURE, R>(P, v, vt, p, y0, RH, halo, reach - 1, c, d_t, full[1]);
    __syncthreads();
    vreg_receive<1, R>(P, v, vt, p, y0, RH);
  }
#pragma unroll
  for (int r = 0; r < R; r++) {
    const int e = (y0 + r) * kHalfW + p;
    if (y0 + r < RH) {
      P.ve[e] = v[0][r];
      P.vo[e] = v[1][r];
    }
  }
  __syncthreads();
}

// The sweeps with registers where the region's rows fit the strips, else
// with every face in shared memory. `smem` is the dynamic shared memory base.
template <bool PRESSURE>
__device__ __forceinline__ void proj_sweeps_fast(float* smem, const Consts& c,
                                                 const StepParams* __restrict__ prm, int sweeps,
                                                 int halo, int TY) {
  const int RH = TY + 2 * halo;
  const int strips = blockDim.x / kHalfW;
  const float d_t = prm->dt;
  if (RH <= 8 * strips)
    proj_sweeps_vreg<PRESSURE, 8>(c, d_t, sweeps, halo, TY);
  else if (RH <= 10 * strips)
    proj_sweeps_vreg<PRESSURE, 10>(c, d_t, sweeps, halo, TY);
  else if (RH <= 12 * strips)
    proj_sweeps_vreg<PRESSURE, 12>(c, d_t, sweeps, halo, TY);
  else if (RH <= 14 * strips)
    proj_sweeps_vreg<PRESSURE, 14>(c, d_t, sweeps, halo, TY);
  else if (RH <= 16 * strips)
    proj_sweeps_vreg<PRESSURE, 16>(c, d_t, sweeps, halo, TY);
  else
    proj_sweeps<PRESSURE>(smem, c, prm, sweeps, halo, TY);
}

// apply_extrapolation_at (src/fluid.cu:720-733) on the owned cells of a
// staged region, in extrapolate_grid's order: the row rules for every owned
// column, then the column rules for every owned row. Each rule reads a cell of
// the tile that writes it as long as the last tile row and column hold at
// least two cells, which the caller checks; the grid's rules then need no
// other tile. Ends with a barrier.
template <bool PRESSURE>
__device__ __forceinline__ void extrapolate_region(float* smem, int RH, int gx0, int gy0,
                                                   int halo, int TX, int TY, int W, int H) {
  const ProjPlanes P = proj_planes<PRESSURE>(smem, RH);
  const int i0 = gx0 + halo, i1 = min(gx0 + halo + TX, W);  // owned global columns
  const int j0 = gy0 + halo, j1 = min(gy0 + halo + TY, H);  // owned global rows
  auto U = [&](int i, int j) -> float& {
    const int x = i - gx0;
    return ((x & 1) ? P.uo : P.ue)[(j - gy0) * kHalfW + (x >> 1)];
  };
  auto V = [&](int i, int j) -> float& {
    const int x = i - gx0;
    return ((x & 1) ? P.vo : P.ve)[(j - gy0) * kHalfW + (x >> 1)];
  };
  const bool bottom = j0 == 0, top = j1 == H;
  if (bottom || top) {
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      if (bottom) {
        U(i, 0) = U(i, 1);
        V(i, 1) = 0.0f;
      }
      if (top) U(i, H - 1) = U(i, H - 2);
    }
  }
  __syncthreads();
  const bool left = i0 == 0, right = i1 == W;
  if (left || right) {
    for (int j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
      if (left) {
        V(0, j) = V(1, j);
        U(1, j) = 0.0f;
      }
      if (right) V(W - 1, j) = V(W - 2, j);
    }
  }
  __syncthreads();
}

// Whether extrapolate_region can stand for the extrapolation kernel on this
// tile grid: the last tile row and column hold at least two cells each.
inline bool extrapolation_tile_local(int W, int H, int TX, int TY) {
  return W >= 3 && H >= 3 && TX >= 2 && TY >= 2 && (W - 1) % TX != 0 && (H - 1) % TY != 0;
}

// Owned cells back out; halo and TX are multiples of 4 when `vec` holds.
template <bool PRESSURE, class S>
__device__ __forceinline__ void proj_stage_out(float* smem, int tx, int ty, S* __restrict__ u_out,
                                               S* __restrict__ v_out, float* __restrict__ p,
                                               const Consts& c, int halo, int TX, int TY) {
  const int RH = TY + 2 * halo;
  const ProjPlanes P = proj_planes<PRESSURE>(smem, RH);
  const int gx0 = tx * TX - halo, gy0 = ty * TY - halo;
  const int W = c.W, H = c.H;
  const bool vec = ((W & 3) == 0) && ((gx0 & 3) == 0);
  for (int it = threadIdx.x; it < TY * kQuads; it += blockDim.x) {
    const int y = halo + it / kQuads, x = 4 * (it % kQuads);
    const int i = gx0 + x, j = gy0 + y;
    if (j >= H || i >= W) continue;
    const int s = y * kHalfW + (x >> 1);
    if (vec && x >= halo && x + 3 < halo + TX) {
      const float2 ue = *reinterpret_cast<const float2*>(P.ue + s);
      const float2 uo = *reinterpret_cast<const float2*>(P.uo + s);
      const float2 ve = *reinterpret_cast<const float2*>(P.ve + s);
      const float2 vo = *reinterpret_cast<const float2*>(P.vo + s);
      store_quad(u_out, W, H, i, j, true, make_float4(ue.x, uo.x, ue.y, uo.y));
      store_quad(v_out, W, H, i, j, true, make_float4(ve.x, vo.x, ve.y, vo.y));
      if (PRESSURE) {
        const float2 pe = *reinterpret_cast<const float2*>(P.pe + s);
        const float2 po = *reinterpret_cast<const float2*>(P.po + s);
        store_quad(p, W, H, i, j, true, make_float4(pe.x, po.x, pe.y, po.y));
      }
      continue;
    }
    for (int d = 0; d < 4; d++) {
      const int xd = x + d;
      if (xd < halo || xd >= halo + TX || i + d >= W) continue;
      const int64_t gk = cell_index(W, H, i + d, j);
      const int sd = y * kHalfW + (xd >> 1);
      st(u_out + gk, (xd & 1) ? P.uo[sd] : P.ue[sd]);
      st(v_out + gk, (xd & 1) ? P.vo[sd] : P.ve[sd]);
      if (PRESSURE) p[gk] = (xd & 1) ? P.po[sd] : P.pe[sd];
    }
  }
}

template <bool PRESSURE, class S>
__device__ __forceinline__ void project_tile(float* smem, int tx, int ty,
                                             const S* __restrict__ u_in,
                                             const S* __restrict__ v_in, S* __restrict__ u_out,
                                             S* __restrict__ v_out, float* __restrict__ p,
                                             const uint8_t* __restrict__ fl, const Consts& c,
                                             const StepParams* __restrict__ prm, int sweeps,
                                             int halo, int TX, int TY, int zero_pressure) {
  proj_stage_in<PRESSURE, S>(smem, tx, ty, u_in, v_in, p, fl, c, halo, TX, TY, zero_pressure);
  __syncthreads();
  proj_sweeps_fast<PRESSURE>(smem, c, prm, sweeps, halo, TY);
  proj_stage_out<PRESSURE, S>(smem, tx, ty, u_out, v_out, p, c, halo, TX, TY);
}

template <bool PRESSURE, class S>
__global__ void __launch_bounds__(kBlockThreads, 1)
k_project_blocked(const S* __restrict__ u_in, const S* __restrict__ v_in,
                  S* __restrict__ u_out, S* __restrict__ v_out, float* __restrict__ p,
                  const uint8_t* __restrict__ fl, Consts c, const StepParams* __restrict__ prm,
                  int sweeps, int halo, int TX, int TY, int tiles_x, int zero_pressure) {
  pdl_entry();
  extern __shared__ __align__(16) float smem[];
  project_tile<PRESSURE, S>(smem, blockIdx.x % tiles_x, blockIdx.x / tiles_x, u_in, v_in, u_out,
                            v_out, p, fl, c, prm, sweeps, halo, TX, TY, zero_pressure);
}

// ---------------------------------------------------------------------------
// Blocked Jacobi diffusion of u.
// ---------------------------------------------------------------------------
// The region of tile (tx, ty) into both buffers A and B (cells that no sweep
// updates keep their value in each).
template <class S, bool CG = false>
__device__ __forceinline__ void diff_stage_in(float* A, float* B, int tx, int ty,
                                              const S* __restrict__ u_in, const Consts& c,
                                              int halo, int TX, int TY) {
  const int RH = TY + 2 * halo;
  const int gx0 = tx * TX - halo, gy0 = ty * TY - halo;
  const int W = c.W, H = c.H;
  const bool vec = ((W & 3) == 0) && ((gx0 & 3) == 0);
  const int items = RH * kQuads;
  for (int base = threadIdx.x; base < items; base += blockDim.x * kInFlight) {
    float4 uq[kInFlight];
#pragma unroll
    for (int r = 0; r < kInFlight; r++) {
      const int it = base + r * blockDim.x;
      const int y = it / kQuads, x = 4 * (it % kQuads);
      const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
      if (CG)
        uq[r] = it < items ? load_quad_cg(u_in, W, H, gx0 + x, gy0 + y, vec) : z;
      else
        uq[r] = it < items ? load_quad(u_in, W, H, gx0 + x, gy0 + y, vec) : z;
    }
#pragma unroll
    for (int r = 0; r < kInFlight; r++) {
      const int it = base + r * blockDim.x;
      if (it >= items) break;
      *reinterpret_cast<float4*>(A + 4 * it) = uq[r];
      *reinterpret_cast<float4*>(B + 4 * it) = uq[r];
    }
  }
}

// One column's run of Jacobi updates, rows e0, e0 + rs, ... (n of them), from
// A into B. The buffers never overlap, so the loads of later rows may be
// issued ahead of earlier rows' stores.
__device__ __forceinline__ void diff_column(const float* __restrict__ A, float* __restrict__ B,
                                            int e0, int rs, int n, float a, float den) {
  float down = A[e0 - rs];
  float centre = A[e0];
  int e = e0;
#pragma unroll 4
  for (int t = 0; t < n; t++, e += rs) {
    const float up = A[e + rs];
    // src/fluid.cu:178-182: neighbours (i-1, j), (i+1, j), (i, j-1), (i, j+1)
    B[e] = fma_rn(a, A[e - 1] + A[e + 1] + down + up, centre) / den;
    down = centre;
    centre = up;
  }
}

// `sweeps` Jacobi sweeps on the staged region, A -> B -> A ...; on return A
// holds the result (the pointers are swapped as the sweeps go). Ends with a
// barrier. With FLIP the region's rows are stored top row first (the order
// of the global layout, as a tensor copy delivers them): region row y sits at
// row RH - 1 - y.
template <bool FLIP = false>
__device__ __forceinline__ void diff_sweeps(float*& A, float*& B, int tx, int ty, const Consts& c,
                                            const StepParams* __restrict__ prm, int sweeps,
                                            int halo, int TX, int TY) {
  const int RH = TY + 2 * halo;
  const int gx0 = tx * TX - halo, gy0 = ty * TY - halo;
  const int W = c.W, H = c.H;
  const float d_t = prm->dt;
  const float a = c.viscosity * d_t / (float)(c.h * c.h);
  // Updated cells: domain interior and not on the region's outer ring. A
  // thread owns one column and a contiguous run of rows, carrying the column
  // neighbours (j-1, j, j+1) in registers.
  const int x = threadIdx.x % kRegionW;
  const int groups = blockDim.x / kRegionW;
  const int i = gx0 + x;
  const int y_lo = max(1, 1 - gy0), y_hi = min(RH - 2, H - 2 - gy0);
  const int chunk = (y_hi - y_lo + groups) / groups;
  const int r0 = y_lo + (threadIdx.x / kRegionW) * chunk;
  const int r1 = min(y_hi + 1, r0 + chunk);
  const bool column = x > 0 && x < kRegionW - 1 && i > 0 && i < W - 1 && r0 < r1;
  const float den = fma_rn(4.0f, a, 1.0f);
  for (int t = 0; t < sweeps; t++) {
    // Only cells within `reach` (sweeps still to come) of the owned tile can
    // still influence it.
    const int reach = sweeps - 1 - t;
    const int ya = max(r0, halo - reach), yb = min(r1, RH - halo + reach);
    if (column && x >= halo - reach && x < kRegionW - halo + reach && ya < yb) {
      const int rs = FLIP ? -kRegionW : kRegionW;     // step to the next region row
      const int base = FLIP ? (RH - 1) * kRegionW : 0;
      diff_column(A, B, base + ya * rs + x, rs, yb - ya, a, den);
    }
    __syncthreads();
    float* T = A;
    A = B;
    B = T;
  }
}

// Owned cells of the region in A back to global (FLIP as in diff_sweeps).
template <class S, bool FLIP = false>
__device__ __forceinline__ void diff_store_owned(const float* A, int tx, int ty,
                                                 S* __restrict__ u_out, const Consts& c, int halo,
                                                 int TX, int TY) {
  const int gx0 = tx * TX - halo, gy0 = ty * TY - halo;
  const int W = c.W, H = c.H;
  const int RH = TY + 2 * halo;
  const bool vec = ((W & 3) == 0) && ((gx0 & 3) == 0);
  for (int it = threadIdx.x; it < TY * kQuads; it += blockDim.x) {
    const int y = halo + it / kQuads, x = 4 * (it % kQuads);
    const int i = gx0 + x, j = gy0 + y;
    if (j >= H || i >= W) continue;
    const float* src = A + (FLIP ? RH - 1 - y : y) * kRegionW + x;
    if (vec && x >= halo && x + 3 < halo + TX) {
      store_quad(u_out, W, H, i, j, true, *reinterpret_cast<const float4*>(src));
      continue;
    }
    for (int d = 0; d < 4; d++) {
      if (x + d < halo || x + d >= halo + TX || i + d >= W) continue;
      st(u_out + cell_index(W, H, i + d, j), src[d]);
    }
  }
}

// ---------------------------------------------------------------------------
// The same pass with each buffer split by column parity: E[y * kHalfW + k] =
// u(2k, y) and O[y * kHalfW + k] = u(2k + 1, y), the odd plane right after the
// even one. A thread owns the column pair (2k, 2k + 1) over a run of rows and
// carries both columns' rows below and above in registers, so a row of the
// pair costs the two loads above, the left neighbour of the even column and
// the right neighbour of the odd one (each the other plane's word at k - 1 or
// k + 1: lanes take consecutive words) and the two stores: three
// shared-memory accesses per cell update instead of four.
// ---------------------------------------------------------------------------
// Quads each thread loads before it stores any: with 8, a whole 256 x 74
// region is in flight at once (one round trip to L2 instead of two).
constexpr int kDiffInFlight = 8;

template <class S>
__device__ __forceinline__ void diff_stage_in_pairs(float* A, float* B, int tx, int ty,
                                                    const S* __restrict__ u_in, const Consts& c,
                                                    int halo, int TX, int TY) {
  const int RH = TY + 2 * halo;
  const int gx0 = tx * TX - halo, gy0 = ty * TY - halo;
  const int W = c.W, H = c.H;
  const bool vec = ((W & 3) == 0) && ((gx0 & 3) == 0);
  const int items = RH * kQuads;
  float* AO = A + RH * kHalfW;
  float* BO = B + RH * kHalfW;
  for (int base = threadIdx.x; base < items; base += blockDim.x * kDiffInFlight) {
    float4 uq[kDiffInFlight];
#pragma unroll
    for (int r = 0; r < kDiffInFlight; r++) {
      const int it = base + r * blockDim.x;
      const int y = it / kQuads, x = 4 * (it % kQuads);
      uq[r] = it < items ? load_quad(u_in, W, H, gx0 + x, gy0 + y, vec)
                         : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int r = 0; r < kDiffInFlight; r++) {
      const int it = base + r * blockDim.x;
      if (it >= items) break;
      const int e = (it / kQuads) * kHalfW + 2 * (it % kQuads);
      const float2 ev = make_float2(uq[r].x, uq[r].z), od = make_float2(uq[r].y, uq[r].w);
      *reinterpret_cast<float2*>(A + e) = ev;
      *reinterpret_cast<float2*>(AO + e) = od;
      *reinterpret_cast<float2*>(B + e) = ev;
      *reinterpret_cast<float2*>(BO + e) = od;
    }
  }
}

// The Jacobi update's division by den = 1 + 4a, as the fast-math division
// gives it (RCP false), or as the product with the reciprocal __fdividef(1,
// den) taken once per sweep (RCP true), which gives the same bits for every
// float input: tests/cpp/reciprocal_product.cu compares the two over all 2^32
// inputs for the divisors of the tested configurations and a spread of others
// in [1, 1e6]. The product is used for den below 2^20.
template <bool RCP>
__device__ __forceinline__ float jacobi_divide(float x, float den, float rden) {
  return RCP ? mul_rn(x, rden) : x / den;
}

// One run of Jacobi updates of a column pair, rows e0, e0 + kHalfW, ... (n of
// them, word offsets in a plane), from A into B; do0 / do1 say which of the
// two columns the sweep updates (each column's left or right neighbour is
// read only when that column is updated, so no read leaves the region).
template <bool RCP>
__device__ __forceinline__ void diff_pair_run(const float* __restrict__ AE,
                                              const float* __restrict__ AO,
                                              float* __restrict__ BE, float* __restrict__ BO,
                                              int e0, int n, bool do0, bool do1, float a,
                                              float den, float rden) {
  float down0 = AE[e0 - kHalfW], down1 = AO[e0 - kHalfW];
  float c0 = AE[e0], c1 = AO[e0];
  int e = e0;
#pragma unroll 4
  for (int t = 0; t < n; t++, e += kHalfW) {
    const float up0 = AE[e + kHalfW], up1 = AO[e + kHalfW];
    const float left = do0 ? AO[e - 1] : 0.0f;   // u(2k - 1)
    const float right = do1 ? AE[e + 1] : 0.0f;  // u(2k + 2)
    // src/fluid.cu:178-182: neighbours (i-1, j), (i+1, j), (i, j-1), (i, j+1)
    if (do0) BE[e] = jacobi_divide<RCP>(fma_rn(a, left + c1 + down0 + up0, c0), den, rden);
    if (do1) BO[e] = jacobi_divide<RCP>(fma_rn(a, c0 + right + down1 + up1, c1), den, rden);
    down0 = c0;
    c0 = up0;
    down1 = c1;
    c1 = up1;
  }
}

// `sweeps` Jacobi sweeps on the split region, A -> B -> A ...; on return A
// holds the result. Ends with a barrier.
__device__ __forceinline__ void diff_sweeps_pairs(float*& A, float*& B, int tx, int ty,
                                                  const Consts& c,
                                                  const StepParams* __restrict__ prm, int sweeps,
                                                  int halo, int TX, int TY) {
  const int RH = TY + 2 * halo;
  const int gx0 = tx * TX - halo, gy0 = ty * TY - halo;
  const int W = c.W, H = c.H;
  const float d_t = prm->dt;
  const float a = c.viscosity * d_t / (float)(c.h * c.h);
  const int k = threadIdx.x % kHalfW;
  const int groups = blockDim.x / kHalfW;
  const int x0 = 2 * k, x1 = 2 * k + 1;
  const int i0 = gx0 + x0, i1 = gx0 + x1;
  const int y_lo = max(1, 1 - gy0), y_hi = min(RH - 2, H - 2 - gy0);
  const int chunk = (y_hi - y_lo + groups) / groups;
  const int r0 = y_lo + (threadIdx.x / kHalfW) * chunk;
  const int r1 = min(y_hi + 1, r0 + chunk);
  // Domain interior and not on the region's outer ring.
  const bool col0 = x0 > 0 && i0 > 0 && i0 < W - 1;
  const bool col1 = x1 < kRegionW - 1 && i1 > 0 && i1 < W - 1;
  const float den = fma_rn(4.0f, a, 1.0f);
  const float rden = __fdividef(1.0f, den);
  const bool use_rcp = den < 1048576.0f;
  for (int t = 0; t < sweeps; t++) {
    // Only cells within `reach` (sweeps still to come) of the owned tile can
    // still influence it.
    const int reach = sweeps - 1 - t;
    const int ya = max(r0, halo - reach), yb = min(r1, RH - halo + reach);
    const bool do0 = col0 && x0 >= halo - reach && x0 < kRegionW - halo + reach;
    const bool do1 = col1 && x1 >= halo - reach && x1 < kRegionW - halo + reach;
    if ((do0 || do1) && ya < yb) {
      if (use_rcp)
        diff_pair_run<true>(A, A + RH * kHalfW, B, B + RH * kHalfW, ya * kHalfW + k, yb - ya,
                            do0, do1, a, den, rden);
      else
        diff_pair_run<false>(A, A + RH * kHalfW, B, B + RH * kHalfW, ya * kHalfW + k, yb - ya,
                             do0, do1, a, den, rden);
    }
    __syncthreads();
    float* T = A;
    A = B;
    B = T;
  }
}

// Owned cells of the split region in A back to global.
template <class S>
__device__ __forceinline__ void diff_store_owned_pairs(const float* A, int tx, int ty,
                                                       S* __restrict__ u_out, const Consts& c,
                                                       int halo, int TX, int TY) {
  const int gx0 = tx * TX - halo, gy0 = ty * TY - halo;
  const int W = c.W, H = c.H;
  const int RH = TY + 2 * halo;
  const float* AO = A + RH * kHalfW;
  const bool vec = ((W & 3) == 0) && ((gx0 & 3) == 0);
  for (int it = threadIdx.x; it < TY * kQuads; it += blockDim.x) {
    const int y = halo + it / kQuads, x = 4 * (it % kQuads);
    const int i = gx0 + x, j = gy0 + y;
    if (j >= H || i >= W) continue;
    const int e = y * kHalfW + (x >> 1);
    const float2 ev = *reinterpret_cast<const float2*>(A + e);
    const float2 od = *reinterpret_cast<const float2*>(AO + e);
    const float q[4] = {ev.x, od.x, ev.y, od.y};
    if (vec && x >= halo && x + 3 < halo + TX) {
      store_quad(u_out, W, H, i, j, true, make_float4(q[0], q[1], q[2], q[3]));
      continue;
    }
    for (int d = 0; d < 4; d++) {
      if (x + d < halo || x + d >= halo + TX || i + d >= W) continue;
      st(u_out + cell_index(W, H, i + d, j), q[d]);
    }
  }
}

template <class S>
__device__ __forceinline__ void diffuse_tile(float* smem, int tx, int ty,
                                             const S* __restrict__ u_in, S* __restrict__ u_out,
                                             const Consts& c, const StepParams* __restrict__ prm,
                                             int sweeps, int halo, int TX, int TY) {
  const int RH = TY + 2 * halo;
  float* A = smem;
  float* B = smem + RH * kRegionW + kArrPad;
  diff_stage_in_pairs<S>(A, B, tx, ty, u_in, c, halo, TX, TY);
  __syncthreads();
  diff_sweeps_pairs(A, B, tx, ty, c, prm, sweeps, halo, TX, TY);
  diff_store_owned_pairs<S>(A, tx, ty, u_out, c, halo, TX, TY);
}

template <class S>
__global__ void __launch_bounds__(kBlockThreads, 1)
k_diffuse_blocked(const S* __restrict__ u_in, S* __restrict__ u_out, Consts c,
                  const StepParams* __restrict__ prm, int sweeps, int halo, int TX, int TY,
                  int tiles_x) {
  pdl_entry();
  extern __shared__ __align__(16) float smem[];
  diffuse_tile<S>(smem, blockIdx.x % tiles_x, blockIdx.x / tiles_x, u_in, u_out, c, prm, sweeps,
                  halo, TX, TY);
}

// ---------------------------------------------------------------------------
// Tensor-memory-accelerator staging of the diffusion region (FP32 fields).
// One thread issues a single 2-D bulk tensor copy of the whole 256 x RH region
// into A, completing on an mbarrier the block waits on; cells off the grid
// arrive as zero, as the vector loads stage them. The copy delivers rows in
// the global (top row first) order, so the sweeps and the write-back run with
// FLIP. Every wait is bounded: a block whose copy does not complete records
// the failure in the error words and returns.
// ---------------------------------------------------------------------------
constexpr int kTmaSpin = 1 << 22;
constexpr int kTmaAlign = 128;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// The box at (x, row) of `map` into dst; x * 4 bytes must be a multiple of 16.
__device__ __forceinline__ void tma_load_2d(float* dst, const CUtensorMap* map, int x, int row,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(row), "r"(smem_u32(bar))
      : "memory");
}

__global__ void __launch_bounds__(kBlockThreads, 1)
k_diffuse_blocked_tma(const __grid_constant__ CUtensorMap in_map, float* __restrict__ u_out,
                      Consts c, const StepParams* __restrict__ prm, int sweeps, int halo, int TX,
                      int TY, int tiles_x, int* __restrict__ err, int* __restrict__ host_err) {
  pdl_entry();
  extern __shared__ __align__(16) float smem_tma[];
  __shared__ __align__(8) uint64_t bar;
  const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
  const int RH = TY + 2 * halo;
  // Both buffers are copy destinations, 128-byte aligned (the launch adds
  // room for the alignment and a 128-byte gap between them).
  float* A = reinterpret_cast<float*>(
      (reinterpret_cast<uintptr_t>(smem_tma) + kTmaAlign - 1) & ~uintptr_t(kTmaAlign - 1));
  float* B = A + RH * kRegionW + kTmaAlign / sizeof(float);
  const int gx0 = tx * TX - halo, gy0 = ty * TY - halo;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    // The region into both buffers (cells no sweep updates keep their value
    // in each), one copy per buffer on the same barrier.
    mbar_expect_tx(&bar, (uint32_t)(2 * RH * kRegionW * sizeof(float)));
    tma_load_2d(A, &in_map, gx0, c.H - gy0 - RH, &bar);
    tma_load_2d(B, &in_map, gx0, c.H - gy0 - RH, &bar);
  }
  bool done = false;
  for (int it = 0; it < kTmaSpin && !done; it++) done = mbar_try_wait(&bar, 0);
  if (__syncthreads_or(!done)) {
    if (threadIdx.x == 0) {
      if (err && atomicCAS(err, 0, 1) == 0 && host_err) {
        *(volatile int*)host_err = 1;
        __threadfence_system();
      }
      // The copy may still land: give it the same bound again before the
      // block's shared memory is released.
      for (int it = 0; it < kTmaSpin && !mbar_try_wait(&bar, 0); it++) {
      }
    }
    __syncthreads();
    return;
  }
  diff_sweeps<true>(A, B, tx, ty, c, prm, sweeps, halo, TX, TY);
  diff_store_owned<float, true>(A, tx, ty, u_out, c, halo, TX, TY);
}

// ---------------------------------------------------------------------------
// Host: tile geometry and pass enqueue.
// ---------------------------------------------------------------------------

// Launch with programmatic stream serialisation when `pdl` (the kernels call
// pdl_entry() first, so the dependency on the previous kernel is kept).
template <class... KArgs, class... Args>
inline void launch_pdl(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                       cudaStream_t st, Args&&... args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

constexpr size_t kMaxSmem = 227 * 1024;
constexpr size_t kStaticSmem = 256;

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
  // kStaticSmem: room for the kernels' own static shared memory.
  while (TY > 2 && smem_of(TY) + kStaticSmem > kMaxSmem) TY -= 2;
  g.TY = TY;
  g.RH = TY + 2 * halo;
  g.tiles_y = (H + TY - 1) / TY;
  g.smem = smem_of(TY);
  return g;
}

// Sweeps per blocked pass as configured: -1 plain, K > 0 fixed, 0 = to be
// chosen by the autotuner once the handle exists.
inline int choose_block_k(const os_handle* h) {
  if (h->cfg.projection_block < 0) return -1;
  if (h->cfg.projection_block > 0) return std::min(h->cfg.projection_block, 32);
  return 0;
}

// Jacobi sweeps per blocked diffusion pass.
inline int diffusion_depth(const os_handle* h) { return h->diff_k > 0 ? h->diff_k : h->block_k; }

// FP32 arithmetic on FP32, FP16 or BF16 storage. With reduced storage a value
// is rounded to storage once per pass (the region stays FP32 in shared
// memory), not once per sweep as in the plain kernels.
template <class S, class A>
inline bool blocked_supported(const os_handle*) {
  return std::is_same<A, float>::value &&
         (std::is_same<S, float>::value || std::is_same<S, __half>::value ||
          std::is_same<S, __nv_bfloat16>::value);
}

inline int sm_count(int device) {
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || n < 1)
    n = 152;
  return n;
}

// Projection: ceil(n / K) passes of up to K sweeps; each pass reads one copy of
// (u, v) and writes the other. `cur_u`/`cur_v` track which copy holds the
// live field (0: u/v, 1: ub/vb) and are updated for the caller.
// `zero_first`: the first pass also performs zero_pressure (inside a step).
template <class S>
inline int enqueue_blocked_projection(os_handle* h, cudaStream_t st, int* cur_u, int* cur_v,
                                      bool zero_first) {
  const int K = h->block_k;
  const bool pressure = h->cfg.enable_pressure != 0;
  const TileGeom g = make_geom(h->W, h->H, 2 * K, true, pressure, sm_count(h->cfg.device));
  S* U[2] = {static_cast<S*>(h->u), static_cast<S*>(h->ub)};
  S* V[2] = {static_cast<S*>(h->v), static_cast<S*>(h->vb)};
  const int tiles = g.tiles_x * g.tiles_y;
  int launches = 0;
  for (int done = 0, pass = 0; done < h->c.n; pass++) {
    const int sweeps = std::min(K, h->c.n - done);
    const S* uin = U[*cur_u];
    const S* vin = V[*cur_v];
    S* uout = U[1 - *cur_u];
    S* vout = V[1 - *cur_v];
    if (pressure) {
      cudaFuncSetAttribute(k_project_blocked<true, S>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem);
      launch_pdl(h->pdl, k_project_blocked<true, S>, tiles, kBlockThreads, g.smem, st,
                 uin, vin, uout, vout, h->p, (const uint8_t*)h->flags, h->c,
                 (const StepParams*)h->d_params, sweeps, g.halo, g.TX, g.TY, g.tiles_x,
                 (zero_first && pass == 0) ? 1 : 0);
    } else {
      cudaFuncSetAttribute(k_project_blocked<false, S>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem);
      launch_pdl(h->pdl, k_project_blocked<false, S>, tiles, kBlockThreads, g.smem, st,
                 uin, vin, uout, vout, h->p, (const uint8_t*)h->flags, h->c,
                 (const StepParams*)h->d_params, sweeps, g.halo, g.TX, g.TY, g.tiles_x, 0);
    }
    launches++;
    *cur_u = 1 - *cur_u;
    *cur_v = 1 - *cur_v;
    done += sweeps;
  }
  return launches;
}

// Dynamic shared memory of k_diffuse_blocked_tma: two 128-byte aligned
// buffers of RH x 256 floats and the alignment slack.
inline size_t tma_diffusion_smem(int RH) {
  return 2 * (size_t)RH * kRegionW * sizeof(float) + 2 * kTmaAlign;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

inline EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// Tensor maps of u and ub (FP32) with a box of one diffusion region, when the
// copy's rules hold: row pitch and region origin multiples of 16 bytes (W and
// the halo K multiples of 4), the box at most 256 rows.
inline bool prepare_tma_diffusion(os_handle* h) {
  const int K = diffusion_depth(h);
  if (h->storage != OS_STORAGE_F32 || K <= 0 || (K & 3) || (h->W & 3)) return false;
  const TileGeom g = make_geom(h->W, h->H, K, false, false, sm_count(h->cfg.device));
  if (g.RH > 256 || (g.TX & 3) || (g.halo & 3)) return false;
  if (tma_diffusion_smem(g.RH) + kStaticSmem > kMaxSmem || K > 8) return false;
  const EncodeTiledFn enc = encode_tiled();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)h->W, (cuuint64_t)h->H};
  const cuuint64_t strides[1] = {(cuuint64_t)h->W * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)kRegionW, (cuuint32_t)g.RH};
  const cuuint32_t elem[2] = {1, 1};
  for (int k = 0; k < 2; k++) {
    if (enc(&h->diff_maps[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, k ? h->ub : h->u, dims,
            strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  return true;
}

template <class S>
inline int enqueue_blocked_diffusion(os_handle* h, cudaStream_t st, int* cur_u) {
  const int K = diffusion_depth(h);
  const TileGeom g = make_geom(h->W, h->H, K, false, false, sm_count(h->cfg.device));
  S* U[2] = {static_cast<S*>(h->u), static_cast<S*>(h->ub)};
  const int tiles = g.tiles_x * g.tiles_y;
  if constexpr (std::is_same<S, float>::value) {
    if (h->tma_diffusion) {
      const size_t smem = tma_diffusion_smem(g.RH);
      cudaFuncSetAttribute(k_diffuse_blocked_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem);
      int launches = 0;
      for (int done = 0; done < h->c.n;) {
        const int sweeps = std::min(K, h->c.n - done);
        launch_pdl(h->pdl, k_diffuse_blocked_tma, tiles, kBlockThreads, smem, st,
                   h->diff_maps[*cur_u], U[1 - *cur_u], h->c, (const StepParams*)h->d_params,
                   sweeps, g.halo, g.TX, g.TY, g.tiles_x, h->rerr, h->d_host_rerr);
        launches++;
        *cur_u = 1 - *cur_u;
        done += sweeps;
      }
      return launches;
    }
  }
  cudaFuncSetAttribute(k_diffuse_blocked<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)g.smem);
  int launches = 0;
  for (int done = 0; done < h->c.n;) {
    const int sweeps = std::min(K, h->c.n - done);
    launch_pdl(h->pdl, k_diffuse_blocked<S>, tiles, kBlockThreads, g.smem, st,
               (const S*)U[*cur_u], U[1 - *cur_u], h->c, (const StepParams*)h->d_params, sweeps,
               g.halo, g.TX, g.TY, g.tiles_x);
    launches++;
    *cur_u = 1 - *cur_u;
    done += sweeps;
  }
  return launches;
}

}  // namespace osg
