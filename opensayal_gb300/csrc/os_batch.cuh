// os_batch.cuh — many independent wind tunnels of different sizes advanced
// together: one CUDA graph per step, one persistent kernel per phase.
//
// Each scenario keeps its own fields (an os_handle each, the reference's
// layout). A scenario occupies a slot; the device plan describes the current
// members:
//   * a descriptor per slot (constants, storage type, field pointers);
//   * the members in order with their cumulative cell counts, for the
//     per-cell phases: each block takes an equal, contiguous range of cells
//     and searches for its first member once;
//   * the tiles of all members sorted by diffusion and by projection passes
//     (descending), one (slot, tx, ty) entry per tile, so that pass p of a
//     phase covers a prefix of its list — the tiles of members with more than
//     p passes — of length items[p];
//   * a remaining-steps count per slot (0: frozen, negative: unlimited),
//     decremented by the last kernel of every step, so that scenarios with
//     different step counts stop exactly on time inside shared steps.
// The plan is O(members + tiles of one pass), so membership changes cost one
// stream-ordered copy; the graph itself does not change. The per-tile and
// per-cell code is the single-grid code for the scenario's storage type, so a
// scenario advances bit for bit as it would alone.
//
// Buffer parity per scenario: diffusion pass p reads copy (p & 1) of u; with D
// diffusion passes, projection pass p reads u copy ((D + p) & 1) and v copy
// (p & 1). Velocity advection then writes the other copies, and the smoke
// kernel copies the live velocity back to the public arrays where needed, so
// between steps every member's state is in its public arrays.
#pragma once

namespace osg {

constexpr int kBatchMaxPasses = 128;  // blocked passes per phase (n <= 128 * K)

struct ScenarioDesc {
  Consts c;
  int storage;       // OS_STORAGE_F32, OS_STORAGE_F16 or OS_STORAGE_BF16
  int smoke_period;
  int smoke_on;      // enable_smoke && wind_tunnel.smoke != 0
  int diff_passes;   // blocked diffusion passes per step (0 when viscosity == 0)
  int proj_passes;   // blocked projection passes per step
  int diff_tiles_x;  // tile columns under the diffusion geometry
  int proj_tiles_x;  // tile columns under the projection geometry
  const StepParams* prm;
  void *u, *v, *ub, *vb, *s, *sb;
  const uint8_t* flags;
  const uint16_t* nbr;  // fluid neighbourhoods (samplers)
};

struct TileRef {
  int slot;
  int16_t tx, ty;
};

// Head of the device plan; the arrays follow at the given byte offsets.
struct PlanHeader {
  int members;
  int admits;     // (slot, steps) pairs in the admit list
  int64_t cells;  // cells over all members
  int off_desc;                       // ScenarioDesc[slots]
  int off_slot;                       // int[members]
  int off_cell_cum;                   // int64_t[members]: cells before member k
  int off_diff_tiles, off_proj_tiles; // TileRef[tiles of pass 0]
  int off_admit;                      // int2[admits]
  int diff_items[kBatchMaxPasses];    // tiles in diffusion pass p
  int proj_items[kBatchMaxPasses];    // tiles in projection pass p
};

template <class T>
__device__ __forceinline__ const T* plan_array(const PlanHeader* P, int off) {
  return reinterpret_cast<const T*>(reinterpret_cast<const char*>(P) + off);
}

// Member whose cell range [cum[k], cum[k+1]) holds cell `it` (cum[0] = 0).
__device__ __forceinline__ int member_of(const int64_t* __restrict__ cum, int n, int64_t it) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (cum[mid] <= it) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Runs fn with a typed null pointer naming the scenario's storage type.
template <class Fn>
__device__ __forceinline__ void with_storage(int storage, Fn&& fn) {
  switch (storage) {
    case OS_STORAGE_F16: fn(static_cast<__half*>(nullptr)); break;
    case OS_STORAGE_BF16: fn(static_cast<__nv_bfloat16*>(nullptr)); break;
    default: fn(static_cast<float*>(nullptr)); break;
  }
}

__device__ __forceinline__ void stage_desc(const ScenarioDesc* src, ScenarioDesc* dst) {
  static_assert(sizeof(ScenarioDesc) % 4 == 0, "descriptor is copied in words");
  constexpr int kWords = sizeof(ScenarioDesc) / 4;
  if (threadIdx.x < kWords)
    reinterpret_cast<uint32_t*>(dst)[threadIdx.x] = reinterpret_cast<const uint32_t*>(src)[threadIdx.x];
}

template <class S>
__device__ __forceinline__ S* copy_of(void* a, void* b, int which) {
  return static_cast<S*>(which ? b : a);
}

// The cells of all members, split into equal contiguous ranges, one per
// block; the member is searched once per block and the range walked row
// segment by row segment. fn(desc, j, i0, i1) handles cells i0..i1-1 of row j
// of a live member.
template <class Fn>
__device__ __forceinline__ void for_cells(const PlanHeader* __restrict__ P,
                                          const int* __restrict__ remaining, Fn&& fn) {
  const int64_t total = P->cells;
  const int64_t per = (total + gridDim.x - 1) / gridDim.x;
  int64_t c = (int64_t)blockIdx.x * per;
  const int64_t end = min(total, c + per);
  if (c >= end) return;
  const int* slot_of = plan_array<int>(P, P->off_slot);
  const int64_t* cum = plan_array<int64_t>(P, P->off_cell_cum);
  const ScenarioDesc* T = plan_array<ScenarioDesc>(P, P->off_desc);
  int k = member_of(cum, P->members, c);
  int64_t base = cum[k];
  while (c < end) {
    const int slot = slot_of[k];
    const ScenarioDesc& d = T[slot];
    const int W = d.c.W;
    const int64_t off = c - base;
    const int j = (int)(off / W);
    const int i0 = (int)(off - (int64_t)j * W);
    const int i1 = (int)min((int64_t)W, (int64_t)i0 + (end - c));
    if (remaining[slot] != 0) fn(d, j, i0, i1);
    c += i1 - i0;
    if (c - base == (int64_t)W * d.c.H) {
      base = c;
      k++;
    }
  }
}

__global__ void k_batch_forces(const PlanHeader* __restrict__ P, const int* __restrict__ remaining) {
  for_cells(P, remaining, [&](const ScenarioDesc& d, int j, int i0, int i1) {
    with_storage(d.storage, [&](auto tag) {
      using S = std::remove_pointer_t<decltype(tag)>;
      S* v = static_cast<S*>(d.v);
      for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const int64_t k = cell_index(d.c.W, d.c.H, i, j);
        st(v + k, forces_cell<S, float>(static_cast<S*>(d.u), static_cast<S*>(d.s),
                                        ld<float>(v + k), d.c, d.smoke_period, d.prm, i, j));
      }
    });
  });
}

__global__ void __launch_bounds__(kBlockThreads, 1)
k_batch_diffuse(const PlanHeader* __restrict__ P, const int* __restrict__ remaining, int pass,
                int K, int halo, int TX, int TY) {
  extern __shared__ __align__(16) float smem[];
  const int n_items = P->diff_items[pass];
  const TileRef* tiles = plan_array<TileRef>(P, P->off_diff_tiles);
  const ScenarioDesc* T = plan_array<ScenarioDesc>(P, P->off_desc);
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const TileRef t = tiles[it];
    const int slot = t.slot;
    if (remaining[slot] == 0) continue;  // uniform over the block
    const ScenarioDesc& d = T[slot];
    const int tx = t.tx, ty = t.ty;
    const int sweeps = min(K, d.c.n - pass * K);
    const int in = pass & 1;
    with_storage(d.storage, [&](auto tag) {
      using S = std::remove_pointer_t<decltype(tag)>;
      diffuse_tile<S>(smem, tx, ty, copy_of<S>(d.u, d.ub, in), copy_of<S>(d.u, d.ub, 1 - in),
                      d.c, d.prm, sweeps, halo, TX, TY);
    });
    __syncthreads();  // the next item restages shared memory
  }
}

__global__ void __launch_bounds__(kBlockThreads, 1)
k_batch_project(const PlanHeader* __restrict__ P, const int* __restrict__ remaining, int pass,
                int K, int halo, int TX, int TY) {
  extern __shared__ __align__(16) float smem[];
  const int n_items = P->proj_items[pass];
  const TileRef* tiles = plan_array<TileRef>(P, P->off_proj_tiles);
  const ScenarioDesc* T = plan_array<ScenarioDesc>(P, P->off_desc);
  // The descriptor is staged in shared memory: its constants are then read
  // from there inside the sweeps instead of being held in registers.
  __shared__ ScenarioDesc sd;
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const TileRef t = tiles[it];
    const int slot = t.slot;
    if (remaining[slot] == 0) continue;
    stage_desc(T + slot, &sd);
    __syncthreads();
    const ScenarioDesc& d = sd;
    const int tx = t.tx, ty = t.ty;
    const int sweeps = min(K, d.c.n - pass * K);
    const int iu = (d.diff_passes + pass) & 1, iv = pass & 1;
    // project_tile in three parts, so that the sweeps are instantiated once.
    with_storage(d.storage, [&](auto tag) {
      using S = std::remove_pointer_t<decltype(tag)>;
      proj_stage_in<false, S>(smem, tx, ty, copy_of<S>(d.u, d.ub, iu), copy_of<S>(d.v, d.vb, iv),
                              nullptr, d.flags, d.c, halo, TX, TY, 0);
    });
    __syncthreads();
    proj_sweeps_fast<false>(smem, d.c, d.prm, sweeps, halo, TY);
    with_storage(d.storage, [&](auto tag) {
      using S = std::remove_pointer_t<decltype(tag)>;
      proj_stage_out<false, S>(smem, tx, ty, copy_of<S>(d.u, d.ub, 1 - iu),
                               copy_of<S>(d.v, d.vb, 1 - iv), nullptr, d.c, halo, TX, TY);
    });
    __syncthreads();
  }
}

__global__ void k_batch_extrapolate(const PlanHeader* __restrict__ P,
                                    const int* __restrict__ remaining) {
  const int* slot_of = plan_array<int>(P, P->off_slot);
  const ScenarioDesc* T = plan_array<ScenarioDesc>(P, P->off_desc);
  for (int k = blockIdx.x; k < P->members; k += gridDim.x) {
    const int slot = slot_of[k];
    if (remaining[slot] == 0) continue;
    const ScenarioDesc& d = T[slot];
    const int iu = (d.diff_passes + d.proj_passes) & 1, iv = d.proj_passes & 1;
    with_storage(d.storage, [&](auto tag) {
      using S = std::remove_pointer_t<decltype(tag)>;
      extrapolate_grid<S>(copy_of<S>(d.u, d.ub, iu), copy_of<S>(d.v, d.vb, iv), d.c);
    });
    __syncthreads();
  }
}

__global__ void k_batch_advect_velocity(const PlanHeader* __restrict__ P,
                                        const int* __restrict__ remaining) {
  for_cells(P, remaining, [&](const ScenarioDesc& d, int j, int i0, int i1) {
    const int iu = (d.diff_passes + d.proj_passes) & 1, iv = d.proj_passes & 1;
    with_storage(d.storage, [&](auto tag) {
      using S = std::remove_pointer_t<decltype(tag)>;
      for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x)
        advect_velocity_cell<S, float>(copy_of<S>(d.u, d.ub, iu), copy_of<S>(d.v, d.vb, iv),
                                       copy_of<S>(d.u, d.ub, 1 - iu),
                                       copy_of<S>(d.v, d.vb, 1 - iv), d.nbr, d.c, d.prm, i, j);
    });
  });
}

// Smoke advection on the advected velocity (copying it back to u, v where it
// sits in a buffer); scenarios without smoke only copy back.
__global__ void k_batch_advect_smoke(const PlanHeader* __restrict__ P,
                                     const int* __restrict__ remaining) {
  for_cells(P, remaining, [&](const ScenarioDesc& d, int j, int i0, int i1) {
    const int iu = 1 - ((d.diff_passes + d.proj_passes) & 1), iv = 1 - (d.proj_passes & 1);
    with_storage(d.storage, [&](auto tag) {
      using S = std::remove_pointer_t<decltype(tag)>;
      S* lu = copy_of<S>(d.u, d.ub, iu);
      S* lv = copy_of<S>(d.v, d.vb, iv);
      S* u = static_cast<S*>(d.u);
      S* v = static_cast<S*>(d.v);
      for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        if (d.smoke_on) {
          advect_smoke_cell<S, float>(lu, lv, static_cast<S*>(d.s), static_cast<S*>(d.sb), u, v,
                                      d.nbr, d.c, d.prm, i, j, iu == 1, iv == 1);
        } else {
          const int64_t q = cell_index(d.c.W, d.c.H, i, j);
          if (iu) u[q] = lu[q];
          if (iv) v[q] = lv[q];
        }
      }
    });
  });
}

__global__ void k_batch_finish_smoke(const PlanHeader* __restrict__ P,
                                     const int* __restrict__ remaining) {
  for_cells(P, remaining, [&](const ScenarioDesc& d, int j, int i0, int i1) {
    if (!d.smoke_on) return;
    with_storage(d.storage, [&](auto tag) {
      using S = std::remove_pointer_t<decltype(tag)>;
      for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x)
        finish_smoke_cell<S, float>(static_cast<S*>(d.sb), static_cast<S*>(d.s), d.c, d.prm,
                                    cell_index(d.c.W, d.c.H, i, j));
    });
  });
}

// End of a step: every live member has one step fewer to go.
__global__ void k_batch_tick(const PlanHeader* __restrict__ P, int* __restrict__ remaining) {
  const int* slot_of = plan_array<int>(P, P->off_slot);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P->members; k += gridDim.x * blockDim.x) {
    const int slot = slot_of[k];
    if (remaining[slot] > 0) remaining[slot]--;
  }
}

// After a plan copy: newly admitted (or cancelled) slots get their step counts.
__global__ void k_batch_admit(const PlanHeader* __restrict__ P, int* __restrict__ remaining) {
  const int2* a = plan_array<int2>(P, P->off_admit);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P->admits; k += gridDim.x * blockDim.x)
    remaining[a[k].x] = a[k].y;
}

}  // namespace osg
