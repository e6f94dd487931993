// os_batch.cuh — many independent wind tunnels of different sizes advanced
// together: one CUDA graph per step, one persistent kernel per phase.
//
// Each scenario keeps its own fields (an os_handle each, the reference's
// layout). A device table describes every scenario; work lists enumerate the
// units of each phase across all scenarios:
//   * row items (scenario, j) for the per-cell phases (forces, velocity and
//     smoke advection, the smoke copy-back);
//   * tile items (scenario, tx, ty) for every blocked diffusion and projection
//     pass; pass p lists only the tiles of scenarios with more than p passes,
//     since projection_n differs between scenarios.
// Persistent kernels (one CTA per SM for the tile phases) walk the lists, so a
// step costs the same ~20 launches whatever the number of scenarios. The
// per-tile and per-cell code is the single-grid code, so a scenario advances
// bit for bit as it would alone.
//
// Buffer parity per scenario: diffusion pass p reads copy (p & 1) of u; with D
// diffusion passes, projection pass p reads u copy ((D + p) & 1) and v copy
// (p & 1). Velocity advection then writes the other copies, and the smoke
// kernel copies the live velocity back to the public arrays where needed.
#pragma once

namespace osg {

struct ScenarioDesc {
  Consts c;
  int smoke_period;
  int smoke_on;      // enable_smoke && wind_tunnel.smoke != 0
  int diff_passes;   // blocked diffusion passes per step (0 when viscosity == 0)
  int proj_passes;   // blocked projection passes per step
  const StepParams* prm;
  float *u, *v, *ub, *vb, *s, *sb;
  const uint8_t* flags;
};

struct TileItem {
  int s, tx, ty;
};

struct RowItem {
  int s, j;
};

__device__ __forceinline__ float* copy_of(float* a, float* b, int which) { return which ? b : a; }

__global__ void k_batch_forces(const RowItem* __restrict__ rows, int n_rows,
                               const ScenarioDesc* __restrict__ T) {
  for (int r = blockIdx.x; r < n_rows; r += gridDim.x) {
    const RowItem it = rows[r];
    const ScenarioDesc& d = T[it.s];
    for (int i = threadIdx.x; i < d.c.W; i += blockDim.x)
      forces_cell<float, float>(d.u, d.v, d.s, d.c, d.smoke_period, d.prm, i, it.j);
  }
}

__global__ void __launch_bounds__(kBlockThreads, 1)
k_batch_diffuse(const TileItem* __restrict__ items, int n_items,
                const ScenarioDesc* __restrict__ T, int pass, int K, int halo, int TX, int TY) {
  extern __shared__ __align__(16) float smem[];
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const TileItem t = items[it];
    const ScenarioDesc& d = T[t.s];
    const int sweeps = min(K, d.c.n - pass * K);
    const int in = pass & 1;
    diffuse_tile<float>(smem, t.tx, t.ty, copy_of(d.u, d.ub, in), copy_of(d.u, d.ub, 1 - in),
                        d.c, d.prm, sweeps, halo, TX, TY);
    __syncthreads();  // the next item restages shared memory
  }
}

__global__ void __launch_bounds__(kBlockThreads, 1)
k_batch_project(const TileItem* __restrict__ items, int n_items,
                const ScenarioDesc* __restrict__ T, int pass, int K, int halo, int TX, int TY) {
  extern __shared__ __align__(16) float smem[];
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const TileItem t = items[it];
    const ScenarioDesc& d = T[t.s];
    const int sweeps = min(K, d.c.n - pass * K);
    const int iu = (d.diff_passes + pass) & 1, iv = pass & 1;
    project_tile<false, float>(smem, t.tx, t.ty, copy_of(d.u, d.ub, iu),
                               copy_of(d.v, d.vb, iv), copy_of(d.u, d.ub, 1 - iu),
                               copy_of(d.v, d.vb, 1 - iv), nullptr, d.flags, d.c, d.prm,
                               sweeps, halo, TX, TY, 0);
    __syncthreads();
  }
}

__global__ void k_batch_extrapolate(const ScenarioDesc* __restrict__ T, int count) {
  for (int s = blockIdx.x; s < count; s += gridDim.x) {
    const ScenarioDesc& d = T[s];
    const int iu = (d.diff_passes + d.proj_passes) & 1, iv = d.proj_passes & 1;
    extrapolate_grid<float>(copy_of(d.u, d.ub, iu), copy_of(d.v, d.vb, iv), d.c);
    __syncthreads();
  }
}

__global__ void k_batch_advect_velocity(const RowItem* __restrict__ rows, int n_rows,
                                        const ScenarioDesc* __restrict__ T) {
  for (int r = blockIdx.x; r < n_rows; r += gridDim.x) {
    const RowItem it = rows[r];
    const ScenarioDesc& d = T[it.s];
    const int iu = (d.diff_passes + d.proj_passes) & 1, iv = d.proj_passes & 1;
    for (int i = threadIdx.x; i < d.c.W; i += blockDim.x)
      advect_velocity_cell<float, float>(copy_of(d.u, d.ub, iu), copy_of(d.v, d.vb, iv),
                                         copy_of(d.u, d.ub, 1 - iu), copy_of(d.v, d.vb, 1 - iv),
                                         d.flags, d.c, d.prm, i, it.j);
  }
}

// Smoke advection on the advected velocity (copying it back to u, v where it
// sits in a buffer); scenarios without smoke only copy back.
__global__ void k_batch_advect_smoke(const RowItem* __restrict__ rows, int n_rows,
                                     const ScenarioDesc* __restrict__ T) {
  for (int r = blockIdx.x; r < n_rows; r += gridDim.x) {
    const RowItem it = rows[r];
    const ScenarioDesc& d = T[it.s];
    const int iu = 1 - ((d.diff_passes + d.proj_passes) & 1), iv = 1 - (d.proj_passes & 1);
    float* lu = copy_of(d.u, d.ub, iu);
    float* lv = copy_of(d.v, d.vb, iv);
    for (int i = threadIdx.x; i < d.c.W; i += blockDim.x) {
      if (d.smoke_on) {
        advect_smoke_cell<float, float>(lu, lv, d.s, d.sb, d.u, d.v, d.flags, d.c, d.prm, i,
                                        it.j, iu == 1, iv == 1);
      } else {
        const int64_t k = cell_index(d.c.W, d.c.H, i, it.j);
        if (iu) d.u[k] = lu[k];
        if (iv) d.v[k] = lv[k];
      }
    }
  }
}

__global__ void k_batch_finish_smoke(const RowItem* __restrict__ rows, int n_rows,
                                     const ScenarioDesc* __restrict__ T) {
  for (int r = blockIdx.x; r < n_rows; r += gridDim.x) {
    const RowItem it = rows[r];
    const ScenarioDesc& d = T[it.s];
    if (!d.smoke_on) continue;
    for (int i = threadIdx.x; i < d.c.W; i += blockDim.x)
      finish_smoke_cell<float, float>(d.sb, d.s, d.c, d.prm, cell_index(d.c.W, d.c.H, i, it.j));
  }
}

}  // namespace osg
