/*
 * fluid_oracle.c — CPU restatement of OpenSayal's simulation step.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the oracle that the parity tests,
 * the smoke check and bench.py's CPU-baseline leg compare the CUDA library
 * against. The product never links, loads or calls it.
 *
 * It restates, function by function, the per-cell device code of the
 * reference (src/fluid.cu, cited line by line below) as host loops, with
 * OpenMP over rows. Arithmetic follows the reference's types exactly: FP32
 * where the reference computes in float, FP64 where it silently promotes
 * ((i + 0.5) * h, h / 2.0, 1.0 / (d + 1e-6), max(x, 0.0)). Where nvcc
 * contracts a multiply feeding an add into one fused multiply-add, this file
 * writes fmaf() explicitly and is compiled with -ffp-contract=off, so the
 * oracle gives the same bits on x86-64 and AArch64.
 *
 * Two behaviours of the reference are undefined or racy and are resolved
 * here on purpose:
 *  - apply_diffusion runs its sweeps in place from many threads at once
 *    (src/fluid.cu:167-190), so each cell sees a timing-dependent mix of old
 *    and new neighbours. The oracle runs Jacobi sweeps (all neighbours old).
 *    The two differ by O(a^2) per sweep, a = viscosity*dt/h^2.
 *  - apply_extrapolation has write/read races at the domain corners
 *    (src/fluid.cu:720-733). The oracle applies the row rules (j == 0,
 *    j == H-1) for every column first and the column rules (i == 0,
 *    i == W-1) afterwards. Only v(W-1, 1) can be observed, and only with the
 *    drain open; this order gives it the value v(W-2, 1) = 0.
 *
 * The reference compiles its device code with --use_fast_math (approximate
 * FP32 divide and sqrt, flush-to-zero). The oracle uses IEEE operations, so
 * it agrees with the GPU to a few ulp per operation, not bit for bit.
 */
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/opensayal_gb300.h"

/* The constants of Fluid as its constructor copies them (src/fluid.cu:41-61,
 * inc/fluid.cuh:40-59). cell_size is an int there: the float key is truncated. */
typedef struct orc_params {
  int W, H;
  float g, density, viscosity, o;
  int h, n;
  float drag;
  int smoke_length, smoke_count, smoke_height;
  float speed;
  int pipe_height;
  float tunnel_smoke;
  int enable_decay, enable_pressure, enable_smoke;
  float decay_rate;
} orc_params;

static orc_params params_of(const os_config* c) {
  orc_params p;
  p.W = c->width;
  p.H = c->height;
  p.g = c->g;
  p.density = c->density;
  p.viscosity = c->viscosity;
  p.o = c->projection_o;
  p.h = (int)c->cell_size;
  p.n = c->projection_n;
  p.drag = c->drag_coeff;
  p.smoke_length = c->smoke_length;
  p.smoke_count = c->smoke_count;
  p.smoke_height = c->smoke_height;
  p.speed = c->tunnel_speed;
  p.pipe_height = c->pipe_height;
  p.tunnel_smoke = c->tunnel_smoke;
  p.enable_decay = c->smoke_enable_decay != 0;
  p.enable_pressure = c->enable_pressure != 0;
  p.enable_smoke = c->enable_smoke != 0;
  p.decay_rate = c->smoke_decay_rate;
  return p;
}

/* Fluid::indx (src/fluid.cu:163-165). 64-bit so that out-of-range probes
 * cannot overflow before index_is_valid rejects them. */
static inline int64_t IX(const orc_params* p, int64_t i, int64_t j) {
  return ((int64_t)p->H - j - 1) * p->W + i;
}

/* Fluid::index_is_valid (src/fluid.cu:356-358). */
static inline int valid(const orc_params* p, int64_t i, int64_t j) {
  return i < p->W && j < p->H && i >= 0 && j >= 0;
}

/* Fluid::is_valid_fluid (src/fluid.cu:360-362). */
static inline int fluid(const orc_params* p, const int32_t* solid, int64_t i,
                        int64_t j) {
  return valid(p, i, j) && !solid[IX(p, i, j)];
}

/* float -> int conversion as the GPU's cvt.rzi.s32.f32 performs it:
 * truncation toward zero, saturating, NaN -> 0 (C leaves these undefined). */
static inline int f2i(float f) {
  if (f != f) return 0;
  if (f >= 2147483648.0f) return INT_MAX;
  if (f <= -2147483648.0f) return INT_MIN;
  return (int)f;
}

/* ------------------------------------------------------------------------ */
/* Construction                                                              */
/* ------------------------------------------------------------------------ */

/* Solid mask and neighbour counts, Fluid::init_device_memory
 * (src/fluid.cu:111-142). The obstacle test is the reference's double
 * expression sqrt(pow(di, 2) + pow(dj, 2)) < radius. total_s starts from zero
 * (the reference malloc()s it without clearing, src/fluid.cu:102-103). */
int orc_init_mask(const os_config* c, int32_t* is_solid, int32_t* total_s) {
  const orc_params P = params_of(c);
  const orc_params* p = &P;
  const int W = p->W, H = p->H;
  for (int i = 0; i < W; i++) {
    for (int j = 0; j < H; j++) {
      const double di = (double)(i - c->obstacle_center_x);
      const double dj = (double)(j - c->obstacle_center_y);
      const int in_obstacle =
          c->obstacle_enable &&
          sqrt(pow(di, 2) + pow(dj, 2)) < (double)c->obstacle_radius;
      const int in_pipe_wall =
          i < c->pipe_length &&
          (j == H / 2 - c->pipe_height / 2 - 1 ||
           j == H / 2 + c->pipe_height / 2 + 1);
      is_solid[IX(p, i, j)] = (i == 0 || j == 0 || j == H - 1 ||
                               (!c->enable_drain && i == W - 1) ||
                               in_obstacle || in_pipe_wall);
    }
  }
  for (int i = 0; i < W; i++) {
    for (int j = 0; j < H; j++) {
      int s = 0;
      if (valid(p, i - 1, j) && is_solid[IX(p, i - 1, j)] == 0) s++;
      if (valid(p, i + 1, j) && is_solid[IX(p, i + 1, j)] == 0) s++;
      if (valid(p, i, j - 1) && is_solid[IX(p, i, j - 1)] == 0) s++;
      if (valid(p, i, j + 1) && is_solid[IX(p, i, j + 1)] == 0) s++;
      total_s[IX(p, i, j)] = s;
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Phases of Fluid::update                                                   */
/* ------------------------------------------------------------------------ */

/* apply_external_forces_at (src/fluid.cu:308-349), every cell. smoke_spacing
 * is only evaluated when smoke_count != 1 (the reference divides by zero
 * otherwise and never uses the value). */
void orc_forces(const os_config* c, const os_source* src, float dt, float* u,
                float* v, float* s) {
  const orc_params P = params_of(c);
  const orc_params* p = &P;
  const int W = p->W, H = p->H;
  const int band_lo = H / 2 - p->pipe_height / 2;
  const int band_hi = H / 2 + p->pipe_height / 2;
  const int smoke_lo = H / 2 - p->smoke_height / 2;
  const int smoke_hi = H / 2 + p->smoke_height / 2;
  int period = 1;
  if (p->smoke_count != 1) {
    const int spacing = (p->pipe_height - p->smoke_count * p->smoke_height) /
                        (p->smoke_count - 1);
    period = spacing + p->smoke_height;
  }
  const float damping = p->drag != 0.0f ? expf(-p->drag * dt) : 1.0f;
  const int active = src && src->active;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < H; j++) {
    for (int i = 0; i < W; i++) {
      const int64_t k = IX(p, i, j);
      if (i <= p->smoke_length && i != 0 && j >= band_lo && j <= band_hi) {
        u[k] = p->speed;
        const int smoke_row =
            (p->smoke_count == 1 && j >= smoke_lo && j <= smoke_hi) ||
            (p->smoke_count != 1 &&
             (H / 2 + p->pipe_height / 2 - j) % period < p->smoke_height);
        if (smoke_row) s[k] = p->tunnel_smoke;
      }
      if (p->drag != 0.0f) {
        u[k] *= damping;
        v[k] *= damping;
      }
      if (active) {
        const int dx = i - src->position_x, dy = j - src->position_y;
        if (dx * dx + dy * dy < 40 * 40) {
          if (src->smoke != 0.0f) s[k] = src->smoke;
          u[k] = fmaf(src->velocity, (float)dx, u[k]);
          v[k] = fmaf(src->velocity, (float)dy, v[k]);
        }
      }
      v[k] = fmaf(p->g, dt, v[k]);
    }
  }
}

/* apply_diffusion_at (src/fluid.cu:176-183) on the interior, as `sweeps`
 * Jacobi sweeps; `scratch` holds W*H floats. */
void orc_diffusion(const os_config* c, float dt, int sweeps, float* u,
                   float* scratch) {
  const orc_params P = params_of(c);
  const orc_params* p = &P;
  const int W = p->W, H = p->H;
  const float a = p->viscosity * dt / (float)(p->h * p->h);
  const float denom = fmaf(4.0f, a, 1.0f);
  for (int t = 0; t < sweeps; t++) {
    memcpy(scratch, u, sizeof(float) * (size_t)W * H);
#pragma omp parallel for schedule(static)
    for (int j = 1; j < H - 1; j++) {
      for (int i = 1; i < W - 1; i++) {
        const float sum = ((scratch[IX(p, i - 1, j)] + scratch[IX(p, i + 1, j)]) +
                           scratch[IX(p, i, j - 1)]) +
                          scratch[IX(p, i, j + 1)];
        u[IX(p, i, j)] = fmaf(a, sum, scratch[IX(p, i, j)]) / denom;
      }
    }
  }
}

/* zero_pressure_at (src/fluid.cu:212-214). */
void orc_zero_pressure(const os_config* c, float* pr) {
  memset(pr, 0, sizeof(float) * (size_t)c->width * c->height);
}

/* apply_projection_at for one cell (src/fluid.cu:229-262), with
 * update_pressure_at (src/fluid.cu:221-227). */
static inline void project_cell(const orc_params* p, const int32_t* solid,
                                const int32_t* total_s, float dt, float* u,
                                float* v, float* pr, int i, int j) {
  const int64_t k = IX(p, i, j);
  if (solid[k]) return;
  const int64_t kr = IX(p, i + 1, j), kt = IX(p, i, j + 1);
  const float d = ((u[kr] - u[k]) + v[kt]) - v[k];
  const float vd = p->o * (d / (float)total_s[k]);
  if (p->enable_pressure) pr[k] += vd * p->density * (float)p->h / dt;
  if (!solid[IX(p, i - 1, j)]) u[k] += vd;
  if (!solid[kr]) u[kr] -= vd;
  if (!solid[IX(p, i, j - 1)]) v[k] += vd;
  if (!solid[kt]) v[kt] -= vd;
}

/* apply_projection (src/fluid.cu:264-295): `sweeps` times, all interior cells
 * with (i + j) even, then all with (i + j) odd. Cells of one colour touch
 * disjoint faces, so the order inside a colour does not matter. */
void orc_projection(const os_config* c, float dt, int sweeps,
                    const int32_t* solid, const int32_t* total_s, float* u,
                    float* v, float* pr) {
  const orc_params P = params_of(c);
  const orc_params* p = &P;
  const int W = p->W, H = p->H;
  for (int t = 0; t < sweeps; t++) {
    for (int colour = 0; colour < 2; colour++) {
#pragma omp parallel for schedule(static)
      for (int j = 1; j < H - 1; j++) {
        int i0 = ((j + colour) & 1) ? 1 : 2;
        for (int i = i0; i < W - 1; i += 2)
          project_cell(p, solid, total_s, dt, u, v, pr, i, j);
      }
    }
  }
}

/* Pressure extrema, the two thrust::reduce calls of update
 * (src/fluid.cu:778-787). */
void orc_pressure_range(const os_config* c, const float* pr, float* mn,
                        float* mx) {
  float lo = INFINITY, hi = -INFINITY;
  const size_t N = (size_t)c->width * c->height;
  for (size_t k = 0; k < N; k++) {
    lo = fminf(lo, pr[k]);
    hi = fmaxf(hi, pr[k]);
  }
  *mn = lo;
  *mx = hi;
}

/* apply_extrapolation_at (src/fluid.cu:720-747), with the race order stated
 * in the header comment: row rules first, then column rules. */
void orc_extrapolation(const os_config* c, float* u, float* v) {
  const orc_params P = params_of(c);
  const orc_params* p = &P;
  const int W = p->W, H = p->H;
  for (int i = 0; i < W; i++) {
    u[IX(p, i, 0)] = u[IX(p, i, 1)];
    v[IX(p, i, 1)] = 0.0f;
    u[IX(p, i, H - 1)] = u[IX(p, i, H - 2)];
  }
  for (int j = 0; j < H; j++) {
    v[IX(p, 0, j)] = v[IX(p, 1, j)];
    u[IX(p, 1, j)] = 0.0f;
    v[IX(p, W - 1, j)] = v[IX(p, W - 2, j)];
  }
}

/* get_general_velocity_x (src/fluid.cu:479-539): masked bilinear u at (x, y)
 * from the four faces around it, with no renormalisation. */
static float sample_u(const orc_params* p, const int32_t* solid,
                      const float* u, float x, float y) {
  const float hf = (float)p->h;
  const int i = f2i(x / hf);
  const int j = f2i(y / hf);
  if (!fluid(p, solid, i, j)) return 0.0f;
  const float in_x = x - (float)(i * p->h);
  const float in_y = y - (float)(j * p->h);
  float acc = 0.0f;
  if ((double)in_y <= p->h / 2.0) {
    const float d_y = (float)(p->h / 2.0 - (double)in_y);
    const float w_x = 1.0f - in_x / hf;
    const float w_y = 1.0f - d_y / hf;
    if (fluid(p, solid, i, j)) acc = fmaf(w_y * w_x, u[IX(p, i, j)], acc);
    if (fluid(p, solid, i + 1, j))
      acc = fmaf(w_y * (1.0f - w_x), u[IX(p, i + 1, j)], acc);
    if (fluid(p, solid, i, j - 1))
      acc = fmaf((1.0f - w_y) * w_x, u[IX(p, i, j - 1)], acc);
    if (fluid(p, solid, i + 1, j - 1))
      acc = fmaf((1.0f - w_y) * (1.0f - w_x), u[IX(p, i + 1, j - 1)], acc);
  } else {
    const float d_y = (float)((double)in_y - p->h / 2.0);
    const float w_x = 1.0f - in_x / hf;
    const float w_y = 1.0f - d_y / hf;
    if (fluid(p, solid, i, j)) acc = fmaf(w_y * w_x, u[IX(p, i, j)], acc);
    if (fluid(p, solid, i, j + 1))
      acc = fmaf((1.0f - w_y) * w_x, u[IX(p, i, j + 1)], acc);
    if (fluid(p, solid, i + 1, j))
      acc = fmaf(w_y * (1.0f - w_x), u[IX(p, i + 1, j)], acc);
    if (fluid(p, solid, i + 1, j + 1))
      acc = fmaf((1.0f - w_y) * (1.0f - w_x), u[IX(p, i + 1, j + 1)], acc);
  }
  return acc;
}

/* get_general_velocity_y (src/fluid.cu:418-477): the mirror of sample_u,
 * with a strict `in_x < h/2` test. */
static float sample_v(const orc_params* p, const int32_t* solid,
                      const float* v, float x, float y) {
  const float hf = (float)p->h;
  const int i = f2i(x / hf);
  const int j = f2i(y / hf);
  if (!fluid(p, solid, i, j)) return 0.0f;
  const float in_x = x - (float)(i * p->h);
  const float in_y = y - (float)(j * p->h);
  float acc = 0.0f;
  if ((double)in_x < p->h / 2.0) {
    const float d_x = (float)(p->h / 2.0 - (double)in_x);
    const float w_x = 1.0f - d_x / hf;
    const float w_y = 1.0f - in_y / hf;
    if (fluid(p, solid, i, j)) acc = fmaf(w_y * w_x, v[IX(p, i, j)], acc);
    if (fluid(p, solid, i - 1, j))
      acc = fmaf(w_y * (1.0f - w_x), v[IX(p, i - 1, j)], acc);
    if (fluid(p, solid, i - 1, j + 1))
      acc = fmaf((1.0f - w_y) * (1.0f - w_x), v[IX(p, i - 1, j + 1)], acc);
    if (fluid(p, solid, i, j + 1))
      acc = fmaf((1.0f - w_y) * w_x, v[IX(p, i, j + 1)], acc);
  } else {
    const float d_x = (float)((double)in_x - p->h / 2.0);
    const float w_x = 1.0f - d_x / hf;
    const float w_y = 1.0f - in_y / hf;
    if (fluid(p, solid, i, j)) acc = fmaf(w_y * w_x, v[IX(p, i, j)], acc);
    if (fluid(p, solid, i, j + 1))
      acc = fmaf((1.0f - w_y) * w_x, v[IX(p, i, j + 1)], acc);
    if (fluid(p, solid, i + 1, j + 1))
      acc = fmaf((1.0f - w_y) * (1.0f - w_x), v[IX(p, i + 1, j + 1)], acc);
    if (fluid(p, solid, i + 1, j))
      acc = fmaf(w_y * (1.0f - w_x), v[IX(p, i + 1, j)], acc);
  }
  return acc;
}

/* apply_velocity_advection_at (src/fluid.cu:598-612) for every cell, with the
 * edge averages of get_vertical_edge_velocity / get_horizontal_edge_velocity
 * (src/fluid.cu:364-416) and the face positions of get_u_position /
 * get_v_position (src/fluid.cu:552-558). Reads u, v; writes u_out, v_out
 * (the reference's d_vel_*_buffer, copied back by src/fluid.cu:614-617). */
void orc_velocity_advection(const os_config* c, float dt, const int32_t* solid,
                            const float* u, const float* v, float* u_out,
                            float* v_out) {
  const orc_params P = params_of(c);
  const orc_params* p = &P;
  const int W = p->W, H = p->H;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < H; j++) {
    for (int i = 0; i < W; i++) {
      const int64_t k = IX(p, i, j);
      /* u on the left face */
      {
        const float x = (float)(i * p->h);
        const float y = (float)((j + 0.5) * p->h);
        float avg_v = v[k];
        int count = 1;
        if (fluid(p, solid, i - 1, j + 1)) { avg_v += v[IX(p, i - 1, j + 1)]; count++; }
        if (fluid(p, solid, i, j + 1)) { avg_v += v[IX(p, i, j + 1)]; count++; }
        if (fluid(p, solid, i - 1, j)) { avg_v += v[IX(p, i - 1, j)]; count++; }
        avg_v /= (float)count;
        const float px = fmaf(-u[k], dt, x);
        const float py = fmaf(-avg_v, dt, y);
        u_out[k] = sample_u(p, solid, u, px, py);
      }
      /* v on the bottom face */
      {
        const float x = (float)((i + 0.5) * p->h);
        const float y = (float)(j * p->h);
        float avg_u = u[k];
        int count = 1;
        if (fluid(p, solid, i + 1, j)) { avg_u += u[IX(p, i + 1, j)]; count++; }
        if (fluid(p, solid, i, j - 1)) { avg_u += u[IX(p, i, j - 1)]; count++; }
        if (fluid(p, solid, i + 1, j - 1)) { avg_u += u[IX(p, i + 1, j - 1)]; count++; }
        avg_u /= (float)count;
        const float px = fmaf(-avg_u, dt, x);
        const float py = fmaf(-v[k], dt, y);
        v_out[k] = sample_v(p, solid, v, px, py);
      }
    }
  }
}

/* interpolate_smoke (src/fluid.cu:644-716): inverse-distance weights to the
 * four nearest cell centres, normalised over all four, summed over the fluid
 * ones only. The distance is get_distance (inc/helper.cuh:77-81); the inverse
 * is taken in double as the reference writes it. */
static float sample_smoke(const orc_params* p, const int32_t* solid,
                          const float* s, float x, float y) {
  const float hf = (float)p->h;
  const int64_t i = f2i(x / hf);
  const int64_t j = f2i(y / hf);
  const float in_x = x - (float)(int)(i * p->h);
  const float in_y = y - (float)(int)(j * p->h);
  int64_t ci[4], cj[4];
  ci[0] = i;
  cj[0] = j;
  const int left = (double)in_x < p->h / 2.0;
  const int below = (double)in_y < p->h / 2.0;
  if (left && below) {
    ci[1] = i - 1; cj[1] = j; ci[2] = i; cj[2] = j - 1; ci[3] = i - 1; cj[3] = j - 1;
  } else if (left) {
    ci[1] = i - 1; cj[1] = j; ci[2] = i; cj[2] = j + 1; ci[3] = i - 1; cj[3] = j + 1;
  } else if (below) {
    ci[1] = i + 1; cj[1] = j; ci[2] = i; cj[2] = j - 1; ci[3] = i + 1; cj[3] = j - 1;
  } else {
    ci[1] = i + 1; cj[1] = j; ci[2] = i; cj[2] = j + 1; ci[3] = i + 1; cj[3] = j + 1;
  }
  float inv[4];
  for (int q = 0; q < 4; q++) {
    const float cx = (float)((ci[q] + 0.5) * p->h);
    const float cy = (float)((cj[q] + 0.5) * p->h);
    const float dx = x - cx, dy = y - cy;
    const float dist = sqrtf(fmaf(dx, dx, dy * dy));
    inv[q] = (float)(1.0 / ((double)dist + 1e-6));
  }
  const float sum_inv = ((inv[0] + inv[1]) + inv[2]) + inv[3];
  float acc = 0.0f;
  for (int q = 0; q < 4; q++) {
    const float w = inv[q] / sum_inv;
    if (fluid(p, solid, ci[q], cj[q])) acc = fmaf(w, s[IX(p, ci[q], cj[q])], acc);
  }
  return acc;
}

/* apply_smoke_advection_at (src/fluid.cu:560-567) for every cell, sampling the
 * velocity at the cell centre (get_general_velocity, src/fluid.cu:541-545).
 * Reads u, v, s; writes s_out (the reference's d_smoke_buffer). */
void orc_smoke_advection(const os_config* c, float dt, const int32_t* solid,
                         const float* u, const float* v, const float* s,
                         float* s_out) {
  const orc_params P = params_of(c);
  const orc_params* p = &P;
  const int W = p->W, H = p->H;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < H; j++) {
    for (int i = 0; i < W; i++) {
      const float x = (float)((i + 0.5) * p->h);
      const float y = (float)((j + 0.5) * p->h);
      const float vx = sample_u(p, solid, u, x, y);
      const float vy = sample_v(p, solid, v, x, y);
      const float px = fmaf(-vx, dt, x);
      const float py = fmaf(-vy, dt, y);
      s_out[IX(p, i, j)] = sample_smoke(p, solid, s, px, py);
    }
  }
}

/* decay_smoke_at (src/fluid.cu:758-762): s = max(s - rate*dt, 0.0) in double. */
void orc_decay(const os_config* c, float dt, float* s) {
  if (!c->smoke_enable_decay) return;
  const size_t N = (size_t)c->width * c->height;
  const float rate = c->smoke_decay_rate;
#pragma omp parallel for schedule(static)
  for (size_t k = 0; k < N; k++) s[k] = (float)fmax((double)fmaf(-rate, dt, s[k]), 0.0);
}

/* Fluid::update (src/fluid.cu:770-795). `work` holds 3*W*H floats of
 * scratch; diffusion runs `diffusion_sweeps` times when viscosity != 0 (the
 * reference's loop counter is uninitialised; its x86-64 g++ -O3 build starts
 * it at zero, so it runs n sweeps). Returns the pressure extrema through
 * pmin/pmax when pressure is enabled. */
void orc_step(const os_config* c, const os_source* src, float dt,
              int diffusion_sweeps, const int32_t* solid,
              const int32_t* total_s, float* u, float* v, float* s, float* pr,
              float* work, float* pmin, float* pmax) {
  const size_t N = (size_t)c->width * c->height;
  float* b0 = work;
  float* b1 = work + N;
  float* b2 = work + 2 * N;
  orc_forces(c, src, dt, u, v, s);
  if (c->enable_pressure) orc_zero_pressure(c, pr);
  if (c->viscosity != 0.0f) orc_diffusion(c, dt, diffusion_sweeps, u, b0);
  orc_projection(c, dt, c->projection_n, solid, total_s, u, v, pr);
  if (c->enable_pressure && pmin && pmax) orc_pressure_range(c, pr, pmin, pmax);
  orc_extrapolation(c, u, v);
  orc_velocity_advection(c, dt, solid, u, v, b0, b1);
  memcpy(u, b0, sizeof(float) * N);
  memcpy(v, b1, sizeof(float) * N);
  if (c->enable_smoke && c->tunnel_smoke != 0.0f) {
    orc_smoke_advection(c, dt, solid, u, v, s, b2);
    memcpy(s, b2, sizeof(float) * N);
    orc_decay(c, dt, s);
  }
}

/* Number of OpenMP threads the oracle's loops use (for the CPU baseline's
 * reported core count). */
int orc_threads(void) {
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}
