/*
 * opensayal_gb300.h — C ABI of the GB300 wind-tunnel simulation step.
 *
 * This library is a drop-in for OpenSayal's `Fluid` class (inc/fluid.cuh:15-116,
 * src/fluid.cu): the same constructor keys, the same per-frame update, the same
 * field layout. Everything is plain C: pointers, sizes and status codes, no C++
 * or torch types, so any FFI (ctypes, cgo, JNI, N-API) can bind it. A C++
 * `class Fluid` with the reference's public members is layered on top in
 * include/opensayal_gb300/fluid.hpp.
 *
 * Field layout (identical to the reference, src/fluid.cu:163-165): every field
 * is a width*height array indexed by indx(i, j) = (height - 1 - j) * width + i,
 * i.e. row-major with j = 0 (the bottom row) stored last. u(i, j) lives on the
 * left face of cell (i, j), v(i, j) on its bottom face, smoke and pressure at
 * the centre.
 *
 * Errors: every entry point returns an os_status. On failure a description is
 * available from os_last_error() (thread-local). The library never calls exit().
 *
 * Threading: one handle must not be used from two host threads at once (the
 * reference's Fluid is not re-entrant either). Distinct handles are independent.
 */
#ifndef OPENSAYAL_GB300_H
#define OPENSAYAL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OS_ABI_VERSION 3

typedef enum os_status {
  OS_OK = 0,
  OS_ERR_INVALID = 1,     /* bad argument or configuration */
  OS_ERR_CUDA = 2,        /* a CUDA runtime call failed */
  OS_ERR_NOMEM = 3,       /* device or host allocation failed */
  OS_ERR_UNSUPPORTED = 4, /* valid request this build does not implement */
  OS_ERR_STATE = 5,       /* call not valid in the handle's current state */
  OS_ERR_TIMEOUT = 6      /* a bounded device wait gave up */
} os_status;

/* Field identifiers for os_upload / os_download. */
typedef enum os_field {
  OS_FIELD_VEL_X = 0,    /* Fluid::d_vel_x   (float) */
  OS_FIELD_VEL_Y = 1,    /* Fluid::d_vel_y   (float) */
  OS_FIELD_SMOKE = 2,    /* Fluid::d_smoke   (float) */
  OS_FIELD_PRESSURE = 3, /* Fluid::d_pressure (float) */
  OS_FIELD_IS_SOLID = 4, /* Fluid::d_is_solid (int32, read-only) */
  OS_FIELD_TOTAL_S = 5   /* Fluid::d_total_s  (int32, read-only) */
} os_field;

/* Storage precision of u, v and smoke. FP32 is the reference's precision. */
typedef enum os_storage {
  OS_STORAGE_F32 = 0,  /* the reference's precision */
  OS_STORAGE_F16 = 1,  /* FP16 u, v, smoke; FP32 arithmetic */
  OS_STORAGE_BF16 = 2, /* BF16 u, v, smoke; FP32 arithmetic */
  OS_STORAGE_F64 = 3   /* FP64 storage and arithmetic: the error yardstick */
} os_storage;

/*
 * Flat mirror of the reference's `Config` (inc/config_parser.hpp:9-115): the
 * thread.cuda, sim and fluid keys that Fluid reads (src/fluid.cu:41-71,111-126).
 * Visual and OpenMP keys do not reach the simulation and are not carried.
 * Booleans are int32 (0 / non-zero). Fill it with os_config_defaults() and then
 * override keys, exactly like an OpenSayal.conf.json overrides the parser's
 * defaults.
 */
typedef struct os_config {
  /* thread.cuda.block_size_{x,y} (config_parser.cpp:30-33). Kept so that the
   * C++ wrapper can expose kernel_grid_dim/kernel_block_dim; the GB300 kernels
   * choose their own launch shapes. */
  int32_t block_size_x;
  int32_t block_size_y;
  /* sim.* */
  int32_t height;
  int32_t width;
  int32_t cell_pixel_size;
  float cell_size; /* truncated to int, as Fluid::cell_size is (inc/fluid.cuh:46) */
  int32_t enable_drain;
  int32_t enable_pressure;
  int32_t enable_smoke;
  int32_t enable_interactive;
  int32_t projection_n;  /* sim.projection.n */
  float projection_o;    /* sim.projection.o */
  int32_t pipe_height;   /* sim.wind_tunnel.pipe_height */
  int32_t pipe_length;   /* sim.wind_tunnel.pipe_length (parser hard-codes 0) */
  int32_t smoke_length;  /* sim.wind_tunnel.smoke_length */
  int32_t smoke_height;  /* sim.wind_tunnel.smoke_height */
  int32_t smoke_count;   /* sim.wind_tunnel.smoke_count */
  float tunnel_speed;    /* sim.wind_tunnel.speed */
  float tunnel_smoke;    /* sim.wind_tunnel.smoke */
  float g;               /* sim.physics.g */
  float d_t;             /* sim.time.d_t */
  int32_t enable_real_time;
  float real_time_multiplier;
  int32_t smoke_enable_decay; /* sim.smoke.enable_decay */
  float smoke_decay_rate;     /* sim.smoke.decay_rate */
  int32_t obstacle_enable;
  int32_t obstacle_center_x;
  int32_t obstacle_center_y;
  float obstacle_radius;
  /* fluid.* */
  float density;
  float drag_coeff;
  float viscosity;
  /* Extensions with no reference key. Zero means "reference behaviour". */
  int32_t storage;          /* os_storage of u, v, smoke; 0 = FP32 */
  int32_t device;           /* CUDA device ordinal */
  int32_t projection_block; /* red/black (and Jacobi) sweeps fused per pass;
                               0 = autotune: os_create times candidate depths
                               on a scratch grid of the same configuration
                               once per process and configuration shape;
                               -1 = one launch per sweep (plain form) */
  int32_t idw_mode;         /* smoke inverse distances 1/(d + 1e-6), which the
                               reference computes in FP64 (src/fluid.cu:
                               690-693): 0 (default) FP32 float-pair
                               arithmetic that rounds like the FP64
                               expression; 1 literal FP64; 2 plain FP32 */
  int32_t projection_resident; /* phases run as one cooperative launch each,
                               tiles kept in shared memory and exchanging
                               halos between passes: a mask, 1 the
                               projection, 2 the diffusion, 3 both, each
                               where the grid fits one co-resident tile per
                               SM (projection: projection_block even;
                               diffusion: a multiple of 4); 0 = the autotuner
                               decides (with projection_block 0; a fixed
                               projection_block runs pass by pass); -1 = never */
  int32_t diffusion_block; /* Jacobi sweeps fused per diffusion pass when the
                               diffusion runs pass by pass (not resident):
                               0 = projection_block's depth, or with
                               projection_block 0 the autotuner's choice
                               (its halo is K cells against the projection's
                               2K, so deeper passes can pay). Single handles
                               only: a batch runs its own depth for every
                               member */
  int32_t reserved[2];
} os_config;

/* The reference's `Source` (inc/fluid.cuh:8-13), the interactive forcing. */
typedef struct os_source {
  int32_t active;
  float smoke;
  float velocity;
  int32_t position_x;
  int32_t position_y;
} os_source;

/* Device pointers of a handle's public fields, laid out by indx(i, j). */
typedef struct os_fields_view {
  int32_t width;
  int32_t height;
  int32_t storage;    /* os_storage of vel_x, vel_y, smoke */
  int32_t projection_block; /* sweeps per blocked pass in use (-1: plain) */
  void* vel_x;        /* Fluid::d_vel_x */
  void* vel_y;        /* Fluid::d_vel_y */
  void* smoke;        /* Fluid::d_smoke */
  float* pressure;    /* Fluid::d_pressure */
  int32_t* is_solid;  /* Fluid::d_is_solid */
  int32_t* total_s;   /* Fluid::d_total_s */
  int32_t projection_resident; /* resident forms in use: bit 0 projection,
                                  bit 1 diffusion */
  int32_t tma_staging;   /* 1: diffusion passes stage their regions with tensor
                            copies; opt-in with the environment variable
                            OPENSAYAL_GB300_TMA=1 at os_create (FP32, W and
                            depth multiples of 4, depth at most 8) */
} os_fields_view;

typedef struct os_handle os_handle;

/* ABI version of the loaded library (OS_ABI_VERSION). */
int32_t os_abi_version(void);

/* Human-readable description of the last failure on this host thread. */
const char* os_last_error(void);

/*
 * ConfigParser defaults for a width x height tunnel (src/config_parser.cpp:
 * 15-184): pipe_height = smoke_height = height/4, obstacle at the centre with
 * radius min(w, h)/30, viscosity 0.001, n = 50, o = 1.9, drain and smoke on.
 * Replaces: ConfigParser::parse() with an empty JSON object.
 */
int os_config_defaults(int32_t width, int32_t height, os_config* out);

/*
 * Allocates the fields, rasterises the solid mask and neighbour counts, zeroes
 * u, v, smoke and pressure. Replaces: Fluid::Fluid(Config) (src/fluid.cu:41-71,
 * 86-161). Unlike the reference it validates the configuration and reports
 * failures instead of proceeding with undefined state.
 */
int os_create(const os_config* cfg, os_handle** out);

/* Frees every device array. Replaces: Fluid::~Fluid() (src/fluid.cu:73-84). */
int os_destroy(os_handle* h);

/*
 * One simulation step, synchronous like the reference (it ends with a device
 * synchronisation). Replaces: Fluid::update(Source, float) (src/fluid.cu:
 * 770-795). `src` may be NULL for an inactive source.
 */
int os_update(os_handle* h, const os_source* src, float dt);

/*
 * `steps` simulation steps enqueued on `stream` (a cudaStream_t, NULL for the
 * handle's own stream) without synchronising; replays one captured CUDA graph
 * per step. No reference counterpart (the reference synchronises every step).
 */
int os_update_async(os_handle* h, const os_source* src, float dt,
                    int32_t steps, void* stream);

/* Waits for all work enqueued on the handle's stream. */
int os_synchronize(os_handle* h);
/* Without waiting: *idle = 1 when everything enqueued on the handle's own
 * stream has completed (and the resident waits reported no failure), else 0.
 * No reference counterpart (the reference's update always synchronises). */
int os_query(os_handle* h, int32_t* idle);

/* Device pointers of the public fields. Replaces: reading Fluid::d_* members. */
int os_fields(os_handle* h, os_fields_view* out);

/* Host <-> device copies of one field; `count` must equal width*height.
 * Float fields are converted from / to the storage precision. */
int os_upload(os_handle* h, int32_t field, const void* host, size_t count);
int os_download(os_handle* h, int32_t field, void* host, size_t count);
/*
 * Without waiting: enqueues on `stream` (NULL: the handle's stream), after
 * the work already there, a copy of a field as it is at that point into a
 * caller-owned device buffer of `count` = width * height 4-byte values
 * (storage fields converted to FP32). With the step on the same stream, a
 * caller reads the copy to the host on a stream of its own while the next
 * step runs: the snapshot is not touched by later steps, while the live
 * field is (the next step's inflow writes smoke at once). No reference
 * counterpart (the reference's callers read the fields after a synchronous
 * update).
 */
int os_snapshot_async(os_handle* h, int32_t field, void* device_dst, size_t count,
                      void* stream);

/* Pressure extrema of the last step with enable_pressure set.
 * Replaces: Fluid::min_pressure / Fluid::max_pressure (src/fluid.cu:778-787). */
int os_pressure_range(os_handle* h, float* min_out, float* max_out);

/*
 * Runs one phase of the step on the current fields (diagnostics and phase-level
 * parity tests). Replaces the private phase methods of Fluid
 * (src/fluid.cu:185-190,216-219,282-295,351-354,591-596,637-642,744-747,764-767).
 */
typedef enum os_phase {
  OS_PHASE_FORCES = 0,         /* apply_external_forces */
  OS_PHASE_ZERO_PRESSURE = 1,  /* zero_pressure */
  OS_PHASE_DIFFUSION = 2,      /* apply_diffusion: n sweeps */
  OS_PHASE_PROJECTION = 3,     /* apply_projection: n red/black sweeps */
  OS_PHASE_PRESSURE_RANGE = 4, /* min/max reduction of pressure */
  OS_PHASE_EXTRAPOLATION = 5,  /* apply_extrapolation */
  OS_PHASE_VEL_ADVECTION = 6,  /* apply_velocity_advection (+ copy back) */
  OS_PHASE_SMOKE_ADVECTION = 7,/* apply_smoke_advection (+ copy back) */
  OS_PHASE_DECAY = 8           /* decay_smoke */
} os_phase;
int os_run_phase(os_handle* h, int32_t phase, const os_source* src, float dt);

/* Number of kernels this library launched on the handle since creation. */
int os_kernel_launches(os_handle* h, int64_t* out);

/*
 * Diagnostics: enqueues `reps` repetitions of one phase on `stream` (NULL for
 * the handle's own stream) between two CUDA events recorded on that stream,
 * waits, and returns the elapsed milliseconds and the number of kernels the
 * repetitions launched. No reference counterpart.
 */
int os_profile_phase(os_handle* h, int32_t phase, const os_source* src, float dt,
                     int32_t reps, void* stream, float* ms_out, int32_t* kernels_out);

/*
 * As os_profile_phase, but the time of each repetition is taken only over the
 * phase's own kernels, as a step runs them: a phase called on its own ends by
 * copying the velocity back to the public fields when its pass count leaves
 * it in the other buffers (a step does not), and that copy is left out of
 * `kernel_ms_out` (summed over the repetitions). `ms_out` is the whole time,
 * as os_profile_phase gives it. No reference counterpart.
 */
int os_profile_phase_kernels(os_handle* h, int32_t phase, const os_source* src, float dt,
                             int32_t reps, void* stream, float* kernel_ms_out, float* ms_out,
                             int32_t* kernels_out);

/*
 * The diffusion phase (n Jacobi sweeps of u, as OS_PHASE_DIFFUSION runs it)
 * on a caller-owned device field, without allocating anything. No counterpart
 * in the reference: it is for callers that may not allocate device memory
 * where they run a step (memory owned by another allocator, a frame loop that
 * cannot afford an allocation's synchronisation, a fixed device footprint).
 *
 * `u` is width*height floats in the reference layout on the calling thread's
 * current device; it is read and overwritten in place. Only width, height,
 * cell_size, projection_n and viscosity of `cfg` are used. The work is
 * enqueued on `stream` (a cudaStream_t; NULL is the legacy default stream)
 * and the call returns without waiting.
 *
 * The ping-pong buffer is one fixed device array inside the library of
 * 1,048,576 floats (4 MiB, held on every GPU that loads the library until it
 * is unloaded); larger grids are rejected with OS_ERR_INVALID. The first call
 * on a device looks up that array's device address (with the device current)
 * and should come before any stream capture. All calls on a device share the
 * array and it keeps the last call's contents; calls that overlap on the GPU
 * (other streams, or other threads) race on it and must be serialised.
 */
int os_diffuse_noalloc(const os_config* cfg, float* u, float dt, void* stream);

/*
 * Headless visuals: the reference's per-frame colouring, velocity arrows and
 * path lines (src/graphics_handler.cu:168-396, src/helper.cu, the
 * `visual.*` and `sim.cell_pixel_size` keys of src/config_parser.cpp:39-40,
 * 120-179), written to caller-owned device buffers on `stream` (NULL: the
 * handle's stream) without waiting. No window or graphics library is used.
 */
typedef struct os_visual_config {
  int32_t cell_pixel_size;        /* sim.cell_pixel_size (1) */
  int32_t arrow_distance;         /* visual.arrows.distance (20) */
  float arrow_length_multiplier;  /* visual.arrows.length_multiplier (0.1) */
  float arrow_disable_threshold;  /* visual.arrows.disable_threshold (0) */
  int32_t arrow_head_length;      /* visual.arrows.head_length (5) */
  int32_t trace_distance;         /* visual.path_line.distance (20) */
  int32_t trace_length;           /* visual.path_line.length (20) */
  int32_t reserved;
} os_visual_config;

/* The reference's ArrowData (inc/graphics_handler.cuh:17-27), pixel
 * coordinates; an entry with valid == 0 carries no other data. */
typedef struct os_arrow {
  int32_t start_x, start_y, end_x, end_y;
  int32_t right_head_end_x, right_head_end_y, left_head_end_x, left_head_end_y;
  int32_t valid;
} os_arrow;

int os_visual_defaults(os_visual_config* out);

/*
 * Parses the text of an OpenSayal.conf.json document (`length` bytes, no
 * terminator needed) as the reference's ConfigParser does: its keys, its
 * defaults (which follow the parsed sim.width and sim.height), and its
 * dotted-key lookup (a key is looked up whole first, then split at its first
 * dot). Fills *cfg (the library's own fields keep os_config_defaults' values)
 * and, when `visual` is not NULL, *visual. Malformed JSON, or a value of the
 * wrong type given whole at the top level, is OS_ERR_INVALID (the reference
 * ends the program); a wrong type inside a nested object yields the default,
 * as the reference's lookup does. Replaces: ConfigParser::parse()
 * (src/config_parser.cpp:15-184, inc/config_parser.hpp:131-150); the C++
 * class ConfigParser in opensayal_gb300/config_parser.hpp reads the file.
 */
int os_config_parse(const char* json_text, size_t length, os_config* cfg,
                    os_visual_config* visual);
/* W*H RGBA words (r << 24 | g << 16 | b << 8 | a) at y * W + x for pixel
 * (x, y) = (i, H - 1 - j), the cell's own index: solid cells grey, the others
 * coloured by smoke and/or pressure as sim.enable_smoke/enable_pressure say
 * (pressure normalised by the last update's extrema); with both off, fluid
 * pixels are left unchanged. */
int os_render_pixels(os_handle* h, int32_t* d_pixels, void* stream);
/* (W / d) x (H / d) arrows, d = arrow_distance, entry (a, b) at
 * (H / d - b - 1) * (W / d) + a for the arrow from cell (a d, b d); entries of
 * solid cells are left unchanged. */
int os_render_arrows(os_handle* h, const os_visual_config* v, os_arrow* d_arrows, void* stream);
/* Path lines of trace_length points from every d-th cell (d = trace_distance),
 * stepped by `dt`: point k of line (a, b) at
 * ((H / d - b - 1) * (W / d) + a) * trace_length + k in d_x and d_y; a solid
 * start cell gets (-1, -1) as its first point only. */
int os_render_traces(os_handle* h, const os_visual_config* v, float dt, int32_t* d_x,
                     int32_t* d_y, void* stream);

/*
 * Failure detection of the resident projection's inter-tile waits, without a
 * fault: one CTA waits on a neighbour flag that nothing sets. Every such wait
 * is bounded; when it gives up it records the failure, and the host call that
 * synchronises reports OS_ERR_TIMEOUT. *status receives what that path
 * reports here (OS_ERR_TIMEOUT when the bound works). No reference
 * counterpart.
 */
int os_selftest_bounded_wait(int32_t device, int32_t* status);

/*
 * Copy bandwidth probe for rooflines (no reference counterpart): allocates
 * two buffers of `bytes` (a positive multiple of 16) on `device`, copies one
 * into the other `reps` times in one launch with cache-at-L2 loads and
 * stores, alternating direction, and reports read + write bytes per second
 * of the timed launch in *gbs (GB/s, 1e9). Buffers that together fit in L2
 * measure the L2 copy bandwidth; larger ones measure HBM.
 */
int os_probe_copy_bandwidth(int32_t device, uint64_t bytes, int32_t reps, float* gbs);

/*
 * FP64 diagnostics of the current fields (no reference counterpart). The
 * residual of a cell is the projection's divergence
 * ((u(i+1,j) - u(i,j)) + v(i,j+1)) - v(i,j) (src/fluid.cu:229-262), taken in
 * FP64 over the cells the projection updates; the sums are FP64 as well and
 * are reduced in a fixed order, so repeated calls on the same fields agree bit
 * for bit. Enqueued on the handle's stream after the work already there, and
 * waits for the result.
 */
typedef struct os_diag {
  double divergence_l2;   /* square root of the sum of squared residuals */
  double divergence_max;  /* largest |residual| */
  double divergence_sum;  /* sum of residuals */
  double smoke_mass;      /* sum of smoke over fluid cells, times cell_size^2 */
  double inflow_flux;     /* sum of u(2, j) between fluid cells (1, j), (2, j), times cell_size */
  double outflow_flux;    /* sum of u(W-1, j) between fluid cells, times cell_size */
  int64_t active_cells;   /* cells the projection updates */
  int64_t reserved;
} os_diag;

int os_diagnose(os_handle* h, os_diag* out);

/*
 * Batched and served scenarios: many independent tunnels of different sizes
 * advanced together, one CUDA graph per step and one persistent kernel per
 * phase that walks the rows or tiles of all members. No reference counterpart
 * (the reference runs one grid). Each member advances exactly as a single
 * handle with the same sweeps-per-pass would: the same per-cell and per-tile
 * code runs, only the schedule differs. Members are FP32, FP16 or BF16 storage
 * with pressure off, on the batch's device, with projection_n at most 128 x
 * block_k; each keeps its own fields, reachable through os_batch_scenario()
 * with the single-handle calls (upload, download, fields). Calls on one batch
 * come from one thread.
 *
 * Membership can change between steps (continuous batching): os_batch_add
 * admits a scenario for a number of steps, it joins at the next os_batch_step
 * and stops on the device after exactly that many of the batch's steps;
 * os_batch_poll reports finished members, whose fields stay readable until
 * os_batch_remove. With a device-memory budget the batch reserves it once and
 * places every member inside it, so os_batch_add says OS_ERR_NOMEM without
 * touching the device when a scenario does not fit.
 */
typedef struct os_batch os_batch;

typedef struct os_batch_stats {
  int32_t scenarios;          /* members, finished or not */
  int32_t block_k;            /* sweeps per blocked pass */
  int32_t kernels_per_step;   /* launches in one step's graph */
  int32_t members_in_plan;    /* members the next step advances */
  int64_t cells;              /* cells over the members in the plan */
  int64_t launches;           /* kernels launched by os_batch_step so far */
  int64_t tile_items_per_step;
  int64_t steps_enqueued;     /* batch steps enqueued so far */
  int64_t steps_completed;    /* of those, seen complete by the host */
  int32_t projection_tile_rows; /* owned rows of a projection tile */
  int32_t diffusion_tile_rows;  /* owned rows of a diffusion tile */
} os_batch_stats;

typedef enum os_member_state {
  OS_MEMBER_WAITING = 0, /* admitted, joins at the next os_batch_step */
  OS_MEMBER_RUNNING = 1,
  OS_MEMBER_DONE = 2     /* all its steps have completed on the device */
} os_member_state;

/* A batch of fixed members, each stepping until the batch is destroyed; member
 * ids are 0..count-1. `block_k`: sweeps per blocked pass (at most 16); 0 =
 * autotune: times a few steps of depths {4, 6, 8, 12} and two tile heights on
 * the new members (whose fields start at zero and are zeroed again), keeping
 * the fastest. */
int os_batch_create(const os_config* cfgs, int32_t count, int32_t block_k, os_batch** out);
/* An empty batch on `device` for continuous batching (`block_k` 0 = 8).
 * `budget_bytes` > 0
 * reserves that much device memory for the members (0: each member allocates
 * its own, without a limit). */
int os_batch_create_dynamic(int32_t device, int32_t block_k, uint64_t budget_bytes,
                            os_batch** out);
/* Admits a scenario for `steps` steps (negative: until removed); its id goes
 * to *id. Its fields start as os_create leaves them and may be uploaded
 * before the next os_batch_step. OS_ERR_NOMEM: it does not fit the budget. */
int os_batch_add(os_batch* b, const os_config* cfg, int32_t steps, int64_t* id);
/* Drops a member and returns its memory (a running member is cancelled; its
 * memory is returned once the steps already enqueued have run). */
int os_batch_remove(os_batch* b, int64_t id);
int os_batch_destroy(os_batch* b);
/* `steps` steps of every member (graph replays) enqueued on `stream` (NULL:
 * the batch's own stream); each member uses its own config's d_t. Membership
 * changes since the last call take effect first, ordered on the same stream. */
int os_batch_step(os_batch* b, int32_t steps, void* stream);
int os_batch_synchronize(os_batch* b);
/* Ids of members whose last step has completed and that were not reported
 * before, at most `cap` of them; with `wait`, blocks until at least one
 * finishes when one is due within the steps already enqueued. */
int os_batch_poll(os_batch* b, int32_t wait, int64_t* ids, int32_t cap, int32_t* count);
/* Blocks until at most `max_in_flight` enqueued steps have not completed
 * (0: all of them), for pacing a loop that enqueues ahead. */
int os_batch_wait(os_batch* b, int64_t max_in_flight);
/* A member's state (os_member_state) and steps still to run (-1: unlimited). */
int os_batch_status(os_batch* b, int64_t id, int32_t* state, int64_t* steps_left);
/* Device bytes held by the members, and the budget (0: none). */
int os_batch_memory(os_batch* b, uint64_t* used, uint64_t* budget);
/* The handle of member `id`, owned by the batch (do not destroy it). */
int os_batch_scenario(os_batch* b, int64_t id, os_handle** out);
int os_batch_info(os_batch* b, os_batch_stats* out);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* OPENSAYAL_GB300_H */
