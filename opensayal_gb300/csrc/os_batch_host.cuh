// os_batch_host.cuh — host side of batched and served scenarios (os_batch_*).
//
// A batch owns its members' handles and advances them with one CUDA graph per
// step. Membership may change between steps: os_batch_add creates a handle
// (out of the batch's device-memory arena when it has a budget, so admission
// is a host-side decision that never stalls the device), and the next
// os_batch_step writes a new device plan with one stream-ordered copy before
// its graph launches; the graph is rebuilt only when the plan needs more
// passes or room than it was built for. Each member has a remaining-steps
// count on the device, so members admitted at different steps and asking for
// different step counts stop exactly on time inside the shared steps; the host
// knows when from the step counter it records with an event after every
// os_batch_step, and os_batch_poll reports the members whose last step has
// completed. A member's device memory goes back to the arena when it is
// removed: at once after it finished (no kernel touches a frozen member), or,
// for a cancelled live member, once the steps already enqueued have completed.
#pragma once

#include <deque>

#include "os_batch.cuh"

struct os_batch {
  struct Member {
    os_handle* h = nullptr;
    int slot = -1;
    int32_t steps = 0;       // requested; negative: unlimited
    int64_t finish_at = -1;  // batch step after which it is done; -1: not yet scheduled
    bool in_plan = false;    // part of the plan most recently written
    bool scheduled = false;  // has been part of a plan
    bool reported = false;
  };
  int device = 0;
  int K = 8;
  int ty_div = 1;  // tile height: the largest that fits, divided by this
  int sms = 152;
  cudaStream_t stream = nullptr;
  Arena* arena = nullptr;  // null: members allocate with cudaMalloc
  TileGeom gd{}, gp{};
  std::map<int64_t, Member> members;  // by id
  int64_t next_id = 0;
  std::vector<int> free_slots;
  int slot_hw = 0;  // slots handed out so far (high-water mark)
  // device plan and countdowns
  PlanHeader* d_plan = nullptr;
  size_t plan_cap = 0;
  int* d_remaining = nullptr;
  int remaining_cap = 0;
  bool dirty = true;
  // pinned plan staging, double-buffered; each guarded by the event recorded
  // after the copy out of it
  char* h_stage[2] = {nullptr, nullptr};
  size_t stage_cap[2] = {0, 0};
  cudaEvent_t stage_ev[2] = {nullptr, nullptr};
  int stage_next = 0;
  // graph
  cudaGraphExec_t graph = nullptr;
  int graph_dpasses = -1, graph_ppasses = -1;
  int kernels_per_step = 0;
  // step accounting
  int64_t steps_enqueued = 0, steps_done = 0;
  std::deque<std::pair<int64_t, cudaEvent_t>> inflight;
  std::vector<cudaEvent_t> event_pool;
  std::vector<std::pair<int64_t, os_handle*>> graveyard;  // release once steps_done reaches
  std::vector<int> graveyard_slots;
  int64_t launches = 0;
  int64_t plan_cells = 0, plan_tiles = 0;
  int plan_members = 0;
};

namespace {

// Largest even tile height whose region fits shared memory, divided by
// `ty_div` (rounded to even): shorter tiles balance better across the SMs at
// the price of more halo rows.
TileGeom batch_geom(int halo, bool projection, int ty_div = 1) {
  TileGeom g{};
  g.halo = halo;
  g.TX = kRegionW - 2 * halo;
  int TY = 2;
  while (true) {
    const int next = TY + 2;
    const size_t sm = projection ? projection_smem(next + 2 * halo, false)
                                 : diffusion_smem(next + 2 * halo);
    if (sm + kStaticSmem > kMaxSmem) break;  // room for the kernels' static shared memory
    TY = next;
  }
  TY = std::max(2, (TY / std::max(1, ty_div)) & ~1);
  g.TY = TY;
  g.RH = TY + 2 * halo;
  g.smem = projection ? projection_smem(g.RH, false) : diffusion_smem(g.RH);
  return g;
}

size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

void release_member(os_handle* h) {
  cudaStreamSynchronize(h->stream);
  free_handle(h);
}

void free_batch(os_batch* b) {
  if (!b) return;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (auto& kv : b->members) release_member(kv.second.h);
  for (auto& g : b->graveyard) release_member(g.second);
  if (b->d_plan) cudaFree(b->d_plan);
  if (b->d_remaining) cudaFree(b->d_remaining);
  for (int i = 0; i < 2; i++) {
    if (b->h_stage[i]) cudaFreeHost(b->h_stage[i]);
    if (b->stage_ev[i]) cudaEventDestroy(b->stage_ev[i]);
  }
  for (auto& f : b->inflight) cudaEventDestroy(f.second);
  for (cudaEvent_t e : b->event_pool) cudaEventDestroy(e);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b->arena;
  delete b;
}

int batch_device(os_batch* b) {
  int cur = -1;
  CUDA_OR_RETURN(cudaGetDevice(&cur));
  if (cur != b->device) CUDA_OR_RETURN(cudaSetDevice(b->device));
  return OS_OK;
}

int build_batch_graph(os_batch* b, int dpasses, int ppasses) {
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  cudaStream_t st = b->stream;
  int kernels = 0;
  const PlanHeader* P = b->d_plan;
  int* R = b->d_remaining;
  const int row_grid = b->sms * 16;
  CUDA_OR_RETURN(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  k_batch_forces<<<row_grid, 128, 0, st>>>(P, R);
  kernels++;
  for (int p = 0; p < dpasses; p++, kernels++)
    k_batch_diffuse<<<b->sms, kBlockThreads, b->gd.smem, st>>>(P, R, p, b->K, b->gd.halo,
                                                                b->gd.TX, b->gd.TY);
  for (int p = 0; p < ppasses; p++, kernels++)
    k_batch_project<<<b->sms, kBlockThreads, b->gp.smem, st>>>(P, R, p, b->K, b->gp.halo,
                                                                b->gp.TX, b->gp.TY);
  k_batch_extrapolate<<<b->sms * 4, 1024, 0, st>>>(P, R);
  k_batch_advect_velocity<<<row_grid, 128, 0, st>>>(P, R);
  k_batch_advect_smoke<<<row_grid, 128, 0, st>>>(P, R);
  k_batch_finish_smoke<<<row_grid, 128, 0, st>>>(P, R);
  k_batch_tick<<<1, 256, 0, st>>>(P, R);
  kernels += 5;
  const cudaError_t le = cudaGetLastError();
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(st, &g);
  if (le != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return set_err(OS_ERR_CUDA, "batch launch: %s", cudaGetErrorString(le));
  }
  if (ce != cudaSuccess) return set_err(OS_ERR_CUDA, "batch capture: %s", cudaGetErrorString(ce));
  const cudaError_t ie = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) return set_err(OS_ERR_CUDA, "batch instantiate: %s", cudaGetErrorString(ie));
  b->graph_dpasses = dpasses;
  b->graph_ppasses = ppasses;
  b->kernels_per_step = kernels;
  return OS_OK;
}

ScenarioDesc describe(const os_batch* b, const os_handle* h) {
  ScenarioDesc d{};
  d.c = h->c;
  d.storage = h->storage;
  d.smoke_period = h->smoke_period;
  d.smoke_on = h->cfg.enable_smoke && h->cfg.tunnel_smoke != 0.0f;
  d.proj_passes = (h->c.n + b->K - 1) / b->K;
  d.diff_passes = h->cfg.viscosity != 0.0f ? d.proj_passes : 0;
  d.diff_tiles_x = (h->W + b->gd.TX - 1) / b->gd.TX;
  d.proj_tiles_x = (h->W + b->gp.TX - 1) / b->gp.TX;
  d.prm = h->d_params;
  d.u = h->u;
  d.v = h->v;
  d.ub = h->ub;
  d.vb = h->vb;
  d.s = h->s;
  d.sb = h->sb;
  d.flags = h->flags;
  d.nbr = h->nbr;
  return d;
}

// Writes the plan for the current members (those with steps still to run
// after the ones already enqueued) and enqueues its copy on `st`; members
// joining now get their step counts set on the device right after the copy.
int write_plan(os_batch* b, cudaStream_t st) {
  struct Entry {
    int64_t id;
    ScenarioDesc d;
    int slot, dtiles, ptiles;
  };
  std::vector<Entry> live;
  std::vector<int2> admits;
  int max_slot = 0, dpasses = 0, ppasses = 0;
  int64_t cells = 0;
  for (auto& kv : b->members) {
    os_batch::Member& m = kv.second;
    const bool was = m.in_plan;
    if (m.finish_at >= 0 && m.finish_at <= b->steps_enqueued) {
      m.in_plan = false;  // done by the time the next step runs
      continue;
    }
    Entry e;
    e.id = kv.first;
    e.d = describe(b, m.h);
    e.slot = m.slot;
    const int ty_d = (m.h->H + b->gd.TY - 1) / b->gd.TY, ty_p = (m.h->H + b->gp.TY - 1) / b->gp.TY;
    e.dtiles = e.d.diff_tiles_x * ty_d;
    e.ptiles = e.d.proj_tiles_x * ty_p;
    live.push_back(e);
    max_slot = std::max(max_slot, m.slot);
    dpasses = std::max(dpasses, e.d.diff_passes);
    ppasses = std::max(ppasses, e.d.proj_passes);
    cells += (int64_t)m.h->N;
    if (!was) {
      admits.push_back(make_int2(m.slot, m.steps < 0 ? -1 : m.steps));
      m.finish_at = m.steps < 0 ? -1 : b->steps_enqueued + m.steps;
      m.in_plan = true;
      m.scheduled = true;
    }
  }
  const int members = (int)live.size();
  const int slots = live.empty() ? 1 : max_slot + 1;

  // Layout: header, descriptors by slot, then the member orders.
  PlanHeader H{};
  size_t off = align16(sizeof(PlanHeader));
  H.off_desc = (int)off;
  off = align16(off + (size_t)slots * sizeof(ScenarioDesc));
  int64_t dtiles = 0, ptiles = 0;
  for (const Entry& e : live) {
    dtiles += e.dtiles;
    ptiles += e.ptiles;
  }
  if (dtiles > INT32_MAX || ptiles > INT32_MAX)
    return set_err(OS_ERR_UNSUPPORTED, "batch has too many tiles");
  H.off_slot = (int)off;
  off = align16(off + (size_t)std::max(members, 1) * sizeof(int));
  H.off_cell_cum = (int)off;
  off = align16(off + (size_t)std::max(members, 1) * sizeof(int64_t));
  H.off_diff_tiles = (int)off;
  off = align16(off + (size_t)std::max<int64_t>(dtiles, 1) * sizeof(TileRef));
  H.off_proj_tiles = (int)off;
  off = align16(off + (size_t)std::max<int64_t>(ptiles, 1) * sizeof(TileRef));
  H.off_admit = (int)off;
  off = align16(off + std::max<size_t>(admits.size(), 1) * sizeof(int2));
  const size_t bytes = off;
  if (bytes > (size_t)INT32_MAX) return set_err(OS_ERR_UNSUPPORTED, "batch plan too large");

  // Device room: the plan and the countdowns; growing either moves it, so the
  // graph (whose kernels hold the pointers) is rebuilt after in-flight steps.
  bool rebuild = b->graph == nullptr || dpasses > b->graph_dpasses || ppasses > b->graph_ppasses;
  if (bytes > b->plan_cap || slots > b->remaining_cap) {
    CUDA_OR_RETURN(cudaStreamSynchronize(st));
    CUDA_OR_RETURN(cudaStreamSynchronize(b->stream));
    if (bytes > b->plan_cap) {
      const size_t cap = std::max(bytes, 2 * b->plan_cap);
      if (b->d_plan) cudaFree(b->d_plan);
      b->d_plan = nullptr;
      b->plan_cap = 0;
      CUDA_OR_RETURN(cudaMalloc(&b->d_plan, cap));
      b->plan_cap = cap;
    }
    if (slots > b->remaining_cap) {
      const int cap = std::max(slots, std::max(256, 2 * b->remaining_cap));
      int* fresh = nullptr;
      CUDA_OR_RETURN(cudaMalloc(&fresh, (size_t)cap * sizeof(int)));
      CUDA_OR_RETURN(cudaMemset(fresh, 0, (size_t)cap * sizeof(int)));
      if (b->d_remaining) {
        CUDA_OR_RETURN(cudaMemcpy(fresh, b->d_remaining, (size_t)b->remaining_cap * sizeof(int),
                                  cudaMemcpyDeviceToDevice));
        cudaFree(b->d_remaining);
      }
      b->d_remaining = fresh;
      b->remaining_cap = cap;
    }
    rebuild = true;
  }
  if (rebuild) {
    if (b->graph) {
      CUDA_OR_RETURN(cudaStreamSynchronize(st));
      CUDA_OR_RETURN(cudaStreamSynchronize(b->stream));
    }
    // Room for n up to the largest seen, so later members rarely force this.
    int rc = build_batch_graph(b, std::max(dpasses, b->graph_dpasses),
                               std::max(ppasses, b->graph_ppasses));
    if (rc) return rc;
  }

  // Staging buffer: wait for the copy that last used it.
  const int sidx = b->stage_next;
  b->stage_next ^= 1;
  CUDA_OR_RETURN(cudaEventSynchronize(b->stage_ev[sidx]));
  if (bytes > b->stage_cap[sidx]) {
    if (b->h_stage[sidx]) cudaFreeHost(b->h_stage[sidx]);
    b->h_stage[sidx] = nullptr;
    b->stage_cap[sidx] = 0;
    const size_t cap = std::max(bytes, 2 * b->stage_cap[sidx ^ 1]);
    CUDA_OR_RETURN(cudaMallocHost(&b->h_stage[sidx], cap));
    b->stage_cap[sidx] = cap;
  }
  char* base = b->h_stage[sidx];
  memset(base, 0, bytes);
  ScenarioDesc* desc = reinterpret_cast<ScenarioDesc*>(base + H.off_desc);
  int* slot_of = reinterpret_cast<int*>(base + H.off_slot);
  int64_t* cell_cum = reinterpret_cast<int64_t*>(base + H.off_cell_cum);
  int64_t total = 0;
  for (int k = 0; k < members; k++) {
    const Entry& e = live[k];
    desc[e.slot] = e.d;
    slot_of[k] = e.slot;
    cell_cum[k] = total;
    total += (int64_t)e.d.c.W * e.d.c.H;
  }
  // Tiles by passes (descending): pass p covers the prefix of members with
  // more than p passes.
  auto order = [&](bool diffusion, TileRef* out, int* items) {
    std::vector<int> idx(members);
    for (int k = 0; k < members; k++) idx[k] = k;
    auto passes = [&](int k) { return diffusion ? live[k].d.diff_passes : live[k].d.proj_passes; };
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int c) { return passes(a) > passes(c); });
    const TileGeom& g = diffusion ? b->gd : b->gp;
    std::vector<int64_t> cum(members + 1);
    int64_t n = 0;
    for (int k = 0; k < members; k++) {
      const Entry& e = live[idx[k]];
      cum[k] = n;
      const int tiles_x = diffusion ? e.d.diff_tiles_x : e.d.proj_tiles_x;
      const int tiles_y = (e.d.c.H + g.TY - 1) / g.TY;
      for (int ty = 0; ty < tiles_y; ty++)
        for (int tx = 0; tx < tiles_x; tx++)
          out[n++] = TileRef{e.slot, (int16_t)tx, (int16_t)ty};
    }
    cum[members] = n;
    int64_t per_step = 0;
    for (int p = 0, k = members; p < kBatchMaxPasses; p++) {
      while (k > 0 && passes(idx[k - 1]) <= p) k--;
      items[p] = (int)cum[k];
      per_step += cum[k];
    }
    return per_step;
  };
  int64_t tiles = order(true, reinterpret_cast<TileRef*>(base + H.off_diff_tiles), H.diff_items);
  tiles += order(false, reinterpret_cast<TileRef*>(base + H.off_proj_tiles), H.proj_items);
  int2* adm = reinterpret_cast<int2*>(base + H.off_admit);
  for (size_t k = 0; k < admits.size(); k++) adm[k] = admits[k];
  H.members = members;
  H.cells = total;
  H.admits = (int)admits.size();
  memcpy(base, &H, sizeof H);

  CUDA_OR_RETURN(cudaMemcpyAsync(b->d_plan, base, bytes, cudaMemcpyHostToDevice, st));
  CUDA_OR_RETURN(cudaEventRecord(b->stage_ev[sidx], st));
  if (!admits.empty()) {
    k_batch_admit<<<1, 256, 0, st>>>(b->d_plan, b->d_remaining);
    CUDA_OR_RETURN(cudaGetLastError());
    b->launches++;
  }
  b->plan_members = members;
  b->plan_cells = cells;
  b->plan_tiles = tiles;
  b->dirty = false;
  return OS_OK;
}

// Completed steps, as far as the recorded events tell without waiting.
int batch_progress(os_batch* b) {
  while (!b->inflight.empty()) {
    const cudaError_t q = cudaEventQuery(b->inflight.front().second);
    if (q == cudaErrorNotReady) break;
    if (q != cudaSuccess) return set_err(OS_ERR_CUDA, "batch step: %s", cudaGetErrorString(q));
    b->steps_done = std::max(b->steps_done, b->inflight.front().first);
    b->event_pool.push_back(b->inflight.front().second);
    b->inflight.pop_front();
  }
  // Cancelled members whose last enqueued steps have completed.
  for (size_t k = 0; k < b->graveyard.size();) {
    if (b->graveyard[k].first <= b->steps_done) {
      release_member(b->graveyard[k].second);
      b->free_slots.push_back(b->graveyard_slots[k]);
      b->graveyard[k] = b->graveyard.back();
      b->graveyard_slots[k] = b->graveyard_slots.back();
      b->graveyard.pop_back();
      b->graveyard_slots.pop_back();
    } else {
      k++;
    }
  }
  return OS_OK;
}

// Blocking depth and tile height for the whole batch; the plan and graph are
// rewritten at the next step.
int set_geometry(os_batch* b, int K, int ty_div) {
  if (b->graph) {
    CUDA_OR_RETURN(cudaStreamSynchronize(b->stream));
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  b->graph_dpasses = b->graph_ppasses = -1;
  b->K = K;
  b->ty_div = ty_div;
  b->gd = batch_geom(K, false, ty_div);
  b->gp = batch_geom(2 * K, true, ty_div);
  cudaFuncSetAttribute(k_batch_diffuse, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)b->gd.smem);
  cudaFuncSetAttribute(k_batch_project, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)b->gp.smem);
  for (auto& kv : b->members) {
    kv.second.h->block_k = K;
    kv.second.h->cfg.projection_block = K;
  }
  b->dirty = true;
  CUDA_OR_RETURN(cudaGetLastError());
  return OS_OK;
}

int write_plan(os_batch* b, cudaStream_t st);

// Autotuner of a fixed batch: times a few steps of every blocking depth and
// tile height on the members' freshly created (all-zero) fields, keeps the
// fastest, and zeroes the fields again, so the members start exactly as
// os_create leaves them.
int tune_batch(os_batch* b) {
  struct Cand {
    int K, div;
  };
  std::vector<Cand> cands;
  for (int K : {4, 6, 8, 12})
    for (int div : {1, 2}) cands.push_back({K, div});
  int max_n = 0;
  for (auto& kv : b->members) max_n = std::max(max_n, kv.second.h->c.n);
  cudaEvent_t a = nullptr, z = nullptr;
  CUDA_OR_RETURN(cudaEventCreate(&a));
  CUDA_OR_RETURN(cudaEventCreate(&z));
  Cand best{b->K, b->ty_div};
  float best_ms = 0.0f;
  int rc = OS_OK;
  for (const Cand& cd : cands) {
    if ((max_n + cd.K - 1) / cd.K > kBatchMaxPasses) continue;
    if ((rc = set_geometry(b, cd.K, cd.div)) || (rc = write_plan(b, b->stream))) break;
    CUDA_OR_RETURN(cudaGraphLaunch(b->graph, b->stream));  // warm-up
    cudaEventRecord(a, b->stream);
    for (int t = 0; t < 3; t++) CUDA_OR_RETURN(cudaGraphLaunch(b->graph, b->stream));
    cudaEventRecord(z, b->stream);
    CUDA_OR_RETURN(cudaEventSynchronize(z));
    float ms = 0.0f;
    CUDA_OR_RETURN(cudaEventElapsedTime(&ms, a, z));
    b->launches += 4LL * b->kernels_per_step;
    if (best_ms == 0.0f || ms < best_ms) {
      best_ms = ms;
      best = cd;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(z);
  if (rc) return rc;
  if ((rc = set_geometry(b, best.K, best.div)) || (rc = write_plan(b, b->stream))) return rc;
  for (auto& kv : b->members) {
    os_handle* h = kv.second.h;
    const size_t fb = h->N * h->esize;
    void* fields[] = {h->u, h->v, h->s, h->ub, h->vb, h->sb};
    for (void* f : fields) CUDA_OR_RETURN(cudaMemsetAsync(f, 0, fb, b->stream));
    CUDA_OR_RETURN(cudaMemsetAsync(h->p, 0, h->N * 4, b->stream));
  }
  CUDA_OR_RETURN(cudaStreamSynchronize(b->stream));
  return OS_OK;
}

int new_batch(int device, int block_k, uint64_t budget, os_batch** out) {
  os_batch* b = new (std::nothrow) os_batch();
  if (!b) return set_err(OS_ERR_NOMEM, "host allocation failed");
  b->K = block_k > 0 ? std::min(block_k, 16) : 8;
  b->device = device;
  auto fail = [&](int code) {
    free_batch(b);
    return code;
  };
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail(set_err(OS_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e)));
  b->sms = sm_count(device);
  if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return fail(set_err(OS_ERR_CUDA, "stream: %s", cudaGetErrorString(e)));
  for (int i = 0; i < 2; i++)
    if ((e = cudaEventCreateWithFlags(&b->stage_ev[i], cudaEventDisableTiming)) != cudaSuccess)
      return fail(set_err(OS_ERR_CUDA, "event: %s", cudaGetErrorString(e)));
  if (budget > 0) {
    b->arena = new (std::nothrow) Arena();
    if (!b->arena) return fail(set_err(OS_ERR_NOMEM, "host allocation failed"));
    if (b->arena->init(budget))
      return fail(set_err(OS_ERR_NOMEM, "device budget of %llu bytes could not be reserved",
                          (unsigned long long)budget));
  }
  b->gd = batch_geom(b->K, false);
  b->gp = batch_geom(2 * b->K, true);
  cudaFuncSetAttribute(k_batch_diffuse, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)b->gd.smem);
  cudaFuncSetAttribute(k_batch_project, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)b->gp.smem);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return fail(set_err(OS_ERR_CUDA, "batch set-up: %s", cudaGetErrorString(e)));
  *out = b;
  return OS_OK;
}

int check_member_config(const os_batch* b, const os_config& c) {
  int rc = validate(&c);
  if (rc) return rc;
  if (c.storage == OS_STORAGE_F64 || c.enable_pressure || c.device != b->device)
    return set_err(OS_ERR_UNSUPPORTED,
                   "batched scenarios are FP32, FP16 or BF16 with pressure off, on the batch's "
                   "device");
  if (c.height / 2 > INT16_MAX || c.width / 16 > INT16_MAX)
    return set_err(OS_ERR_UNSUPPORTED, "grid too large for a batch's tile numbering");
  if ((c.projection_n + b->K - 1) / b->K > kBatchMaxPasses)
    return set_err(OS_ERR_UNSUPPORTED, "sim.projection.n above %d at %d sweeps per pass",
                   kBatchMaxPasses * b->K, b->K);
  return OS_OK;
}

int add_member(os_batch* b, const os_config& cfg, int32_t steps, int64_t* id) {
  os_config c = cfg;
  c.projection_block = b->K;
  os_handle* h = nullptr;
  int rc = create_handle(&c, b->arena, &h);
  if (rc) return rc;
  if ((rc = push_params(h, nullptr, c.d_t, h->stream))) {
    release_member(h);
    return rc;
  }
  const cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    release_member(h);
    return set_err(OS_ERR_CUDA, "scenario set-up: %s", cudaGetErrorString(e));
  }
  os_batch::Member m;
  m.h = h;
  m.steps = steps;
  if (!b->free_slots.empty()) {
    std::sort(b->free_slots.begin(), b->free_slots.end(), std::greater<int>());
    m.slot = b->free_slots.back();
    b->free_slots.pop_back();
  } else {
    m.slot = b->slot_hw++;
  }
  const int64_t mid = b->next_id++;
  b->members[mid] = m;
  b->dirty = true;
  *id = mid;
  return OS_OK;
}

}  // namespace

extern "C" {

int os_batch_create(const os_config* cfgs, int32_t count, int32_t block_k, os_batch** out) {
  if (!cfgs || !out || count < 1) return set_err(OS_ERR_INVALID, "bad argument");
  *out = nullptr;
  for (int i = 0; i < count; i++) {
    int rc = validate(&cfgs[i]);
    if (rc) return rc;
    if (cfgs[i].device != cfgs[0].device)
      return set_err(OS_ERR_UNSUPPORTED, "batched scenarios share one device (scenario %d)", i);
  }
  os_batch* b = nullptr;
  int rc = new_batch(cfgs[0].device, block_k, 0, &b);
  if (rc) return rc;
  for (int i = 0; i < count; i++) {
    int64_t id;
    if ((rc = check_member_config(b, cfgs[i])) || (rc = add_member(b, cfgs[i], -1, &id))) {
      free_batch(b);
      return rc;
    }
  }
  if ((rc = write_plan(b, b->stream))) {
    free_batch(b);
    return rc;
  }
  const char* env = std::getenv("OPENSAYAL_GB300_AUTOTUNE");
  if (block_k == 0 && !(env && env[0] == '0') && (rc = tune_batch(b))) {
    free_batch(b);
    return rc;
  }
  *out = b;
  return OS_OK;
}

int os_batch_create_dynamic(int32_t device, int32_t block_k, uint64_t budget_bytes, os_batch** out) {
  if (!out) return set_err(OS_ERR_INVALID, "null argument");
  *out = nullptr;
  return new_batch(device, block_k, budget_bytes, out);
}

int os_batch_add(os_batch* b, const os_config* cfg, int32_t steps, int64_t* id) {
  if (!b || !cfg || !id) return set_err(OS_ERR_INVALID, "null argument");
  if (steps == 0) return set_err(OS_ERR_INVALID, "steps must be positive (or negative: unlimited)");
  int rc = check_member_config(b, *cfg);
  if (rc) return rc;
  if ((rc = batch_device(b))) return rc;
  return add_member(b, *cfg, steps, id);
}

int os_batch_remove(os_batch* b, int64_t id) {
  if (!b) return set_err(OS_ERR_INVALID, "null batch");
  auto it = b->members.find(id);
  if (it == b->members.end()) return set_err(OS_ERR_INVALID, "no scenario %lld", (long long)id);
  int rc = batch_device(b);
  if (rc) return rc;
  if ((rc = batch_progress(b))) return rc;
  os_batch::Member m = it->second;
  b->members.erase(it);
  if (!m.scheduled || (m.finish_at >= 0 && m.finish_at <= b->steps_done)) {
    // Never stepped, or frozen on the device: nothing in flight touches it.
    release_member(m.h);
    b->free_slots.push_back(m.slot);
    return OS_OK;
  }
  // Steps that touch it are still enqueued: keep it until they have run, and
  // take it out of the plan before the next step.
  const int64_t last = m.finish_at >= 0 ? std::min(m.finish_at, b->steps_enqueued)
                                        : b->steps_enqueued;
  b->graveyard.push_back({last, m.h});
  b->graveyard_slots.push_back(m.slot);
  if (m.in_plan) b->dirty = true;
  return OS_OK;
}

int os_batch_destroy(os_batch* b) {
  if (!b) return OS_OK;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  for (auto& f : b->inflight) cudaEventSynchronize(f.second);
  free_batch(b);
  return OS_OK;
}

int os_batch_step(os_batch* b, int32_t steps, void* stream) {
  if (!b || steps < 0) return set_err(OS_ERR_INVALID, "bad argument");
  int rc = batch_device(b);
  if (rc) return rc;
  if (steps == 0) return OS_OK;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : b->stream;
  if ((rc = batch_progress(b))) return rc;
  // Members whose last step is already enqueued leave the plan.
  for (auto& kv : b->members)
    if (kv.second.in_plan && kv.second.finish_at >= 0 && kv.second.finish_at <= b->steps_enqueued)
      b->dirty = true;
  if (b->dirty && (rc = write_plan(b, st))) return rc;
  for (int t = 0; t < steps; t++) CUDA_OR_RETURN(cudaGraphLaunch(b->graph, st));
  b->steps_enqueued += steps;
  b->launches += (int64_t)steps * b->kernels_per_step;
  cudaEvent_t ev;
  if (!b->event_pool.empty()) {
    ev = b->event_pool.back();
    b->event_pool.pop_back();
  } else {
    CUDA_OR_RETURN(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  }
  CUDA_OR_RETURN(cudaEventRecord(ev, st));
  b->inflight.push_back({b->steps_enqueued, ev});
  return OS_OK;
}

int os_batch_synchronize(os_batch* b) {
  if (!b) return set_err(OS_ERR_INVALID, "null batch");
  int rc = batch_device(b);
  if (rc) return rc;
  CUDA_OR_RETURN(cudaStreamSynchronize(b->stream));
  for (auto& f : b->inflight) CUDA_OR_RETURN(cudaEventSynchronize(f.second));
  return batch_progress(b);
}

int os_batch_poll(os_batch* b, int32_t wait, int64_t* ids, int32_t cap, int32_t* count) {
  if (!b || !count || (cap > 0 && !ids)) return set_err(OS_ERR_INVALID, "null argument");
  *count = 0;
  int rc = batch_device(b);
  if (rc) return rc;
  auto collect = [&]() {
    int n = 0;
    for (auto& kv : b->members) {
      os_batch::Member& m = kv.second;
      if (m.reported || m.finish_at < 0 || m.finish_at > b->steps_done) continue;
      if (n >= cap) break;
      ids[n++] = kv.first;
      m.reported = true;
    }
    return n;
  };
  if ((rc = batch_progress(b))) return rc;
  int n = collect();
  // Waiting: block on enqueued steps, oldest first, until something finishes.
  while (wait && n == 0 && cap > 0 && !b->inflight.empty()) {
    bool pending = false;
    for (auto& kv : b->members)
      if (!kv.second.reported && kv.second.finish_at >= 0 &&
          kv.second.finish_at <= b->steps_enqueued)
        pending = true;
    if (!pending) break;
    CUDA_OR_RETURN(cudaEventSynchronize(b->inflight.front().second));
    if ((rc = batch_progress(b))) return rc;
    n = collect();
  }
  *count = n;
  return OS_OK;
}

int os_batch_wait(os_batch* b, int64_t max_in_flight) {
  if (!b || max_in_flight < 0) return set_err(OS_ERR_INVALID, "bad argument");
  int rc = batch_device(b);
  if (rc) return rc;
  if ((rc = batch_progress(b))) return rc;
  while (b->steps_enqueued - b->steps_done > max_in_flight && !b->inflight.empty()) {
    CUDA_OR_RETURN(cudaEventSynchronize(b->inflight.front().second));
    if ((rc = batch_progress(b))) return rc;
  }
  return OS_OK;
}

int os_batch_status(os_batch* b, int64_t id, int32_t* state, int64_t* steps_left) {
  if (!b || !state || !steps_left) return set_err(OS_ERR_INVALID, "null argument");
  auto it = b->members.find(id);
  if (it == b->members.end()) return set_err(OS_ERR_INVALID, "no scenario %lld", (long long)id);
  int rc = batch_progress(b);
  if (rc) return rc;
  const os_batch::Member& m = it->second;
  if (!m.scheduled) {
    *state = OS_MEMBER_WAITING;
    *steps_left = m.steps;
  } else if (m.finish_at < 0) {
    *state = OS_MEMBER_RUNNING;
    *steps_left = -1;
  } else if (m.finish_at <= b->steps_done) {
    *state = OS_MEMBER_DONE;
    *steps_left = 0;
  } else {
    *state = OS_MEMBER_RUNNING;
    *steps_left = std::min<int64_t>(m.steps, m.finish_at - b->steps_done);
  }
  return OS_OK;
}

int os_batch_memory(os_batch* b, uint64_t* used, uint64_t* budget) {
  if (!b || !used || !budget) return set_err(OS_ERR_INVALID, "null argument");
  if (b->arena) {
    *used = b->arena->used();
    *budget = b->arena->capacity();
  } else {
    uint64_t sum = 0;
    for (auto& kv : b->members) sum += kv.second.h->device_bytes;
    *used = sum;
    *budget = 0;
  }
  return OS_OK;
}

int os_batch_scenario(os_batch* b, int64_t id, os_handle** out) {
  if (!b || !out) return set_err(OS_ERR_INVALID, "null argument");
  auto it = b->members.find(id);
  if (it == b->members.end()) return set_err(OS_ERR_INVALID, "no scenario %lld", (long long)id);
  *out = it->second.h;
  return OS_OK;
}

int os_batch_info(os_batch* b, os_batch_stats* out) {
  if (!b || !out) return set_err(OS_ERR_INVALID, "null argument");
  memset(out, 0, sizeof *out);
  out->scenarios = (int32_t)b->members.size();
  out->block_k = b->K;
  out->kernels_per_step = b->kernels_per_step;
  out->members_in_plan = b->plan_members;
  out->cells = b->plan_cells;
  out->launches = b->launches;
  out->tile_items_per_step = b->plan_tiles;
  out->steps_enqueued = b->steps_enqueued;
  out->steps_completed = b->steps_done;
  out->projection_tile_rows = b->gp.TY;
  out->diffusion_tile_rows = b->gd.TY;
  return OS_OK;
}

}  // extern "C"
