#!/usr/bin/env python
"""Throughput of the GB300 wind-tunnel step in cell-steps/s.

Workload: the reference's default tunnel, 1920x1080, n=50 red/black sweeps,
viscosity 0.001 (n Jacobi diffusion sweeps), smoke on, drain on, g=-5,
dt=0.05, seeded uniform[-0.01, 0.01] velocity perturbation (synthetic: the
reference has no dataset). A step is one Fluid::update.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

value  : W*H*K / (sum of the K per-step CUDA-event times), fields resident in
         HBM, L2 flushed between steps (a 256 MiB write outside the timed
         events; the step's own working set fits in the 129 MB L2).
e2e    : the same metric through the C ABI as the reference's frame loop uses
         it: a synchronous os_update() (whose new d_t goes host->device) and a
         device->host read of the smoke field into pinned memory, every step.
N > 1  : independent replicas, one grid per GPU (the path does not shard);
         value = all ranks' cell-steps / the slowest rank's time.
--impl reference: the reference's per-cell update as a CPU loop on all host
         cores (the oracle port; the reference has no CPU build of its own),
         plus, where a GPU is present, the reference's own CUDA kernels driven
         as its Fluid::update drives them.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-steps/s (incl. n sweeps) 1920x1080 & batched; serve p50/p99 vs plain, same GPU"
UNIT = "cell-steps/s"
FALLBACK_HBM_GBS = 6800.0
L2_FLUSH_BYTES = 256 << 20


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": FALLBACK_HBM_GBS, "source": "fallback"}


def l2_copy_peak(device: int) -> dict:
    """The L2 copy bandwidth, measured live: the library's bandwidth probe
    (one launch copying a buffer back and forth `reps` times with
    cache-at-L2 loads and stores) on buffers whose pair fits in the 129 MB
    L2; the best of three runs per size is kept. The stencil phases keep
    their sweeps on the SM and exchange through L2, so this is the level
    their effective rate is compared with."""
    import ctypes as C
    from opensayal_gb300 import native
    lib = native.load()
    best = {"gbs": 0.0}
    for mib in (8, 16, 24):
        for _ in range(3):
            g = C.c_float()
            native.check(lib.os_probe_copy_bandwidth(device, mib << 20, 200, C.byref(g)))
            if g.value > best["gbs"]:
                best = {"gbs": float(g.value), "buffer_mib": mib}
    best["how"] = ("os_probe_copy_bandwidth: two buffers of 8-24 MiB copied back and forth 200 "
                   "times in one launch (ld/st.global.cg), read+write bytes / CUDA-event time, "
                   "best of 3 per size")
    return best


def bytes_per_cell_step(n: int, viscous: bool) -> int:
    """Compulsory FP32 traffic of an unfused phase-per-pass schedule (1-byte
    flags): forces 8, diffusion 8/sweep, projection 17/sweep, advection 17+17."""
    return (25 if viscous else 17) * n + 42


class Clocks:
    """nvidia-smi samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        self.samples = []
        if self.proc is None:
            return
        time.sleep(0.3)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        for line in out.strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def summary(self) -> dict:
        if not getattr(self, "samples", None):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        reasons = set()
        for s in self.samples:
            for name, val in zip(self.NAMES, s[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def dist_max(world, x: float) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() and dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(world, x: float) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() and dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t)
    return float(t.item())


def cpu_baseline(cfg, budget_s: float = 15.0, max_steps: int = 400) -> dict:
    """The oracle port on the host cores (rank 0, N=1 only)."""
    import oracle
    from opensayal_gb300 import scenarios
    o = oracle.OracleFluid(cfg)
    u, v = scenarios.perturbation(2, o.is_solid)
    o.u[:], o.v[:] = u, v
    o.update(None, cfg.d_t)  # first touch of the working set
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps:
        o.update(None, cfg.d_t)
        steps += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return {"value": cfg.width * cfg.height * steps / el, "unit": UNIT,
            "cores": oracle.oracle_threads(), "kind": "port",
            "sample": f"{steps} full {cfg.width}x{cfg.height} steps of the C/OpenMP restatement "
                      f"({el:.1f} s)"}


def workload_config(name: str):
    from opensayal_gb300 import scenarios
    return {"default": scenarios.default_tunnel_config, "small": scenarios.small_config,
            "large": scenarios.large_config}[name]()


def config_record(cfg, name: str, world: int) -> dict:
    """The workload, and only the workload: both arms print the same record."""
    return {"workload": f"{name}: {cfg.width}x{cfg.height} tunnel, n={cfg.projection_n}, "
                        f"o={cfg.projection_o:g}, viscosity={cfg.viscosity:g}, g={cfg.g:g}, "
                        f"dt={cfg.d_t:g}, drain={cfg.enable_drain}, smoke={cfg.enable_smoke}",
            "width": cfg.width, "height": cfg.height, "projection_n": cfg.projection_n,
            "storage": ["f32", "f16", "bf16", "f64"][cfg.storage],
            "l2": "GPU steps: flushed between timed steps (256 MiB write outside the events)",
            "parallelism": "replicas" if world > 1 else "single", "global_batch": world}


def time_visuals(f, cfg, sptr, stream, pk) -> dict:
    """Headless visuals on the workload's fields: pixel colours (reads smoke
    and the flag byte, writes one word: 9 B per cell), and the arrows and path
    lines at the reference's default spacing; CUDA events, 20 calls each."""
    import torch
    from opensayal_gb300.fluid import visual_defaults
    from opensayal_gb300.native import OsArrow
    import ctypes as C
    v = visual_defaults()
    cells = cfg.width * cfg.height
    pix = torch.empty(cells, dtype=torch.int32, device="cuda")
    aw, ah = cfg.width // v.arrow_distance, cfg.height // v.arrow_distance
    arrows = torch.empty(max(1, aw * ah) * C.sizeof(OsArrow) // 4, dtype=torch.int32, device="cuda")
    tw, th = cfg.width // v.trace_distance, cfg.height // v.trace_distance
    tx = torch.empty(max(1, tw * th * v.trace_length), dtype=torch.int32, device="cuda")
    ty = torch.empty_like(tx)
    calls = {
        "pixels": lambda: f.render_pixels(pix.data_ptr(), sptr),
        "arrows": lambda: f.render_arrows(v, arrows.data_ptr(), sptr),
        "traces": lambda: f.render_traces(v, cfg.d_t, tx.data_ptr(), ty.data_ptr(), sptr),
    }
    out = {}
    for name, fn in calls.items():
        fn()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(20):
            fn()
        b.record(stream)
        b.synchronize()
        out[name + "_us"] = a.elapsed_time(b) / 20 * 1e3
    gbs = 9 * cells / (out["pixels_us"] * 1e-6) / 1e9
    out["pixels_gbs"] = gbs
    out["pixels_frac"] = gbs / pk["hbm_gbs"]
    out["note"] = "pixels: 9 B/cell (smoke, flag, pixel word); L2-warm back-to-back calls"
    return out


def run_gb300(args, world, rank, local) -> dict | None:
    import torch
    from opensayal_gb300 import Fluid, native, scenarios
    from opensayal_gb300.build import build_library
    build_library()
    torch.cuda.set_device(local)
    cfg = workload_config(args.workload)
    cfg.device = local
    if args.block is not None:
        cfg.projection_block = args.block
    if args.resident is not None:
        cfg.projection_resident = args.resident
    if args.diffusion_block is not None:
        cfg.diffusion_block = args.diffusion_block
    cells = cfg.width * cfg.height
    f = Fluid(cfg)
    u, v = scenarios.perturbation(2, f.download("is_solid"))
    f.upload("vel_x", u)
    f.upload("vel_y", v)
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    dt = cfg.d_t
    with torch.cuda.stream(stream):
        f.update_async(None, dt, max(args.warmup, 3), sptr)
    stream.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    launches0 = f.kernel_launches
    dist_barrier(world)
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        wall0 = time.perf_counter()
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.add_(1.0)
                starts[k].record(stream)
                f.update_async(None, dt, 1, sptr)
                ends[k].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    dist_barrier(world)
    launches = f.kernel_launches - launches0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_s = dist_max(world, sum(step_ms) / 1e3)
    value = world * cells * args.steps / total_s

    # e2e: the step and the read-back of its smoke field through the C ABI,
    # every step: the new d_t goes host->device (it alternates by one ulp, as
    # real-time mode changes it every frame), os_update_async enqueues the
    # step, os_snapshot_async copies the smoke into one of two device
    # buffers, and a second stream copies that buffer into pinned host memory
    # while the next step runs. Timed on the host clock from the first
    # enqueue to the last copy's completion.
    cells_f = cells
    pinned = [torch.empty(cells_f, dtype=torch.float32, pin_memory=True) for _ in range(2)]
    snap = [torch.empty(cells_f, dtype=torch.float32, device="cuda") for _ in range(2)]
    copy_stream = torch.cuda.Stream()
    copied = [torch.cuda.Event() for _ in range(2)]
    dts = [dt, float(np.nextafter(np.float32(dt), np.float32(1.0)))]
    # At least 200 steps, after 10 untimed ones of the same pattern, so that a
    # single host-side delay does not decide a run of a few milliseconds.
    e2e_steps = max(args.steps, 200)

    def pipelined(nsteps):
        for k in range(nsteps):
            b = k & 1
            f.update_async(None, dts[b], 1, sptr)
            if k >= 2:
                stream.wait_event(copied[b])  # copy k-2 has read snap[b]
            f.snapshot_async("smoke", snap[b].data_ptr(), sptr)
            ready = torch.cuda.Event()
            ready.record(stream)
            copy_stream.wait_event(ready)
            with torch.cuda.stream(copy_stream):
                pinned[b].copy_(snap[b], non_blocking=True)
            copied[b].record(copy_stream)
        torch.cuda.synchronize()

    pipelined(10)
    dist_barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pipelined(e2e_steps)
    e2e_s = dist_max(world, time.perf_counter() - t0)
    # the reference's pattern, for comparison: synchronous update, then the read-back
    pinned_np = pinned[0].numpy()
    for k in range(10):
        f.update(None, dts[k & 1])
        f.download("smoke", out=pinned_np)
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        f.update(None, dts[k & 1])
        f.download("smoke", out=pinned_np)
    sync_s = dist_max(world, time.perf_counter() - t0)
    e2e = {"value": world * cells * e2e_steps / e2e_s, "unit": UNIT, "steps": e2e_steps,
           "h2d_bytes_per_step": 32, "d2h_bytes_per_step": 4 * cells,
           "how": "os_update_async + os_snapshot_async on the step's stream, the device-to-"
                  "host copy of each step's smoke on a second stream overlapping the next step",
           "synchronous": {"value": world * cells * e2e_steps / sync_s,
                           "how": "os_update (synchronous) then os_download of the smoke, "
                                  "every step, as the reference's frame loop does"}}

    # roofline of the dominant phase (projection), timed alone on the same
    # stream: CUDA events around the phase's own kernels, as the step runs
    # them (a phase called on its own also copies the velocity back to the
    # public fields when its pass count leaves it in the other buffers; that
    # copy is timed apart and left out)
    pk = peaks()
    proj_kms, proj_ms, proj_kernels = f.profile_phase_kernels(native.PHASE_PROJECTION, None, dt,
                                                              3, sptr)
    proj_s = proj_kms / 3 / 1e3
    proj_bytes = 17 * cfg.projection_n * cells
    diff_kms, diff_ms, diff_kernels = f.profile_phase_kernels(native.PHASE_DIFFUSION, None, dt,
                                                              3, sptr)
    achieved = proj_bytes / proj_s / 1e9
    # DRAM bytes of the projection phase: per launch from the ncu capture
    # summarised in profiles/ (same workload and blocking depth) or scaled
    # from one, as the entry says, times the phase's launches; null when the
    # configuration was not captured.
    traffic, traffic_source, on_chip = None, "not captured for this configuration", None
    # launches of the projection kernel in one phase: one resident launch, or
    # one blocked launch per pass
    k_proj = (1 if f.fields().projection_resident else
              -(-cfg.projection_n // max(1, f.fields().projection_block)))
    tfile = ROOT / "profiles" / "roofline_traffic.json"
    if tfile.exists():
        key = f"{args.workload}:block{f.fields().projection_block}" + (
            ":resident" if f.fields().projection_resident else "")
        entry = json.loads(tfile.read_text()).get(key)
        if entry:
            traffic = entry["bytes_per_launch"] * k_proj
            traffic_source = entry["source"]
            if "smsp__issue_active" in entry:
                on_chip = {"smsp__issue_active": entry["smsp__issue_active"],
                           "l1tex__throughput": entry["l1tex__throughput"],
                           "source": "the same capture"}
    step_bytes = bytes_per_cell_step(cfg.projection_n, cfg.viscosity != 0.0)
    l2 = l2_copy_peak(local)
    ms_per_step = total_s * 1e3 / args.steps
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": ["f32", "f16", "bf16", "f64"][cfg.storage], "data": "synthetic",
        "config": config_record(cfg, args.workload, world),
        "tuning": {"kernels_per_step": launches // max(1, args.steps),
                   "projection_block": f.fields().projection_block,
                   "projection_resident": f.fields().projection_resident,
                   "projection_block_source": "autotuned" if cfg.projection_block == 0 else "fixed"},
        "e2e": e2e,
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved / pk["hbm_gbs"], "traffic": traffic,
                     "traffic_source": traffic_source,
                     "kernel": "projection phase (17 B/cell per red/black sweep x n sweeps)",
                     "kernels_per_phase_timed": k_proj,
                     "launches_per_phase_with_copy_back": proj_kernels // 3,
                     "peak_source": pk["source"]},
        # The projection's sweeps run in shared memory and its halo exchanges
        # go through L2; DRAM sees the fields about once per phase. The level
        # that binds is on-chip, so the same algorithmic rate is also given
        # against a live L2-resident copy.
        "roofline_l2": {"bound": "l2", "achieved": achieved, "peak": l2["gbs"], "unit": "GB/s",
                        "frac": achieved / l2["gbs"], "peak_source": "measured live: " + l2["how"],
                        "peak_buffer_mib": l2.get("buffer_mib"),
                        # the binding pipes: instruction issue and shared memory
                        "on_chip": on_chip},
        "step_roofline": {"bytes_per_cell_step": step_bytes,
                          "achieved": step_bytes * value / world / 1e9, "unit": "GB/s",
                          "frac": step_bytes * value / world / 1e9 / pk["hbm_gbs"]},
        "phase_ms": {"projection": proj_kms / 3, "diffusion": diff_kms / 3,
                     "how": "CUDA events around each phase's own kernels, timed alone; "
                            "with_copy_back adds the copy to the public fields that a "
                            "phase called on its own ends with and a step does not run",
                     "with_copy_back": {"projection": proj_ms / 3, "diffusion": diff_ms / 3}},
        "phase_launches": {"projection": proj_kernels // 3, "diffusion": diff_kernels // 3},
        "wall_s": wall,
        "clocks": clk.summary(),
    }
    result["visual"] = time_visuals(f, cfg, sptr, stream, pk)
    f.close()
    del flush
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(cfg)
    if args.workload == "default" and not args.no_legs:
        # The other two legs of the metric: batched uneven tunnels and served
        # Poisson arrivals, each against one-at-a-time solves on the same GPU.
        result["batched"] = batched_measure(world, rank, local, args.scenarios, args.steps,
                                            args.warmup, baselines=not args.no_cpu_baseline)
        result["serving"] = serving_measure(world, rank, local, args.leg_serve_rate,
                                            args.leg_serve_seconds, args.leg_serve_drain,
                                            args.serve_budget_gb, args.serve_slots or None,
                                            args.serve_chunk, serial=not args.no_serial,
                                            lanes=args.serve_lanes,
                                            saturation_mcells=args.serve_saturation_mcells or None)
    return result if rank == 0 else None


BATCHED_WORKLOAD = ("batched: {count} uneven tunnels (seed 4), W,H in 128..1024 step 32, "
                    "n in {{50,100,200}}, pipe H/4, inflow U[0.5,3], dt 0.05")


def batched_measure(world, rank, local, count: int, steps: int, warmup: int, *,
                    mixed: bool = False, block: int = 0, sample_every: int = 8,
                    baselines: bool = True) -> dict:
    """The batched scenarios (seed 4): `count` uneven tunnels advanced together
    by one graph per step, timed over `steps` steps with CUDA events; then,
    every step, the batch step plus every scenario's smoke read back (e2e);
    then, on every `sample_every`-th scenario, the same scenarios one at a time
    (this library's plain per-sweep launch sequence, which is the reference's
    launch pattern and synchronises every step, and its blocked handles)."""
    import torch
    from opensayal_gb300 import Fluid, scenarios
    from opensayal_gb300.batch import Batch
    from opensayal_gb300.build import build_library
    build_library()
    torch.cuda.set_device(local)
    cfgs = scenarios.batched_scenarios(count, seed=4 + 1000 * rank)
    for i, c in enumerate(cfgs):
        c.device = local
        if mixed and i % 2:
            c.storage = 2  # OS_STORAGE_BF16
    cells = sum(c.width * c.height for c in cfgs)
    t_setup = time.perf_counter()
    b = Batch(cfgs, block_k=block if block and block > 0 else 0)
    for i, c in enumerate(cfgs):
        view = b.scenario(i)
        u, v = scenarios.perturbation(4000 + i, view.download("is_solid"))
        view.upload("vel_x", u)
        view.upload("vel_y", v)
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    b.step(warmup, sptr)
    stream.synchronize()
    setup_s = time.perf_counter() - t_setup
    launches0 = b.stats().launches
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist_barrier(world)
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        start.record(stream)
        b.step(steps, sptr)
        end.record(stream)
        torch.cuda.synchronize()
    dist_barrier(world)
    total_s = dist_max(world, start.elapsed_time(end) / 1e3)
    value = world * cells * steps / total_s
    st = b.stats()
    launches = int(st.launches - launches0)

    # e2e: every step, the batch step and every scenario's smoke read back to
    # pinned host memory: each member's smoke is copied on the step's stream
    # into its slice of one device buffer (os_snapshot_async), and a second
    # stream copies that buffer to the host while the next step runs.
    offsets, off = [], 0
    for c in cfgs:
        offsets.append(off)
        off += c.width * c.height
    views = [b.scenario(i) for i in range(len(cfgs))]
    snap = [torch.empty(cells, dtype=torch.float32, device="cuda") for _ in range(2)]
    host = [torch.empty(cells, dtype=torch.float32, pin_memory=True) for _ in range(2)]
    copy_stream = torch.cuda.Stream()
    copied = [torch.cuda.Event() for _ in range(2)]
    e2e_steps = min(steps, 5)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        s_ = k & 1
        b.step(1, sptr)
        if k >= 2:
            stream.wait_event(copied[s_])
        base = snap[s_].data_ptr()
        for view, o in zip(views, offsets):
            view.snapshot_async("smoke", base + 4 * o, sptr)
        ready = torch.cuda.Event()
        ready.record(stream)
        copy_stream.wait_event(ready)
        with torch.cuda.stream(copy_stream):
            host[s_].copy_(snap[s_], non_blocking=True)
        copied[s_].record(copy_stream)
    torch.cuda.synchronize()
    e2e_s = dist_max(world, time.perf_counter() - t0)
    del snap, host
    b.close()

    def one_at_a_time(block_k: int, sample: list, per: int) -> float:
        t = 0.0
        done = 0
        for c in sample:
            cc = c.copy()
            cc.projection_block = block_k
            with Fluid(cc) as f:
                f.update(None, cc.d_t)
                t1 = time.perf_counter()
                for _ in range(per):
                    f.update(None, cc.d_t)
                t += time.perf_counter() - t1
                done += cc.width * cc.height * per
        return done / t

    alone = None
    if baselines:
        sample = cfgs[::sample_every]
        alone = {"plain_per_sweep_sync": one_at_a_time(-1, sample, 2),
                 "blocked_graph_sync": one_at_a_time(8, sample, 2), "unit": UNIT,
                 "steps_per_scenario": 2,
                 "sample": f"every {sample_every}th scenario ({len(sample)} of {count}), "
                           "host wall clock around synchronous updates"}
    return {
        "value": value, "unit": UNIT, "steps": steps, "warmup": warmup,
        "ms_per_step": total_s * 1e3 / steps,
        "workload": BATCHED_WORKLOAD.format(count=count) + (" (BF16 for half)" if mixed else ""),
        "scenarios": count, "cells": cells, "setup_s": setup_s,
        "tuning": {"block_k": st.block_k, "kernels_per_step": st.kernels_per_step,
                   "tile_items_per_step": st.tile_items_per_step},
        "l2": f"inputs larger than L2 ({cells * 37 / 1e9:.1f} GB of fields)",
        "e2e": {"value": world * cells * e2e_steps / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 4 * cells,
                "steps": e2e_steps,
                "how": "every member's smoke snapshot on the step's stream, one device-to-host "
                       "copy per step on a second stream overlapping the next step"},
        "gpu_launches": launches,
        "one_at_a_time": alone,
        "clocks": clk.summary(),
    }


def run_batched(args, world, rank, local) -> dict | None:
    """The batched scenarios as the line's own workload (--workload batched)."""
    m = batched_measure(world, rank, local, args.scenarios, args.steps, args.warmup,
                        mixed=args.mixed, block=args.block or 0,
                        baselines=not args.no_cpu_baseline)
    res = {
        "metric": METRIC, "value": m["value"], "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": m["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32/bf16" if args.mixed else "f32", "data": "synthetic",
        "config": {"workload": m["workload"], "scenarios": m["scenarios"], "cells": m["cells"],
                   "l2": m["l2"], "parallelism": "replicas" if world > 1 else "single"},
        "tuning": m["tuning"], "e2e": m["e2e"], "gpu_launches": m["gpu_launches"],
        "one_at_a_time": m["one_at_a_time"], "clocks": m["clocks"],
    }
    return res if rank == 0 else None


SERVING_WORKLOAD = ("serving: Poisson {rate:g}/s for {seconds:g} s (seed 5), tunnels as batched, "
                    "steps U[100,5000], BF16 storage p=0.5")


def serving_measure(world, rank, local, rate: float, seconds: float, drain: float,
                    budget_gb: float, slots: int | None, chunk: int, serial: bool = True,
                    lanes: int = 4, saturation_mcells: float | None = 32.0) -> dict:
    """Poisson arrivals (seed 5) of tunnels drawn as in the batched workload,
    steps U[100, 5000], BF16 or FP32 storage (p = 0.5), served by continuous
    batching within a device-memory budget; the same arrival trace served one
    request at a time by single handles is the baseline. Both stop at the
    horizon (arrival window plus a drain allowance) or when every request is
    done."""
    import torch
    from opensayal_gb300 import scenarios
    from opensayal_gb300.build import build_library
    from opensayal_gb300.serving import Server, serve_serial
    build_library()
    torch.cuda.set_device(local)
    reqs = scenarios.serving_requests(rate, seconds, seed=5 + 1000 * rank)
    for r in reqs:
        r.config.device = local
    horizon = seconds + drain
    # Warm the library and the graph path on two small requests first.
    warm = scenarios.serving_requests(1000.0, 0.002, seed=99)[:2]
    for r in warm:
        r.config.device = local
        r.steps = 3
    with Server(budget_bytes=1 << 30, block_k=8, max_members=2, lanes=1) as w:
        w.run(warm, 60.0)
    budget = int(budget_gb * 1e9)
    sat = int(saturation_mcells * 1e6) if saturation_mcells else None
    dist_barrier(world)
    with Clocks(local) as clk:
        with Server(budget_bytes=budget, block_k=8, max_members=slots, chunk=chunk, lanes=lanes,
                    saturation_cells=sat) as srv:
            rep = srv.run(reqs, horizon)
            st = srv.batch.stats()
    served = rep.summary()
    serial_rep = serve_serial(reqs, horizon, block_k=8).summary() if serial else None
    value = dist_sum(world, float(rep.cell_steps)) / dist_max(world, rep.wall_s)
    return {
        "value": value, "unit": UNIT,
        "workload": SERVING_WORKLOAD.format(rate=rate, seconds=seconds),
        "budget_gb": budget_gb, "max_members": slots, "lanes": lanes,
        "saturation_mcells": saturation_mcells, "chunk": chunk, "horizon_s": horizon,
        "block_k": st.block_k, "requests": len(reqs),
        "serving": served, "serial_single_handles": serial_rep,
        "e2e": {"value": value, "unit": UNIT,
                "h2d_bytes_per_step": rep.h2d_bytes // max(1, st.steps_enqueued),
                "d2h_bytes_per_step": rep.d2h_bytes // max(1, st.steps_enqueued)},
        "gpu_launches": int(st.launches), "steps_enqueued": int(st.steps_enqueued),
        "wall_s": rep.wall_s, "clocks": clk.summary(),
    }


def run_serving(args, world, rank, local) -> dict | None:
    """The served scenarios as the line's own workload (--workload serving)."""
    m = serving_measure(world, rank, local, args.serve_rate, args.serve_seconds,
                        args.serve_drain, args.serve_budget_gb, args.serve_slots or None,
                        args.serve_chunk, serial=not args.no_serial, lanes=args.serve_lanes,
                        saturation_mcells=args.serve_saturation_mcells or None)
    steps = max(1, m["steps_enqueued"])
    res = {
        "metric": "served cell-steps/s (continuous batching, Poisson arrivals)",
        "value": m["value"], "unit": UNIT, "n_gpus": world, "steps": steps,
        "warmup": 1, "ms_per_step": m["wall_s"] * 1e3 / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/bf16",
        "data": "synthetic",
        "config": {"workload": m["workload"], "budget_gb": m["budget_gb"],
                   "max_members": m["max_members"], "lanes": m["lanes"],
                   "saturation_mcells": m["saturation_mcells"], "chunk": m["chunk"],
                   "horizon_s": m["horizon_s"],
                   "l2": "inputs larger than L2 (tens of members, ~12 MB each)",
                   "parallelism": "replicas" if world > 1 else "single"},
        "serving": m["serving"], "serial_single_handles": m["serial_single_handles"],
        "e2e": m["e2e"], "gpu_launches": m["gpu_launches"], "clocks": m["clocks"],
    }
    return res if rank == 0 else None


def run_precision(args, world, rank, local) -> dict | None:
    """Storage precision against an FP64 run of the same scheme: the 4096x4096
    tunnel (n = 200, dt = 0.02) from the same seeded state, in FP32, FP16 and
    BF16 storage (FP32 arithmetic) and in FP64 storage and arithmetic; the
    per-field relative L2 against FP64 at every checkpoint of
    `--precision-steps` (cumulative step counts), and the FP64 diagnostics of
    every run at the last one. The grid can be scaled down with
    --precision-size (256 gives the 256x128-shaped small tunnel)."""
    import torch
    from opensayal_gb300 import Fluid, scenarios
    from opensayal_gb300.build import build_library
    build_library()
    torch.cuda.set_device(local)
    if args.precision_size == 256:
        base = scenarios.small_config()
    else:
        base = scenarios.large_config()
        if args.precision_size:
            sc = args.precision_size / base.width
            base.width = base.height = args.precision_size
            base.pipe_height = int(base.pipe_height * sc)
            base.obstacle_center_x = base.obstacle_center_y = args.precision_size // 2
            base.obstacle_radius = base.obstacle_radius * sc
            base.smoke_height = base.height // 4
    base.device = local
    if args.precision_inviscid:
        base.viscosity = 0.0  # no diffusion: separates its rounding from the rest
    checkpoints = sorted({int(x) for x in str(args.precision_steps).split(",") if x})
    fields = ("vel_x", "vel_y", "smoke")
    runs = {}
    for name, storage in (("f64", 3), ("f32", 0), ("f16", 1), ("bf16", 2)):
        cfg = base.copy()
        cfg.storage = storage
        f = Fluid(cfg)
        u, v = scenarios.perturbation(3, f.download("is_solid"))
        f.upload("vel_x", u)
        f.upload("vel_y", v)
        snaps, done, elapsed = {}, 0, 0.0
        for cp in checkpoints:
            t0 = time.perf_counter()
            f.update_async(None, cfg.d_t, cp - done)
            f.synchronize()
            elapsed += time.perf_counter() - t0
            done = cp
            snaps[cp] = {k: f.download(k).astype(np.float64) for k in fields}
        runs[name] = {"snaps": snaps, "diag": f.diagnose(), "ms_per_step": elapsed * 1e3 / done,
                      "projection_block": f.fields().projection_block,
                      "projection_resident": f.fields().projection_resident}
        f.close()
    ref = runs["f64"]
    out = {}
    for name, r in runs.items():
        curve = {}
        for cp in checkpoints:
            rel = {}
            for k in fields:
                want = ref["snaps"][cp][k]
                den = float(np.linalg.norm(want)) or 1.0
                rel[k] = float(np.linalg.norm(r["snaps"][cp][k] - want)) / den
            curve[str(cp)] = rel
        dr = {}
        for k in ("divergence_l2", "smoke_mass", "inflow_flux", "outflow_flux"):
            den = abs(ref["diag"][k]) or 1.0
            dr[k] = abs(r["diag"][k] - ref["diag"][k]) / den
        out[name] = {"rel_l2_vs_f64": curve, "diag": r["diag"], "diag_rel_err_vs_f64": dr,
                     "ms_per_step": r["ms_per_step"], "projection_block": r["projection_block"],
                     "projection_resident": r["projection_resident"]}
    last = str(checkpoints[-1])
    cells = base.width * base.height
    res = {
        "metric": "relative L2 vs FP64 run of the same scheme",
        "value": out["bf16"]["rel_l2_vs_f64"][last]["vel_x"],
        "unit": "relative L2 (u, bf16 storage, last checkpoint)", "n_gpus": world,
        "steps": checkpoints[-1], "warmup": 0,
        "ms_per_step": out["f32"]["ms_per_step"], "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/f16/bf16 vs f64", "data": "synthetic",
        "config": dict(config_record(base, "precision", world), cells=cells,
                       checkpoints=checkpoints),
        "variants": out,
    }
    return res if rank == 0 else None


def run_reference(args, world, rank, local) -> dict | None:
    if rank != 0:
        return None
    import oracle
    from opensayal_gb300 import scenarios
    cfg = workload_config(args.workload)
    cells = cfg.width * cfg.height
    o = oracle.OracleFluid(cfg)
    u, v = scenarios.perturbation(2, o.is_solid)
    o.u[:], o.v[:] = u, v
    for _ in range(min(args.warmup, 1)):
        o.update(None, cfg.d_t)
    budget = 150.0
    t0 = time.perf_counter()
    done = 0
    while done < args.steps:
        o.update(None, cfg.d_t)
        done += 1
        if time.perf_counter() - t0 > budget:
            break
    el = time.perf_counter() - t0
    value = cells * done / el
    sample = (f"{done} of {args.steps} requested full {cfg.width}x{cfg.height} steps "
              f"({el:.1f} s; capped at {budget:.0f} s)")
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el * 1e3 / done, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config_record(cfg, args.workload, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.oracle_threads(),
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    result["reference_cuda"] = reference_cuda(cfg, args)
    if args.workload == "default" and not args.no_legs:
        result["batched"] = reference_batched(args)
        result["serving"] = reference_serving(args)
    libs = repo_libraries_mapped()
    # This arm runs the oracle and the reference's own kernels only: the
    # library under test must not be mapped into its process.
    assert not any("libopensayal_gb300" in x for x in libs), libs
    result["native_libraries"] = libs
    return result


def repo_libraries_mapped() -> list[str]:
    """Shared objects and cubins of this repository mapped into this process."""
    try:
        text = Path("/proc/self/maps").read_text()
    except OSError:
        return []
    root = str(ROOT) + "/"
    out = set()
    for line in text.splitlines():
        parts = line.split(None, 5)
        if len(parts) == 6 and parts[5].startswith(root):
            out.add(parts[5][len(root):])
    return sorted(out)


def reference_batched(args, sample_every: int = 8, per: int = 2) -> dict:
    """The batched scenarios (seed 4) one at a time through the reference's own
    kernels, as its Fluid::update runs them (one launch per sweep, a device
    synchronisation per step): every `sample_every`-th of the 512 scenarios,
    one warm step then `per` timed steps each, host wall clock."""
    import oracle
    try:
        import torch
        if not torch.cuda.is_available() or not oracle.reference_available():
            return {"unavailable": "no GPU or no reference cubin"}
        from opensayal_gb300 import scenarios
        cfgs = scenarios.batched_scenarios(args.scenarios, seed=4)[::sample_every]
        t, done = 0.0, 0
        for i, c in enumerate(cfgs):
            r = oracle.RefFluid(c)
            u, v = scenarios.perturbation(4000 + i * sample_every, r.is_solid)
            r.upload("vel_x", u)
            r.upload("vel_y", v)
            r.update(None, c.d_t)
            t0 = time.perf_counter()
            for _ in range(per):
                r.update(None, c.d_t)
            t += time.perf_counter() - t0
            done += c.width * c.height * per
            r.close()
        return {"value": done / t, "unit": UNIT,
                "workload": BATCHED_WORKLOAD.format(count=args.scenarios),
                "sample": f"every {sample_every}th scenario ({len(cfgs)} of {args.scenarios}), "
                          f"{per} steps each after one warm step",
                "timing": "host wall clock around Fluid::update, which synchronises each step"}
    except Exception as exc:  # the arm must still print its line
        return {"unavailable": f"{type(exc).__name__}: {exc}"}


def reference_serving(args) -> dict:
    """The served leg's arrival trace (seed 5) through the reference's own
    kernels, one request at a time in arrival order (the reference has one
    Fluid per process and no batching), to the same horizon. Requests that
    ask for BF16 storage run in FP32: the reference has no other storage."""
    import oracle
    try:
        import torch
        if not torch.cuda.is_available() or not oracle.reference_available():
            return {"unavailable": "no GPU or no reference cubin"}
        from opensayal_gb300 import scenarios
        from opensayal_gb300.serving import ServeReport
        reqs = scenarios.serving_requests(args.leg_serve_rate, args.leg_serve_seconds, seed=5)
        horizon = args.leg_serve_seconds + args.leg_serve_drain
        warm = oracle.RefFluid(reqs[0].config)
        warm.update(None, reqs[0].config.d_t)
        warm.close()
        rep = ServeReport()
        t0 = time.perf_counter()
        for req in reqs:
            now = time.perf_counter() - t0
            if now >= horizon:
                break
            if req.arrival > now:
                time.sleep(min(req.arrival - now, horizon - now))
                if time.perf_counter() - t0 >= horizon:
                    break
            rep.arrived += 1
            rep.admitted += 1
            rep.offered_cell_steps += req.cells * req.steps
            c = req.config.copy()
            c.storage = 0
            r = oracle.RefFluid(c)
            u, v = scenarios.perturbation(req.seed, r.is_solid)
            r.upload("vel_x", u)
            r.upload("vel_y", v)
            done = 0
            while done < req.steps and time.perf_counter() - t0 < horizon:
                r.update(None, c.d_t)
                done += 1
            rep.cell_steps += req.cells * done
            if done == req.steps:
                r.download("smoke")
                rep.latencies_s.append(time.perf_counter() - t0 - req.arrival)
                rep.finished += 1
            r.close()
        rep.wall_s = time.perf_counter() - t0
        rep.arrived = sum(1 for r in reqs if r.arrival < rep.wall_s)
        out = rep.summary()
        return {"value": out["cell_steps_per_s"], "unit": UNIT,
                "workload": SERVING_WORKLOAD.format(rate=args.leg_serve_rate,
                                                    seconds=args.leg_serve_seconds),
                "horizon_s": horizon, "requests": len(reqs), "serial_reference": out}
    except Exception as exc:  # the arm must still print its line
        return {"unavailable": f"{type(exc).__name__}: {exc}"}


def reference_cuda(cfg, args) -> dict:
    """The reference's own kernels (unmodified src/fluid.cu device code), driven
    with its launch shapes and its per-step device synchronisation."""
    import oracle
    try:
        import torch
        if not torch.cuda.is_available() or not oracle.reference_available():
            return {"unavailable": "no GPU or no reference cubin"}
        from opensayal_gb300 import scenarios
        r = oracle.RefFluid(cfg)
        u, v = scenarios.perturbation(2, r.is_solid)
        r.upload("vel_x", u)
        r.upload("vel_y", v)
        for _ in range(max(args.warmup, 3)):
            r.update(None, cfg.d_t)
        steps = min(args.steps, 200)
        t0 = time.perf_counter()
        for _ in range(steps):
            r.update(None, cfg.d_t)
        el = time.perf_counter() - t0
        r.close()
        return {"value": cfg.width * cfg.height * steps / el, "unit": UNIT, "steps": steps,
                "ms_per_step": el * 1e3 / steps,
                "timing": "host wall clock around Fluid::update, which synchronises each step"}
    except Exception as exc:  # the arm must still print its line
        return {"unavailable": f"{type(exc).__name__}: {exc}"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="default",
                    choices=["default", "small", "large", "batched", "serving", "precision"])
    ap.add_argument("--scenarios", type=int, default=512, help="batched workload size")
    ap.add_argument("--block", type=int, default=None,
                    help="red/black sweeps per blocked pass (0 autotune, -1 plain)")
    ap.add_argument("--diffusion-block", type=int, default=None,
                    help="Jacobi sweeps per diffusion pass (0: the projection's depth or, "
                         "autotuned, the autotuner's)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--resident", type=int, default=None, choices=[-1, 0, 1, 2, 3],
                    help="phases as resident cooperative launches: mask 1 projection, "
                         "2 diffusion, 3 both; -1 never; 0 autotuner decides")
    ap.add_argument("--mixed", action="store_true",
                    help="batched: BF16 storage for half of the scenarios")
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--serve-drain", type=float, default=30.0)
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--serve-slots", type=int, default=0,
                    help="members the batch may hold (0: bounded by memory and saturation)")
    ap.add_argument("--serve-lanes", type=int, default=4,
                    help="latency lanes: requests run on single handles of their own")
    ap.add_argument("--serve-saturation-mcells", type=float, default=32.0,
                    help="cells (millions) the batch holds at most (0: memory only)")
    ap.add_argument("--serve-chunk", type=int, default=2)
    ap.add_argument("--no-serial", action="store_true")
    ap.add_argument("--no-legs", action="store_true",
                    help="default workload: skip the batched and served legs")
    ap.add_argument("--leg-serve-rate", type=float, default=1.0,
                    help="served leg of the default run: Poisson arrivals per second")
    ap.add_argument("--leg-serve-seconds", type=float, default=20.0)
    ap.add_argument("--leg-serve-drain", type=float, default=40.0)
    ap.add_argument("--precision-size", type=int, default=0,
                    help="precision: square grid size instead of 4096 (256: the small tunnel)")
    ap.add_argument("--precision-steps", default="100,250,500,1000",
                    help="precision: cumulative step counts at which the errors are taken")
    ap.add_argument("--precision-inviscid", action="store_true",
                    help="precision: viscosity 0 (the diffusion's increments are what 16-bit "
                         "storage rounds away)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup()
    if args.impl == "reference":
        res = run_reference(args, world, rank, local)
    else:
        runner = {"batched": run_batched, "serving": run_serving,
                  "precision": run_precision}.get(args.workload, run_gb300)
        res = runner(args, world, rank, local)
    if res is not None:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
