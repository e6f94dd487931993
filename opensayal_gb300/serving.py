"""Serving wind-tunnel scenarios as they arrive (continuous batching).

`Server.run` takes requests with arrival times and serves them through one
dynamic Batch: arrivals queue in order; a request is admitted when a member
slot is free and its fields fit the device-memory budget (the batch refuses
what does not fit without touching the device); admitted requests join the
shared steps, each stops after exactly its own step count, and its result
(the smoke field) is read back as soon as its last step has completed, which
frees its memory for the next request. `serve_serial` is the baseline: the
same requests one at a time through a single Fluid handle each.

Time-to-result is measured from a request's arrival to the end of its result's
device-to-host read. A run ends at the horizon; requests not finished by then
are reported, not dropped from the count.
"""
from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from .batch import Batch, BudgetFull
from .fluid import Fluid
from .scenarios import Request, perturbation


@dataclass
class ServeReport:
    arrived: int = 0
    finished: int = 0
    admitted: int = 0
    wall_s: float = 0.0
    latencies_s: list = field(default_factory=list)  # finished requests
    cell_steps: int = 0        # completed cell-steps, finished or not
    offered_cell_steps: int = 0
    h2d_bytes: int = 0
    d2h_bytes: int = 0
    peak_members: int = 0
    peak_device_bytes: int = 0
    budget_refusals: int = 0

    def percentiles(self) -> dict:
        """p50/p99 over finished requests, and over all arrived requests with
        unfinished ones counted as unbounded (None when the percentile falls
        on an unfinished request)."""
        out = {}
        lat = np.sort(np.asarray(self.latencies_s, dtype=np.float64))
        for q in (50, 99):
            out[f"p{q}_finished_s"] = float(np.percentile(lat, q)) if lat.size else None
            if self.arrived:
                rank = int(np.ceil(q / 100.0 * self.arrived)) - 1
                out[f"p{q}_all_s"] = float(lat[rank]) if rank < lat.size else None
            else:
                out[f"p{q}_all_s"] = None
        return out

    def summary(self) -> dict:
        d = {
            "arrived": self.arrived, "admitted": self.admitted, "finished": self.finished,
            "unfinished": self.arrived - self.finished, "wall_s": round(self.wall_s, 3),
            "cell_steps_per_s": self.cell_steps / self.wall_s if self.wall_s else 0.0,
            "offered_cell_steps_per_s": self.offered_cell_steps / self.wall_s if self.wall_s else 0.0,
            "h2d_bytes": self.h2d_bytes, "d2h_bytes": self.d2h_bytes,
            "peak_members": self.peak_members, "peak_device_bytes": self.peak_device_bytes,
            "budget_refusals": self.budget_refusals,
        }
        d.update(self.percentiles())
        return d


def _initial_fields(view: Fluid, req: Request) -> int:
    """Seeded perturbation of u, v on the fluid cells; returns bytes uploaded."""
    solid = view.download("is_solid")
    u, v = perturbation(req.seed, solid)
    view.upload("vel_x", u)
    view.upload("vel_y", v)
    return u.nbytes + v.nbytes


class Server:
    """Continuous batching over one dynamic Batch.

    max_members bounds the requests on the GPU at once (the batch's step time
    grows with their cells); chunk is the number of steps enqueued per loop
    turn and depth the chunks allowed in flight before the loop waits. `batch`
    replaces the dynamic Batch the server would create (any object with its
    add/remove/step/wait/poll/status/memory/scenario/stats/synchronize)."""

    def __init__(self, budget_bytes: int, block_k: int = 8, max_members: int = 64,
                 chunk: int = 2, depth: int = 2, device: int = 0, batch=None):
        self.batch = batch if batch is not None else Batch.dynamic(
            block_k=block_k, device=device, budget_bytes=budget_bytes)
        self.max_members = max_members
        self.chunk = chunk
        self.depth = depth

    def close(self):
        self.batch.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def run(self, requests: list[Request], horizon_s: float, results: dict | None = None,
            clock=time.perf_counter, sleep=time.sleep) -> ServeReport:
        b = self.batch
        rep = ServeReport()
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        queue: deque[Request] = deque()
        active: dict[int, tuple[Request, int]] = {}  # id -> (request, steps_enqueued at admit)
        t0 = clock()
        while True:
            now = clock() - t0
            while pending and pending[0].arrival <= now:
                queue.append(pending.popleft())
                rep.arrived += 1
                rep.offered_cell_steps += queue[-1].cells * queue[-1].steps
            while queue and len(active) < self.max_members:
                req = queue[0]
                try:
                    mid = b.add(req.config, req.steps)
                except BudgetFull:
                    rep.budget_refusals += 1
                    break
                rep.h2d_bytes += _initial_fields(b.scenario(mid), req)
                queue.popleft()
                active[mid] = (req, b.stats().steps_enqueued)
                rep.admitted += 1
            rep.peak_members = max(rep.peak_members, len(active))
            rep.peak_device_bytes = max(rep.peak_device_bytes, b.memory()[0])
            if active:
                b.step(self.chunk)
                b.wait(self.depth * self.chunk)
            for mid in b.poll():
                req, _ = active.pop(mid)
                smoke = b.scenario(mid).download("smoke")
                rep.d2h_bytes += smoke.nbytes
                rep.latencies_s.append(clock() - t0 - req.arrival)
                rep.finished += 1
                rep.cell_steps += req.cells * req.steps
                if results is not None:
                    results[req.index] = smoke
                b.remove(mid)
            now = clock() - t0
            if now >= horizon_s or (not pending and not queue and not active):
                break
            if not active and not queue and pending:
                sleep(max(0.0, min(pending[0].arrival - now, horizon_s - now)))
        # Progress of the unfinished members counts toward the served work.
        b.synchronize()
        for mid, (req, _) in active.items():
            state, left = b.status(mid)
            rep.cell_steps += req.cells * (req.steps - max(left, 0))
        rep.wall_s = clock() - t0
        # Requests that arrived before the end but were never taken up.
        rep.arrived += sum(1 for r in pending if r.arrival < rep.wall_s)
        return rep


def serve_serial(requests: list[Request], horizon_s: float, block_k: int = 8,
                 chunk: int = 50, results: dict | None = None,
                 clock=time.perf_counter) -> ServeReport:
    """The same requests one at a time, each through its own Fluid handle
    (first come, first served), within the same horizon."""
    rep = ServeReport()
    pending = deque(sorted(requests, key=lambda r: r.arrival))
    t0 = clock()
    while pending:
        now = clock() - t0
        if now >= horizon_s:
            break
        req = pending[0]
        if req.arrival > now:
            time.sleep(min(req.arrival - now, horizon_s - now))
            continue
        pending.popleft()
        rep.arrived += 1
        rep.offered_cell_steps += req.cells * req.steps
        rep.admitted += 1
        c = req.config.copy()
        c.projection_block = block_k
        with Fluid(c) as f:
            rep.h2d_bytes += _initial_fields(f, req)
            done = 0
            while done < req.steps and clock() - t0 < horizon_s:
                k = min(chunk, req.steps - done)
                f.update_async(None, c.d_t, k)
                f.synchronize()
                done += k
            rep.cell_steps += req.cells * done
            if done == req.steps:
                smoke = f.download("smoke")
                rep.d2h_bytes += smoke.nbytes
                rep.latencies_s.append(clock() - t0 - req.arrival)
                rep.finished += 1
                if results is not None:
                    results[req.index] = smoke
    rep.wall_s = clock() - t0
    # Requests that arrived before the horizon but were never started.
    rep.arrived += sum(1 for r in pending if r.arrival < rep.wall_s)
    return rep
