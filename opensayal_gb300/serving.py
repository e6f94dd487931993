"""Serving wind-tunnel scenarios as they arrive (continuous batching).

`Server.run` takes requests with arrival times and serves them as they
arrive: waiting requests are taken shortest remaining work first (with an
ageing bound); a request runs in a latency lane (a single handle on its own
stream, concurrent with the others) when one is free, and otherwise joins
one dynamic Batch, admitted while its fields fit the device-memory budget
(the batch refuses what does not fit without touching the device) and the
batch is below the size at which its throughput saturates. Every request
stops after exactly its own step count, and its result (the smoke field) is
read back as soon as its last step has completed, which frees its lane or
memory for the next request. `serve_serial` is the baseline: the same
requests one at a time, in arrival order, through a single Fluid handle
each.

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


class HandleLane:
    """One request on a single handle of its own, stepping on the handle's own
    stream: lanes run concurrently with one another and with the batch. Steps
    are enqueued in chunks; a chunk that finished in under `target_s` doubles
    the next one (up to 256 steps), so short steps do not leave the device
    waiting for the host."""

    def __init__(self, req: Request, block_k: int = 8, target_s: float = 0.01,
                 clock=time.perf_counter):
        c = req.config.copy()
        c.projection_block = block_k
        self.req, self.clock, self.target_s = req, clock, target_s
        self.f = Fluid(c)
        self.h2d_bytes = _initial_fields(self.f, req)
        self.device_bytes = 40 * req.cells  # u, v, smoke (+buffers), p, masks, flags
        self.done = 0         # steps known complete
        self.in_flight = 0    # steps enqueued and not yet known complete
        self.chunk = 16
        self.t_enq = 0.0

    def pump(self) -> None:
        """Record a completed chunk and enqueue the next one; never waits."""
        if self.in_flight:
            if not self.f.idle():
                return
            self.done += self.in_flight
            if self.clock() - self.t_enq < self.target_s:
                self.chunk = min(256, self.chunk * 2)
            self.in_flight = 0
        left = self.req.steps - self.done
        if left > 0:
            k = min(self.chunk, left)
            self.f.update_async(None, self.req.config.d_t, k)
            self.in_flight = k
            self.t_enq = self.clock()

    @property
    def finished(self) -> bool:
        return self.done == self.req.steps

    def result(self) -> np.ndarray:
        return self.f.download("smoke")

    def wait(self) -> None:
        self.f.synchronize()
        self.done += self.in_flight
        self.in_flight = 0

    def close(self) -> None:
        self.f.close()


class Server:
    """Continuous batching over one dynamic Batch, with latency lanes.

    Waiting requests are taken shortest remaining work first (cells x steps),
    except that a request that has waited `age_limit_s` goes ahead of all
    younger ones in arrival order, so that no request starves. A request goes
    to a free lane when there is one (`lanes` single handles, each on its own
    stream, running concurrently: at light load a request runs at the speed
    of a grid alone, without queueing behind the one before it); otherwise it
    joins the batch, which steps all its members with one graph per step. The
    batch admits members while their fields fit the device-memory budget and
    the cells in it stay within `saturation_cells` (beyond which the batch's
    throughput no longer grows and every member only slows down), and, when
    `max_members` is set, while it has fewer members. `chunk` is the number
    of batch steps enqueued per loop turn and `depth` the chunks allowed in
    flight before the loop waits. `batch` replaces the dynamic Batch the
    server would create (any object with its add/remove/step/wait/poll/status/
    memory/scenario/stats/synchronize) and `lane_factory` the lanes (a
    callable taking a request; the result needs pump/finished/result/wait/
    close and h2d_bytes/device_bytes)."""

    def __init__(self, budget_bytes: int, block_k: int = 8, max_members: int | None = None,
                 chunk: int = 2, depth: int = 2, device: int = 0, batch=None, lanes: int = 0,
                 saturation_cells: int | None = None, age_limit_s: float = 30.0,
                 lane_factory=None):
        self.batch = batch if batch is not None else Batch.dynamic(
            block_k=block_k, device=device, budget_bytes=budget_bytes)
        self.max_members = max_members
        self.chunk = chunk
        self.depth = depth
        self.lanes = lanes
        self.saturation_cells = saturation_cells
        self.age_limit_s = age_limit_s
        self.lane_factory = lane_factory or (lambda req: HandleLane(req, block_k))

    def close(self):
        self.batch.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _pick(self, queue: list, now: float) -> int:
        """Index of the next request to serve: the oldest of those past the age
        limit, else the least work (cells x steps), ties in arrival order."""
        best, best_key = 0, None
        for k, r in enumerate(queue):
            aged = now - r.arrival >= self.age_limit_s
            key = (0, r.arrival) if aged else (1, r.cells * r.steps, r.arrival)
            if best_key is None or key < best_key:
                best, best_key = k, key
        return best

    def run(self, requests: list[Request], horizon_s: float, results: dict | None = None,
            clock=time.perf_counter, sleep=time.sleep) -> ServeReport:
        b = self.batch
        rep = ServeReport()
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        queue: list[Request] = []
        active: dict[int, Request] = {}  # batch member id -> request
        lanes: list = []
        batch_cells = 0
        t0 = clock()

        def finish(req, smoke, now):
            rep.d2h_bytes += smoke.nbytes
            rep.latencies_s.append(now - req.arrival)
            rep.finished += 1
            rep.cell_steps += req.cells * req.steps
            if results is not None:
                results[req.index] = smoke

        while True:
            now = clock() - t0
            while pending and pending[0].arrival <= now:
                r = pending.popleft()
                queue.append(r)
                rep.arrived += 1
                rep.offered_cell_steps += r.cells * r.steps
            # Lanes first, then the batch, each taking the best waiting request.
            while queue and len(lanes) < self.lanes:
                req = queue.pop(self._pick(queue, now))
                lane = self.lane_factory(req)
                rep.h2d_bytes += lane.h2d_bytes
                rep.admitted += 1
                lanes.append(lane)
            while queue and (self.max_members is None or len(active) < self.max_members):
                k = self._pick(queue, now)
                req = queue[k]
                if (self.saturation_cells is not None and active
                        and batch_cells + req.cells > self.saturation_cells):
                    break
                try:
                    mid = b.add(req.config, req.steps)
                except BudgetFull:
                    rep.budget_refusals += 1
                    break
                queue.pop(k)
                rep.h2d_bytes += _initial_fields(b.scenario(mid), req)
                active[mid] = req
                batch_cells += req.cells
                rep.admitted += 1
            rep.peak_members = max(rep.peak_members, len(active) + len(lanes))
            rep.peak_device_bytes = max(rep.peak_device_bytes,
                                        b.memory()[0] + sum(x.device_bytes for x in lanes))
            for lane in lanes:
                lane.pump()
            if active:
                b.step(self.chunk)
                b.wait(self.depth * self.chunk)
            for mid in b.poll():
                req = active.pop(mid)
                batch_cells -= req.cells
                finish(req, b.scenario(mid).download("smoke"), clock() - t0)
                b.remove(mid)
            for lane in [x for x in lanes if x.finished]:
                finish(lane.req, lane.result(), clock() - t0)
                lane.close()
                lanes.remove(lane)
            now = clock() - t0
            if now >= horizon_s or (not pending and not queue and not active and not lanes):
                break
            if not active and not queue and not lanes and pending:
                sleep(max(0.0, min(pending[0].arrival - now, horizon_s - now)))
            elif not active and lanes:
                sleep(0.0005)  # lanes only: poll their streams without spinning hard
        # Progress of the unfinished members and lanes counts toward the served work.
        b.synchronize()
        for mid, req in active.items():
            state, left = b.status(mid)
            rep.cell_steps += req.cells * (req.steps - max(left, 0))
        for lane in lanes:
            lane.wait()
            rep.cell_steps += lane.req.cells * lane.done
            lane.close()
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
