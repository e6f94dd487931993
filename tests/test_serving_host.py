"""The serving loop's host logic on the CPU, against stand-ins for the
dynamic batch and the latency lanes with a simulated clock: waiting requests
are taken shortest work first with an ageing bound, lanes take requests
before the batch, admission respects the member limit, the saturation size
and the memory budget (a refused request waits), a member's result is read
back when its last step has run, the horizon cuts the run, and the report
counts unfinished requests and the partial progress of unfinished members."""
import numpy as np
import pytest

from opensayal_gb300 import native, scenarios
from opensayal_gb300.batch import BudgetFull
from opensayal_gb300.fluid import default_config
from opensayal_gb300.scenarios import Request
from opensayal_gb300.serving import ServeReport, Server


class Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, s):
        self.t += s


class View:
    """A member's fields as the server touches them."""

    def __init__(self, cfg):
        self.n = cfg.width * cfg.height
        self.fields = {"is_solid": np.zeros(self.n, np.int32),
                       "smoke": np.zeros(self.n, np.float32)}

    def download(self, name):
        return self.fields[name].copy()

    def upload(self, name, a):
        self.fields[name] = np.asarray(a).copy()


class Stats:
    def __init__(self, steps):
        self.steps_enqueued = steps


class FakeBatch:
    """Members advance `step(k)` steps at `seconds_per_step` of simulated time
    each; device memory is 10 bytes per cell against `budget` (0: none)."""

    def __init__(self, clock, seconds_per_step=0.01, budget=0):
        self.clock, self.sps, self.budget = clock, seconds_per_step, budget
        self.left, self.views, self.done, self.enqueued = {}, {}, set(), 0
        self.used = 0
        self.next_id = 0
        self.admitted = []
        self.admitted_steps = []

    def add(self, cfg, steps):
        need = 10 * cfg.width * cfg.height
        if self.budget and self.used + need > self.budget:
            raise BudgetFull(native.OS_ERR_NOMEM, "budget")
        mid = self.next_id
        self.next_id += 1
        self.left[mid] = steps
        self.views[mid] = View(cfg)
        self.used += need
        self.admitted.append(mid)
        self.admitted_steps.append(steps)
        return mid

    def remove(self, mid):
        self.used -= 10 * self.views[mid].n
        del self.left[mid]
        del self.views[mid]

    def step(self, k):
        self.enqueued += k
        for mid in self.left:
            if self.left[mid] > 0:
                self.left[mid] = max(0, self.left[mid] - k)
        self.clock.t += k * self.sps

    def wait(self, max_in_flight=0):
        pass

    def synchronize(self):
        pass

    def poll(self):
        out = [m for m, l in self.left.items() if l == 0 and m not in self.done]
        self.done.update(out)
        for m in out:
            self.views[m].fields["smoke"][:] = m  # the member's "result"
        return out

    def status(self, mid):
        left = self.left[mid]
        return (native.MEMBER_DONE if left == 0 else native.MEMBER_RUNNING), left

    def memory(self):
        return self.used, self.budget

    def scenario(self, mid):
        return self.views[mid]

    def stats(self):
        return Stats(self.enqueued)


def requests(arrivals, steps, w=32, h=16):
    out = []
    for k, (t, n) in enumerate(zip(arrivals, steps)):
        out.append(Request(k, t, default_config(w, h), n, seed=k))
    return out


def test_every_request_finishes_in_order_with_its_latency():
    clock = Clock()
    fb = FakeBatch(clock)
    srv = Server(0, max_members=4, chunk=2, batch=fb)
    reqs = requests([0.0, 0.0, 0.05, 1.0], [10, 20, 10, 4])
    results = {}
    rep = srv.run(reqs, horizon_s=100.0, results=results, clock=clock, sleep=clock.sleep)
    assert rep.arrived == rep.admitted == rep.finished == 4
    assert fb.admitted == [0, 1, 2, 3]  # first come, first admitted
    assert sorted(results) == [0, 1, 2, 3]
    assert all(np.all(results[k] == k) for k in range(4))  # each its own result
    assert rep.cell_steps == sum(r.cells * r.steps for r in reqs)
    # Request 0 finishes first: 10 steps from t = 0 at 0.01 s per step.
    assert rep.latencies_s[0] == pytest.approx(0.10)
    # The last request arrives at 1.0 s, after an idle wait, and needs 4 steps.
    assert rep.latencies_s[-1] == pytest.approx(0.04)
    assert rep.h2d_bytes == 4 * 2 * 32 * 16 * 4 and rep.d2h_bytes == 4 * 32 * 16 * 4


def test_member_limit_and_budget_make_requests_wait():
    clock = Clock()
    fb = FakeBatch(clock, budget=2 * 10 * 32 * 16)  # room for two members
    srv = Server(0, max_members=8, chunk=2, batch=fb)
    reqs = requests([0.0] * 5, [6] * 5)
    rep = srv.run(reqs, horizon_s=100.0, clock=clock, sleep=clock.sleep)
    assert rep.finished == 5
    assert rep.peak_members == 2
    assert rep.budget_refusals > 0
    assert rep.peak_device_bytes <= fb.budget
    lat = sorted(rep.latencies_s)
    assert lat[0] == pytest.approx(0.06) and lat[-1] > lat[0]


def test_horizon_counts_unfinished_requests_and_partial_progress():
    clock = Clock()
    fb = FakeBatch(clock)
    srv = Server(0, max_members=2, chunk=2, batch=fb)
    # 100 arrivals within the horizon, each 1000 steps: two run, the rest queue.
    reqs = requests(list(np.linspace(0.0, 0.5, 100)), [1000] * 100)
    rep = srv.run(reqs, horizon_s=1.0, clock=clock, sleep=clock.sleep)
    assert rep.finished == 0 and rep.arrived == 100 and rep.admitted == 2
    # Progress of the two running members counts toward the served work.
    done = sum(reqs[m].cells * (1000 - left) for m, left in fb.left.items())
    assert rep.cell_steps == done > 0
    pct = rep.percentiles()
    assert pct["p50_finished_s"] is None and pct["p99_all_s"] is None
    s = rep.summary()
    assert s["unfinished"] == 100 and s["offered_cell_steps_per_s"] > s["cell_steps_per_s"]


def test_percentiles_over_all_arrivals():
    rep = ServeReport(arrived=4, finished=3, latencies_s=[1.0, 2.0, 3.0])
    p = rep.percentiles()
    assert p["p50_finished_s"] == pytest.approx(2.0)
    assert p["p50_all_s"] == pytest.approx(2.0)  # rank 2 of 4 is finished
    assert p["p99_all_s"] is None                # rank 4 of 4 is not


class FakeLane:
    """A lane that completes one step per pump."""

    def __init__(self, req, log):
        self.req, self.done = req, 0
        self.h2d_bytes, self.device_bytes = 8 * req.cells, 40 * req.cells
        log.append(req.index)

    def pump(self):
        self.done = min(self.req.steps, self.done + 1)

    @property
    def finished(self):
        return self.done == self.req.steps

    def result(self):
        return np.full(self.req.cells, -1.0 - self.req.index, np.float32)

    def wait(self):
        pass

    def close(self):
        pass


def test_shortest_work_first_then_ageing():
    # Three requests wait at t = 0 for a batch of one member. Without ageing
    # they run shortest first; with a 0.05 s ageing bound the two left when
    # the first finishes (t = 0.1 s) have both aged and go in arrival order.
    for age, want in ((100.0, [10, 30, 50]), (0.05, [10, 50, 30])):
        clock = Clock()
        fb = FakeBatch(clock)
        srv = Server(0, max_members=1, chunk=2, batch=fb, age_limit_s=age)
        rep = srv.run(requests([0.0, 0.0, 0.0], [50, 10, 30]), horizon_s=100.0, clock=clock,
                      sleep=clock.sleep)
        assert rep.finished == 3
        assert fb.admitted_steps == want
        assert rep.latencies_s[0] == pytest.approx(0.10)


def test_lanes_take_requests_before_the_batch():
    clock = Clock()
    fb = FakeBatch(clock)
    log = []
    srv = Server(0, chunk=2, batch=fb, lanes=2, lane_factory=lambda r: FakeLane(r, log))
    reqs = requests([0.0] * 5, [8, 4, 6, 2, 10])
    results = {}
    rep = srv.run(reqs, horizon_s=100.0, results=results, clock=clock, sleep=clock.sleep)
    assert rep.finished == rep.admitted == 5
    assert log[:2] == [3, 1]          # the two shortest go to the lanes
    assert len(fb.admitted) == 3      # the rest join the batch at once
    for k in log:
        assert np.all(results[k] == -1.0 - k)
    assert rep.peak_members == 5
    assert rep.cell_steps == sum(r.cells * r.steps for r in reqs)


def test_saturation_bounds_the_batch_and_the_slot_count_does_not():
    clock = Clock()
    fb = FakeBatch(clock)
    cells = 32 * 16
    srv = Server(0, chunk=2, batch=fb, saturation_cells=3 * cells)
    reqs = requests([0.0] * 8, [6] * 8)
    rep = srv.run(reqs, horizon_s=100.0, clock=clock, sleep=clock.sleep)
    assert rep.finished == 8 and rep.peak_members == 3
    clock = Clock()
    fb = FakeBatch(clock)
    srv = Server(0, chunk=2, batch=fb)  # neither slots nor saturation: all join
    rep = srv.run(requests([0.0] * 8, [6] * 8), horizon_s=100.0, clock=clock,
                  sleep=clock.sleep)
    assert rep.peak_members == 8
