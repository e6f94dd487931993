"""Continuous batching: members join at different steps, ask for different
step counts, use different storage types, and leave (finished or cancelled)
while others run; each finished member's fields are bit for bit those of the
same scenario run alone through Fluid.update for the same number of steps.
Admission against a device-memory budget refuses what does not fit and
accepts it once memory is returned."""
import numpy as np
import pytest

from opensayal_gb300 import native
from opensayal_gb300.batch import Batch, BudgetFull
from opensayal_gb300.fluid import Fluid, default_config
from tests.parity_cases import FIELDS, perturbed_state, same_bits

pytestmark = pytest.mark.gpu

F32, F16, BF16 = 0, 1, 2


def cfg_of(w, h, n, storage, k):
    c = default_config(w, h)
    c.tunnel_speed = 0.6 + 0.3 * k
    c.g = -1.0 * k
    c.projection_n = n
    c.obstacle_radius = 3.0 + k
    c.storage = storage
    return c


def alone(cfg, state, steps, block_k):
    c = cfg.copy()
    c.projection_block = block_k
    with Fluid(c) as f:
        for k, a in state.items():
            f.upload(k, a)
        for _ in range(steps):
            f.update(None, c.d_t)
        return {field: f.download(field) for field in FIELDS}


def test_members_joining_and_leaving_match_alone_runs(gpu):
    K = 4
    plan = {  # name: (config, steps)
        "a": (cfg_of(128, 96, 20, F32, 0), 7),
        "b": (cfg_of(300, 160, 13, F16, 1), 3),
        "c": (cfg_of(97, 250, 7, BF16, 2), 10),
        "d": (cfg_of(640, 384, 20, F32, 3), 4),
        "e": (cfg_of(160, 128, 33, BF16, 4), 5),
        "f": (cfg_of(33, 3, 4, F16, 5), 6),
    }
    plan["c"][0].viscosity = 0.0
    plan["e"][0].enable_smoke = 0
    states = {k: perturbed_state(c, 40 + i) for i, (k, (c, _)) in enumerate(plan.items())}
    ids, results = {}, {}

    def admit(b, name):
        c, steps = plan[name]
        ids[name] = b.add(c, steps)
        view = b.scenario(ids[name])
        for k, a in states[name].items():
            view.upload(k, a)

    def collect(b, wait=False):
        for mid in b.poll(wait=wait):
            name = next(k for k, v in ids.items() if v == mid)
            view = b.scenario(mid)
            results[name] = {field: view.download(field) for field in FIELDS}
            b.remove(mid)

    with Batch.dynamic(block_k=K, budget_bytes=1 << 30) as b:
        for name in "abc":
            admit(b, name)
        b.step(2)
        admit(b, "d")
        admit(b, "e")
        b.step(1)
        b.step(3)                 # b finishes after batch step 3
        collect(b, wait=True)
        assert "b" in results
        admit(b, "f")             # reuses b's slot
        state, left = b.status(ids["c"])
        assert state == native.MEMBER_RUNNING and 0 < left <= 10
        b.remove(ids["c"])        # cancelled while running
        b.step(2)
        b.step(8)
        b.synchronize()
        collect(b)
        assert b.stats().scenarios == 0
        assert not b.poll()
        used, budget = b.memory()
        assert used == 0 and budget >= 1 << 30
    assert set(results) == {"a", "b", "d", "e", "f"}
    for name, got in results.items():
        c, steps = plan[name]
        want = alone(c, states[name], steps, K)
        for field in FIELDS:
            x, y = got[field], want[field]
            assert same_bits(x, y), f"{name} {field}: {int((x != y).sum())} differ"


def test_budget_admission_waits_for_memory(gpu):
    c = cfg_of(256, 128, 8, F32, 0)
    with Batch.dynamic(block_k=8, budget_bytes=1 << 20) as probe:
        with pytest.raises(BudgetFull):
            probe.add(c, 5)
    with Batch.dynamic(block_k=8) as free:
        free.add(c, 5)
        used, budget = free.memory()
        assert budget == 0 and used > 0
    one = used
    with Batch.dynamic(block_k=8, budget_bytes=2 * one + one // 2) as b:
        first = b.add(c, 3)
        second = b.add(c, 6)
        with pytest.raises(BudgetFull):
            b.add(c, 2)
        b.step(3)
        done = b.poll(wait=True)
        assert done == [first]
        b.remove(first)
        third = b.add(c, 2)        # fits again
        b.step(3)
        b.synchronize()
        assert sorted(b.poll()) == sorted([second, third])
        for mid in (second, third):
            assert np.isfinite(b.scenario(mid).download("smoke")).all()


def test_unlimited_member_runs_until_removed(gpu):
    c = cfg_of(128, 64, 8, F32, 1)
    with Batch.dynamic(block_k=8) as b:
        mid = b.add(c, -1)
        b.step(5)
        b.synchronize()
        assert b.poll() == []
        assert b.status(mid) == (native.MEMBER_RUNNING, -1)
        st = b.stats()
        assert st.steps_enqueued == 5 and st.steps_completed == 5 and st.members_in_plan == 1
        b.remove(mid)
        b.step(1)
        b.synchronize()
        assert b.stats().members_in_plan == 0


@pytest.mark.parametrize("lanes", [0, 2])
def test_served_results_equal_serial_solves(gpu, lanes):
    from opensayal_gb300.scenarios import Request
    from opensayal_gb300.serving import Server, serve_serial
    rng = np.random.default_rng(11)
    reqs = []
    for i in range(7):
        w, h = int(rng.choice([64, 96, 160, 224])), int(rng.choice([48, 96, 128]))
        c = cfg_of(w, h, int(rng.choice([9, 16, 30])), BF16 if i % 2 else F32, i)
        reqs.append(Request(i, 0.002 * i, c, int(rng.integers(5, 40)), 1000 + i))
    got, want = {}, {}
    with Server(budget_bytes=64 << 20, block_k=8, max_members=3, chunk=2, lanes=lanes) as s:
        rep = s.run(reqs, horizon_s=300.0, results=got)
    assert rep.finished == rep.arrived == len(reqs) and rep.peak_members <= 3 + lanes
    assert rep.cell_steps == sum(r.cells * r.steps for r in reqs)
    serial = serve_serial(reqs, horizon_s=300.0, block_k=8, results=want)
    assert serial.finished == len(reqs)
    for i in range(len(reqs)):
        assert same_bits(got[i], want[i]), f"request {i}: {int((got[i] != want[i]).sum())} differ"
