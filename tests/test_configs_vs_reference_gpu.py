"""The configurations the measurements are quoted on, checked directly against
the reference's own kernels (the unmodified src/fluid.cu device code through
oracle/ref_harness.cpp), in the form the measurements run them:

* the 1920x1080 default tunnel with the autotuned kernels (temporally blocked,
  resident projection), 100 steps;
* batched uneven tunnels (seed 4, n in {50, 100, 200}, non-integer radii)
  advanced together inside one Batch, each member against its own reference
  run;
* the 4096x4096 tunnel (n = 200) on the pass-by-pass blocked engine.

Bars (relative L2 per field): 1e-5, the bar this path is held to; 1e-4 with
the drain open, where the reference's extrapolation races on v(W-1, 1)
(src/fluid.cu:720-733) and two runs of the reference itself differ.
"""
import numpy as np
import pytest

import oracle
from opensayal_gb300 import Fluid, scenarios
from opensayal_gb300.batch import Batch
from tests.parity_cases import FIELDS, perturbed_state

pytestmark = pytest.mark.gpu

REL_L2_BAR = 1e-5
DRAIN_RACE_BAR = 1e-4


def bar(cfg) -> float:
    return DRAIN_RACE_BAR if cfg.enable_drain else REL_L2_BAR


def check_fields(got: dict, ref: "oracle.RefFluid", cfg, label: str) -> None:
    for field in FIELDS:
        b = ref.download(field)
        a = got[field]
        assert np.isfinite(a).all(), f"{label}/{field}: non-finite values"
        e = oracle.rel_l2(a, b)
        assert e <= bar(cfg), f"{label}/{field}: rel L2 {e:.3e} > {bar(cfg):g}"


def run_ref(cfg, state: dict, steps: int) -> "oracle.RefFluid":
    r = oracle.RefFluid(cfg)
    for k, a in state.items():
        r.upload(k, a)
    for _ in range(steps):
        r.update(None, cfg.d_t)
    return r


@pytest.mark.parametrize("drain", [1, 0])
def test_default_tunnel_as_benched_100_steps(gpu, drain):
    cfg = scenarios.default_tunnel_config()  # depths and forms autotuned
    cfg.enable_drain = drain
    state = perturbed_state(cfg, 2)
    with Fluid(cfg) as f:
        view = f.fields()
        assert view.projection_block > 0, "the benched form is temporally blocked"
        for k, a in state.items():
            f.upload(k, a)
        f.update_async(None, cfg.d_t, 100)
        f.synchronize()
        got = {k: f.download(k) for k in FIELDS}
        label = (f"1920x1080 drain={drain} block={view.projection_block} "
                 f"resident={view.projection_resident}")
    ref = run_ref(cfg, state, 100)
    check_fields(got, ref, cfg, label)
    ref.close()


def batched_members(drain: int | None):
    cfgs = scenarios.batched_scenarios(512, seed=4)
    # Eight members that cover the three sweep counts, small and large grids.
    picks = [0, 1, 2, 3, 5, 8, 13, 21]
    out = []
    for i in picks:
        c = cfgs[i]
        if drain is not None:
            c.enable_drain = drain
        out.append((i, c))
    return out


@pytest.mark.parametrize("drain", [None, 0], ids=["as_drawn", "drain_off"])
def test_batched_scenarios_vs_reference_20_steps(gpu, drain):
    members = batched_members(drain)
    ns = {c.projection_n for _, c in members}
    assert ns == {50, 100, 200}, ns
    cfgs = [c for _, c in members]
    states = []
    with Batch(cfgs) as b:
        for m, (i, c) in enumerate(members):
            view = b.scenario(m)
            st = perturbed_state(c, 4000 + i)
            for k, a in st.items():
                view.upload(k, a)
            states.append(st)
        b.step(20)
        b.synchronize()
        got = [{k: b.scenario(m).download(k) for k in FIELDS} for m in range(len(members))]
    for m, (i, c) in enumerate(members):
        ref = run_ref(c, states[m], 20)
        check_fields(got[m], ref, c, f"scenario {i} ({c.width}x{c.height}, n={c.projection_n}, "
                                     f"r={c.obstacle_radius:.3f})")
        ref.close()


@pytest.mark.parametrize("drain", [1, 0])
def test_large_grid_3_steps(gpu, drain):
    cfg = scenarios.large_config()
    cfg.enable_drain = drain
    state = perturbed_state(cfg, 3)
    with Fluid(cfg) as f:
        for k, a in state.items():
            f.upload(k, a)
        for _ in range(3):
            f.update(None, cfg.d_t)
        got = {k: f.download(k) for k in FIELDS}
        assert f.fields().projection_block > 0
    ref = run_ref(cfg, state, 3)
    check_fields(got, ref, cfg, f"4096x4096 drain={drain}")
    ref.close()
