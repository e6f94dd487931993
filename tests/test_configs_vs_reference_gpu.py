"""The configurations the measurements are quoted on, checked directly against
the reference's own kernels (the unmodified src/fluid.cu device code through
oracle/ref_harness.cpp), in the form the measurements run them:

* the 1920x1080 default tunnel with the autotuned kernels (temporally blocked,
  resident projection), 100 steps, viscous and inviscid; without diffusion
  and with the drain closed nothing races, and the fields must be identical;
* batched uneven tunnels (seed 4, n in {50, 100, 200}, non-integer radii)
  advanced together inside one Batch, each member against its own reference
  run;
* the 4096x4096 tunnel (n = 200) on the pass-by-pass blocked engine.

The reference is not deterministic: its diffusion sweeps u in place from
racing threads (src/fluid.cu:167-190), and with the drain open its
extrapolation writes v(W-1, 1) from two threads (src/fluid.cu:720-733). Each
case therefore runs the reference twice and measures its own spread s (the
relative L2 between its two runs). The bar for the library against the
reference is max(1e-5, 2 s) per field: 1e-5 where the reference repeats
itself, and twice its own disagreement where it does not.

The drain race is different in kind. The library writes 0 there (the
outcome the reference gives most often), while the reference's outcome can
change from step to step and from one GPU to another: the 1920x1080 tunnel
without diffusion has ended 3.7e-6 from the library on one GB300 and 1.1e-4
on another, and a 448x704 member 1.1e-4, each time with the reference's two
runs agreeing to a few 1e-6. With the drain open a case is therefore held to
max(1e-5, 2 s, 5e-4), about five times the largest effect of the race seen,
and every such case has a twin with the drain closed (no race) held to
max(1e-5, 2 s).
"""
import numpy as np
import pytest

import oracle
from opensayal_gb300 import Fluid, scenarios
from opensayal_gb300.batch import Batch
from tests.parity_cases import FIELDS, perturbed_state

pytestmark = pytest.mark.gpu

FLOOR = 1e-5
DRAIN_RACE_BAR = 5e-4


def run_ref(cfg, state: dict, steps: int) -> dict:
    r = oracle.RefFluid(cfg)
    for k, a in state.items():
        r.upload(k, a)
    for _ in range(steps):
        r.update(None, cfg.d_t)
    out = {k: r.download(k) for k in FIELDS}
    r.close()
    return out


def check_against_reference(got: dict, cfg, state: dict, steps: int, label: str) -> dict:
    a = run_ref(cfg, state, steps)
    b = run_ref(cfg, state, steps)
    report = {}
    for field in FIELDS:
        x = got[field]
        assert np.isfinite(x).all(), f"{label}/{field}: non-finite values"
        spread = oracle.rel_l2(b[field], a[field])
        bar = max(FLOOR, 2 * spread, DRAIN_RACE_BAR if cfg.enable_drain else 0.0)
        e = oracle.rel_l2(x, a[field])
        report[field] = (e, spread)
        assert e <= bar, (f"{label}/{field}: rel L2 {e:.3e} > {bar:.1e} (reference spread "
                          f"{spread:.1e})")
    return report


@pytest.mark.parametrize("drain", [1, 0])
@pytest.mark.parametrize("viscosity", [0.001, 0.0])
def test_default_tunnel_as_benched_100_steps(gpu, drain, viscosity):
    cfg = scenarios.default_tunnel_config()  # depths and forms autotuned
    cfg.enable_drain = drain
    cfg.viscosity = viscosity
    state = perturbed_state(cfg, 2)
    with Fluid(cfg) as f:
        view = f.fields()
        assert view.projection_block > 0, "the benched form is temporally blocked"
        for k, a in state.items():
            f.upload(k, a)
        f.update_async(None, cfg.d_t, 100)
        f.synchronize()
        got = {k: f.download(k) for k in FIELDS}
        label = (f"1920x1080 drain={drain} viscosity={viscosity} "
                 f"block={view.projection_block} resident={view.projection_resident}")
    report = check_against_reference(got, cfg, state, 100, label)
    if not drain and viscosity == 0.0:
        # No race anywhere: the reference repeats itself, and the library
        # equals it bit for bit after 100 steps.
        for field, (e, spread) in report.items():
            assert e == 0.0 and spread == 0.0, (label, field, e, spread)


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
        check_against_reference(got[m], c, states[m], 20,
                                f"scenario {i} ({c.width}x{c.height}, n={c.projection_n}, "
                                f"r={c.obstacle_radius:.3f}, drain={c.enable_drain})")


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
    check_against_reference(got, cfg, state, 3, f"4096x4096 drain={drain}")


def test_default_tunnel_with_pressure_20_steps(gpu):
    """sim.enable_pressure on the benchmarked grid: the resident projection
    accumulates p in its sweeps and the extrema come from the warp-shuffle
    reduction. Without diffusion and with the drain closed nothing races, so
    every field, pressure included, must equal the reference's bit for bit,
    and so must the extrema (the reference's Thrust reductions)."""
    cfg = scenarios.default_tunnel_config()
    cfg.enable_pressure = 1
    cfg.enable_drain = 0
    cfg.viscosity = 0.0
    state = perturbed_state(cfg, 6)
    with Fluid(cfg) as f:
        assert f.fields().projection_block > 0
        for k, a in state.items():
            f.upload(k, a)
        for _ in range(20):
            f.update(None, cfg.d_t)
        got = {k: f.download(k) for k in FIELDS + ("pressure",)}
        lo, hi = f.min_pressure, f.max_pressure
    r = oracle.RefFluid(cfg)
    for k, a in state.items():
        r.upload(k, a)
    for _ in range(20):
        r.update(None, cfg.d_t)
    for field in FIELDS + ("pressure",):
        want = r.download(field)
        assert np.array_equal(got[field], want), (field, int((got[field] != want).sum()))
    rlo, rhi = r.pressure_range
    r.close()
    assert (lo, hi) == (rlo, rhi)
