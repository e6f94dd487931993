"""Pins the CPU oracle to golden fixtures produced by the reference's own
kernels (tests/golden/make_golden.py, run on a GPU).

Bars: masks and counts bit-exact; one phase at a time within 1e-5 relative L2
(the oracle rounds exactly where the reference's fast-math build rounds
approximately: a few ulp per operation); 20 pressure steps within 1e-4 and
100 viscous steps within 2e-4 (coherent drift of the fast-math division by
1 + 4a across ~5000 diffusion sweeps, see tests/test_parity_gpu.py).
"""
from pathlib import Path

import numpy as np
import pytest

import oracle
from opensayal_gb300 import native, scenarios
from tests.golden.make_golden import PHASE_WRITES, golden_phase_config
from tests.parity_cases import load_oracle, perturbed_state
from tests.test_parity_gpu import PHASES, race_sites

GOLDEN = Path(__file__).resolve().parent / "golden"


def fixture(name):
    path = GOLDEN / name
    if not path.exists():
        pytest.fail(f"missing golden fixture {path}")
    return np.load(path)


@pytest.mark.parametrize("name,steps,bar", [("small_100.npz", 100, 2e-4),
                                            ("small_p_20.npz", 20, 1e-4)])
def test_oracle_full_steps_against_reference_kernels(oracle_built, name, steps, bar):
    g = fixture(name)
    cfg = scenarios.small_config()
    if "pressure_range" in g.files:
        cfg.enable_pressure = 1
    assert int(g["steps"]) == steps
    o = load_oracle(cfg, perturbed_state(cfg, int(g["seed"])))
    assert np.array_equal(o.is_solid, g["is_solid"])
    assert np.array_equal(o.total_s, g["total_s"])
    for _ in range(steps):
        o.update(None, cfg.d_t)
    fields = ("vel_x", "vel_y", "smoke") + (("pressure",) if cfg.enable_pressure else ())
    for f in fields:
        e = oracle.rel_l2(o.fields()[f], g[f])
        assert e <= bar, f"{name}/{f}: {e:.3e}"
    if cfg.enable_pressure:
        lo, hi = g["pressure_range"]
        assert abs(o.min_pressure - lo) <= 1e-3 * abs(lo)
        assert abs(o.max_pressure - hi) <= 1e-3 * abs(hi)


@pytest.mark.parametrize("drain", [0, 1])
@pytest.mark.parametrize("name,phase,src", PHASES + [("diffusion", native.PHASE_DIFFUSION, None)],
                         ids=[p[0] for p in PHASES] + ["diffusion"])
def test_oracle_phase_against_reference_kernels(oracle_built, name, phase, src, drain):
    g = fixture("phases_64x40.npz")
    cfg = golden_phase_config(drain)
    state = {k: g[f"in_d{drain}_{k}"] for k in ("vel_x", "vel_y", "smoke", "pressure")}
    o = load_oracle(cfg, state)
    o.phase(phase, src, 0.05)
    racy = race_sites(cfg) if phase == native.PHASE_EXTRAPOLATION else {}
    for f in PHASE_WRITES[name]:
        mine = o.fields()[f].copy()
        ref = g[f"out_d{drain}_{name}_{f}"]
        for k in racy.get(f, []):
            mine[k] = ref[k]
        e = oracle.rel_l2(mine, ref)
        assert e <= 1e-5, f"{name}/{f}: {e:.3e}"
