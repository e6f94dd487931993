"""Generate the golden fixtures from the reference's own kernels.

Runs on a machine with a GPU: the unmodified src/fluid.cu device code
(oracle/_ref/fluid_ref.cubin) driven by oracle/ref_harness.cpp, on seeded
inputs. The fixtures pin the CPU oracle (tests/test_golden.py) without a GPU.

    python tests/golden/make_golden.py [outdir]

Fixtures:
  small_100.npz     256x128 parity case, seed-1 perturbation, 100 steps.
  small_p_20.npz    the same with pressure on, 20 steps.
  phases_64x40.npz  one reference phase at a time on a random 64x40 state.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from opensayal_gb300 import native, scenarios  # noqa: E402
from tests.parity_cases import ACTIVE_SOURCE, load_ref, perturbed_state, random_state  # noqa: E402
from tests.test_parity_gpu import PHASES, phase_config  # noqa: E402


# Fields each reference phase writes (src/fluid.cu).
PHASE_WRITES = {
    "forces": ("vel_x", "vel_y", "smoke"),
    "forces_inactive": ("vel_x", "vel_y", "smoke"),
    "zero_pressure": ("pressure",),
    "projection": ("vel_x", "vel_y", "pressure"),
    "extrapolation": ("vel_x", "vel_y"),
    "velocity_advection": ("vel_x", "vel_y"),
    "smoke_advection": ("smoke",),
    "decay": ("smoke",),
    "diffusion": ("vel_x",),
}


def golden_phase_config(drain: int):
    """64x40 grid with every phase switched on (pressure, decay, drag, gravity)."""
    return phase_config(enable_drain=drain, width=64, height=40, obstacle_center_x=30,
                        obstacle_center_y=19, obstacle_radius=6.5, pipe_height=14,
                        smoke_height=8)


def run_case(cfg, seed, steps):
    ref = load_ref(cfg, perturbed_state(cfg, seed))
    for _ in range(steps):
        ref.update(None, cfg.d_t)
    out = {k: ref.download(k) for k in ("vel_x", "vel_y", "smoke", "pressure")}
    out["is_solid"] = ref.download("is_solid")
    out["total_s"] = ref.download("total_s")
    out["steps"] = np.int32(steps)
    out["seed"] = np.int32(seed)
    if cfg.enable_pressure:
        out["pressure_range"] = np.array(ref.pressure_range, np.float32)
    return out


def main(outdir: Path) -> None:
    outdir.mkdir(parents=True, exist_ok=True)
    cfg = scenarios.small_config()
    np.savez_compressed(outdir / "small_100.npz", **run_case(cfg, 1, 100))
    cfg_p = scenarios.small_config()
    cfg_p.enable_pressure = 1
    np.savez_compressed(outdir / "small_p_20.npz", **run_case(cfg_p, 1, 20))
    phases = {}
    for drain in (0, 1):
        c = golden_phase_config(drain)
        base = oracle.OracleFluid(c)
        state = random_state(c, 11, base.is_solid)
        for k, a in state.items():
            phases[f"in_d{drain}_{k}"] = a
        for name, ph, src in PHASES + [("diffusion", native.PHASE_DIFFUSION, None)]:
            ref = load_ref(c, state)
            ref.phase(ph, src, 0.05)
            for k in PHASE_WRITES[name]:
                phases[f"out_d{drain}_{name}_{k}"] = ref.download(k)
    np.savez_compressed(outdir / "phases_64x40.npz", **phases)
    print("wrote", sorted(p.name for p in outdir.glob("*.npz")))


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent)
