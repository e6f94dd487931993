"""Shared set-up for the parity tests: one scenario run three ways (the GB300
library, the reference's own kernels, the CPU oracle) on identical inputs."""
from __future__ import annotations

import numpy as np

import oracle
from opensayal_gb300 import Fluid, scenarios
from opensayal_gb300.fluid import Source

FIELDS = ("vel_x", "vel_y", "smoke")


def random_state(cfg, seed: int, solid: np.ndarray) -> dict:
    """A generic mid-simulation state: O(1) velocities on fluid faces, smoke in
    [0, 1] everywhere, pressure O(1)."""
    rng = np.random.default_rng(seed)
    n = cfg.width * cfg.height
    fluid = solid == 0
    return {
        "vel_x": np.where(fluid, rng.uniform(-2, 2, n), 0).astype(np.float32),
        "vel_y": np.where(fluid, rng.uniform(-2, 2, n), 0).astype(np.float32),
        "smoke": rng.uniform(0, 1, n).astype(np.float32),
        "pressure": rng.uniform(-1, 1, n).astype(np.float32),
    }


def load_lib(cfg, state: dict) -> Fluid:
    f = Fluid(cfg)
    for k, a in state.items():
        f.upload(k, a)
    return f


def load_ref(cfg, state: dict) -> "oracle.RefFluid":
    r = oracle.RefFluid(cfg)
    for k, a in state.items():
        r.upload(k, a)
    return r


def load_oracle(cfg, state: dict) -> "oracle.OracleFluid":
    o = oracle.OracleFluid(cfg)
    for k, a in state.items():
        o.fields()[k][:] = a
    return o


def perturbed_state(cfg, seed: int) -> dict:
    o = oracle.OracleFluid(cfg)
    u, v = scenarios.perturbation(seed, o.is_solid)
    n = cfg.width * cfg.height
    z = np.zeros(n, np.float32)
    return {"vel_x": u, "vel_y": v, "smoke": z, "pressure": z.copy()}


def same_bits(a: np.ndarray, b: np.ndarray) -> bool:
    """Bit-for-bit equality, except that +0.0 and -0.0 compare equal."""
    return bool(np.array_equal(a, b) and np.array_equal(np.isnan(a), np.isnan(b)))


ACTIVE_SOURCE = Source(active=True, smoke=0.7, velocity=0.3, position=(40, 30))
