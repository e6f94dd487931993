"""Seeded synthetic wind-tunnel scenarios: the workloads the library is measured on.

Every key not named here keeps its ConfigParser default
(src/config_parser.cpp:21-179), in particular viscosity = 0.001 (diffusion on).
The initial velocity perturbation is uniform[-0.01, 0.01] on u and v of every
non-solid cell, drawn from a counter-based generator (SplitMix64 of the seed,
the field and the cell index) so that any implementation can reproduce it.
"""
from __future__ import annotations

import numpy as np

from .fluid import default_config
from .native import OsConfig

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(x: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser applied to x + golden (vectorised, wrapping uint64)."""
    with np.errstate(over="ignore"):
        z = x.astype(np.uint64) + _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, stream: int, count: int, lo: float, hi: float) -> np.ndarray:
    """`count` float32 draws in [lo, hi) from (seed, stream, index)."""
    idx = np.arange(count, dtype=np.uint64)
    with np.errstate(over="ignore"):
        key = (np.uint64(seed) * _GOLDEN) ^ (np.uint64(stream) << np.uint64(48)) ^ idx
    bits = splitmix64(key) >> np.uint64(40)  # 24 random bits
    u01 = bits.astype(np.float64) / float(1 << 24)
    return (lo + (hi - lo) * u01).astype(np.float32)


def perturbation(seed: int, is_solid: np.ndarray, amplitude: float = 0.01):
    """(u, v) initial fields: uniform[-a, a] on non-solid cells, 0 on solid ones.
    `is_solid` is the W*H mask in the reference layout."""
    n = is_solid.size
    fluid = (is_solid == 0)
    u = np.where(fluid, uniform(seed, 1, n, -amplitude, amplitude), 0).astype(np.float32)
    v = np.where(fluid, uniform(seed, 2, n, -amplitude, amplitude), 0).astype(np.float32)
    return u, v


def small_config() -> OsConfig:
    """256x128 parity case: pipe 32 rows, inflow 2.0 with smoke 1, obstacle r=12
    at (128, 64), g=0, dt=0.05, n=50, o=1.9, drain off, decay off."""
    c = default_config(256, 128)
    c.pipe_height = 32
    c.tunnel_speed = 2.0
    c.tunnel_smoke = 1.0
    c.obstacle_center_x, c.obstacle_center_y, c.obstacle_radius = 128, 64, 12.0
    c.g = 0.0
    c.d_t = 0.05
    c.density = 1.0
    c.projection_n, c.projection_o = 50, 1.9
    c.enable_drain = 0
    c.smoke_enable_decay = 0
    return c


def default_tunnel_config() -> OsConfig:
    """1920x1080 reference default: pipe 270, inflow 2.0 with smoke 1, obstacle
    (960, 540) r=36, g=-5, dt=0.05, n=50, o=1.9, drain on, smoke on."""
    c = default_config(1920, 1080)
    c.pipe_height = 270
    c.tunnel_speed = 2.0
    c.tunnel_smoke = 1.0
    c.obstacle_center_x, c.obstacle_center_y, c.obstacle_radius = 960, 540, 36.0
    c.g = -5.0
    c.d_t = 0.05
    c.projection_n, c.projection_o = 50, 1.9
    return c


def large_config() -> OsConfig:
    """4096x4096 bandwidth-bound grid: pipe 1024, obstacle r=128 at the centre,
    g=-5, dt=0.02, n=200, o=1.9."""
    c = default_config(4096, 4096)
    c.pipe_height = 1024
    c.tunnel_speed = 2.0
    c.tunnel_smoke = 1.0
    c.obstacle_center_x, c.obstacle_center_y, c.obstacle_radius = 2048, 2048, 128.0
    c.g = -5.0
    c.d_t = 0.02
    c.projection_n, c.projection_o = 200, 1.9
    return c


CONFIGS = {
    "small": (small_config, 1, 100),
    "default": (default_tunnel_config, 2, 1000),
    "large": (large_config, 3, 500),
}


def _draw_scenario(rng: np.random.Generator) -> OsConfig:
    sizes = np.arange(128, 1025, 32)
    w = int(rng.choice(sizes))
    h = int(rng.choice(sizes))
    c = default_config(w, h)
    c.pipe_height = h // 4
    c.tunnel_speed = float(rng.uniform(0.5, 3.0))
    c.tunnel_smoke = 1.0
    c.obstacle_center_x = int(rng.integers(w // 4, 3 * w // 4 + 1))
    c.obstacle_center_y = int(rng.integers(h // 4, 3 * h // 4 + 1))
    c.obstacle_radius = float(rng.uniform(4.0, 0.1 * h))
    c.g = float(rng.uniform(-10.0, 0.0))
    c.projection_n = int(rng.choice([50, 100, 200]))
    c.projection_o = 1.9
    c.d_t = 0.05
    return c


def batched_scenarios(count: int = 512, seed: int = 4) -> list[OsConfig]:
    """Uneven grids: W, H uniform in {128, 160, ..., 1024}, pipe H/4, inflow
    U[0.5, 3], obstacle centre integer-uniform over the middle half, radius
    U[4, 0.1 H], g U[-10, 0], n in {50, 100, 200}, o 1.9, dt 0.05."""
    rng = np.random.default_rng(seed)
    return [_draw_scenario(rng) for _ in range(count)]


class Request:
    """One served scenario: arrival time (s), config, step count and the seed
    of its initial velocity perturbation."""

    __slots__ = ("index", "arrival", "config", "steps", "seed")

    def __init__(self, index, arrival, config, steps, seed):
        self.index, self.arrival, self.config, self.steps, self.seed = (
            index, arrival, config, steps, seed)

    @property
    def cells(self) -> int:
        return self.config.width * self.config.height


def serving_requests(rate: float = 200.0, seconds: float = 60.0, seed: int = 5,
                     mixed_share: float = 0.5) -> list[Request]:
    """Poisson arrivals at `rate` per second for `seconds`; each request is a
    scenario drawn as in batched_scenarios with a step count uniform in
    [100, 5000] and, with probability `mixed_share`, BF16 storage of u, v and
    smoke (FP32 otherwise)."""
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t >= seconds:
            return out
        c = _draw_scenario(rng)
        steps = int(rng.integers(100, 5001))
        if rng.random() < mixed_share:
            c.storage = 2  # OS_STORAGE_BF16
        out.append(Request(len(out), t, c, steps, seed * 1_000_003 + len(out)))
