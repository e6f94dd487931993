"""The CPU oracle (oracle/fluid_oracle.c) against independent restatements of
the reference's construction rules and against the scheme's invariants."""
import numpy as np
import pytest

import oracle
from opensayal_gb300 import scenarios
from opensayal_gb300.fluid import default_config


def numpy_mask(cfg):
    """src/fluid.cu:111-142 restated with numpy (double obstacle test)."""
    W, H = cfg.width, cfg.height
    j, i = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")  # logical (j, i)
    dist = np.sqrt((i - cfg.obstacle_center_x).astype(np.float64) ** 2 +
                   (j - cfg.obstacle_center_y).astype(np.float64) ** 2)
    solid = (i == 0) | (j == 0) | (j == H - 1)
    if not cfg.enable_drain:
        solid |= (i == W - 1)
    if cfg.obstacle_enable:
        solid |= dist < np.float64(np.float32(cfg.obstacle_radius))
    pipe = (i < cfg.pipe_length) & ((j == H // 2 - cfg.pipe_height // 2 - 1) |
                                   (j == H // 2 + cfg.pipe_height // 2 + 1))
    solid |= pipe
    fluid = ~solid
    s = np.zeros((H, W), np.int32)
    s[:, 1:] += fluid[:, :-1]
    s[:, :-1] += fluid[:, 1:]
    s[1:, :] += fluid[:-1, :]
    s[:-1, :] += fluid[1:, :]
    # logical row j is stored at memory row H-1-j
    return solid[::-1].astype(np.int32).reshape(-1), s[::-1].reshape(-1)


@pytest.mark.parametrize("make", [
    scenarios.small_config,
    lambda: (lambda c: (setattr(c, "obstacle_radius", 7.3), setattr(c, "enable_drain", 1), c)[-1])(scenarios.small_config()),
    lambda: (lambda c: (setattr(c, "pipe_length", 40), c)[-1])(default_config(96, 64)),
])
def test_mask_and_counts_bit_exact(oracle_built, make):
    cfg = make()
    o = oracle.OracleFluid(cfg)
    solid, total_s = numpy_mask(cfg)
    assert np.array_equal(o.is_solid, solid)
    assert np.array_equal(o.total_s, total_s)


def test_small_config_sets(oracle_built):
    """Inflow band: ph+1 rows (inclusive bounds, src/fluid.cu:317-319); the
    left column is solid and the drain column closed when drain is off."""
    cfg = scenarios.small_config()
    o = oracle.OracleFluid(cfg)
    o.phase(0, None, cfg.d_t)  # forces only: the step's extrapolation clears u(1, j)
    W, H = cfg.width, cfg.height
    u = o.u.reshape(H, W)[::-1]  # logical [j, i]
    inflow_rows = np.nonzero(u[:, 1] == np.float32(2.0))[0]
    assert inflow_rows.tolist() == list(range(64 - 16, 64 + 16 + 1))
    solid = o.is_solid.reshape(H, W)[::-1]
    assert solid[:, 0].all() and solid[:, W - 1].all()
    assert solid[0].all() and solid[H - 1].all()
    disc = solid[1:H - 1, 1:W - 1].sum()
    assert disc == 437  # cells with sqrt(di^2 + dj^2) < 12


def test_projection_reduces_divergence(oracle_built):
    cfg = scenarios.small_config()
    rng = np.random.default_rng(0)
    res = []
    for n in (1, 10, 50):
        c = cfg.copy()
        c.projection_n = n
        o = oracle.OracleFluid(c)
        o.u[:] = np.where(o.is_solid == 0, rng.standard_normal(o.u.size), 0).astype(np.float32)
        o.v[:] = np.where(o.is_solid == 0, rng.standard_normal(o.v.size), 0).astype(np.float32)
        rng = np.random.default_rng(0)
        o.phase(3, None, cfg.d_t)  # projection
        W, H = c.width, c.height
        u = o.u.reshape(H, W)[::-1]
        v = o.v.reshape(H, W)[::-1]
        d = (u[1:-1, 2:] - u[1:-1, 1:-1]) + (v[2:, 1:-1] - v[1:-1, 1:-1])
        act = (o.is_solid.reshape(H, W)[::-1][1:-1, 1:-1] == 0)
        res.append(float(np.sqrt((d[act] ** 2).mean())))
    assert res[0] > res[1] > res[2]


def test_smoke_stays_bounded(oracle_built):
    cfg = scenarios.small_config()
    o = oracle.OracleFluid(cfg)
    u, v = scenarios.perturbation(1, o.is_solid)
    o.u[:], o.v[:] = u, v
    for _ in range(20):
        o.update(None, cfg.d_t)
    assert np.isfinite(o.u).all() and np.isfinite(o.v).all()
    assert o.s.min() >= 0.0 and o.s.max() <= max(1.0, cfg.tunnel_smoke) + 1e-6


def test_perturbation_is_seeded_and_bounded(lib_built):
    solid = np.zeros(1000, np.int32)
    solid[::7] = 1
    u1, v1 = scenarios.perturbation(3, solid)
    u2, v2 = scenarios.perturbation(3, solid)
    assert np.array_equal(u1, u2) and np.array_equal(v1, v2)
    assert not np.array_equal(u1, scenarios.perturbation(4, solid)[0])
    assert (u1[solid == 1] == 0).all()
    assert np.abs(u1).max() <= 0.01 and np.abs(v1).max() <= 0.01
    assert np.abs(u1[solid == 0]).min() >= 0.0 and u1.std() > 0.004


def test_batched_scenarios_distribution(lib_built):
    scs = scenarios.batched_scenarios(64, seed=4)
    assert len(scs) == 64
    for c in scs:
        assert 128 <= c.width <= 1024 and c.width % 32 == 0
        assert 128 <= c.height <= 1024 and c.height % 32 == 0
        assert c.pipe_height == c.height // 4
        assert 0.5 <= c.tunnel_speed <= 3.0
        assert c.width // 4 <= c.obstacle_center_x <= 3 * c.width // 4
        assert 4.0 <= c.obstacle_radius <= 0.1 * c.height
        assert -10.0 <= c.g <= 0.0 and c.projection_n in (50, 100, 200)


def test_serving_requests_distribution(lib_built):
    """Poisson arrivals at 200/s for 60 s: about 12,000 requests in order, the
    batched scenario mix, steps in [100, 5000], half in BF16 storage."""
    reqs = scenarios.serving_requests(200.0, 60.0, seed=5)
    n = len(reqs)
    assert abs(n - 12000) < 5 * np.sqrt(12000)
    t = np.array([r.arrival for r in reqs])
    assert (np.diff(t) > 0).all() and t[0] > 0 and t[-1] < 60.0
    gaps = np.diff(t)
    assert abs(gaps.mean() - 1 / 200.0) < 0.1 / 200.0  # exponential gaps, mean 1/rate
    steps = np.array([r.steps for r in reqs])
    assert steps.min() >= 100 and steps.max() <= 5000
    assert abs(steps.mean() - 2550) < 100
    bf16 = np.mean([r.config.storage == 2 for r in reqs])
    assert 0.45 < bf16 < 0.55
    assert all(r.index == k for k, r in enumerate(reqs))
    assert len({r.seed for r in reqs}) == n  # one perturbation seed per request
    again = scenarios.serving_requests(200.0, 60.0, seed=5)
    assert [(r.arrival, r.steps) for r in again] == [(r.arrival, r.steps) for r in reqs]
