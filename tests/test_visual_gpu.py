"""Headless visuals against the reference's own device code on the same
fields: pixel colours (the reference's hsv_to_rgb / map_rgba / clamp), path
lines (the reference's Fluid::trace) and velocity arrows (the reference's
get_general_velocity, make_arrow_data restated), all bit for bit; entries the
reference leaves alone stay as they were."""
import math

import numpy as np
import pytest

import oracle
from opensayal_gb300 import native
from opensayal_gb300.fluid import Fluid, default_config, visual_defaults
from tests.parity_cases import load_lib, random_state

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SENTINEL = 0x1234567


def scene(w, h, seed, **over):
    c = default_config(w, h)
    c.tunnel_speed = 1.5
    c.obstacle_radius = 9.0
    c.projection_block = 4
    for k, v in over.items():
        setattr(c, k, v)
    solid = oracle.OracleFluid(c).is_solid
    state = random_state(c, seed, solid)
    rng = np.random.default_rng(seed)
    n = w * h
    state["smoke"] = rng.uniform(0.0, 1.0, n).astype(np.float32)
    state["pressure"] = rng.uniform(-3.0, 5.0, n).astype(np.float32)
    state["vel_x"] = rng.uniform(-2.0, 2.0, n).astype(np.float32)
    state["vel_y"] = rng.uniform(-2.0, 2.0, n).astype(np.float32)
    return c, state


def both(c, state):
    f = load_lib(c, state)
    r = oracle.RefFluid(c)
    for k, a in state.items():
        r.upload(k, a)
    return f, r


@pytest.mark.parametrize("pressure,smoke", [(0, 1), (1, 0), (1, 1), (0, 0)])
def test_pixels_match_reference(gpu, pressure, smoke):
    c, state = scene(203, 117, 5, enable_pressure=pressure, enable_smoke=smoke)
    f, r = both(c, state)
    f.run_phase(native.PHASE_PRESSURE_RANGE, None, c.d_t)
    r.phase(native.PHASE_PRESSURE_RANGE, None, c.d_t)
    lo, hi = r.pressure_range
    if pressure:
        assert (f.min_pressure, f.max_pressure) == (lo, hi)
    n = c.width * c.height
    init = np.full(n, SENTINEL, np.int32)
    d = torch.tensor(init, device="cuda")
    f.render_pixels(d.data_ptr())
    f.synchronize()
    got = d.cpu().numpy()
    want = r.render_pixels(f.min_pressure, f.max_pressure, init)
    assert np.array_equal(got, want), f"{int((got != want).sum())} pixels differ"
    f.close()


@pytest.mark.parametrize("distance,length", [(7, 15), (20, 20), (1, 4)])
def test_traces_match_reference(gpu, distance, length):
    c, state = scene(150, 96, 8)
    f, r = both(c, state)
    v = visual_defaults()
    v.trace_distance, v.trace_length = distance, length
    tw, th = c.width // distance, c.height // distance
    init = np.full(tw * th * length, SENTINEL, np.int32)
    dx, dy = torch.tensor(init, device="cuda"), torch.tensor(init, device="cuda")
    f.render_traces(v, 0.05, dx.data_ptr(), dy.data_ptr())
    f.synchronize()
    wx, wy = r.render_traces(0.05, distance, length, init, init)
    gx, gy = dx.cpu().numpy(), dy.cpu().numpy()
    assert np.array_equal(gx, wx) and np.array_equal(gy, wy), \
        f"{int((gx != wx).sum() + (gy != wy).sum())} points differ"
    f.close()


@pytest.mark.parametrize("cell_px,distance", [(1, 5), (3, 8), (1, 1)])
def test_arrows_match_reference(gpu, cell_px, distance):
    c, state = scene(160, 90, 13)
    f, r = both(c, state)
    v = visual_defaults()
    v.cell_pixel_size, v.arrow_distance = cell_px, distance
    v.arrow_length_multiplier, v.arrow_disable_threshold, v.arrow_head_length = 6.0, 0.4, 7
    aw, ah = c.width // distance, c.height // distance
    init = np.full(aw * ah * 9, SENTINEL, np.int32)
    d = torch.tensor(init, device="cuda")
    f.render_arrows(v, d.data_ptr())
    f.synchronize()
    got = d.cpu().numpy().reshape(-1, 9)
    want = r.render_arrows(cell_px, v.arrow_length_multiplier, v.arrow_disable_threshold,
                           float(v.arrow_head_length), np.float32(math.pi / 8).item(), distance,
                           init)
    untouched = (want[:, 0] == SENTINEL) & (want[:, 8] == (SENTINEL & 0xFF))
    assert np.array_equal(got[untouched], init.reshape(-1, 9)[untouched])
    written = ~untouched
    assert np.array_equal(got[written, 8] != 0, want[written, 8] != 0), "valid flags differ"
    valid = written & (want[:, 8] != 0)
    assert valid.sum() > 0
    assert np.array_equal(got[valid, :8], want[valid, :8]), \
        f"{int((got[valid, :8] != want[valid, :8]).any(axis=1).sum())} arrows differ"
    f.close()
