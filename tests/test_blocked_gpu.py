"""The temporally blocked projection and diffusion give exactly the bits of
the plain per-sweep kernels (which match the reference's kernels, see
test_parity_gpu.py): the red/black ordering and the Jacobi update are exact,
so tiling, halos and sweeps-per-pass must not change a single result."""
import numpy as np
import pytest

import oracle
from opensayal_gb300 import native, scenarios
from opensayal_gb300.fluid import default_config
from tests.parity_cases import FIELDS, load_lib, perturbed_state, random_state, same_bits

pytestmark = pytest.mark.gpu

SIZES = [(96, 64), (256, 128), (300, 77), (1920, 1080), (513, 260), (17, 9)]


def tunnel(w, h, **over):
    c = default_config(w, h)
    c.tunnel_speed = 2.0
    c.g = -5.0
    c.projection_n = 13
    c.enable_pressure = 1
    for k, v in over.items():
        setattr(c, k, v)
    return c


@pytest.mark.parametrize("w,h", SIZES)
@pytest.mark.parametrize("k", [1, 3, 4, 8])
@pytest.mark.parametrize("phase", [native.PHASE_PROJECTION, native.PHASE_DIFFUSION])
def test_blocked_phase_equals_plain(gpu, w, h, k, phase):
    base = tunnel(w, h, viscosity=0.02)
    solid = oracle.OracleFluid(base).is_solid
    state = random_state(base, 21, solid)
    plain_cfg = base.copy()
    plain_cfg.projection_block = -1
    blocked_cfg = base.copy()
    blocked_cfg.projection_block = k
    a, b = load_lib(plain_cfg, state), load_lib(blocked_cfg, state)
    a.run_phase(phase, None, 0.05)
    b.run_phase(phase, None, 0.05)
    for field in FIELDS + ("pressure",):
        x, y = a.download(field), b.download(field)
        assert same_bits(x, y), f"{field}: {int((x != y).sum())} cells differ"
    a.close()
    b.close()


@pytest.mark.parametrize("pressure", [0, 1])
@pytest.mark.parametrize("k", [2, 4, 6])
def test_blocked_steps_equal_plain(gpu, pressure, k):
    cfg = scenarios.small_config()
    cfg.enable_pressure = pressure
    cfg.enable_drain = 1
    cfg.g = -3.0
    state = perturbed_state(cfg, 8)
    plain_cfg = cfg.copy()
    plain_cfg.projection_block = -1
    blocked_cfg = cfg.copy()
    blocked_cfg.projection_block = k
    a, b = load_lib(plain_cfg, state), load_lib(blocked_cfg, state)
    for _ in range(10):
        a.update(None, cfg.d_t)
        b.update(None, cfg.d_t)
    for field in FIELDS + (("pressure",) if pressure else ()):
        x, y = a.download(field), b.download(field)
        assert same_bits(x, y), f"{field}: {int((x != y).sum())} cells differ"
    if pressure:
        assert a.min_pressure == b.min_pressure and a.max_pressure == b.max_pressure


def test_default_workload_blocked_equals_plain(gpu):
    cfg = scenarios.default_tunnel_config()
    state = perturbed_state(cfg, 2)
    plain_cfg = cfg.copy()
    plain_cfg.projection_block = -1
    a, b = load_lib(plain_cfg, state), load_lib(cfg, state)
    for _ in range(3):
        a.update(None, cfg.d_t)
        b.update(None, cfg.d_t)
    for field in FIELDS:
        assert same_bits(a.download(field), b.download(field)), field


@pytest.mark.parametrize("w,h", [(1920, 1080), (300, 77), (17, 9)])
@pytest.mark.parametrize("k,dk", [(8, 16), (4, 12), (8, 20), (2, 32)])
def test_diffusion_depth_apart_from_projection(gpu, w, h, k, dk):
    """diffusion_block sets the Jacobi sweeps per diffusion pass apart from
    the projection's depth; the results stay those of the plain kernels."""
    base = tunnel(w, h, viscosity=0.02, projection_n=37)
    solid = oracle.OracleFluid(base).is_solid
    state = random_state(base, 33, solid)
    plain_cfg = base.copy()
    plain_cfg.projection_block = -1
    blocked_cfg = base.copy()
    blocked_cfg.projection_block = k
    blocked_cfg.diffusion_block = dk
    blocked_cfg.projection_resident = -1
    a, b = load_lib(plain_cfg, state), load_lib(blocked_cfg, state)
    a.run_phase(native.PHASE_DIFFUSION, None, 0.05)
    b.run_phase(native.PHASE_DIFFUSION, None, 0.05)
    ms, launches = b.profile_phase(native.PHASE_DIFFUSION, None, 0.05, 1)
    # ceil(37 / dk) passes, plus a copy back when their count is odd
    passes = -(-37 // dk)
    assert launches == passes + (passes % 2)
    b.run_phase(native.PHASE_DIFFUSION, None, 0.05)
    a.run_phase(native.PHASE_DIFFUSION, None, 0.05)
    a.run_phase(native.PHASE_DIFFUSION, None, 0.05)
    for field in FIELDS:
        x, y = a.download(field), b.download(field)
        assert same_bits(x, y), f"{field}: {int((x != y).sum())} cells differ"
    a.close()
    b.close()


def test_diffusion_depth_in_steps_with_resident_projection(gpu):
    cfg = scenarios.default_tunnel_config()
    state = perturbed_state(cfg, 5)
    plain_cfg = cfg.copy()
    plain_cfg.projection_block = -1
    deep = cfg.copy()
    deep.projection_block = 8
    deep.projection_resident = 1
    deep.diffusion_block = 16
    a, b = load_lib(plain_cfg, state), load_lib(deep, state)
    assert b.fields().projection_resident == 1
    for _ in range(3):
        a.update(None, cfg.d_t)
        b.update(None, cfg.d_t)
    for field in FIELDS:
        assert same_bits(a.download(field), b.download(field)), field


@pytest.mark.parametrize("phase", [native.PHASE_PROJECTION, native.PHASE_DIFFUSION])
def test_phase_kernel_timing_leaves_the_phase_as_run(gpu, phase):
    """os_profile_phase_kernels times each repetition's own kernels apart from
    the copy back, and the fields end as after the same phases run one by
    one."""
    cfg = scenarios.default_tunnel_config()
    cfg.projection_block, cfg.projection_resident = 8, 1
    state = perturbed_state(cfg, 7)
    a, b = load_lib(cfg, state), load_lib(cfg, state)
    kms, ms, launches = b.profile_phase_kernels(phase, None, cfg.d_t, 3)
    for _ in range(3):
        a.run_phase(phase, None, cfg.d_t)
    assert 0.0 < kms <= ms
    _, launches_plain = b.profile_phase(phase, None, cfg.d_t, 3)
    assert launches == launches_plain
    for _ in range(3):
        a.run_phase(phase, None, cfg.d_t)
    for field in FIELDS:
        x, y = a.download(field), b.download(field)
        assert same_bits(x, y), f"{field}: {int((x != y).sum())} cells differ"
    a.close()
    b.close()
