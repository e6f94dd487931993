"""The resident projection (one cooperative launch per phase, tiles kept in
shared memory, halos exchanged between passes through bounded neighbour
waits) gives exactly the bits of the pass-by-pass engine and of the plain
per-sweep kernels; its waits give up and report instead of hanging."""
import numpy as np
import pytest

import oracle
from opensayal_gb300 import native, scenarios
from opensayal_gb300.fluid import Fluid, default_config
from tests.parity_cases import FIELDS, load_lib, perturbed_state, random_state, same_bits

pytestmark = pytest.mark.gpu

# Sizes whose tiles fit one per SM: several tile rows and columns, a width that
# is not a multiple of 4 (scalar staging), a grid with one tile row.
SIZES = [(1920, 1080), (513, 260), (300, 77), (1000, 40), (2048, 1200)]


def tunnel(w, h, **over):
    c = default_config(w, h)
    c.tunnel_speed = 2.0
    c.g = -5.0
    c.projection_n = 21
    for k, v in over.items():
        setattr(c, k, v)
    return c


def pair(base, state, k):
    passes = base.copy()
    passes.projection_block = k
    passes.projection_resident = -1
    resident = base.copy()
    resident.projection_block = k
    resident.projection_resident = 1
    a, b = load_lib(passes, state), load_lib(resident, state)
    assert a.fields().projection_resident == 0
    if not b.fields().projection_resident & 1:
        a.close()
        b.close()
        pytest.skip("tiles of this size do not fit one per SM in shared memory")
    return a, b


@pytest.mark.parametrize("w,h", SIZES)
@pytest.mark.parametrize("k", [2, 4, 8])
@pytest.mark.parametrize("pressure", [0, 1])
def test_resident_projection_equals_passes(gpu, w, h, k, pressure):
    base = tunnel(w, h, enable_pressure=pressure)
    solid = oracle.OracleFluid(base).is_solid
    state = random_state(base, 31, solid)
    a, b = pair(base, state, k)
    a.run_phase(native.PHASE_PROJECTION, None, 0.05)
    b.run_phase(native.PHASE_PROJECTION, None, 0.05)
    for field in FIELDS + ("pressure",):
        x, y = a.download(field), b.download(field)
        assert same_bits(x, y), f"{field}: {int((x != y).sum())} cells differ"
    a.close()
    b.close()


@pytest.mark.parametrize("w,h", SIZES)
@pytest.mark.parametrize("k", [4, 8, 12])
def test_resident_diffusion_equals_passes(gpu, w, h, k):
    base = tunnel(w, h, viscosity=0.02)
    solid = oracle.OracleFluid(base).is_solid
    state = random_state(base, 37, solid)
    passes = base.copy()
    passes.projection_block = k
    passes.projection_resident = -1
    resident = base.copy()
    resident.projection_block = k
    resident.projection_resident = 2
    a, b = load_lib(passes, state), load_lib(resident, state)
    if not b.fields().projection_resident & 2:
        a.close()
        b.close()
        pytest.skip("tiles of this size do not fit one per SM in shared memory")
    a.run_phase(native.PHASE_DIFFUSION, None, 0.05)
    b.run_phase(native.PHASE_DIFFUSION, None, 0.05)
    for field in FIELDS:
        x, y = a.download(field), b.download(field)
        assert same_bits(x, y), f"{field}: {int((x != y).sum())} cells differ"
    a.close()
    b.close()


@pytest.mark.parametrize("storage", [0, 1, 2])
def test_resident_steps_equal_plain(gpu, storage):
    cfg = scenarios.default_tunnel_config()
    cfg.storage = storage
    cfg.projection_n = 30
    state = perturbed_state(cfg, 12)
    plain = cfg.copy()
    plain.projection_block = -1
    res = cfg.copy()
    res.projection_block = 4
    res.projection_resident = 3
    a, b = load_lib(plain, state), load_lib(res, state)
    assert b.fields().projection_resident == 3  # projection and diffusion
    for _ in range(6):
        a.update(None, cfg.d_t)
        b.update(None, cfg.d_t)
    if storage == 0:
        for field in FIELDS:
            x, y = a.download(field), b.download(field)
            assert same_bits(x, y), f"{field}: {int((x != y).sum())} cells differ"
    else:
        # 16-bit storage rounds once per pass in the blocked forms and once per
        # sweep in the plain one; compare with the pass engine instead.
        p = cfg.copy()
        p.projection_block = 4
        p.projection_resident = -1
        c = load_lib(p, state)
        for _ in range(6):
            c.update(None, cfg.d_t)
        for field in FIELDS:
            x, y = c.download(field), b.download(field)
            assert same_bits(x, y), f"{field}: {int((x != y).sum())} cells differ"
        c.close()
    a.close()
    b.close()


def test_resident_falls_back_when_grid_does_not_fit(gpu):
    cfg = scenarios.large_config()
    cfg.projection_n = 8
    cfg.projection_block = 4
    cfg.projection_resident = 3
    with Fluid(cfg) as f:
        assert f.fields().projection_resident == 0  # 4096 x 4096 needs more tiles than SMs
        f.update(None, cfg.d_t)


def test_bounded_wait_reports_timeout_and_context_survives(gpu):
    import ctypes as C
    lib = native.load()
    status = C.c_int32(-1)
    native.check(lib.os_selftest_bounded_wait(0, C.byref(status)))
    assert status.value == native.OS_ERR_TIMEOUT
    # The context is still usable: a resident step runs and is finite.
    cfg = tunnel(512, 256, projection_block=4, projection_resident=3)
    with Fluid(cfg) as f:
        f.update(None, cfg.d_t)
        assert np.isfinite(f.download("vel_x")).all()
