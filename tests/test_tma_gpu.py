"""Diffusion passes staged by tensor copies (one 2-D bulk copy of the region
into each Jacobi buffer, rows arriving in the global top-first order) give
exactly the bits of the vector-load staging; where the copy's alignment rules
do not hold (or at depths above 8, where it measured slower) the handle keeps
the vector loads. The staging is opt-in (OPENSAYAL_GB300_TMA=1): inside a step
it measured slower than the vector loads."""
import os

import pytest

import oracle
from opensayal_gb300 import native, scenarios
from opensayal_gb300.fluid import Fluid, default_config
from tests.parity_cases import FIELDS, load_lib, perturbed_state, random_state, same_bits

pytestmark = pytest.mark.gpu


def with_tma(fn, *args):
    os.environ["OPENSAYAL_GB300_TMA"] = "1"
    try:
        return fn(*args)
    finally:
        del os.environ["OPENSAYAL_GB300_TMA"]


def without_tma(cfg, state):
    return load_lib(cfg, state)


@pytest.mark.parametrize("w,h", [(1920, 1080), (300, 77), (96, 64), (2048, 1200), (4, 3)])
@pytest.mark.parametrize("k", [4, 8])
def test_tma_diffusion_equals_vector_staging(gpu, w, h, k):
    c = default_config(w, h)
    c.viscosity = 0.02
    c.projection_n = 23
    c.projection_block = k
    c.projection_resident = -1
    solid = oracle.OracleFluid(c).is_solid
    state = random_state(c, 41, solid)
    a, b = with_tma(load_lib, c, state), without_tma(c, state)
    assert a.fields().tma_staging == 1 and b.fields().tma_staging == 0
    a.run_phase(native.PHASE_DIFFUSION, None, 0.05)
    b.run_phase(native.PHASE_DIFFUSION, None, 0.05)
    for field in FIELDS:
        x, y = a.download(field), b.download(field)
        assert same_bits(x, y), f"{field}: {int((x != y).sum())} cells differ"
    a.close()
    b.close()


def test_tma_steps_equal_vector_staging(gpu):
    cfg = scenarios.default_tunnel_config()
    cfg.projection_block = 8
    state = perturbed_state(cfg, 3)
    a, b = with_tma(load_lib, cfg, state), without_tma(cfg, state)
    assert a.fields().tma_staging == 1
    for _ in range(5):
        a.update(None, cfg.d_t)
        b.update(None, cfg.d_t)
    for field in FIELDS:
        x, y = a.download(field), b.download(field)
        assert same_bits(x, y), f"{field}: {int((x != y).sum())} cells differ"
    a.close()
    b.close()


@pytest.mark.parametrize("w,k,storage", [(513, 8, 0), (1920, 6, 0), (1920, 8, 2), (1920, 12, 0)])
def test_tma_not_used_where_its_rules_fail(gpu, w, k, storage):
    c = default_config(w, 64)
    c.projection_block = k
    c.storage = storage
    with with_tma(Fluid, c) as f:
        assert f.fields().tma_staging == 0
        f.update(None, c.d_t)
