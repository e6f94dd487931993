"""Parity of the GB300 library with the reference's own CUDA kernels (the
unmodified src/fluid.cu device code, run through oracle/ref_harness.cpp) and
with the CPU oracle, on identical seeded inputs.

Bars (relative L2 unless stated):
* masks, neighbour counts, inflow/drain sets: bit-exact;
* every deterministic phase against the reference kernels, smoke advection
  included: bit-exact (the library performs the same FP32/FP64 operations in
  the same order, with the same multiply-adds fused);
* diffusion against the reference kernels: the reference sweeps in place from
  racing threads, the library runs Jacobi; they differ by <= 64 a^2 per sweep
  (a = viscosity*dt/h^2);
* 100 full FP32 steps of the 256x128 case against the reference kernels:
  1e-5 (the bar this path is held to). With the drain open the reference races on
  v(W-1, 1) (src/fluid.cu:720-733) and two runs of the reference itself
  differ by up to ~3e-5, so that variant is held to 1e-4;
* against the CPU oracle: 1e-5 per phase and for inviscid runs; viscous runs
  drift because the reference's fast-math division by 1 + 4a (applied ~5000
  times in 100 steps) rounds coherently while the oracle divides exactly:
  2e-4 after 100 steps, 1e-5 after 10.
"""
import numpy as np
import pytest

import oracle
from opensayal_gb300 import Fluid, native, scenarios
from opensayal_gb300.fluid import default_config
from tests.parity_cases import (ACTIVE_SOURCE, FIELDS, load_lib, load_oracle, load_ref,
                                perturbed_state, random_state, same_bits)

pytestmark = pytest.mark.gpu

REL_L2_BAR = 1e-5
DRAIN_RACE_BAR = 1e-4
ORACLE_VISCOUS_100 = 2e-4


def phase_config(**over):
    c = scenarios.small_config()
    c.width, c.height = 96, 64
    c.obstacle_center_x, c.obstacle_center_y, c.obstacle_radius = 48, 30, 9.5
    c.pipe_height = 20
    c.smoke_height = 12
    c.g = -5.0
    c.enable_pressure = 1
    c.smoke_enable_decay = 1
    c.smoke_decay_rate = 0.3
    c.drag_coeff = 0.2
    c.projection_n = 7
    c.projection_block = -1
    for k, v in over.items():
        setattr(c, k, v)
    return c


def test_masks_bit_exact(gpu):
    for cfg in (scenarios.small_config(), scenarios.default_tunnel_config(),
                scenarios.batched_scenarios(3, seed=9)[2]):
        f = Fluid(cfg)
        o = oracle.OracleFluid(cfg)
        assert np.array_equal(f.download("is_solid"), o.is_solid)
        assert np.array_equal(f.download("total_s"), o.total_s)
        f.close()


PHASES = [
    ("forces", native.PHASE_FORCES, ACTIVE_SOURCE),
    ("forces_inactive", native.PHASE_FORCES, None),
    ("zero_pressure", native.PHASE_ZERO_PRESSURE, None),
    ("projection", native.PHASE_PROJECTION, None),
    ("extrapolation", native.PHASE_EXTRAPOLATION, None),
    ("velocity_advection", native.PHASE_VEL_ADVECTION, None),
    ("smoke_advection", native.PHASE_SMOKE_ADVECTION, None),
    ("decay", native.PHASE_DECAY, None),
]


def race_sites(cfg) -> dict:
    """Faces that apply_extrapolation_at writes from racing threads
    (src/fluid.cu:720-733): u(1,0), u(1,H-1), u(0,0), v(0,1), v(W-1,1)."""
    W, H = cfg.width, cfg.height
    idx = lambda i, j: (H - 1 - j) * W + i  # noqa: E731
    return {"vel_x": [idx(1, 0), idx(1, H - 1), idx(0, 0)], "vel_y": [idx(0, 1), idx(W - 1, 1)]}


def ulp_diff(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Distance in units in the last place between float32 arrays."""
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7FFFFFFF), ia)
    ib = np.where(ib < 0, -(ib & 0x7FFFFFFF), ib)
    return np.abs(ia - ib)


@pytest.mark.parametrize("drain", [0, 1])
@pytest.mark.parametrize("name,phase,src", PHASES, ids=[p[0] for p in PHASES])
def test_phase_vs_reference_kernels(gpu, name, phase, src, drain):
    cfg = phase_config(enable_drain=drain)
    base = oracle.OracleFluid(cfg)
    state = random_state(cfg, 11, base.is_solid)
    lib, ref = load_lib(cfg, state), load_ref(cfg, state)
    dt = 0.05
    lib.run_phase(phase, src, dt)
    ref.phase(phase, src, dt)
    racy = race_sites(cfg) if phase == native.PHASE_EXTRAPOLATION else {}
    for field in FIELDS + ("pressure",):
        a, b = lib.download(field), ref.download(field)
        for k in racy.get(field, []):
            a[k] = b[k]  # either outcome of the race is the reference's
        assert same_bits(a, b), (
            f"{name}/{field}: {int((a != b).sum())} cells differ, max |d| = "
            f"{float(np.nanmax(np.abs(a.astype(np.float64) - b)))}")


def test_diffusion_matches_reference_to_race_order(gpu):
    cfg = phase_config(viscosity=0.05)  # a = 2.5e-3: races visible in the last bits
    base = oracle.OracleFluid(cfg)
    state = random_state(cfg, 12, base.is_solid)
    lib, ref = load_lib(cfg, state), load_ref(cfg, state)
    lib.run_phase(native.PHASE_DIFFUSION, None, 0.05)
    ref.phase(native.PHASE_DIFFUSION, None, 0.05)
    a, b = lib.download("vel_x"), ref.download("vel_x")
    # Per sweep a cell sees at most four neighbours that moved by a*|lap u| <=
    # a*16 (|u| <= 2), i.e. it differs by <= 64 a^2; n = 7 sweeps.
    bound = 7 * 64 * (2.5e-3) ** 2 + 1e-6
    assert np.abs(a.astype(np.float64) - b).max() < bound
    assert same_bits(lib.download("vel_y"), ref.download("vel_y"))


@pytest.mark.parametrize("block", [-1, 3])
def test_diffusion_bit_exact_where_reference_is_race_free(gpu, block):
    """On a 33x3 grid the reference's interior cells (i = 1..31, j = 1) are all
    threads of one warp of one block (block_size_x = 64), which load before
    they store: its in-place sweep is then exactly Jacobi, so the library must
    match it bit for bit, sweep after sweep."""
    cfg = default_config(33, 3)
    cfg.viscosity = 7.0  # a = 0.35: every sweep changes every interior bit
    cfg.projection_n = 9
    cfg.projection_block = block
    state = random_state(cfg, 14, np.zeros(33 * 3, np.int32))
    lib, ref = load_lib(cfg, state), load_ref(cfg, state)
    lib.run_phase(native.PHASE_DIFFUSION, None, 0.05)
    ref.phase(native.PHASE_DIFFUSION, None, 0.05)
    assert same_bits(lib.download("vel_x"), ref.download("vel_x"))


@pytest.mark.parametrize("name,phase,src", PHASES + [("diffusion", native.PHASE_DIFFUSION, None)],
                         ids=[p[0] for p in PHASES] + ["diffusion"])
def test_phase_vs_oracle(gpu, name, phase, src):
    cfg = phase_config(projection_n=50)
    base = oracle.OracleFluid(cfg)
    state = random_state(cfg, 13, base.is_solid)
    lib, orc = load_lib(cfg, state), load_oracle(cfg, state)
    lib.run_phase(phase, src, 0.05)
    orc.phase(phase, src, 0.05)
    racy = race_sites(cfg) if phase == native.PHASE_EXTRAPOLATION else {}
    for field in FIELDS + ("pressure",):
        a, b = lib.download(field), orc.fields()[field].copy()
        for k in racy.get(field, []):
            a[k] = b[k]
        assert oracle.rel_l2(a, b) <= REL_L2_BAR, (name, field, oracle.rel_l2(a, b))


def run_steps(obj, steps, dt, src=None):
    for _ in range(steps):
        obj.update(src, dt)


def field_error(a: np.ndarray, b: np.ndarray) -> float:
    """Relative L2 over finite entries; NaN/inf must sit in the same cells."""
    fa, fb = np.isfinite(a), np.isfinite(b)
    assert np.array_equal(fa, fb), "non-finite values in different cells"
    return oracle.rel_l2(a[fa], b[fb])


@pytest.mark.parametrize("variant", ["plain", "pressure", "drain_gravity", "inviscid"])
def test_small_case_100_steps(gpu, variant):
    """256x128, n=50, 100 steps, seeded perturbation, against the reference
    kernels and the oracle (bars in the module docstring)."""
    cfg = scenarios.small_config()
    if variant == "pressure":
        cfg.enable_pressure = 1
    elif variant == "drain_gravity":
        cfg.enable_drain = 1
        cfg.g = -5.0
    elif variant == "inviscid":
        cfg.viscosity = 0.0
    state = perturbed_state(cfg, 1)
    lib, ref, orc = load_lib(cfg, state), load_ref(cfg, state), load_oracle(cfg, state)
    steps = 100
    run_steps(lib, steps, cfg.d_t)
    run_steps(ref, steps, cfg.d_t)
    run_steps(orc, steps, cfg.d_t)
    ref_bar = DRAIN_RACE_BAR if cfg.enable_drain else REL_L2_BAR
    orc_bar = ORACLE_VISCOUS_100 if cfg.viscosity != 0.0 else REL_L2_BAR
    fields = FIELDS + (("pressure",) if cfg.enable_pressure else ())
    for field in fields:
        mine = lib.download(field)
        e_ref = oracle.rel_l2(mine, ref.download(field))
        e_orc = oracle.rel_l2(mine, orc.fields()[field])
        assert e_ref <= ref_bar, f"{variant}/{field} vs reference kernels: {e_ref:.3e}"
        assert e_orc <= orc_bar, f"{variant}/{field} vs oracle: {e_orc:.3e}"
    if cfg.enable_pressure:
        lo, hi = lib.min_pressure, lib.max_pressure
        p = lib.download("pressure")
        assert lo == p.min() and hi == p.max()
        rlo, rhi = ref.download("pressure").min(), ref.download("pressure").max()
        assert abs(lo - rlo) <= 1e-4 * max(1.0, abs(rlo))
        assert abs(hi - rhi) <= 1e-4 * max(1.0, abs(rhi))


def test_small_case_10_steps_vs_oracle(gpu):
    cfg = scenarios.small_config()
    state = perturbed_state(cfg, 1)
    lib, orc = load_lib(cfg, state), load_oracle(cfg, state)
    run_steps(lib, 10, cfg.d_t)
    run_steps(orc, 10, cfg.d_t)
    for field in FIELDS:
        e = oracle.rel_l2(lib.download(field), orc.fields()[field])
        assert e <= REL_L2_BAR, f"{field}: {e:.3e}"


def test_source_drag_decay_steps(gpu):
    """The interactive source, drag and decay paths over 20 full steps."""
    cfg = phase_config(projection_n=20, viscosity=0.001)
    state = perturbed_state(cfg, 5)
    lib, ref = load_lib(cfg, state), load_ref(cfg, state)
    for t in range(20):
        src = ACTIVE_SOURCE if t % 3 == 0 else None
        lib.update(src, 0.05)
        ref.update(src, 0.05)
    for field in FIELDS + ("pressure",):
        e = oracle.rel_l2(lib.download(field), ref.download(field))
        assert e <= REL_L2_BAR, f"{field}: {e:.3e}"


@pytest.mark.parametrize("w,h", [(3, 3), (8, 5), (131, 67), (200, 9), (97, 250)])
def test_ragged_sizes(gpu, w, h):
    """Grids that are no multiple of any tile or warp, down to 3x3."""
    cfg = default_config(w, h)
    cfg.tunnel_speed = 1.0
    cfg.enable_drain = 0
    cfg.projection_n = 5
    state = perturbed_state(cfg, 7)
    lib, ref = load_lib(cfg, state), load_ref(cfg, state)
    run_steps(lib, 5, 0.05)
    run_steps(ref, 5, 0.05)
    for field in FIELDS:
        a, b = lib.download(field), ref.download(field)
        for k in race_sites(cfg).get(field, []):
            a[k] = b[k]
        e = field_error(a, b)
        assert e <= REL_L2_BAR, f"{w}x{h}/{field}: {e:.3e}"


def test_update_async_matches_update(gpu):
    """Graph replays on a caller stream give the same bits as synchronous steps."""
    import torch
    cfg = scenarios.small_config()
    state = perturbed_state(cfg, 3)
    a, b = load_lib(cfg, state), load_lib(cfg, state)
    run_steps(a, 7, cfg.d_t)
    s = torch.cuda.Stream()
    b.update_async(None, cfg.d_t, 7, s.cuda_stream)
    s.synchronize()
    for field in FIELDS:
        assert same_bits(a.download(field), b.download(field))
