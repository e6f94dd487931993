"""Batched scenarios advance exactly as each scenario does alone: the batch
runs the single-grid per-cell and per-tile code under a different schedule
(work lists, persistent kernels, one graph per step), and temporal blocking is
bit-exact whatever the tiling."""
import numpy as np
import pytest

from opensayal_gb300 import scenarios
from opensayal_gb300.batch import Batch
from opensayal_gb300.fluid import Fluid, default_config
from tests.parity_cases import FIELDS, perturbed_state, same_bits

pytestmark = pytest.mark.gpu


def mixed_configs():
    out = []
    for k, (w, h, n) in enumerate([(128, 96, 50), (300, 160, 13), (97, 250, 7), (640, 384, 20),
                                   (33, 3, 4), (512, 128, 9)]):
        c = default_config(w, h)
        c.tunnel_speed = 0.5 + 0.4 * k
        c.g = -1.5 * k
        c.projection_n = n
        c.obstacle_radius = 3.5 + k
        if k == 2:
            c.viscosity = 0.0
        if k == 3:
            c.enable_smoke = 0
        if k == 5:
            c.enable_drain = 0
            c.smoke_enable_decay = 1
        out.append(c)
    return out


@pytest.mark.parametrize("block_k", [3, 8])
def test_batch_equals_scenarios_alone(gpu, block_k):
    cfgs = mixed_configs()
    states = [perturbed_state(c, 10 + i) for i, c in enumerate(cfgs)]
    steps = 6
    with Batch(cfgs, block_k=block_k) as b:
        for i, st in enumerate(states):
            view = b.scenario(i)
            for k, a in st.items():
                view.upload(k, a)
        b.step(steps)
        b.synchronize()
        stats = b.stats()
        assert stats.scenarios == len(cfgs) and stats.block_k == block_k
        assert stats.cells == sum(c.width * c.height for c in cfgs)
        for i, (c, st) in enumerate(zip(cfgs, states)):
            alone_cfg = c.copy()
            alone_cfg.projection_block = block_k
            with Fluid(alone_cfg) as f:
                for k, a in st.items():
                    f.upload(k, a)
                for _ in range(steps):
                    f.update(None, c.d_t)
                view = b.scenario(i)
                for field in FIELDS:
                    x, y = view.download(field), f.download(field)
                    assert same_bits(x, y), f"scenario {i} {field}: {int((x != y).sum())} differ"


def test_batch_of_generated_scenarios_runs(gpu):
    cfgs = scenarios.batched_scenarios(24, seed=4)
    with Batch(cfgs) as b:
        b.step(2)
        b.synchronize()
        for i in range(len(cfgs)):
            s = b.scenario(i).download("smoke")
            assert np.isfinite(s).all()
        st = b.stats()
        passes = -(-max(c.projection_n for c in cfgs) // st.block_k)
        assert st.kernels_per_step == 2 * passes + 6
        assert st.block_k in (4, 6, 8, 12) and st.projection_tile_rows >= 2


def test_batch_rejects_pressure(gpu):
    from opensayal_gb300.native import NativeError
    c = default_config(64, 32)
    c.enable_pressure = 1
    with pytest.raises(NativeError):
        Batch([c])
