"""os_diffuse_noalloc: the diffusion phase for callers that may not allocate
device memory where they run it (memory owned by another allocator, a frame
loop that cannot stall on an allocation, a fixed device footprint).

It must give exactly what the handle's own diffusion phase gives (the same
per-sweep arithmetic; only the ping-pong buffer differs: a fixed array inside
the library instead of the handle's buffer), call after call, although every
call reuses the same array. This file sorts last so that a failure here does
not hide the results of the other GPU tests.
"""
import ctypes as C

import numpy as np
import pytest

from opensayal_gb300 import native
from opensayal_gb300.fluid import Fluid, default_config
from tests.parity_cases import same_bits

pytestmark = pytest.mark.gpu


def tunnel(w, h, n):
    cfg = default_config(w, h)
    cfg.viscosity = 0.05
    cfg.projection_n = n
    cfg.projection_block = -1
    return cfg


def via_handle(cfg, u0, dt):
    f = Fluid(cfg)
    f.upload("vel_x", u0)
    f.run_phase(native.PHASE_DIFFUSION, None, dt)
    out = f.download("vel_x")
    f.close()
    return out


def via_noalloc(cfg, u0, dt):
    import torch
    lib = native.load()
    dev = torch.from_numpy(u0.copy()).to("cuda:0")
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    rc = lib.os_diffuse_noalloc(C.byref(cfg), C.c_void_p(dev.data_ptr()), C.c_float(dt),
                                C.c_void_p(stream.cuda_stream))
    native.check(rc)
    stream.synchronize()
    return dev.cpu().numpy()


@pytest.mark.parametrize("w,h,n", [(300, 161, 7), (300, 161, 8),
                                   (1024, 1024, 5)])  # the largest grid it accepts, odd n
def test_noalloc_diffusion_equals_handle_diffusion_twice(gpu, w, h, n):
    rng = np.random.default_rng(n)
    cfg = tunnel(w, h, n)
    for call in range(2):  # the second call starts from the first call's leftovers
        u0 = rng.uniform(-2, 2, cfg.width * cfg.height).astype(np.float32)
        want = via_handle(cfg, u0, 0.05)
        got = via_noalloc(cfg, u0, 0.05)
        assert same_bits(got, want), f"call {call}: {int((got != want).sum())} cells differ"


def test_noalloc_rejects_grids_beyond_its_scratch(gpu):
    import torch
    lib = native.load()
    cfg = tunnel(1025, 1024, 3)  # 1,049,600 cells > 1,048,576
    dev = torch.zeros(cfg.width * cfg.height, dtype=torch.float32, device="cuda:0")
    rc = lib.os_diffuse_noalloc(C.byref(cfg), C.c_void_p(dev.data_ptr()), C.c_float(0.05), None)
    assert rc == native.OS_ERR_INVALID
    assert b"scratch" in lib.os_last_error()
    assert float(dev.abs().max()) == 0.0
