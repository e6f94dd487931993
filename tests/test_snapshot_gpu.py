"""os_snapshot_async: a field copied on the step's stream into a device buffer
of the caller, read back on another stream while the next step runs, gives
each step's field exactly as a synchronous update and download do."""
import numpy as np
import pytest

from opensayal_gb300 import Fluid, native, scenarios
from tests.parity_cases import perturbed_state, same_bits

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage", [native.STORAGE_F32, native.STORAGE_BF16])
def test_snapshot_equals_download(gpu, storage):
    import torch
    cfg = scenarios.small_config()
    cfg.storage = storage
    state = perturbed_state(cfg, 8)
    with Fluid(cfg) as f:
        for k, a in state.items():
            f.upload(k, a)
        for _ in range(3):
            f.update(None, cfg.d_t)
        for field, dtype in (("vel_x", torch.float32), ("smoke", torch.float32),
                             ("is_solid", torch.int32)):
            buf = torch.full((cfg.width * cfg.height,), -7, dtype=dtype, device="cuda")
            f.snapshot_async(field, buf.data_ptr())
            f.synchronize()
            assert same_bits(buf.cpu().numpy(), f.download(field)), field


def test_overlapped_read_back_gives_every_step(gpu):
    """The bench's e2e pattern: two snapshot buffers, the device-to-host copy of
    step k on a second stream while step k + 1 runs."""
    import torch
    cfg = scenarios.small_config()
    state = perturbed_state(cfg, 9)
    n = cfg.width * cfg.height
    steps = 6
    want = []
    with Fluid(cfg) as f:
        for k, a in state.items():
            f.upload(k, a)
        for _ in range(steps):
            f.update(None, cfg.d_t)
            want.append(f.download("smoke"))
    got = []
    with Fluid(cfg) as f:
        for k, a in state.items():
            f.upload(k, a)
        stream, copy_stream = torch.cuda.Stream(), torch.cuda.Stream()
        snap = [torch.empty(n, dtype=torch.float32, device="cuda") for _ in range(2)]
        host = [torch.empty(n, dtype=torch.float32, pin_memory=True) for _ in range(steps)]
        copied = [torch.cuda.Event() for _ in range(2)]
        for k in range(steps):
            b = k & 1
            f.update_async(None, cfg.d_t, 1, stream.cuda_stream)
            if k >= 2:
                stream.wait_event(copied[b])
            f.snapshot_async("smoke", snap[b].data_ptr(), stream.cuda_stream)
            ready = torch.cuda.Event()
            ready.record(stream)
            copy_stream.wait_event(ready)
            with torch.cuda.stream(copy_stream):
                host[k].copy_(snap[b], non_blocking=True)
            copied[b].record(copy_stream)
        torch.cuda.synchronize()
        got = [h.numpy().copy() for h in host]
    for k in range(steps):
        assert same_bits(got[k], want[k]), f"step {k}"
    assert not same_bits(want[0], want[-1])


def test_snapshot_rejects_bad_arguments(gpu):
    import ctypes as C
    lib = native.load()
    cfg = scenarios.small_config()
    with Fluid(cfg) as f:
        h = C.c_void_p(f.handle)
        assert lib.os_snapshot_async(h, native.FIELD_SMOKE, None, cfg.width * cfg.height,
                                     None) == native.OS_ERR_INVALID
        assert lib.os_snapshot_async(h, 99, C.c_void_p(16), cfg.width * cfg.height,
                                     None) == native.OS_ERR_INVALID
        assert lib.os_snapshot_async(h, native.FIELD_SMOKE, C.c_void_p(16), 5,
                                     None) == native.OS_ERR_INVALID
        np.testing.assert_equal(lib.os_snapshot_async(None, 0, None, 0, None),
                                native.OS_ERR_INVALID)
