"""Batched scenarios: many tunnels of different sizes advanced together by one
CUDA graph per step (os_batch_* in include/opensayal_gb300.h)."""
from __future__ import annotations

import ctypes as C

from . import native
from .fluid import Fluid
from .native import OsBatchStats, OsConfig, check


class Batch:
    """Owns the scenarios' fields; `scenario(i)` gives a Fluid view of one."""

    def __init__(self, configs: list[OsConfig], block_k: int = 0):
        self._lib = native.load()
        arr = (OsConfig * len(configs))(*[c.copy() for c in configs])
        h = C.c_void_p()
        check(self._lib.os_batch_create(arr, len(configs), int(block_k), C.byref(h)))
        self._h = h
        self.configs = [c.copy() for c in configs]

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            check(self._lib.os_batch_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self) -> int:
        return len(self.configs)

    def step(self, steps: int = 1, stream: int | None = None) -> None:
        check(self._lib.os_batch_step(self._h, int(steps),
                                      C.c_void_p(stream) if stream else None))

    def synchronize(self) -> None:
        check(self._lib.os_batch_synchronize(self._h))

    def scenario(self, index: int) -> Fluid:
        h = C.c_void_p()
        check(self._lib.os_batch_scenario(self._h, int(index), C.byref(h)))
        return Fluid.view(h, self.configs[index])

    def stats(self) -> OsBatchStats:
        s = OsBatchStats()
        check(self._lib.os_batch_info(self._h, C.byref(s)))
        return s
