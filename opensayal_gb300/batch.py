"""Batched and served scenarios: many tunnels of different sizes advanced
together by one CUDA graph per step (os_batch_* in include/opensayal_gb300.h).

`Batch(configs)` holds a fixed set that steps until closed (member ids
0..len-1). `Batch.dynamic(budget_bytes=...)` starts empty for continuous
batching: `add` admits a scenario for a number of steps, it joins at the next
`step`, and `poll` reports the members whose steps have all completed."""
from __future__ import annotations

import ctypes as C

from . import native
from .fluid import Fluid
from .native import OS_ERR_NOMEM, NativeError, OsBatchStats, OsConfig, check


class BudgetFull(NativeError):
    """The scenario does not fit the batch's device-memory budget now."""


class Batch:
    """Owns the members' fields; `scenario(id)` gives a Fluid view of one."""

    def __init__(self, configs: list[OsConfig] | None = None, block_k: int = 0, *,
                 device: int = 0, budget_bytes: int = 0):
        self._lib = native.load()
        self._h = None
        h = C.c_void_p()
        self.configs: dict[int, OsConfig] = {}
        if configs is None:
            check(self._lib.os_batch_create_dynamic(int(device), int(block_k),
                                                    int(budget_bytes), C.byref(h)))
        else:
            arr = (OsConfig * len(configs))(*[c.copy() for c in configs])
            check(self._lib.os_batch_create(arr, len(configs), int(block_k), C.byref(h)))
            self.configs = {i: c.copy() for i, c in enumerate(configs)}
        self._h = h

    @classmethod
    def dynamic(cls, block_k: int = 0, device: int = 0, budget_bytes: int = 0) -> "Batch":
        return cls(None, block_k, device=device, budget_bytes=budget_bytes)

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

    def add(self, config: OsConfig, steps: int) -> int:
        """Admit `config` for `steps` steps (negative: until removed); returns
        its id. Raises BudgetFull when it does not fit the budget now."""
        mid = C.c_int64()
        rc = self._lib.os_batch_add(self._h, C.byref(config), int(steps), C.byref(mid))
        if rc == OS_ERR_NOMEM:
            raise BudgetFull(rc, self._lib.os_last_error().decode())
        check(rc)
        self.configs[mid.value] = config.copy()
        return mid.value

    def remove(self, mid: int) -> None:
        check(self._lib.os_batch_remove(self._h, int(mid)))
        self.configs.pop(mid, None)

    def step(self, steps: int = 1, stream: int | None = None) -> None:
        check(self._lib.os_batch_step(self._h, int(steps),
                                      C.c_void_p(stream) if stream else None))

    def synchronize(self) -> None:
        check(self._lib.os_batch_synchronize(self._h))

    def poll(self, wait: bool = False, cap: int = 1024) -> list[int]:
        """Ids of members finished since the last poll."""
        ids = (C.c_int64 * cap)()
        n = C.c_int32()
        check(self._lib.os_batch_poll(self._h, int(bool(wait)), ids, cap, C.byref(n)))
        return list(ids[: n.value])

    def wait(self, max_in_flight: int = 0) -> None:
        """Block until at most `max_in_flight` enqueued steps are incomplete."""
        check(self._lib.os_batch_wait(self._h, int(max_in_flight)))

    def status(self, mid: int) -> tuple[int, int]:
        """(state, steps left): state is native.MEMBER_WAITING/RUNNING/DONE."""
        state, left = C.c_int32(), C.c_int64()
        check(self._lib.os_batch_status(self._h, int(mid), C.byref(state), C.byref(left)))
        return state.value, left.value

    def memory(self) -> tuple[int, int]:
        """(device bytes held by members, budget; 0 when unbudgeted)."""
        used, budget = C.c_uint64(), C.c_uint64()
        check(self._lib.os_batch_memory(self._h, C.byref(used), C.byref(budget)))
        return used.value, budget.value

    def scenario(self, mid: int) -> Fluid:
        h = C.c_void_p()
        check(self._lib.os_batch_scenario(self._h, int(mid), C.byref(h)))
        return Fluid.view(h, self.configs[mid])

    def stats(self) -> OsBatchStats:
        s = OsBatchStats()
        check(self._lib.os_batch_info(self._h, C.byref(s)))
        return s
