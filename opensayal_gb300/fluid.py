"""Python mirror of the reference's simulation interface.

`Fluid(config)` / `Fluid.update(source, d_t)` follow the reference's class
`Fluid` (inc/fluid.cuh:15-116, src/fluid.cu:41-71,770-795); `Source` follows
inc/fluid.cuh:8-13; `load_config` follows ConfigParser (inc/config_parser.hpp:
131-150, src/config_parser.cpp:15-184). Every call goes through the C ABI of
libopensayal_gb300.so; the arithmetic runs on the GPU only.
"""
from __future__ import annotations

import ctypes as C
import json
from dataclasses import dataclass
from pathlib import Path
from typing import Any

import numpy as np

from . import native
from .native import OsConfig, OsFieldsView, OsSource, check


@dataclass
class Source:
    """The reference's Source: an interactive forcing disc of radius 40 cells."""

    active: bool = False
    smoke: float = 0.0
    velocity: float = 0.0
    position: tuple[int, int] = (0, 0)

    def to_native(self) -> OsSource:
        return OsSource(int(bool(self.active)), float(self.smoke), float(self.velocity),
                        int(self.position[0]), int(self.position[1]))


def default_config(width: int = 1920, height: int = 1080) -> OsConfig:
    """ConfigParser defaults for a width x height tunnel (src/config_parser.cpp:21-179).

    Filled in here, without loading the CUDA library, so that configurations
    can be built where the library is absent or must not be mapped (the CPU
    checkers). The C ABI's os_config_defaults gives the same structure, field
    for field (tests/test_abi.py compares the two)."""
    if width < 1 or height < 1:
        raise ValueError(f"bad size {width}x{height}")
    cfg = OsConfig()  # zero-filled: storage F32, device 0, autotuned depths
    cfg.block_size_x, cfg.block_size_y = 64, 1
    cfg.height, cfg.width = height, width
    cfg.cell_pixel_size = 1
    cfg.cell_size = 1.0
    cfg.enable_drain, cfg.enable_pressure, cfg.enable_smoke, cfg.enable_interactive = 1, 0, 1, 0
    cfg.projection_n, cfg.projection_o = 50, 1.9
    cfg.pipe_height = height // 4
    cfg.pipe_length = 0  # hard-coded by the parser (src/config_parser.cpp:64)
    cfg.smoke_length = 1
    cfg.smoke_height = height // 4
    cfg.smoke_count = 1
    cfg.tunnel_speed, cfg.tunnel_smoke = 0.0, 1.0
    cfg.g = 0.0
    cfg.d_t = 0.05
    cfg.enable_real_time, cfg.real_time_multiplier = 0, 1.0
    cfg.smoke_enable_decay, cfg.smoke_decay_rate = 0, 0.05
    cfg.obstacle_enable = 1
    cfg.obstacle_center_x, cfg.obstacle_center_y = width // 2, height // 2
    # std::min(height, width) / 30.0f: an FP32 division
    cfg.obstacle_radius = float(np.float32(min(height, width)) / np.float32(30.0))
    cfg.density, cfg.drag_coeff, cfg.viscosity = 1.0, 0.0, 0.001
    return cfg


# Reference config key -> (os_config field, type). src/config_parser.cpp:21-179.
CONFIG_KEYS: dict[str, tuple[str, type]] = {
    "thread.cuda.block_size_x": ("block_size_x", int),
    "thread.cuda.block_size_y": ("block_size_y", int),
    "sim.height": ("height", int),
    "sim.width": ("width", int),
    "sim.cell_pixel_size": ("cell_pixel_size", int),
    "sim.cell_size": ("cell_size", float),
    "sim.enable_drain": ("enable_drain", bool),
    "sim.enable_pressure": ("enable_pressure", bool),
    "sim.enable_smoke": ("enable_smoke", bool),
    "sim.enable_interactive": ("enable_interactive", bool),
    "sim.projection.n": ("projection_n", int),
    "sim.projection.o": ("projection_o", float),
    "sim.wind_tunnel.pipe_height": ("pipe_height", int),
    "sim.wind_tunnel.smoke_length": ("smoke_length", int),
    "sim.wind_tunnel.smoke_height": ("smoke_height", int),
    "sim.wind_tunnel.smoke_count": ("smoke_count", int),
    "sim.wind_tunnel.speed": ("tunnel_speed", float),
    "sim.wind_tunnel.smoke": ("tunnel_smoke", float),
    "sim.physics.g": ("g", float),
    "sim.time.d_t": ("d_t", float),
    "sim.time.enable_real_time": ("enable_real_time", bool),
    "sim.time.real_time_multiplier": ("real_time_multiplier", float),
    "sim.smoke.enable_decay": ("smoke_enable_decay", bool),
    "sim.smoke.decay_rate": ("smoke_decay_rate", float),
    "sim.obstacle.enable": ("obstacle_enable", bool),
    "sim.obstacle.center_x": ("obstacle_center_x", int),
    "sim.obstacle.center_y": ("obstacle_center_y", int),
    "sim.obstacle.radius": ("obstacle_radius", float),
    "fluid.density": ("density", float),
    "fluid.drag_coeff": ("drag_coeff", float),
    "fluid.viscosity": ("viscosity", float),
}


class _WrongType(TypeError):
    pass


def _convert(value: Any, typ: type, key: str) -> Any:
    """The conversions of the reference's JSON library: a boolean key needs a
    JSON boolean; numbers (and booleans) convert to int by truncation and to
    float by rounding."""
    if typ is bool:
        if not isinstance(value, bool):
            raise _WrongType(f"config key {key!r} must be a boolean, got {value!r}")
        return int(value)
    if not isinstance(value, (bool, int, float)):
        raise _WrongType(f"config key {key!r} must be a number, got {value!r}")
    return int(value) if typ is int else float(value)


def _get_or(obj: Any, key: str, typ: type, default: Any, top: bool = True) -> Any:
    """ConfigParser::get_or (inc/config_parser.hpp:131-150): the whole dotted key
    at this level first, then recurse on the part after the first dot inside
    the member named by the part before it. A wrong type found below the top
    level yields the default (the reference's catch-all around the
    recursion); at the top level it is an error."""
    if isinstance(obj, dict) and key in obj:
        try:
            return _convert(obj[key], typ, key)
        except _WrongType:
            if top:
                raise
            return default
    if key == "" or "." not in key:
        return default
    parent, child = key.split(".", 1)
    if not isinstance(obj, dict) or parent not in obj:
        return default
    return _get_or(obj[parent], child, typ, default, top=False)


def visual_defaults() -> native.OsVisualConfig:
    """The `visual.*` and `sim.cell_pixel_size` defaults of
    src/config_parser.cpp:39-40, 120-179."""
    v = native.OsVisualConfig()
    v.cell_pixel_size = 1
    v.arrow_distance = 20
    v.arrow_length_multiplier = 0.1
    v.arrow_disable_threshold = 0.0
    v.arrow_head_length = 5
    v.trace_distance = 20
    v.trace_length = 20
    return v


def load_config(source: dict | str | Path) -> OsConfig:
    """Parse an OpenSayal.conf.json (a path, JSON text or a dict) with the reference's
    defaults and dotted-key lookup. Size-dependent defaults (pipe and smoke
    heights, obstacle centre and radius) follow the parsed width and height."""
    if isinstance(source, dict):
        obj = source
    elif isinstance(source, Path) or not str(source).lstrip().startswith(("{", "[")):
        obj = json.loads(Path(source).read_text())
    else:
        obj = json.loads(source)
    width = _get_or(obj, "sim.width", int, 1920)
    height = _get_or(obj, "sim.height", int, 1080)
    cfg = default_config(width, height)
    for key, (field, typ) in CONFIG_KEYS.items():
        setattr(cfg, field, _get_or(obj, key, typ, getattr(cfg, field)))
    return cfg


FIELD_IDS = {
    "vel_x": native.FIELD_VEL_X,
    "vel_y": native.FIELD_VEL_Y,
    "smoke": native.FIELD_SMOKE,
    "pressure": native.FIELD_PRESSURE,
    "is_solid": native.FIELD_IS_SOLID,
    "total_s": native.FIELD_TOTAL_S,
}


class Fluid:
    """The reference's Fluid on the GB300 library. Fields stay in device memory
    in the reference layout indx(i, j) = (height - 1 - j) * width + i."""

    def __init__(self, config: OsConfig):
        self._lib = native.load()
        self.config = config.copy()
        h = C.c_void_p()
        check(self._lib.os_create(C.byref(self.config), C.byref(h)))
        self._h = h
        self._owned = True
        self._set_shape(config)

    def _set_shape(self, config: OsConfig) -> None:
        self.width = config.width
        self.height = config.height
        self.n = config.projection_n
        self.o = config.projection_o
        self.cell_size = int(config.cell_size)

    @classmethod
    def view(cls, handle: C.c_void_p, config: OsConfig) -> "Fluid":
        """A Fluid over a handle owned elsewhere (a batch scenario)."""
        f = cls.__new__(cls)
        f._lib = native.load()
        f.config = config.copy()
        f._h = C.c_void_p(handle.value)
        f._owned = False
        f._set_shape(config)
        return f

    # -- lifecycle -----------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            if self._owned:
                check(self._lib.os_destroy(self._h))
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

    # -- the step ------------------------------------------------------------
    def update(self, source: Source | None, d_t: float) -> None:
        """Fluid::update(Source, float): one synchronous step."""
        src = (source or Source()).to_native()
        check(self._lib.os_update(self._h, C.byref(src), C.c_float(d_t)))

    def update_async(self, source: Source | None, d_t: float, steps: int = 1,
                     stream: int | None = None) -> None:
        """`steps` graph replays on `stream` (a cudaStream_t value) without waiting."""
        src = (source or Source()).to_native()
        check(self._lib.os_update_async(self._h, C.byref(src), C.c_float(d_t), int(steps),
                                        C.c_void_p(stream) if stream else None))

    def synchronize(self) -> None:
        check(self._lib.os_synchronize(self._h))

    def idle(self) -> bool:
        """True when every step enqueued on the handle's own stream has run."""
        out = C.c_int32()
        check(self._lib.os_query(self._h, C.byref(out)))
        return bool(out.value)

    def run_phase(self, phase: int, source: Source | None, d_t: float) -> None:
        src = (source or Source()).to_native()
        check(self._lib.os_run_phase(self._h, int(phase), C.byref(src), C.c_float(d_t)))

    def profile_phase(self, phase: int, source: Source | None, d_t: float, reps: int,
                      stream: int | None = None) -> tuple[float, int]:
        """(milliseconds, kernels) for `reps` repetitions of one phase, timed with
        CUDA events on the stream the kernels run on."""
        src = (source or Source()).to_native()
        ms, kern = C.c_float(), C.c_int32()
        check(self._lib.os_profile_phase(self._h, int(phase), C.byref(src), C.c_float(d_t),
                                         int(reps), C.c_void_p(stream) if stream else None,
                                         C.byref(ms), C.byref(kern)))
        return ms.value, kern.value

    def profile_phase_kernels(self, phase: int, source: Source | None, d_t: float, reps: int,
                              stream: int | None = None) -> tuple[float, float, int]:
        """(milliseconds of the phase's own kernels, milliseconds in all, kernels)
        for `reps` repetitions of one phase: the first leaves out the copy back
        to the public fields that a diffusion or projection phase called on its
        own ends with and a step does not run."""
        src = (source or Source()).to_native()
        kms, ms, kern = C.c_float(), C.c_float(), C.c_int32()
        check(self._lib.os_profile_phase_kernels(
            self._h, int(phase), C.byref(src), C.c_float(d_t), int(reps),
            C.c_void_p(stream) if stream else None, C.byref(kms), C.byref(ms), C.byref(kern)))
        return kms.value, ms.value, kern.value

    # -- state ---------------------------------------------------------------
    def indx(self, i: int, j: int) -> int:
        return (self.height - j - 1) * self.width + i

    def fields(self) -> OsFieldsView:
        view = OsFieldsView()
        check(self._lib.os_fields(self._h, C.byref(view)))
        return view

    def download(self, field: str | int, out: np.ndarray | None = None) -> np.ndarray:
        fid = FIELD_IDS[field] if isinstance(field, str) else field
        dtype = np.int32 if fid in (native.FIELD_IS_SOLID, native.FIELD_TOTAL_S) else np.float32
        n = self.width * self.height
        if out is None:
            out = np.empty(n, dtype=dtype)
        assert out.dtype == dtype and out.size == n and out.flags.c_contiguous
        check(self._lib.os_download(self._h, fid, out.ctypes.data_as(C.c_void_p), n))
        return out

    def snapshot_async(self, field: str | int, d_dst: int, stream: int | None = None) -> None:
        """Enqueue a copy of `field` (as FP32 or int32, width * height values)
        into the device buffer at `d_dst` on `stream`, without waiting."""
        fid = FIELD_IDS[field] if isinstance(field, str) else field
        check(self._lib.os_snapshot_async(self._h, fid, C.c_void_p(d_dst),
                                          self.width * self.height,
                                          C.c_void_p(stream) if stream else None))

    def upload(self, field: str | int, data: np.ndarray) -> None:
        fid = FIELD_IDS[field] if isinstance(field, str) else field
        arr = np.ascontiguousarray(data, dtype=np.float32).reshape(-1)
        check(self._lib.os_upload(self._h, fid, arr.ctypes.data_as(C.c_void_p), arr.size))

    @property
    def min_pressure(self) -> float:
        lo, hi = C.c_float(), C.c_float()
        check(self._lib.os_pressure_range(self._h, C.byref(lo), C.byref(hi)))
        return lo.value

    @property
    def max_pressure(self) -> float:
        lo, hi = C.c_float(), C.c_float()
        check(self._lib.os_pressure_range(self._h, C.byref(lo), C.byref(hi)))
        return hi.value

    # Headless visuals into caller-owned device buffers (device pointers as
    # integers, e.g. a torch tensor's data_ptr()); enqueued without waiting.
    def render_pixels(self, d_pixels: int, stream: int | None = None) -> None:
        check(self._lib.os_render_pixels(self._h, C.c_void_p(d_pixels),
                                         C.c_void_p(stream) if stream else None))

    def render_arrows(self, visual: "native.OsVisualConfig", d_arrows: int,
                      stream: int | None = None) -> None:
        check(self._lib.os_render_arrows(self._h, C.byref(visual), C.c_void_p(d_arrows),
                                         C.c_void_p(stream) if stream else None))

    def render_traces(self, visual: "native.OsVisualConfig", d_t: float, d_x: int, d_y: int,
                      stream: int | None = None) -> None:
        check(self._lib.os_render_traces(self._h, C.byref(visual), C.c_float(d_t),
                                         C.c_void_p(d_x), C.c_void_p(d_y),
                                         C.c_void_p(stream) if stream else None))

    def diagnose(self) -> dict:
        """FP64 divergence residual (l2, max, sum over the projected cells),
        smoke mass and inflow/outflow fluxes of the current fields."""
        d = native.OsDiag()
        check(self._lib.os_diagnose(self._h, C.byref(d)))
        return {name: getattr(d, name) for name, _ in native.OsDiag._fields_ if name != "reserved"}

    @property
    def kernel_launches(self) -> int:
        out = C.c_int64()
        check(self._lib.os_kernel_launches(self._h, C.byref(out)))
        return out.value

    @property
    def handle(self) -> int:
        return self._h.value
