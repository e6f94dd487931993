"""ctypes binding of the C ABI in include/opensayal_gb300.h.

The structures below mirror the header field for field. Loading fails loudly
when the CUDA library has not been built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from .build import LIB_PATH

OS_OK = 0
OS_ERR_INVALID = 1
OS_ERR_CUDA = 2
OS_ERR_NOMEM = 3
OS_ERR_UNSUPPORTED = 4
OS_ERR_STATE = 5
OS_ERR_TIMEOUT = 6

FIELD_VEL_X, FIELD_VEL_Y, FIELD_SMOKE, FIELD_PRESSURE, FIELD_IS_SOLID, FIELD_TOTAL_S = range(6)
STORAGE_F32, STORAGE_F16, STORAGE_BF16, STORAGE_F64 = range(4)
(PHASE_FORCES, PHASE_ZERO_PRESSURE, PHASE_DIFFUSION, PHASE_PROJECTION,
 PHASE_PRESSURE_RANGE, PHASE_EXTRAPOLATION, PHASE_VEL_ADVECTION,
 PHASE_SMOKE_ADVECTION, PHASE_DECAY) = range(9)


class OsConfig(C.Structure):
    """os_config: flat mirror of the reference's Config (inc/config_parser.hpp:9-115)."""

    _fields_ = [
        ("block_size_x", C.c_int32),
        ("block_size_y", C.c_int32),
        ("height", C.c_int32),
        ("width", C.c_int32),
        ("cell_pixel_size", C.c_int32),
        ("cell_size", C.c_float),
        ("enable_drain", C.c_int32),
        ("enable_pressure", C.c_int32),
        ("enable_smoke", C.c_int32),
        ("enable_interactive", C.c_int32),
        ("projection_n", C.c_int32),
        ("projection_o", C.c_float),
        ("pipe_height", C.c_int32),
        ("pipe_length", C.c_int32),
        ("smoke_length", C.c_int32),
        ("smoke_height", C.c_int32),
        ("smoke_count", C.c_int32),
        ("tunnel_speed", C.c_float),
        ("tunnel_smoke", C.c_float),
        ("g", C.c_float),
        ("d_t", C.c_float),
        ("enable_real_time", C.c_int32),
        ("real_time_multiplier", C.c_float),
        ("smoke_enable_decay", C.c_int32),
        ("smoke_decay_rate", C.c_float),
        ("obstacle_enable", C.c_int32),
        ("obstacle_center_x", C.c_int32),
        ("obstacle_center_y", C.c_int32),
        ("obstacle_radius", C.c_float),
        ("density", C.c_float),
        ("drag_coeff", C.c_float),
        ("viscosity", C.c_float),
        ("storage", C.c_int32),
        ("device", C.c_int32),
        ("projection_block", C.c_int32),
        ("idw_mode", C.c_int32),
        ("projection_resident", C.c_int32),
        ("diffusion_block", C.c_int32),
        ("reserved", C.c_int32 * 2),
    ]

    def copy(self) -> "OsConfig":
        out = OsConfig()
        C.memmove(C.byref(out), C.byref(self), C.sizeof(OsConfig))
        return out

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


class OsSource(C.Structure):
    """os_source: the reference's Source (inc/fluid.cuh:8-13)."""

    _fields_ = [
        ("active", C.c_int32),
        ("smoke", C.c_float),
        ("velocity", C.c_float),
        ("position_x", C.c_int32),
        ("position_y", C.c_int32),
    ]


class OsFieldsView(C.Structure):
    _fields_ = [
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("storage", C.c_int32),
        ("projection_block", C.c_int32),
        ("vel_x", C.c_void_p),
        ("vel_y", C.c_void_p),
        ("smoke", C.c_void_p),
        ("pressure", C.c_void_p),
        ("is_solid", C.c_void_p),
        ("total_s", C.c_void_p),
        ("projection_resident", C.c_int32),
        ("tma_staging", C.c_int32),
    ]


# Every entry point declared in include/opensayal_gb300.h: (name, restype, argtypes).
SIGNATURES = [
    ("os_abi_version", C.c_int32, []),
    ("os_last_error", C.c_char_p, []),
    ("os_config_defaults", C.c_int, [C.c_int32, C.c_int32, C.POINTER(OsConfig)]),
    ("os_create", C.c_int, [C.POINTER(OsConfig), C.POINTER(C.c_void_p)]),
    ("os_destroy", C.c_int, [C.c_void_p]),
    ("os_update", C.c_int, [C.c_void_p, C.POINTER(OsSource), C.c_float]),
    ("os_update_async", C.c_int, [C.c_void_p, C.POINTER(OsSource), C.c_float, C.c_int32, C.c_void_p]),
    ("os_synchronize", C.c_int, [C.c_void_p]),
    ("os_query", C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    ("os_fields", C.c_int, [C.c_void_p, C.POINTER(OsFieldsView)]),
    ("os_upload", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t]),
    ("os_download", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t]),
    ("os_snapshot_async", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t,
                                    C.c_void_p]),
    ("os_pressure_range", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    ("os_run_phase", C.c_int, [C.c_void_p, C.c_int32, C.POINTER(OsSource), C.c_float]),
    ("os_kernel_launches", C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    ("os_profile_phase", C.c_int, [C.c_void_p, C.c_int32, C.POINTER(OsSource), C.c_float,
                                   C.c_int32, C.c_void_p, C.POINTER(C.c_float),
                                   C.POINTER(C.c_int32)]),
    ("os_profile_phase_kernels", C.c_int, [C.c_void_p, C.c_int32, C.POINTER(OsSource),
                                           C.c_float, C.c_int32, C.c_void_p,
                                           C.POINTER(C.c_float), C.POINTER(C.c_float),
                                           C.POINTER(C.c_int32)]),
    ("os_diffuse_noalloc", C.c_int, [C.POINTER(OsConfig), C.c_void_p, C.c_float, C.c_void_p]),
    ("os_diagnose", C.c_int, [C.c_void_p, C.c_void_p]),
    ("os_visual_defaults", C.c_int, [C.c_void_p]),
    ("os_config_parse", C.c_int, [C.c_char_p, C.c_size_t, C.POINTER(OsConfig), C.c_void_p]),
    ("os_render_pixels", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("os_render_arrows", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("os_render_traces", C.c_int, [C.c_void_p, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p,
                                   C.c_void_p]),
    ("os_selftest_bounded_wait", C.c_int, [C.c_int32, C.POINTER(C.c_int32)]),
    ("os_probe_copy_bandwidth", C.c_int, [C.c_int32, C.c_uint64, C.c_int32,
                                          C.POINTER(C.c_float)]),
    ("os_batch_create", C.c_int, [C.POINTER(OsConfig), C.c_int32, C.c_int32,
                                  C.POINTER(C.c_void_p)]),
    ("os_batch_create_dynamic", C.c_int, [C.c_int32, C.c_int32, C.c_uint64,
                                          C.POINTER(C.c_void_p)]),
    ("os_batch_add", C.c_int, [C.c_void_p, C.POINTER(OsConfig), C.c_int32,
                               C.POINTER(C.c_int64)]),
    ("os_batch_remove", C.c_int, [C.c_void_p, C.c_int64]),
    ("os_batch_destroy", C.c_int, [C.c_void_p]),
    ("os_batch_step", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    ("os_batch_synchronize", C.c_int, [C.c_void_p]),
    ("os_batch_poll", C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int64), C.c_int32,
                                C.POINTER(C.c_int32)]),
    ("os_batch_wait", C.c_int, [C.c_void_p, C.c_int64]),
    ("os_batch_status", C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_int32),
                                  C.POINTER(C.c_int64)]),
    ("os_batch_memory", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    ("os_batch_scenario", C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_void_p)]),
    ("os_batch_info", C.c_int, [C.c_void_p, C.c_void_p]),
]


class OsDiag(C.Structure):
    _fields_ = [
        ("divergence_l2", C.c_double),
        ("divergence_max", C.c_double),
        ("divergence_sum", C.c_double),
        ("smoke_mass", C.c_double),
        ("inflow_flux", C.c_double),
        ("outflow_flux", C.c_double),
        ("active_cells", C.c_int64),
        ("reserved", C.c_int64),
    ]


class OsVisualConfig(C.Structure):
    _fields_ = [
        ("cell_pixel_size", C.c_int32),
        ("arrow_distance", C.c_int32),
        ("arrow_length_multiplier", C.c_float),
        ("arrow_disable_threshold", C.c_float),
        ("arrow_head_length", C.c_int32),
        ("trace_distance", C.c_int32),
        ("trace_length", C.c_int32),
        ("reserved", C.c_int32),
    ]


class OsArrow(C.Structure):
    _fields_ = [(name, C.c_int32) for name in (
        "start_x", "start_y", "end_x", "end_y", "right_head_end_x", "right_head_end_y",
        "left_head_end_x", "left_head_end_y", "valid")]


class OsBatchStats(C.Structure):
    _fields_ = [
        ("scenarios", C.c_int32),
        ("block_k", C.c_int32),
        ("kernels_per_step", C.c_int32),
        ("members_in_plan", C.c_int32),
        ("cells", C.c_int64),
        ("launches", C.c_int64),
        ("tile_items_per_step", C.c_int64),
        ("steps_enqueued", C.c_int64),
        ("steps_completed", C.c_int64),
        ("projection_tile_rows", C.c_int32),
        ("diffusion_tile_rows", C.c_int32),
    ]


MEMBER_WAITING, MEMBER_RUNNING, MEMBER_DONE = 0, 1, 2

_lib = None


class NativeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[os status {code}] {msg}")
        self.code = code


def load(path: Path | str | None = None) -> C.CDLL:
    """Load the built library. Raises if it is missing (build it first with
    opensayal_gb300.build.build_library())."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is not built; run opensayal_gb300.build.build_library() "
            "(the GB300 library has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != OS_OK:
        msg = load().os_last_error().decode(errors="replace")
        raise NativeError(rc, msg)
