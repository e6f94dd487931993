"""Test infrastructure: the oracle for OpenSayal's simulation step.

Only tests/, __graft_entry__.smoke() and bench.py (its CPU-baseline leg and its
reference arm) import this package. The library never does.

* `OracleFluid` runs fluid_oracle.c, the CPU restatement of src/fluid.cu.
* `RefFluid` runs the reference's own kernels (the unmodified src/fluid.cu device
  code, compiled to _ref/fluid_ref.cubin) through ref_harness.cpp on a GPU.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "build" / "liboracle.so"
HARNESS_SO = HERE / "build" / "libref_harness.so"
REF_CUBIN = HERE / "_ref" / "fluid_ref.cubin"
VISUAL_CUBIN = HERE / "_ref" / "visual_ref.cubin"

# The reference's x86-64 g++ 13 -O3 build starts the uninitialised diffusion
# loop counter (src/fluid.cu:186) at zero: n diffusion sweeps per step.
def reference_diffusion_sweeps(n: int) -> int:
    return n


def build(with_reference: bool | None = None) -> None:
    """Build the checkers with oracle/Makefile: the C restatement, the harness
    for the reference's kernels and, where the reference sources are present
    (the Makefile's REFERENCE, overridable with OPENSAYAL_REFERENCE), the
    reference cubins. Elsewhere the cubins already in _ref/ are used."""
    targets = ["all"]
    env_ref = os.environ.get("OPENSAYAL_REFERENCE")
    if with_reference is None:
        probe = subprocess.run(["make", "-s", "-C", str(HERE), "--no-print-directory",
                                "print-reference"] + ([f"REFERENCE={env_ref}"] if env_ref else []),
                               capture_output=True, text=True)
        ref_dir = Path(probe.stdout.strip() or "/nonexistent")
        with_reference = (ref_dir / "src" / "fluid.cu").exists()
    if with_reference:
        targets.append("ref")
    extra = [f"REFERENCE={env_ref}"] if env_ref else []
    res = subprocess.run(["make", "-s", "-C", str(HERE), *targets, *extra],
                         capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")


_oracle = None
_harness = None
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def _load_oracle():
    global _oracle
    if _oracle is None:
        if not ORACLE_SO.exists():
            build()
        lib = C.CDLL(str(ORACLE_SO))
        cfgp = C.c_void_p
        lib.orc_init_mask.argtypes = [cfgp, _i32p, _i32p]
        lib.orc_forces.argtypes = [cfgp, C.c_void_p, C.c_float, _f32p, _f32p, _f32p]
        lib.orc_diffusion.argtypes = [cfgp, C.c_float, C.c_int, _f32p, _f32p]
        lib.orc_zero_pressure.argtypes = [cfgp, _f32p]
        lib.orc_projection.argtypes = [cfgp, C.c_float, C.c_int, _i32p, _i32p, _f32p, _f32p, _f32p]
        lib.orc_pressure_range.argtypes = [cfgp, _f32p, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        lib.orc_extrapolation.argtypes = [cfgp, _f32p, _f32p]
        lib.orc_velocity_advection.argtypes = [cfgp, C.c_float, _i32p, _f32p, _f32p, _f32p, _f32p]
        lib.orc_smoke_advection.argtypes = [cfgp, C.c_float, _i32p, _f32p, _f32p, _f32p, _f32p]
        lib.orc_decay.argtypes = [cfgp, C.c_float, _f32p]
        lib.orc_step.argtypes = [cfgp, C.c_void_p, C.c_float, C.c_int, _i32p, _i32p,
                                 _f32p, _f32p, _f32p, _f32p, _f32p,
                                 C.POINTER(C.c_float), C.POINTER(C.c_float)]
        lib.orc_threads.restype = C.c_int
        _oracle = lib
    return _oracle


def oracle_threads() -> int:
    return _load_oracle().orc_threads()


class OracleFluid:
    """CPU restatement of Fluid with the same fields (reference layout)."""

    def __init__(self, config, diffusion_sweeps: int | None = None):
        self.lib = _load_oracle()
        self.cfg = config.copy()
        self._cp = C.cast(C.pointer(self.cfg), C.c_void_p)
        self.W, self.H = self.cfg.width, self.cfg.height
        n = self.W * self.H
        self.is_solid = np.zeros(n, np.int32)
        self.total_s = np.zeros(n, np.int32)
        self.lib.orc_init_mask(self._cp, self.is_solid, self.total_s)
        self.u = np.zeros(n, np.float32)
        self.v = np.zeros(n, np.float32)
        self.s = np.zeros(n, np.float32)
        self.p = np.zeros(n, np.float32)
        self.work = np.zeros(3 * n, np.float32)
        self.diffusion_sweeps = (reference_diffusion_sweeps(self.cfg.projection_n)
                                 if diffusion_sweeps is None else diffusion_sweeps)
        self.min_pressure = 0.0
        self.max_pressure = 0.0

    def fields(self) -> dict:
        return {"vel_x": self.u, "vel_y": self.v, "smoke": self.s, "pressure": self.p}

    def _src(self, source):
        if source is None:
            return None
        from opensayal_gb300.native import OsSource
        self._srcbuf = source.to_native() if not isinstance(source, OsSource) else source
        return C.cast(C.pointer(self._srcbuf), C.c_void_p)

    def update(self, source, d_t: float) -> None:
        lo, hi = C.c_float(), C.c_float()
        self.lib.orc_step(self._cp, self._src(source), d_t, self.diffusion_sweeps,
                          self.is_solid, self.total_s, self.u, self.v, self.s, self.p,
                          self.work, C.byref(lo), C.byref(hi))
        if self.cfg.enable_pressure:
            self.min_pressure, self.max_pressure = lo.value, hi.value

    # single phases, mirroring os_run_phase
    def phase(self, phase: int, source, d_t: float) -> None:
        from opensayal_gb300 import native as nv
        L, cp, n = self.lib, self._cp, self.W * self.H
        if phase == nv.PHASE_FORCES:
            L.orc_forces(cp, self._src(source), d_t, self.u, self.v, self.s)
        elif phase == nv.PHASE_ZERO_PRESSURE:
            L.orc_zero_pressure(cp, self.p)
        elif phase == nv.PHASE_DIFFUSION:
            L.orc_diffusion(cp, d_t, self.diffusion_sweeps, self.u, self.work[:n])
        elif phase == nv.PHASE_PROJECTION:
            L.orc_projection(cp, d_t, self.cfg.projection_n, self.is_solid, self.total_s,
                             self.u, self.v, self.p)
        elif phase == nv.PHASE_PRESSURE_RANGE:
            lo, hi = C.c_float(), C.c_float()
            L.orc_pressure_range(cp, self.p, C.byref(lo), C.byref(hi))
            self.min_pressure, self.max_pressure = lo.value, hi.value
        elif phase == nv.PHASE_EXTRAPOLATION:
            L.orc_extrapolation(cp, self.u, self.v)
        elif phase == nv.PHASE_VEL_ADVECTION:
            ub, vb = np.empty_like(self.u), np.empty_like(self.v)
            L.orc_velocity_advection(cp, d_t, self.is_solid, self.u, self.v, ub, vb)
            self.u[:], self.v[:] = ub, vb
        elif phase == nv.PHASE_SMOKE_ADVECTION:
            sb = np.empty_like(self.s)
            L.orc_smoke_advection(cp, d_t, self.is_solid, self.u, self.v, self.s, sb)
            self.s[:] = sb
        elif phase == nv.PHASE_DECAY:
            L.orc_decay(cp, d_t, self.s)
        else:
            raise ValueError(phase)


def _load_harness():
    global _harness
    if _harness is None:
        if not HARNESS_SO.exists():
            build()
        lib = C.CDLL(str(HARNESS_SO))
        lib.ref_last_error.restype = C.c_char_p
        lib.ref_open.argtypes = [C.c_char_p]
        lib.ref_create.argtypes = [C.c_void_p, _i32p, _i32p]
        lib.ref_create.restype = C.c_void_p
        lib.ref_destroy.argtypes = [C.c_void_p]
        lib.ref_upload.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        lib.ref_download.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        lib.ref_phase.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_float, C.c_int]
        lib.ref_update.argtypes = [C.c_void_p, C.c_void_p, C.c_float, C.c_int]
        lib.ref_pressure_range.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        lib.ref_visual_open.argtypes = [C.c_char_p]
        lib.ref_render_pixels.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_void_p]
        lib.ref_render_traces.argtypes = [C.c_void_p, C.c_float, C.c_int, C.c_int, C.c_void_p,
                                          C.c_void_p]
        lib.ref_render_arrows.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_float,
                                          C.c_float, C.c_int, C.c_void_p]
        lib.ref_sample_velocity.argtypes = [C.c_void_p, C.c_int, _f32p, _f32p, _f32p, _f32p]
        rc = lib.ref_open(str(REF_CUBIN).encode())
        if rc != 0:
            raise RuntimeError(f"reference cubin: {lib.ref_last_error().decode()}")
        if VISUAL_CUBIN.exists() and lib.ref_visual_open(str(VISUAL_CUBIN).encode()) != 0:
            raise RuntimeError(f"visual cubin: {lib.ref_last_error().decode()}")
        _harness = lib
    return _harness


def reference_available() -> bool:
    return REF_CUBIN.exists()


class RefFluid:
    """The reference's own kernels on the GPU, driven as Fluid::update drives them."""

    FIELDS = {"vel_x": 0, "vel_y": 1, "smoke": 2, "pressure": 3, "is_solid": 4, "total_s": 5}

    def __init__(self, config, diffusion_sweeps: int | None = None):
        self.lib = _load_harness()
        self.cfg = config.copy()
        self._cp = C.cast(C.pointer(self.cfg), C.c_void_p)
        self.W, self.H = self.cfg.width, self.cfg.height
        n = self.W * self.H
        # Host construction work of the reference (mask, counts) is deterministic
        # host code; the oracle's restatement of it is reused here.
        self.is_solid = np.zeros(n, np.int32)
        self.total_s = np.zeros(n, np.int32)
        _load_oracle().orc_init_mask(self._cp, self.is_solid, self.total_s)
        self.h = self.lib.ref_create(self._cp, self.is_solid, self.total_s)
        if not self.h:
            raise RuntimeError(self.lib.ref_last_error().decode())
        self.diffusion_sweeps = (reference_diffusion_sweeps(self.cfg.projection_n)
                                 if diffusion_sweeps is None else diffusion_sweeps)

    def close(self):
        if self.h:
            self.lib.ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _src(self, source):
        if source is None:
            return None
        from opensayal_gb300.native import OsSource
        self._srcbuf = source.to_native() if not isinstance(source, OsSource) else source
        return C.cast(C.pointer(self._srcbuf), C.c_void_p)

    def upload(self, field: str, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr, dtype=np.int32 if field in ("is_solid", "total_s") else np.float32)
        if self.lib.ref_upload(self.h, self.FIELDS[field], a.ctypes.data_as(C.c_void_p)):
            raise RuntimeError(self.lib.ref_last_error().decode())

    def download(self, field: str) -> np.ndarray:
        dt = np.int32 if field in ("is_solid", "total_s") else np.float32
        out = np.empty(self.W * self.H, dt)
        if self.lib.ref_download(self.h, self.FIELDS[field], out.ctypes.data_as(C.c_void_p)):
            raise RuntimeError(self.lib.ref_last_error().decode())
        return out

    def update(self, source, d_t: float) -> None:
        if self.lib.ref_update(self.h, self._src(source), d_t, self.diffusion_sweeps):
            raise RuntimeError(self.lib.ref_last_error().decode())

    def phase(self, phase: int, source, d_t: float) -> None:
        if self.lib.ref_phase(self.h, phase, self._src(source), d_t, self.diffusion_sweeps):
            raise RuntimeError(self.lib.ref_last_error().decode())

    @property
    def pressure_range(self):
        lo, hi = C.c_float(), C.c_float()
        self.lib.ref_pressure_range(self.h, C.byref(lo), C.byref(hi))
        return lo.value, hi.value

    # Visuals (ref_visual.cu): `init` arrays are the buffers' prior contents.
    def render_pixels(self, min_pressure: float, max_pressure: float, init: np.ndarray) -> np.ndarray:
        out = np.ascontiguousarray(init, dtype=np.int32).copy()
        if self.lib.ref_render_pixels(self.h, min_pressure, max_pressure,
                                      out.ctypes.data_as(C.c_void_p)):
            raise RuntimeError(self.lib.ref_last_error().decode())
        return out

    def render_traces(self, dt: float, distance: int, length: int, init_x: np.ndarray,
                      init_y: np.ndarray):
        xs = np.ascontiguousarray(init_x, dtype=np.int32).copy()
        ys = np.ascontiguousarray(init_y, dtype=np.int32).copy()
        if self.lib.ref_render_traces(self.h, dt, distance, length, xs.ctypes.data_as(C.c_void_p),
                                      ys.ctypes.data_as(C.c_void_p)):
            raise RuntimeError(self.lib.ref_last_error().decode())
        return xs, ys

    def sample_velocity(self, px: np.ndarray, py: np.ndarray):
        """The reference's get_general_velocity at the points (px, py)."""
        px = np.ascontiguousarray(px, dtype=np.float32)
        py = np.ascontiguousarray(py, dtype=np.float32)
        ou, ov = np.empty_like(px), np.empty_like(py)
        if self.lib.ref_sample_velocity(self.h, px.size, px, py, ou, ov):
            raise RuntimeError(self.lib.ref_last_error().decode())
        return ou, ov

    def render_arrows(self, cell_size: int, length_multiplier: float, disable_threshold: float,
                      head_length: float, head_angle: float, distance: int,
                      init: np.ndarray) -> np.ndarray:
        """ArrowData records as an (n, 9) int32 array; column 8 is `valid` (its
        first byte; the padding bytes are masked off)."""
        raw = np.ascontiguousarray(init, dtype=np.int32).copy()
        if self.lib.ref_render_arrows(self.h, cell_size, length_multiplier, disable_threshold,
                                      head_length, head_angle, distance,
                                      raw.ctypes.data_as(C.c_void_p)):
            raise RuntimeError(self.lib.ref_last_error().decode())
        raw = raw.reshape(-1, 9)
        raw[:, 8] &= 0xFF
        return raw


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    """||a - b|| / ||b|| in float64 (0 when both are zero)."""
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    den = np.linalg.norm(b)
    num = np.linalg.norm(a - b)
    if den == 0.0:
        return 0.0 if num == 0.0 else float("inf")
    return float(num / den)
