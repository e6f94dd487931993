"""The C++ drop-in header: a program written against the reference's
interface compiles against include/opensayal_gb300/fluid.hpp (CPU test) and
gives the same fields as the Python binding (GPU test)."""
import subprocess

import numpy as np
import pytest

from opensayal_gb300 import Fluid
from opensayal_gb300.build import LIB_DIR
from opensayal_gb300.fluid import default_config
from tests.conftest import ROOT

SRC = ROOT / "tests" / "cpp" / "drop_in_main.cpp"
EXE = ROOT / "oracle" / "build" / "drop_in_main"


def build_program():
    deps = [SRC, *(ROOT / "include").rglob("*.h*"), LIB_DIR / "libopensayal_gb300.so"]
    if EXE.exists() and all(d.stat().st_mtime <= EXE.stat().st_mtime for d in deps):
        return EXE
    EXE.parent.mkdir(parents=True, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O2", f"-I{ROOT / 'include'}", "-I/usr/local/cuda/include",
           str(SRC), "-o", str(EXE), f"-L{LIB_DIR}", "-lopensayal_gb300",
           f"-Wl,-rpath,{LIB_DIR}", "-L/usr/local/cuda/lib64", "-lcudart",
           "-Wl,-rpath,/usr/local/cuda/lib64"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return EXE


def test_program_compiles_against_the_header(lib_built):
    assert build_program().exists()


@pytest.mark.gpu
def test_program_matches_python_binding(gpu):
    exe = build_program()
    out = subprocess.run([str(exe), "256", "128", "10"], check=True, capture_output=True,
                         text=True).stdout.split()
    su, sv, ss, pmin, pmax, idx = float(out[0]), float(out[1]), float(out[2]), float(out[3]), \
        float(out[4]), int(out[5])
    c = default_config(256, 128)
    c.enable_drain, c.enable_pressure, c.g = 0, 1, -5.0
    c.tunnel_speed, c.tunnel_smoke = 2.0, 1.0
    c.obstacle_radius = 9.5
    with Fluid(c) as f:
        for _ in range(10):
            f.update(None, 0.05)
        # sequential FP64 sums, as the program forms them
        for name, total in (("vel_x", su), ("vel_y", sv), ("smoke", ss)):
            assert total == float(np.cumsum(f.download(name).astype(np.float64))[-1]), name
        assert pmin == np.float32(f.min_pressure) and pmax == np.float32(f.max_pressure)
        assert idx == f.indx(3, 0)


HELPERS_SRC = ROOT / "tests" / "cpp" / "device_helpers_main.cu"
HELPERS_EXE = ROOT / "oracle" / "build" / "device_helpers_main"


def build_helpers_program():
    """The caller-kernel program, compiled by nvcc with the reference's
    Release flags (CMakeLists.txt:21) so that its helper arithmetic rounds as
    the reference's does."""
    import os
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    deps = [HELPERS_SRC, *(ROOT / "include").rglob("*.h*"), LIB_DIR / "libopensayal_gb300.so"]
    if HELPERS_EXE.exists() and all(d.stat().st_mtime <= HELPERS_EXE.stat().st_mtime
                                    for d in deps):
        return HELPERS_EXE
    HELPERS_EXE.parent.mkdir(parents=True, exist_ok=True)
    cmd = [nvcc, "-std=c++17", "-O3", "--use_fast_math", "-gencode",
           "arch=compute_103a,code=sm_103a", f"-I{ROOT / 'include'}", str(HELPERS_SRC),
           "-o", str(HELPERS_EXE), f"-L{LIB_DIR}", "-lopensayal_gb300",
           "-Xlinker", "-rpath", "-Xlinker", str(LIB_DIR)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return HELPERS_EXE


def test_helpers_program_compiles_against_the_header(lib_built):
    assert build_helpers_program().exists()


@pytest.mark.gpu
def test_device_helpers_match_reference_kernels(gpu, tmp_path):
    """get_general_velocity and trace called from the caller's own kernel
    through fluid.d_this give the bits the reference's own device functions
    give on the same fields (oracle/ref_visual.cu's ref_sample and
    ref_traces)."""
    import json

    import oracle
    from opensayal_gb300.fluid import load_config
    exe = build_helpers_program()
    doc = {"sim": {"width": 256, "height": 128, "enable_drain": False,
                   "projection": {"n": 20}, "physics": {"g": -5.0},
                   "wind_tunnel": {"speed": 2.0, "pipe_height": 32},
                   "obstacle": {"radius": 9.5}}}
    conf = tmp_path / "OpenSayal.conf.json"
    conf.write_text(json.dumps(doc))
    cfg = load_config(conf)
    W, H = cfg.width, cfg.height
    rng = np.random.default_rng(21)
    n = 4096
    px = rng.uniform(-3, W + 3, n).astype(np.float32)
    py = rng.uniform(-3, H + 3, n).astype(np.float32)
    # exact half-cell and whole-cell positions, where the branches switch
    px[:256] = (rng.integers(0, W, 256) + rng.choice([0.0, 0.5], 256)).astype(np.float32)
    py[:256] = (rng.integers(0, H, 256) + rng.choice([0.0, 0.5], 256)).astype(np.float32)
    pts = tmp_path / "points.bin"
    with open(pts, "wb") as fh:
        fh.write(np.int32(n).tobytes())
        fh.write(px.tobytes())
        fh.write(py.tobytes())
    out = tmp_path / "out.bin"
    subprocess.run([str(exe), str(conf), "10", str(pts), str(out)], check=True,
                   capture_output=True, text=True)
    raw = out.read_bytes()
    cells = W * H
    d, length = 8, 12
    tn = (W // d) * (H // d) * length
    f32 = np.frombuffer(raw[: 4 * (2 * cells + 2 * n)], dtype=np.float32)
    u, v = f32[:cells], f32[cells:2 * cells]
    su, sv = f32[2 * cells:2 * cells + n], f32[2 * cells + n:]
    i32 = np.frombuffer(raw[4 * (2 * cells + 2 * n):], dtype=np.int32)
    xs, ys = i32[:tn], i32[tn:]
    assert np.abs(u).max() > 0.1, "the flow should have developed"
    ref = oracle.RefFluid(cfg)
    ref.upload("vel_x", u)
    ref.upload("vel_y", v)
    ru, rv = ref.sample_velocity(px, py)
    assert np.array_equal(su, ru), int((su != ru).sum())
    assert np.array_equal(sv, rv), int((sv != rv).sum())
    rx, ry = ref.render_traces(cfg.d_t, d, length, np.zeros(tn, np.int32), np.zeros(tn, np.int32))
    assert np.array_equal(xs, rx) and np.array_equal(ys, ry)
    ref.close()
