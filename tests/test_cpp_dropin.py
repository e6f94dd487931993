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
