"""The all-fluid path of the projection sweeps divides by s = 4 as a product
by 0.25. That must give the bits of the reference's fast-math division by a
run-time s = 4 (apply_projection_at, src/fluid.cu:240) for every input:
compared over all 2^32 float bit patterns on the GPU."""
import os
import subprocess

import pytest

from tests.conftest import ROOT

SRC = ROOT / "tests" / "cpp" / "quarter_division.cu"
EXE = ROOT / "oracle" / "build" / "quarter_division"


def build_program():
    if EXE.exists() and SRC.stat().st_mtime <= EXE.stat().st_mtime:
        return EXE
    EXE.parent.mkdir(parents=True, exist_ok=True)
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    # the reference's Release flags (CMakeLists.txt:21), which the library shares
    cmd = [nvcc, "-std=c++17", "-O3", "--use_fast_math", "-gencode",
           "arch=compute_103a,code=sm_103a", str(SRC), "-o", str(EXE)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return EXE


def test_program_compiles():
    assert build_program().exists()


@pytest.mark.gpu
def test_quarter_product_equals_division_by_four_everywhere(gpu):
    out = subprocess.run([str(build_program())], check=True, capture_output=True, text=True,
                         timeout=120).stdout.split()
    assert out[0] == "0", f"{out[0]} inputs differ, the first {out[1]}"
