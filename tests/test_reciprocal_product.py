"""The diffusion passes on column-parity planes take the Jacobi update's
division by den = 1 + 4a (apply_diffusion_at, src/fluid.cu:178-182) as the
product with __fdividef(1, den). That must give the bits of the reference's
fast-math division for every input: compared over all 2^32 float bit
patterns on the GPU, for the divisors of a spread of viscosities, steps and
cell sizes and for further divisors up to 1e6."""
import os
import subprocess

import pytest

from tests.conftest import ROOT

SRC = ROOT / "tests" / "cpp" / "reciprocal_product.cu"
EXE = ROOT / "oracle" / "build" / "reciprocal_product"


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
def test_reciprocal_product_equals_division_everywhere(gpu):
    out = subprocess.run([str(build_program())], check=True, capture_output=True, text=True,
                         timeout=300).stdout.strip().splitlines()
    assert len(out) == 89
    bad = [line for line in out if line.split()[1] != "0"]
    assert not bad, f"divisors whose product differs: {bad}"
