"""In-tree build of the CUDA library (sm_103a).

`build_library()` compiles opensayal_gb300/csrc into
opensayal_gb300/lib/libopensayal_gb300.so with nvcc, for GB300 only
(`-gencode arch=compute_103a,code=sm_103a`) and with `--use_fast_math`, the
reference's own Release flag (CMakeLists.txt:21), so that FP32 divisions and
square roots round the way the reference's kernels do.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB_DIR = PKG / "lib"
LIB_PATH = LIB_DIR / "libopensayal_gb300.so"
HEADER = ROOT / "include" / "opensayal_gb300.h"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-std=c++17", "-O3", "--use_fast_math", "-lineinfo",
    "-Xcompiler", "-fPIC", "-shared", "-diag-suppress", "177",
]


def _nvcc() -> str:
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = Path(cuda_home) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    found = shutil.which("nvcc")
    if not found:
        raise RuntimeError("nvcc not found: the GB300 library cannot be built")
    return found


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + [HEADER]


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    """Compile the library if any source is newer than the built .so."""
    if not force and not _stale(LIB_PATH, _sources()):
        return LIB_PATH
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [_nvcc(), *NVCC_FLAGS, *ARCH_FLAGS, "-o", str(tmp), str(CSRC / "os_fluid.cu")]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed ({' '.join(cmd)}):\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(res.stderr)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build_library(force=True, verbose=True))
