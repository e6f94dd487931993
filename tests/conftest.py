import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the compute path")


@pytest.fixture(scope="session")
def lib_built():
    from opensayal_gb300.build import build_library
    return build_library()


@pytest.fixture(scope="session")
def oracle_built():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu(lib_built, oracle_built):
    import torch
    if torch.cuda.device_count() == 0:
        pytest.skip("no CUDA device in this machine")
    return 0
