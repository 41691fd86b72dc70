"""pytest configuration: the `gpu` marker and shared fixtures.

`-m "not gpu"` runs everything that needs no GPU (oracle pins, fixtures,
host logic, the C ABI's exports and validation).  `-m gpu` runs the parity
tests proper: the CUDA core through the C ABI against the oracle.
"""
import os
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(REPO / "tests"))
sys.path.insert(0, str(REPO))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (sm_103) and the built CUDA core")


@pytest.fixture(scope="session")
def lib():
    import common  # noqa: F401
    import are_gb300 as are
    return are.load()


@pytest.fixture(scope="session")
def gpu_lib(lib):
    n = lib.are_device_count()
    assert n > 0, "GPU test run without a visible CUDA device"
    return lib


@pytest.fixture(scope="session")
def oracle():
    from oracle.orc import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def nthreads():
    return max(1, min(16, os.cpu_count() or 1))
