"""Shared test setup.

Markers: `gpu` tests need a GB300 and the CUDA library; everything else runs
on a CPU-only machine (compilation with NVRTC works without a device).
"""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and libskelcl_cuda.so")


@pytest.fixture(scope="session")
def built():
    """Build libskelcl_cuda.so and the oracle once per session."""
    from skelcl_gb300 import build as b
    b.build()
    return True


@pytest.fixture(scope="session")
def scl(built):
    """The ctypes module, initialised on device 0 (GPU tests only)."""
    import skelcl_gb300 as s
    s.init(0)
    yield s


@pytest.fixture(scope="session")
def orc(built):
    import oracle
    return oracle
