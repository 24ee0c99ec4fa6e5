import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libsph_gb300.so)")


@pytest.fixture(scope="session")
def orc():
    """The CPU oracle (test infrastructure), built on first use."""
    import oracle
    if not os.path.exists(oracle.LIB_PATH):
        oracle.build()
    oracle.set_threads(min(16, os.cpu_count() or 1))
    return oracle


@pytest.fixture(scope="session")
def sphlib():
    """The product library, built on first use (nvcc, sm_103a)."""
    from cudasphnew_gb300 import _build, lib
    _build.build()
    lib.load()
    return lib
