import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "fastcc-benchmark_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the package libraries and the oracle once per session (no-ops
    when they are up to date)."""
    import build_lib
    import oracle
    build_lib.build_all()
    oracle.build()
    yield


@pytest.fixture(scope="session")
def ctx():
    import fastcc_gpu
    c = fastcc_gpu.Context(0)
    yield c
    c.close()
