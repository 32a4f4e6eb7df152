"""Shared fixtures.  GPU tests are marked ``gpu`` and call the engine through
its C ABI; everything else runs on the CPU (oracle, host logic, ABI load)."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the engine")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from highperformanceseismicstacking_gb300 import build
    build.build_oracle()
    build.build_engine()
    yield


@pytest.fixture(scope="session")
def engine():
    from highperformanceseismicstacking_gb300 import capi
    eng = capi.Engine(0)
    yield eng
    eng.close()
