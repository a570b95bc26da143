import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA engine through the C ABI)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the native libraries once (fast no-op when up to date)."""
    from simbody_gb300.build import build_oracle, build_workloads
    build_workloads()
    build_oracle()
    yield


@pytest.fixture(scope="session")
def engine():
    """The CUDA engine; GPU tests fail loudly if it is missing."""
    from simbody_gb300.build import build_engine
    build_engine()
    import simbody_gb300 as sbg
    if sbg.device_count() < 1:
        pytest.fail("no CUDA device visible to the engine")
    return sbg
