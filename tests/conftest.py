import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the engine's kernels)")


@pytest.fixture(scope="session")
def engine():
    """The built engine library; builds it if needed."""
    from everett_gb300 import build
    build.build()
    from everett_gb300 import _native
    return _native.lib()


@pytest.fixture(scope="session")
def gpu(engine):
    from everett_gb300 import _native
    if _native.device_count() < 1:
        pytest.fail("no CUDA device visible to the engine")
    return True
