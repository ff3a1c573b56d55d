import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def cflib():
    """The built libcellflow.so (built on demand; there is no CPU fallback)."""
    from cellflow_gb300 import _lib, build

    build.build()
    return _lib.load()
