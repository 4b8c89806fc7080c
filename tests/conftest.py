import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libswiftest_gb300.so")


@pytest.fixture(scope="session")
def ctx():
    """One CUDA context for the GPU tests; fails loudly when the library is missing."""
    from swiftest_gb300 import build as B
    B.build()
    from swiftest_gb300.api import Context
    c = Context(0)
    yield c
    c.close()
