import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds libtacogb (nvcc cross-compiles without a GPU) and the oracle once per session."""
    from taco_gb300 import build as B
    B.build()
    from oracle import oracle as O
    O.build()
