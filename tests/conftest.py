import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 (sm_103a) device")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the engine library and the oracle once per session (nvcc cross-compiles)."""
    from cnt_film_monte_carlo_gb300 import build
    from oracle import oracle

    build.build()
    oracle.build()
    yield
