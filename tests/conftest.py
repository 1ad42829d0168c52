import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sampler on the device)")


@pytest.fixture(scope="session", autouse=True)
def built_library():
    """Build libgnuts.so and the oracle once per session (incremental)."""
    from cmdstan_gb300 import build
    build.build()
    yield
