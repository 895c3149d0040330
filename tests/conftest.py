import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and librtgpu.so")


@pytest.fixture(scope="session")
def rtlib():
    """Build (if stale) and load librtgpu.so."""
    from raytracer_gb300 import build
    build.build()
    import raytracer_gb300 as R
    return R


@pytest.fixture(scope="session")
def ctx(rtlib):
    c = rtlib.Context(0)
    yield c
    c.close()
