import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "one-mxll-to-rule-them-all_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the oracle (gcc) and the GPU library (nvcc, sm_103a) once per session."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_oracle

    build_oracle.build()
    sys.path.insert(0, PKG)
    import build as gpu_build

    gpu_build.build()
    yield


@pytest.fixture(scope="session")
def orc():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    return oracle


@pytest.fixture(scope="session")
def omx():
    import omx as m

    return m
