import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "quantumopticsbase.jl_gb300"), os.path.join(ROOT, "oracle"),
          os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and libqobgpu.so")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    """Build the oracle (gcc) once per session; the GPU library is built by
    __graft_entry__.build() (nvcc), which the GPU tests require."""
    import oracle

    oracle.build()
    yield
