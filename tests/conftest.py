import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "fast-bc_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C ABI of libfbcgpu.so)")


@pytest.fixture(scope="session")
def fg():
    """The engine's Python binding, initialised on cuda:0."""
    import fastbc_gpu

    fastbc_gpu.init(0)
    return fastbc_gpu
