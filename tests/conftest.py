import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "axia-fem_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libaxia_gpu.so")


def gpu_available():
    """True when an NVIDIA device node is visible; the GPU tests then must pass
    (a missing library or a failing context is an error, not a skip)."""
    return any(os.path.exists(f"/dev/nvidia{i}") for i in range(8))


@pytest.fixture(scope="session")
def gpu_ctx():
    if not gpu_available():
        pytest.skip("no CUDA device")
    from axia_gpu import GpuContext
    ctx = GpuContext(0)
    yield ctx
    ctx.close()
