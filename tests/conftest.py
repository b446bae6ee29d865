import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs through libbmxg.so)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O
    O.build(ref=False)
    return O


@pytest.fixture(scope="session")
def gpu_lib():
    """libbmxg.so built for sm_103a and a visible device; no fallback."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("the gpu tests need a CUDA device")
    from boltzmannmfx_gb300 import build, runtime
    build.build()
    torch.cuda.init()
    return runtime.load_library()
