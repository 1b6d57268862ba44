import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def cuda_lib():
    """Builds (incrementally) and loads libtotri_gb300.so; requires a GPU."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from totri_gb300 import build, _lib
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def cuda_free_lib():
    """Builds (incrementally) and loads libtotri_gb300.so for its host-only
    entry points and argument checks (no GPU needed)."""
    from totri_gb300 import build, _lib
    build.build()
    return _lib.load()
