import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libfdfd_cuda.so")


@pytest.fixture(scope="session")
def fdfd():
    return __graft_entry__.load_package()


@pytest.fixture(scope="session")
def lib(fdfd):
    """The CUDA library, built on demand (nvcc cross-compiles without a GPU)."""
    __graft_entry__.build()
    return fdfd._lib.load()


@pytest.fixture(scope="session")
def oracle():
    import fdfd_oracle
    return fdfd_oracle
