import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libfdfd_cuda.so")
    config.addinivalue_line("markers", "big_oracle(*names): full-size oracle results the test reads")


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


# Full-size oracle results (tests/_big_oracle.py): a GPU test that needs one
# names it with @pytest.mark.big_oracle("name"); the jobs start in spawned
# processes as soon as collection ends, so they overlap the other GPU tests.
def pytest_collection_finish(session):
    names = set()
    for item in session.items:
        for m in item.iter_markers("big_oracle"):
            names.update(m.args)
    if names:
        import _big_oracle
        _big_oracle.start(sorted(names))


def pytest_sessionfinish(session, exitstatus):
    mod = sys.modules.get("_big_oracle")
    if mod is not None:
        mod.shutdown()


@pytest.fixture(scope="session")
def big_oracle():
    import _big_oracle
    return _big_oracle.result
