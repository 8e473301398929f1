import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    config.addinivalue_line("markers", "slow: long-running")


def _lib_built():
    return os.path.exists(os.path.join(ROOT, "batoid_gb300", "libbatoid_gb300.so"))


@pytest.fixture(scope="session", autouse=True)
def _build_native():
    """Build the CUDA library and the oracle if they are missing."""
    if not _lib_built():
        import __graft_entry__
        __graft_entry__.build()
    if not os.path.exists(os.path.join(ROOT, "oracle", "liboracle.so")):
        import oracle as ora
        ora.build()
    yield
