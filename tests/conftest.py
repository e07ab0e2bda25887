import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# the reference source tree, when a test wants to read it directly (unset: skip)
REFERENCE = os.environ.get("MRFMAP_REFERENCE_DIR")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def native_lib():
    """The C-ABI library, built in-tree if missing."""
    from mrfmap_gb300 import _build, lib
    if not os.path.exists(lib.LIB_PATH):
        _build.build_lib()
    return lib.load()


@pytest.fixture(scope="session")
def small_room():
    from mrfmap_gb300 import synthetic
    return synthetic.small_room(0)
