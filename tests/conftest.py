import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the libscft kernels")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as orc

    if not os.path.exists(os.path.join(orc.BUILD_DIR, "liboracle.so")):
        orc.build(with_reference=False)
    return orc.Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle import oracle as orc

    if not orc.Reference.available() and orc.reference_dir() is not None:
        orc.build(with_reference=True)
    if not orc.Reference.available():
        pytest.skip("reference routines not built (reference sources absent on this host)")
    return orc.Reference()


@pytest.fixture(scope="session")
def lib():
    from scft_gb300 import _lib

    return _lib.load()
