import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("ssbl-cuda-xpbd_gb300", "oracle", "tests"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built sm_103a library")


@pytest.fixture(scope="session")
def oracle_lib():
    import xpbd_oracle

    xpbd_oracle.build()
    return xpbd_oracle


@pytest.fixture(scope="session")
def gpu_lib():
    """The product library, built for sm_103a; fails loudly when missing."""
    from xpbd_gb300 import build, native

    build.build()
    lib = native._load_library()
    return native
