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


@pytest.fixture(scope="session", autouse=True)
def _oracle_key_division():
    """Most GPU tests compare the solver with the CPU oracle bit for bit, so
    the solvers the tests create use the oracle's IEEE cell-key division.  The
    library's default, the reference's own division, is checked against the
    reference solver in test_gpu_ref_parity.py, whose solvers ask for it by
    name (and by the smoke check of the entry module)."""
    from xpbd_gb300 import build, native

    if not os.path.exists(build.library_path()):
        yield
        return
    native.set_default_key_division("ieee")
    yield
    native.set_default_key_division("reference")
