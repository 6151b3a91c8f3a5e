import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle.Oracle()


@pytest.fixture(scope="session")
def ref():
    """The reference library compiled from its own sources (only where they exist)."""
    from oracle import pyoracle
    from zfp_gb300 import capi
    path = pyoracle.build_ref()
    if not path or not os.path.exists(path):
        pytest.skip("reference sources not available here")
    return capi.ZfpLib(path)


@pytest.fixture(scope="session")
def lib():
    import zfp_gb300
    from zfp_gb300 import build
    build.build()
    return zfp_gb300.load()


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU test needs a CUDA device")
    return torch
