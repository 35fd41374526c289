import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels through the C ABI)")


@pytest.fixture(scope="session")
def native_lib():
    """Build (if needed) and load libsphgpu.so."""
    from spheral_gb300 import build, _native
    build.build()
    return _native.lib()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as orc
    orc.build()
    return orc
