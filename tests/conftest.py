import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gbmd_lib():
    from exastamp_gb300 import build as B
    B.build()
    from exastamp_gb300 import _capi
    return _capi


@pytest.fixture(scope="session")
def gpu(gbmd_lib):
    """The C-ABI binding, with a GPU present (GPU tests only)."""
    return gbmd_lib
