import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


@pytest.fixture(scope="session")
def product_lib():
    from pbf_gb300 import build
    build.build()
    from pbf_gb300 import _capi
    return _capi.load()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def gpu(product_lib):
    if not HAS_GPU:
        pytest.fail("a CUDA GPU is required for -m gpu tests")
    return product_lib
