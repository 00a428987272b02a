import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "proland-4.0_gb300")
for p in (ROOT, PKG, os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    from oracle import build
    build.build()
    return oracle


@pytest.fixture(scope="session")
def product():
    """The product library; built here if needed (the build only needs nvcc)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("proland_gb300_build", os.path.join(PKG, "build.py"))
    pbuild = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pbuild)
    pbuild.build()
    import proland_gb300
    return proland_gb300


@pytest.fixture(scope="session")
def gpu(product):
    if not product.device_available():
        pytest.fail("GPU test collected but no CUDA device is visible")
    return product
