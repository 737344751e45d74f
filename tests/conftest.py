import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

PKG = "masterarbeit_parallele_konstruktion_der_burrows-wheeler-transformation_auf_der_gpu_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")
    config.addinivalue_line("markers", "slow: long-running (full-size workloads)")


@pytest.fixture(scope="session")
def pkg():
    """The package with libgbwt.so built (nvcc cross-compiles without a GPU)."""
    importlib.import_module(PKG + ".build").build()
    return importlib.import_module(PKG)


@pytest.fixture(scope="session")
def wl():
    return importlib.import_module(PKG + ".workloads")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def storage(pkg):
    st = pkg.Storage(1 << 20)
    yield st
    st.close()
