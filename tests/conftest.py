import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session", autouse=True)
def _oracle_built():
    """The oracle is test infrastructure; build it on first use (g++, seconds)."""
    from oracle import build as obuild

    if not os.path.isfile(obuild.ORACLE_SO):
        assert obuild.build_oracle().wait() == 0
    yield


@pytest.fixture(scope="session")
def native_lib_path():
    """libnrgb300.so, built here when missing (nvcc cross-compiles without a GPU)."""
    from newrecon_gb300 import _build

    if not os.path.isfile(_build.LIB):
        _build.build()
    return _build.LIB


def golden(name):
    import numpy as np

    return np.load(os.path.join(ROOT, "tests", "golden", f"{name}.npz"))
