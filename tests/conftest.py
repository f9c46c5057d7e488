import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libxpbi.so")


@pytest.fixture(scope="session")
def xp():
    """The package (its directory name is not an identifier)."""
    return importlib.import_module("xpbi-webgpu_gb300")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def built_lib(xp):
    from importlib import import_module
    b = import_module("xpbi-webgpu_gb300.build")
    b.build()
    return xp.lib()


def field_rel_err(a, b):
    """Normwise relative error max|a-b| / max|b| of one field."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.abs(b).max(), 1e-30)
    return float(np.abs(a - b).max() / scale)
