import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA library)")


@pytest.fixture(scope="session")
def table():
    from mitos_gb300.perturb import load_table
    return load_table()


@pytest.fixture(scope="session")
def spline(table):
    import mitos_gb300.lib as ml
    return ml.Spline(table)


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
