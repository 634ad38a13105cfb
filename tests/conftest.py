"""Shared test fixtures.  Tests marked ``gpu`` need a CUDA device and the built engine; the
rest run on the CPU (oracle, host logic, ABI surface)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the compiled engine")


@pytest.fixture(scope="session")
def restatement():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle.Restatement()


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    return load


@pytest.fixture(scope="session")
def engine_lib():
    """The engine library (built here if missing and nvcc is available)."""
    import omega2d_gb300 as og
    if not os.path.exists(og.LIB_PATH):
        from omega2d_gb300 import _build
        try:
            _build.build()
        except Exception as e:  # no toolkit on this machine
            pytest.skip(f"engine library not built and cannot be built here: {e}")
    return og.lib()


@pytest.fixture(scope="session")
def ctx():
    import omega2d_gb300 as og
    c = og.Context(0)
    yield c
    c.close()


def rel_err(ref, got):
    """Normwise max relative error ||got - ref||_inf / ||ref||_inf."""
    ref = np.asarray(ref, np.float64)
    got = np.asarray(got, np.float64)
    den = np.max(np.abs(ref))
    return float(np.max(np.abs(got - ref)) / (den if den > 0 else 1.0))
