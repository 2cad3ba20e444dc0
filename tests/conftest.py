import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run on the GB300 box)")


@pytest.fixture(scope="session")
def fz():
    import __graft_entry__ as g
    return g.load_package()


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def synth(fz):
    from importlib import import_module
    return import_module("fz_gpu_gb300.synth")


def error_tolerance(x, eb_abs):
    """Per-point bound of |x - x'| for float dual-quantisation: x' = fl(round(fl(x r)) e)
    with r = (float)(1/2eb), e = (float)(2eb): |x - x'| <= eb (1 + 2u) + 4u |x|,
    u = 2^-24.  The test uses eb (1 + 2^-21) + 2^-21 |x|."""
    import numpy as np
    return eb_abs * (1 + 2.0 ** -21) + np.abs(x.astype(np.float64)) * 2.0 ** -21
