import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as orc
    if not os.path.exists(orc.LIB_ORACLE):
        orc.build(with_ref=False)
    return orc.Oracle()


@pytest.fixture(scope="session")
def msk():
    import utr_public_gb300 as m
    if not os.path.exists(m.LIB_PATH):
        from utr_public_gb300 import _build
        _build.build()
    m.load()
    return m


@pytest.fixture(scope="session")
def ctx(msk):
    c = msk.Context(0)
    yield c
    c.close()


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def rel_l2(a, b):
    """Relative L2 distance ||a - b|| / ||b|| over every element.  Complex
    arrays are compared as complex128 (real and imaginary parts both count);
    interleaved (..., 2) float arrays as they are."""
    a, b = np.asarray(a), np.asarray(b)
    dt = np.complex128 if (np.iscomplexobj(a) or np.iscomplexobj(b)) else np.float64
    a = a.astype(dt)
    b = b.astype(dt)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
