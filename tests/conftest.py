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
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
