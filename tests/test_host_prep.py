"""Host side of libmsk without a GPU: the C ABI loads and exports what
include/msk.h declares, and the reference-exact host preparation (Shell
sort, rotation, slice assignment, potential tables) equals the oracle and the
reference's golden outputs bit for bit."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden
from utr_public_gb300 import specimen as sp


def declared_functions():
    hdrs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
            if f.endswith(".h")]
    names = set()
    for h in hdrs:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(msk_\w+)\s*\(", text))
    return sorted(names)


def test_abi_exports_every_declared_symbol(msk):
    names = declared_functions()
    assert "msk_calculate" in names and "msk_tilt_series" in names
    L = msk.load()
    for n in names:
        assert hasattr(L, n), n
    assert set(msk.EXPORTS) <= set(names)


def test_missing_library_fails_loudly(monkeypatch):
    """Without libmsk.so the package raises at load: there is no CPU
    fallback for any call."""
    import utr_public_gb300 as m
    monkeypatch.setattr(m, "_lib", None)
    monkeypatch.setattr(m, "LIB_PATH", os.path.join(ROOT, "no_such_dir", "libmsk.so"))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        m.load()
    with pytest.raises(RuntimeError):
        m.Context(0)


def test_status_strings(msk):
    L = msk.load()
    for st in (0, -1, -2, -3, -4, -5, -6, -7, -8):
        assert L.msk_status_string(st)
    assert L.msk_status_string(-99) == b"unknown status"


def test_null_context_is_rejected(msk):
    L = msk.load()
    z = np.zeros(200, np.float32)
    assert L.msk_calculate(None, None, None, z, 0, None, None, None, None, None, None, 1.0, 1.0,
                           0, 0, None) == msk.MSK_EINVAL


def test_sort_matches_reference_and_oracle(msk, oracle):
    g = golden("ref_sort.npz")
    s = sp.plain_specimen(1001)
    idx = np.arange(s.natom, dtype=np.float32)
    _, _, _, zs, perm = msk.sort_by_z(s.Znum, s.x, s.y, s.z, idx)
    assert np.array_equal(perm.astype(np.int32), g["perm"])
    s2 = sp.tilt_specimen(1002)
    a = msk.sort_by_z(s2.Znum, s2.x, s2.y, s2.z, s2.occ)
    b = oracle.sort_by_z(s2.Znum, s2.x, s2.y, s2.z, s2.occ)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


@pytest.mark.parametrize("angZ,angY", [(0.0, 0.0), (0.0, 0.7853981633974483),
                                       (1.2, 2.9), (3.0, -0.4)])
def test_rotation_matches_oracle(msk, oracle, angZ, angY):
    s = sp.tilt_specimen(1002)
    a = msk.rotate(160.0, angZ, angY, s.x, s.y, s.z, 0.5, -0.25, 1.0)
    b = oracle.rotate(160.0, angZ, angY, s.x, s.y, s.z, 0.5, -0.25, 1.0)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


@pytest.mark.parametrize("dz,box", [(2.0, 64.0), (1.0, 160.0), (1.25, 100.0), (0.7, 33.3)])
def test_slice_assignment_matches_oracle(msk, oracle, dz, box):
    s = sp.random_specimen(5000, box, 0.0, box, 77)
    _, _, _, zs, _ = oracle.sort_by_z(s.Znum, s.x, s.y, s.z, s.occ)
    a, na = msk.slice_assign(dz, box, zs)
    b, nb = oracle.slice_assign(dz, box, zs)
    assert na == nb == msk.slice_count(dz, box) == oracle.slice_count(dz, box)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("Z", [1, 6, 7, 8, 16, 29, 79, 103])
def test_potential_table_matches_oracle(msk, oracle, Z):
    knots, coef = msk.potential_table(Z)
    ok, oy, ob, oc, od = oracle.lut_table(Z)
    assert np.array_equal(knots, ok)
    assert np.array_equal(coef[:, 0], oy)
    assert np.array_equal(coef[:, 1], ob)
    assert np.array_equal(coef[:, 2], oc)
    assert np.array_equal(coef[:, 3], od)
    with pytest.raises(Exception):
        msk.potential_table(0)
