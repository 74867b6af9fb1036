"""The potential spline's interval lookup (spline_vz in msk_passes.cuh): a
byte table per bucket of r^2 (the float's exponent and top four mantissa
bits, 2^-20 to 2^5) gives the last knot at or below the bucket's start, and
one compare with the next knot finishes it.  That is seval's bisection
interval (TemsimLibrary/slicelib.cpp:2402-2425: knot[i] <= r^2 < knot[i+1],
clamped to [0, 98]) only if no bucket holds two knots; the knots are the
reference's fixed log-spaced r grid (0.01 to 5 A, 100 points, squared), as
the host tables build them.  Restated here in numpy and checked for every
bucket and on random r^2 against a bisection."""
import numpy as np

KN = 100
SHIFT = 23 - 4
BASE = (127 - 20) << 4
NB = 25 << 4


def knots_f32():
    dlnr = np.log(5.0 / 0.01) / (KN - 1)
    r = 0.01 * np.exp(np.arange(KN) * dlnr)
    return (r * r).astype(np.float32)


def bucket_table(k):
    lo = ((BASE + np.arange(NB)).astype(np.uint32) << SHIFT).view(np.float32)
    i0 = np.searchsorted(k[1:KN - 1], lo, side="right")  # knots[i0 + 1] <= lo advances
    return np.minimum(i0, KN - 2).astype(np.int64), lo


def lookup(k, table, rsq):
    b = (rsq.astype(np.float32).view(np.uint32) >> SHIFT).astype(np.int64) - BASE
    b = np.clip(b, 0, NB - 1)
    i = table[b]
    up = (rsq >= k[i + 1]) & (i < KN - 2)
    return i + up


def bisection(k, rsq):
    i = np.searchsorted(k, rsq, side="right") - 1  # knot[i] <= rsq < knot[i+1]
    return np.clip(i, 0, KN - 2)


def test_no_bucket_holds_two_knots():
    k = knots_f32()
    table, lo = bucket_table(k)
    hi = np.append(lo[1:], np.float32(2.0 ** 5))
    for b in range(NB):
        i0 = table[b]
        if i0 + 2 <= KN - 1:
            assert k[i0 + 2] >= hi[b], b


def test_lookup_equals_bisection():
    k = knots_f32()
    table, lo = bucket_table(k)
    rng = np.random.default_rng(5)
    rsq = np.concatenate([
        np.exp(rng.uniform(np.log(1e-6), np.log(9.0), 200000)).astype(np.float32),
        k[:KN - 1], np.nextafter(k[:KN - 1], np.float32(0)), lo[(lo >= 1e-6) & (lo <= 9.0)],
        np.float32([9.0, 1e-6])])
    rsq = rsq[(rsq > 0) & (rsq <= 9.0)]
    assert np.array_equal(lookup(k, table, rsq), bisection(k, rsq))
