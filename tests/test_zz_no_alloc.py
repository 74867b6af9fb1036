"""msk_calculate_static: calculate() for callers that cannot allocate device
memory (a plug-in whose host framework owns every device byte through its own
pool, or a loop that cannot afford cudaMalloc's latency and implicit
synchronisation).  Its scratch is a fixed array compiled into libmsk.so, so
this file checks, through the C ABI, that consecutive calls of different
sizes -- each reusing what the previous call left in that array -- give the
same exit wave as msk_calculate while the library's device-allocation count
stays unchanged, and that sizes beyond the array's limits are refused.  It is collected last so that a run stopping at its first failure
has already run every other test; it also passes alone in a fresh process.
"""
import numpy as np
import pytest

from conftest import golden, rel_l2
from utr_public_gb300 import specimen as sp

pytestmark = pytest.mark.gpu

# tolerance of the GPU parity tests (relative L2 over the grid)
TOL = 1e-5


def cases(msk):
    g = golden("ref_exit_c1_256.npz")
    s = sp.plain_specimen(int(g["seed"]))
    n = int(g["natom"])
    big = (msk.make_param(64.0, 64.0, 256, 256, 200.0, 2.0),
           (s.Znum[:n], s.x[:n], s.y[:n], s.z[:n], s.occ[:n]), 64.0, 64.0)
    r = sp.random_specimen(300, 32.0, 3.0, 29.0, 77)
    small = (msk.make_param(32.0, 32.0, 64, 128, 300.0, 1.0),
             (r.Znum, r.x, r.y, r.z, r.occ), 32.0, 32.0)
    return big, small


def test_static_entry_matches_calculate_on_consecutive_calls(ctx, msk):
    big, small = cases(msk)
    seq = (big, small, big)  # a smaller grid over what the big call left, then big again
    refs = [ctx.calculate(param, *atoms, box, boxz) for param, atoms, box, boxz in seq]
    # the counter counts: a new context's first call allocates its buffers
    n0 = msk.device_allocations()
    c2 = msk.Context(0)
    try:
        c2.calculate(*small[:1], *small[1], small[2], small[3])
    finally:
        c2.close()
    assert msk.device_allocations() > n0
    # ... and the entry point allocates nothing, on any of its calls
    n1 = msk.device_allocations()
    for (param, atoms, box, boxz), ref in zip(seq, refs):
        out = msk.calculate_static(param, *atoms, box, boxz)
        assert np.isfinite(out).all()
        assert rel_l2(out, ref) < TOL
    assert msk.device_allocations() == n1


def test_static_entry_refuses_sizes_beyond_its_scratch(msk):
    r = sp.random_specimen(10, 64.0, 10.0, 54.0, 5)
    atoms = (r.Znum, r.x, r.y, r.z, r.occ)
    with pytest.raises(msk.MskError) as e:
        msk.calculate_static(msk.make_param(64.0, 64.0, 1024, 512, 200.0, 2.0), *atoms, 64.0, 64.0)
    assert e.value.status == msk.MSK_ETOOLARGE
    many = sp.random_specimen(70000, 64.0, 10.0, 54.0, 6)
    with pytest.raises(msk.MskError) as e:
        msk.calculate_static(msk.make_param(64.0, 64.0, 64, 64, 200.0, 2.0), many.Znum, many.x,
                             many.y, many.z, many.occ, 64.0, 64.0)
    assert e.value.status == msk.MSK_ETOOLARGE
