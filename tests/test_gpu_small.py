"""Small grids (64^2 to 256^2) run their whole slice loop in one launch: one
thread-block cluster per unit (msk_small.cuh).  The potentials, multipliers
and atom order are those of the launch-per-pass loop (MSK_SMALL_GRID=0
selects it); the line transforms use another radix split (16 points a
thread), so the two paths agree to FP32 rounding (relative L2 2e-6) and both
must match the FP64 oracle within 1e-5.  The reference golden at 256^2 (C1's
grid) is checked through the cluster path by test_gpu_parity, and repeated
calls through it are bit-stable (test_gpu_parity.test_deterministic)."""
import os

import numpy as np
import pytest

from conftest import rel_l2
from utr_public_gb300 import specimen as sp

pytestmark = pytest.mark.gpu


def both_paths(fn):
    os.environ["MSK_SMALL_GRID"] = "0"
    try:
        loop = fn()
    finally:
        os.environ.pop("MSK_SMALL_GRID", None)
    return fn(), loop


@pytest.mark.parametrize("n,fov,v0,dz", [(64, 32.0, 200.0, 2.0), (128, 48.0, 300.0, 1.0),
                                          (256, 64.0, 200.0, 2.0)])
def test_calculate_cluster_path_equals_pass_loop(ctx, msk, oracle, n, fov, v0, dz):
    s = sp.random_specimen(400, fov, 0.1 * fov, 0.9 * fov, 900 + n)
    atoms = (s.Znum, s.x, s.y, s.z, s.occ)
    param = msk.make_param(fov, fov, n, n, v0, dz)
    fast, loop = both_paths(lambda: ctx.calculate(param, *atoms, fov, fov))
    assert rel_l2(fast, loop) < 2e-6
    ref64 = oracle.calculate(param, *atoms, fov, fov, fp64=True)
    assert rel_l2(fast, ref64) < 1e-5 and rel_l2(loop, ref64) < 1e-5


def test_calculate_cluster_path_with_incident_wave_and_tilt(ctx, msk, oracle):
    s = sp.random_specimen(300, 32.0, 4.0, 28.0, 917)
    atoms = (s.Znum, s.x, s.y, s.z, s.occ)
    param = msk.make_param(32.0, 32.0, 128, 128, 200.0, 1.0, ctiltx=0.003, ctilty=-0.002)
    rng = np.random.default_rng(8)
    ph = rng.uniform(0, 2 * np.pi, (128, 128))
    w0 = np.stack([np.cos(ph), np.sin(ph)], -1).astype(np.float32)
    fast, loop = both_paths(lambda: ctx.calculate(param, *atoms, 32.0, 32.0, wave0=w0))
    assert rel_l2(fast, loop) < 2e-6
    ref64 = oracle.calculate(param, *atoms, 32.0, 32.0, wave0=w0.astype(np.float64), fp64=True)
    assert rel_l2(fast, ref64) < 1e-5


def test_tilt_series_cluster_path_equals_pass_loop(ctx, msk):
    """Several units in one launch (one cluster each; the path takes calls whose
    units fit in one wave of clusters), slices without atoms at both ends of the
    box, two defoci: images and exit waves as the loop's; every unit of the
    launch equal to the same orientation computed alone."""
    spec = sp.random_specimen(700, 64.0, 14.0, 50.0, 931)
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    s = msk.Series()
    s.nx = s.ny = 256
    s.ctblength = s.ctblengthz = 64.0
    s.v0, s.deltaz = 300.0, 1.0
    angY = np.deg2rad([0.0, 35.0, 80.0, 125.0])
    angZ = np.linspace(0.0, 0.5, len(angY))
    run = lambda: ctx.tilt_series(s, *atoms, angZ, angY, [0.0, 400.0], want_exit=True)
    (fi, fe, fk), (li, le, lk) = both_paths(run)
    assert np.array_equal(fk, lk)
    for a in range(len(angY)):
        assert rel_l2(fe[a], le[a]) < 2e-6, a
        for d in range(2):
            assert rel_l2(fi[a, d], li[a, d]) < 2e-6, (a, d)
    one, ew1, _ = ctx.tilt_series(s, *atoms, angZ[2:3], angY[2:3], [0.0, 400.0], want_exit=True)
    assert np.array_equal(one[0], fi[2]) and np.array_equal(ew1[0], fe[2])
