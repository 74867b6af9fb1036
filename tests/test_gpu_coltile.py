"""The column passes' schedules (chosen per grid and pass by timing at run
time: the FFT plan -- 32 or 16 points a thread -- and two tile widths each).
A tilt series run with each variant forced (MSK_COL_TILE) in its own process:
the two tile widths of one plan compute every column identically (bit for
bit), every variant and the tuned choice match the FP64 oracle within 1e-5,
and the tuner reports the schedule it chose (msk_column_plan).  64^2 and
256^2 run their slice loop as one cluster launch, so only their free-space
step takes a column pass; 1024^2 and 2048^2 take all of them."""
import concurrent.futures as cf
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = ((64, 32.0), (256, 64.0), (1024, 96.0), (2048, 96.0))
ANGLES = (10.0, 50.0)

SCRIPT = r"""
import sys, json, numpy as np
sys.path.insert(0, %r)
import utr_public_gb300 as msk
from utr_public_gb300 import specimen as sp
ctx = msk.Context(0)
out, plans = {}, {}
for n, fov in %r:
    spec = sp.random_specimen(400, fov, 0.2 * fov, 0.8 * fov, 1041)
    s = msk.Series()
    s.nx = s.ny = n
    s.ctblength = s.ctblengthz = fov
    s.v0, s.deltaz, s.aobj = 300.0, 2.0, 0.02
    imgs, ew, _ = ctx.tilt_series(s, spec.Znum, spec.x, spec.y, spec.z, spec.occ, [0.0, 0.3],
                                  np.deg2rad(%r), [0.0, 200.0], want_exit=True)
    out["img%%d" %% n], out["ew%%d" %% n] = imgs, ew
    plans[str(n)] = {p: msk.column_plan(0, n, n, p) for p in msk.COLUMN_PASSES}
np.savez(sys.argv[1], **out)
print(json.dumps(plans))
""" % (ROOT, CASES, list(ANGLES))


def run(tmp_path, variant):
    env = dict(os.environ)
    env.pop("MSK_COL_TILE", None)
    if variant is not None:
        env["MSK_COL_TILE"] = str(variant)
    path = str(tmp_path / ("variant_%s.npz" % variant))
    r = subprocess.run([sys.executable, "-c", SCRIPT, path], check=True, env=env, timeout=900,
                       capture_output=True, text=True)
    return np.load(path), json.loads(r.stdout.strip().splitlines()[-1])


def test_column_schedules(tmp_path, oracle):
    from oracle.oracle import SeriesParams
    from utr_public_gb300 import specimen as sp
    res = {v: run(tmp_path, v) for v in (0, 1, 2, 3, None)}
    for k in res[0][0].files:
        assert np.array_equal(res[0][0][k].view(np.uint32), res[1][0][k].view(np.uint32)), k
        assert np.array_equal(res[2][0][k].view(np.uint32), res[3][0][k].view(np.uint32)), k
    # forced variants are reported as such; the tuned choice is one of them
    assert res[2][1]["1024"]["band_limit"]["points_per_thread"] == 16
    assert res[0][1]["1024"]["propagate"]["points_per_thread"] == 32
    for n in ("1024", "2048"):
        for p, info in res[None][1][n].items():
            if p in ("band_limit", "propagate", "free_space"):
                assert info is not None and info["variant"] in (0, 1, 2, 3), (n, p)

    def ref(job):
        n, fov, a = job
        spec = sp.random_specimen(400, fov, 0.2 * fov, 0.8 * fov, 1041)
        p = SeriesParams()
        p.ax, p.ctblengthz, p.nx, p.ny, p.v0, p.deltaz = fov, fov, n, n, 300.0, 2.0
        p.aobj, p.max_slices, p.min_slice = 0.02, -1, 0
        img, ew, _ = oracle.orientation(p, spec.Znum, spec.x, spec.y, spec.z, spec.occ,
                                        [0.0, 0.3][a], np.deg2rad(ANGLES[a]),
                                        np.array([0.0, 200.0]), fp64=True, want_exit=True)
        return job, img, ew

    jobs = [(n, fov, a) for n, fov in CASES for a in (0, 1)]
    with cf.ThreadPoolExecutor(8) as ex:
        refs = list(ex.map(ref, jobs))
    for (n, fov, a), img, ew in refs:
        for v in (0, 2, None):
            got = res[v][0]
            assert rel_l2(got["ew%d" % n][a, 0], ew) < 1e-5, (n, a, v)
            for d in range(2):
                assert rel_l2(got["img%d" % n][a, d], img[d]) < 1e-5, (n, a, v, d)
