"""The transmit's schedules (chosen per grid by timing at run time: the row
FFT plan, 32 or 16 points a thread, and the CTA width).  A tilt series run
with each schedule forced (MSK_ROW_PLAN) in its own process and with the
tuner's choice: every one matches the FP64 oracle within 1e-5, the two CTA
widths of the 32-point plan compute every row identically (bit for bit), the
two plans agree to FP32 rounding, and the tuner reports the schedule it ran
(msk_row_plan).
Grids of 512^2 and up (and a 256 x 1024 grid: 1024-point rows) run the
launch-per-pass slice loop, so every slice takes the transmit."""
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
CASES = ((512, 512, 64.0), (1024, 1024, 96.0), (2048, 2048, 96.0), (256, 1024, 64.0))
ANGLES = (10.0, 50.0)

SCRIPT = r"""
import sys, json, numpy as np
sys.path.insert(0, %r)
import utr_public_gb300 as msk
from utr_public_gb300 import specimen as sp
ctx = msk.Context(0)
out, plans = {}, {}
for nx, ny, fov in %r:
    spec = sp.random_specimen(400, fov, 0.2 * fov, 0.8 * fov, 1042)
    s = msk.Series()
    s.nx, s.ny = nx, ny
    s.ctblength = s.ctblengthz = fov
    s.v0, s.deltaz, s.aobj = 300.0, 2.0, 0.02
    imgs, ew, _ = ctx.tilt_series(s, spec.Znum, spec.x, spec.y, spec.z, spec.occ, [0.0, 0.3],
                                  np.deg2rad(%r), [0.0, 200.0], want_exit=True)
    k = "%%d_%%d" %% (nx, ny)
    out["img" + k], out["ew" + k] = imgs, ew
    plans[k] = msk.row_plan(0, nx, ny)
np.savez(sys.argv[1], **out)
print(json.dumps(plans))
""" % (ROOT, CASES, list(ANGLES))


def run(tmp_path, variant):
    env = dict(os.environ)
    env.pop("MSK_ROW_PLAN", None)
    if variant is not None:
        env["MSK_ROW_PLAN"] = str(variant)
    path = str(tmp_path / ("rowplan_%s.npz" % variant))
    r = subprocess.run([sys.executable, "-c", SCRIPT, path], check=True, env=env, timeout=900,
                       capture_output=True, text=True)
    return np.load(path), json.loads(r.stdout.strip().splitlines()[-1])


def test_transmit_schedules(tmp_path, oracle):
    from oracle.oracle import SeriesParams
    from utr_public_gb300 import specimen as sp
    res = {v: run(tmp_path, v) for v in (0, 1, 2, None)}
    for k in res[0][0].files:
        assert np.array_equal(res[0][0][k].view(np.uint32), res[1][0][k].view(np.uint32)), k
    for nx, ny, _ in CASES:
        k = "%d_%d" % (nx, ny)
        assert res[0][1][k] == {"variant": 0, "points_per_thread": 32,
                                "rows_per_cta": max(1, 64 // (ny // 32))}, k
        assert res[1][1][k] == {"variant": 1, "points_per_thread": 32,
                                "rows_per_cta": max(1, 128 // (ny // 32))}, k
        assert res[2][1][k]["variant"] == 2 and res[2][1][k]["points_per_thread"] == 16, k
        assert res[None][1][k]["variant"] in (0, 1, 2), k
        # another radix split of the same transforms: FP32 rounding apart
        assert rel_l2(res[2][0]["ew" + k], res[0][0]["ew" + k]) < 5e-6, k

    def ref(job):
        nx, ny, fov, a = job
        spec = sp.random_specimen(400, fov, 0.2 * fov, 0.8 * fov, 1042)
        p = SeriesParams()
        p.ax, p.ctblengthz, p.nx, p.ny, p.v0, p.deltaz = fov, fov, nx, ny, 300.0, 2.0
        p.aobj, p.max_slices, p.min_slice = 0.02, -1, 0
        img, ew, _ = oracle.orientation(p, spec.Znum, spec.x, spec.y, spec.z, spec.occ,
                                        [0.0, 0.3][a], np.deg2rad(ANGLES[a]),
                                        np.array([0.0, 200.0]), fp64=True, want_exit=True)
        return job, img, ew

    jobs = [(nx, ny, fov, a) for nx, ny, fov in CASES for a in (0, 1)]
    with cf.ThreadPoolExecutor(8) as ex:
        refs = list(ex.map(ref, jobs))
    for (nx, ny, fov, a), img, ew in refs:
        k = "%d_%d" % (nx, ny)
        for v in (0, 2, None):
            got = res[v][0]
            assert rel_l2(got["ew" + k][a, 0], ew) < 1e-5, (k, a, v)
            for d in range(2):
                assert rel_l2(got["img" + k][a, d], img[d]) < 1e-5, (k, a, v, d)
