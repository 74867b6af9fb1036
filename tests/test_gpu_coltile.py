"""The column passes' two tile widths (chosen per grid and pass by timing at
run time) compute every column identically: a tilt series run with either
width forced (MSK_COL_TILE, read once per process) gives the same images and
exit waves bit for bit, and so does the tuned choice."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, %r)
import utr_public_gb300 as msk
from utr_public_gb300 import specimen as sp
ctx = msk.Context(0)
out = {}
for n, fov in ((64, 32.0), (256, 64.0), (2048, 96.0)):
    spec = sp.random_specimen(400, fov, 0.2 * fov, 0.8 * fov, 1041)
    s = msk.Series()
    s.nx = s.ny = n
    s.ctblength = s.ctblengthz = fov
    s.v0, s.deltaz, s.aobj = 300.0, 2.0, 0.02
    imgs, ew, _ = ctx.tilt_series(s, spec.Znum, spec.x, spec.y, spec.z, spec.occ, [0.0, 0.3],
                                  np.deg2rad([10.0, 50.0]), [0.0, 200.0], want_exit=True)
    out["img%%d" %% n], out["ew%%d" %% n] = imgs, ew
np.savez(sys.argv[1], **out)
""" % ROOT


def run(tmp_path, tile):
    env = dict(os.environ)
    env.pop("MSK_COL_TILE", None)
    if tile is not None:
        env["MSK_COL_TILE"] = str(tile)
    path = str(tmp_path / ("tile_%s.npz" % tile))
    subprocess.run([sys.executable, "-c", SCRIPT, path], check=True, env=env, timeout=600)
    return np.load(path)


def test_column_tiles_give_identical_results(tmp_path):
    a, b, tuned = run(tmp_path, 0), run(tmp_path, 1), run(tmp_path, None)
    for k in a.files:
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k
        assert np.array_equal(a[k].view(np.uint32), tuned[k].view(np.uint32)), k
