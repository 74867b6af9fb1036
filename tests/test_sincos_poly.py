"""exp(i x) of the transmission function (sincos_poly.cuh: Cody-Waite
reduction by pi/2, Taylor polynomials on |r| <= pi/4) compiled for the host,
against double precision: over the phases the splat meets (|x| of a few
radians, dense near 0) and out to the range limit, within a few units in the
last place of 1.  No GPU."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="needs nvcc")
def test_expi_poly_against_double(tmp_path):
    from utr_public_gb300 import _build
    exe = str(tmp_path / "sincos_poly_host")
    subprocess.run([_build.nvcc()] + _build.ARCH + ["-O3", "-std=c++17",
                    "-I" + os.path.join(ROOT, "utr_public_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "sincos_poly_host.cu"), "-o", exe], check=True)
    rng = np.random.default_rng(7)
    x = np.concatenate([rng.uniform(-4.0, 4.0, 200000), rng.uniform(-1e-3, 1e-3, 20000),
                        rng.uniform(-4096.0, 4096.0, 50000),
                        np.array([0.0, -0.0, np.pi / 4, np.pi / 2, np.pi, 3 * np.pi / 2])]
                       ).astype(np.float32)
    inp, out = tmp_path / "x.bin", tmp_path / "y.bin"
    x.tofile(inp)
    subprocess.run([exe, str(inp), str(out)], check=True)
    y = np.fromfile(out, np.float32).reshape(-1, 2).astype(np.float64)
    xd = x.astype(np.float64)
    err = np.hypot(y[:, 0] - np.cos(xd), y[:, 1] - np.sin(xd))
    small = np.abs(xd) <= 8.0
    assert err[small].max() < 2.5e-7, err[small].max()     # ~2 ulp of 1
    assert err.max() < 1.0e-6, err.max()                  # reduction error grows with |k|
    assert y[np.where(x == 0.0)[0][0]].tolist() == [1.0, 0.0]  # exp(i 0) = 1 exactly
