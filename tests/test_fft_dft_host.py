"""The in-register DFT blocks of the line FFT (fft_line.cuh: radix 2..32, the
FMA tangent-form butterflies) compiled for the host and checked against a
double-precision DFT in numpy, in the cfpix sign convention (forward
exp(+2 pi i jk/R), inverse exp(-2 pi i jk/R), both unnormalised).  No GPU."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

RADICES = (2, 4, 8, 16, 32)


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="needs nvcc")
def test_register_dft_matches_double_dft(tmp_path):
    from utr_public_gb300 import _build
    exe = str(tmp_path / "fft_dft_host")
    subprocess.run([_build.nvcc()] + _build.ARCH + ["-O3", "-std=c++17",
                    "-I" + os.path.join(ROOT, "utr_public_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "fft_dft_host.cu"), "-o", exe], check=True)
    reps = 200
    rng = np.random.default_rng(11)
    blocks = []
    for _ in range(reps):
        for r in RADICES:
            for inv in (0, 1):
                blocks.append((r, inv, (rng.standard_normal(r) + 1j * rng.standard_normal(r))
                               .astype(np.complex64)))
    x = np.concatenate([b[2] for b in blocks])
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    x.tofile(inp)
    subprocess.run([exe, str(inp), str(out), str(reps)], check=True)
    y = np.fromfile(out, np.complex64)
    o = 0
    worst = {}
    for r, inv, v in blocks:
        j = np.arange(r)
        sign = -1.0 if inv else 1.0
        mat = np.exp(sign * 2j * np.pi * np.outer(j, j) / r)
        want = mat @ v.astype(np.complex128)
        got = y[o:o + r].astype(np.complex128)
        o += r
        e = np.linalg.norm(got - want) / np.linalg.norm(want)
        worst[r] = max(worst.get(r, 0.0), e)
    # FP32: a few units in the last place, growing like log2(R)
    for r in RADICES:
        assert worst[r] < 2.0e-7 * np.log2(r) + 1e-7, (r, worst[r])
