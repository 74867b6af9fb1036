"""The C++ drop-in for the reference's autoslic class compiles against the
reference's own headers and links against libmsk.so (where the reference tree
is present; it is not shipped with this repository)."""
import os
import subprocess

import pytest

from conftest import ROOT

REF = "/root/reference"


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "TemsimLibrary")),
                    reason="reference tree not present")
def test_dropin_builds_against_reference_headers(msk, tmp_path):
    src = os.path.join(ROOT, "utr_public_gb300", "dropin", "autoslic_msk.cpp")
    obj = str(tmp_path / "autoslic_msk.o")
    inc = ["-I" + os.path.join(REF, "TemsimLibrary"), "-I" + os.path.join(REF, "fftwlib"),
           "-I" + os.path.join(ROOT, "include")]
    subprocess.run(["g++", "-std=gnu++17", "-fPIC", "-Wall", "-c", src, "-o", obj] + inc,
                   check=True)
    # with the reference's own cfpix / slicelib objects (built by the oracle's
    # recipe) and the FFTW-API shim, nothing may stay unresolved
    from oracle import oracle as orc
    orc.build(with_ref=True)
    ref = os.path.join(ROOT, "oracle", "_ref")
    so = str(tmp_path / "libautoslic_msk.so")
    objs = [os.path.join(ref, f) for f in ("cfpix.o", "slicelib.o", "fftw_shim.o", "fft_cpu.o")]
    subprocess.run(["g++", "-shared", "-o", so, obj] + objs + [msk.LIB_PATH, "-Wl,--no-undefined",
                    "-lpthread"], check=True)
    syms = subprocess.run(["nm", "-DC", so], capture_output=True, text=True).stdout
    assert "autoslic::calculate(" in syms
    assert "msk_calculate" in syms
