"""The C++ drop-in for the reference's autoslic class
(utr_public_gb300/dropin/autoslic_msk.cpp, replacing TemsimLibrary/autoslic.cpp
behind autoslic.hpp:166-169).

* Built against interface stand-ins (tests/dropin_iface/: the cfpix layout,
  the autoslic declaration, the param[] offsets), it links against libmsk.so
  with nothing unresolved (CPU), and on the GPU two host threads -- one
  autoslic object each, as MsctKirkland's per-orientation workers hold them --
  call autoslic::calculate() at once: each exit wave matches the reference's
  own FP32 result (golden) within 2e-5 and the two are equal bit for bit.
* Where the reference tree is present (MSK_REFERENCE_TREE, or the tree the
  oracle's reference build recorded), the drop-in also compiles against the
  reference's own headers and links with the reference's cfpix / slicelib
  objects.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden, rel_l2

IFACE = os.path.join(ROOT, "tests", "dropin_iface")
DROPIN = os.path.join(ROOT, "utr_public_gb300", "dropin", "autoslic_msk.cpp")


def build_dropin(msk, out_dir):
    """libdropin.so: the drop-in, the stand-in cfpix and the threaded driver,
    linked against libmsk.so with every symbol resolved."""
    so = os.path.join(str(out_dir), "libdropin.so")
    cmd = ["g++", "-std=gnu++17", "-O2", "-fPIC", "-Wall", "-shared", "-o", so, DROPIN,
           os.path.join(IFACE, "dropin_driver.cpp"), "-I" + IFACE,
           "-I" + os.path.join(ROOT, "include"), msk.LIB_PATH,
           "-Wl,-rpath," + os.path.dirname(msk.LIB_PATH), "-Wl,--no-undefined", "-lpthread"]
    subprocess.run(cmd, check=True)
    return so


def test_dropin_builds_against_interface(msk, tmp_path):
    so = build_dropin(msk, tmp_path)
    syms = subprocess.run(["nm", "-DC", so], capture_output=True, text=True).stdout
    assert "autoslic::calculate(" in syms and "dropin_threads" in syms


@pytest.mark.gpu
def test_dropin_calculate_two_threads_on_gpu(msk, tmp_path):
    g = golden("ref_exit_c1_256.npz")
    from utr_public_gb300 import specimen as sp
    s = sp.plain_specimen(int(g["seed"]))
    n = int(g["natom"])
    fov, nx, ny = float(g["fov"]), int(g["nx"]), int(g["ny"])
    param = msk.make_param(fov, fov, nx, ny, float(g["v0"]), float(g["deltaz"]))
    L = C.CDLL(build_dropin(msk, tmp_path))
    fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
    ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
    L.dropin_threads.argtypes = [C.c_int, fp, C.c_int, ip, fp, fp, fp, fp, C.c_float, C.c_float,
                                 fp, C.c_char_p, C.c_int]
    out = np.zeros((2, nx, ny, 2), np.float32)
    err = C.create_string_buffer(512)
    a = [np.ascontiguousarray(v[:n], dt) for v, dt in
         ((s.Znum, np.int32), (s.x, np.float32), (s.y, np.float32), (s.z, np.float32),
          (s.occ, np.float32))]
    rc = L.dropin_threads(2, np.ascontiguousarray(param, np.float32), n, *a, fov, fov, out, err, 512)
    assert rc == 0, err.value.decode()
    for k in range(2):
        assert rel_l2(out[k], g["pix"]) < 2e-5
    assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32))


def test_dropin_builds_against_reference_headers(msk, tmp_path):
    from oracle import oracle as orc
    ref_tree = orc.reference_tree()
    if ref_tree is None:
        pytest.skip("reference tree not present")
    obj = str(tmp_path / "autoslic_msk.o")
    inc = ["-I" + os.path.join(ref_tree, "TemsimLibrary"), "-I" + os.path.join(ref_tree, "fftwlib"),
           "-I" + os.path.join(ROOT, "include")]
    subprocess.run(["g++", "-std=gnu++17", "-fPIC", "-Wall", "-c", DROPIN, "-o", obj] + inc,
                   check=True)
    # with the reference's own cfpix / slicelib objects (built by the oracle's
    # recipe) and the FFTW-API shim, nothing may stay unresolved
    orc.build(with_ref=True)
    ref = os.path.join(ROOT, "oracle", "_ref")
    so = str(tmp_path / "libautoslic_msk.so")
    objs = [os.path.join(ref, f) for f in ("cfpix.o", "slicelib.o", "fftw_shim.o", "fft_cpu.o")]
    subprocess.run(["g++", "-shared", "-o", so, obj] + objs + [msk.LIB_PATH, "-Wl,--no-undefined",
                    "-lpthread"], check=True)
    syms = subprocess.run(["nm", "-DC", so], capture_output=True, text=True).stdout
    assert "autoslic::calculate(" in syms
    assert "msk_calculate" in syms
