"""MsctKirkland's file formats (no GPU): the GRD and GRC layouts of
ReadmeMsctKirkland.txt and a baseline 32-bit float TIFF, parsed back byte by
byte, and the two orientation-file formats (.txt, .relionnew)."""
import struct

import numpy as np
import pytest


def image(nx=24, ny=16, seed=0):
    return np.random.default_rng(seed).standard_normal((nx, ny)).astype(np.float32)


def test_grd_layout(msk, tmp_path):
    img = image()
    p = tmp_path / "a.grd"
    msk.write_grd(p, img, 0.0, 12.0, -1.0, 7.0)
    b = p.read_bytes()
    assert b[:4] == b"DSBB"
    nx, ny = struct.unpack_from("<hh", b, 4)
    assert (nx, ny) == img.shape
    xlo, xhi, ylo, yhi, zlo, zhi = struct.unpack_from("<6d", b, 8)
    assert (xlo, xhi, ylo, yhi) == (0.0, 12.0, -1.0, 7.0)
    assert zlo == float(img.min()) and zhi == float(img.max())
    vals = np.frombuffer(b, "<f4", offset=56)
    # rows along y, x fastest: the [ny][nx] transpose of the [nx][ny] image
    assert np.array_equal(vals.reshape(ny, nx), img.T)


def test_grc_layout(msk, tmp_path):
    amp = np.stack([image(seed=1), image(seed=2)], axis=-1)
    p = tmp_path / "a.grc"
    msk.write_grc(p, amp, 0.0197, 0.0, 12.0, 0.0, 8.0)
    b = p.read_bytes()
    assert struct.unpack_from("<h", b, 0)[0] == -5
    assert struct.unpack_from("<d", b, 2)[0] == 0.0197
    assert struct.unpack_from("<hh", b, 10) == amp.shape[:2]
    assert struct.unpack_from("<4d", b, 14) == (0.0, 12.0, 0.0, 8.0)
    vals = np.frombuffer(b, "<f4", offset=46).reshape(amp.shape[1], amp.shape[0], 2)
    assert np.array_equal(vals, amp.transpose(1, 0, 2))


def read_tiff(b):
    """A baseline little-endian TIFF with one strip: (tags, pixel bytes)."""
    assert b[:4] == b"II*\x00"
    ifd = struct.unpack_from("<I", b, 4)[0]
    n = struct.unpack_from("<H", b, ifd)[0]
    tags = {}
    for k in range(n):
        tag, typ, cnt = struct.unpack_from("<HHI", b, ifd + 2 + 12 * k)
        off = ifd + 2 + 12 * k + 8
        tags[tag] = struct.unpack_from("<H" if typ == 3 else "<I", b, off)[0]
    start, size = tags[273], tags[279]
    return tags, b[start:start + size]


def test_tiff32_layout(msk, tmp_path):
    img = image(20, 12, 3)
    p = tmp_path / "a.tif"
    msk.write_tiff32(p, img)
    tags, pix = read_tiff(p.read_bytes())
    assert tags[256] == 20 and tags[257] == 12           # width = nx, height = ny
    assert tags[258] == 32 and tags[339] == 3 and tags[259] == 1
    assert np.array_equal(np.frombuffer(pix, "<f4").reshape(12, 20), img.T)


def test_orientations_txt(msk, tmp_path):
    p = tmp_path / "angles.txt"
    p.write_text("//Z Y' Z''1 defocus1 Z''2 defocus2\n"
                 "// a comment line\n"
                 "10.5 20.25 30 100.5 40 -50\n"
                 "\n"
                 "1 2 3 4\n")
    angles, planes, shifts = msk.read_orientations(p)
    assert np.array_equal(angles, [[10.5, 20.25], [1.0, 2.0]])
    assert np.array_equal(planes[0][:, :2], [[30.0, 100.5], [40.0, -50.0]])
    assert np.array_equal(planes[1][:, :2], [[3.0, 4.0]])
    assert not shifts.any() and not planes[0][:, 2:].any()


def test_orientations_relion(msk, tmp_path):
    p = tmp_path / "angles.relionnew"
    p.write_text("0 img0001.mrcs 1.5 -2.5 1000 800 30 10 20 -40\n"
                 "1 img0002.mrcs 0 0 500 500 -12 -5 90 180\n")
    angles, planes, shifts = msk.read_orientations(p)
    # every number but the astigmatism angle changes sign
    assert np.array_equal(angles, [[-10.0, -20.0], [5.0, -90.0]])
    assert np.array_equal(shifts, [[-1.5, 2.5], [0.0, 0.0]])
    assert np.array_equal(planes[0], [[40.0, -900.0, -100.0, 30.0, 0.0]])
    assert np.array_equal(planes[1], [[-180.0, -500.0, 0.0, -12.0, 0.0]])


def test_orientations_errors(msk, tmp_path):
    bad = tmp_path / "angles.txt"
    bad.write_text("1 2 3\n")  # an unpaired plane entry
    with pytest.raises(msk.MskError):
        msk.read_orientations(bad)
    other = tmp_path / "angles.csv"
    other.write_text("1 2\n")
    with pytest.raises(msk.MskError):
        msk.read_orientations(other)


SHIPPED = "DefocusRand108_2_NEW2.txt"


def shipped_numpy():
    """The reference's shipped orientation file parsed by numpy: two '//'
    header lines, then 108 lines of six tab-separated numbers (Z, Y', then the
    Z'' rotation and defocus of each of two detector planes)."""
    import os
    from conftest import GOLDEN
    return np.loadtxt(os.path.join(GOLDEN, SHIPPED), comments="//", delimiter="\t")


def test_reads_the_reference_orientation_file(msk):
    """msk_read_orientations on the file the reference ships beside MsctKirkland
    (MultisliceCppTest/MsctKirkland/DefocusRand108_2_NEW2.txt; its readers,
    MultisliceT.cpp:264-277): every angle and plane equal to numpy's parse."""
    import os
    from conftest import GOLDEN
    want = shipped_numpy()
    assert want.shape == (108, 6)
    angles, planes, shifts = msk.read_orientations(os.path.join(GOLDEN, SHIPPED))
    assert angles.shape == (108, 2) and np.array_equal(angles, want[:, :2])
    assert len(planes) == 108 and all(p.shape == (2, 5) for p in planes)
    pl = np.stack(planes)
    assert np.array_equal(pl[:, :, 0], want[:, [2, 4]])   # Z'' rotations
    assert np.array_equal(pl[:, :, 1], want[:, [3, 5]])   # defoci
    assert not pl[:, :, 2:].any() and not shifts.any()     # no astigmatism, no shifts
