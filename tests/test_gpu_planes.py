"""Per-orientation detector planes (msk_tilt_series_planes) and runs from
MsctKirkland orientation files.  Every image must equal, bit for bit, the image
msk_tilt_series makes for that orientation with the same plane given as its
common plane: the same kernels run on the same waves; only the grouping of
planes into launches differs."""
import numpy as np
import pytest

from utr_public_gb300 import specimen as sp

pytestmark = pytest.mark.gpu


def series(msk, n=64, fov=48.0):
    s = msk.Series()
    s.nx = s.ny = n
    s.ctblength = s.ctblengthz = fov
    s.v0, s.deltaz, s.aobj, s.cs3 = 300.0, 1.0, 0.015, 1e6
    return s


def specimen():
    spec = sp.random_specimen(500, 48.0, 8.0, 40.0, 1031)
    return (spec.Znum, spec.x, spec.y, spec.z, spec.occ)


def single(ctx, msk, atoms, aZ, aY, plane, shift, nconfig=1, disp=None):
    """One orientation, one plane, through msk_tilt_series."""
    s = series(msk)
    s.astig, s.astig_angle = plane[2], plane[3]
    rot = np.array([plane[1]])
    s.rotation = rot.ctypes.data
    s.xshift, s.yshift = shift
    img, _ = ctx.tilt_series(s, *atoms, [aZ], [aY], [plane[0]], nconfig=nconfig,
                             displacements=disp)
    return img[0, 0]


def test_planes_per_orientation_equal_single_orientation_calls(ctx, msk):
    atoms = specimen()
    aZ = np.array([0.1, 0.0, 0.7])
    aY = np.deg2rad([10.0, 55.0, 130.0])
    planes = [
        [(0.0, 0.0, 0.0, 0.0), (200.0, 0.4, 30.0, 0.3)],
        [(80.0, 0.0, 0.0, 0.0)],
        [(0.0, 0.0, 0.0, 0.0), (-60.0, -1.2, 0.0, 0.0), (200.0, 0.4, 30.0, 0.3)],
    ]
    shifts = np.array([[0.0, 0.0], [1.1, -0.6], [0.0, 0.0]])
    imgs, _ = ctx.tilt_series_planes(series(msk), *atoms, aZ, aY, planes, shifts=shifts)
    k = 0
    for a in range(3):
        for q in planes[a]:
            ref = single(ctx, msk, atoms, aZ[a], aY[a], q, tuple(shifts[a]))
            assert np.array_equal(imgs[k], ref), (a, q)
            k += 1
    assert k == imgs.shape[0]


def test_common_planes_equal_tilt_series(ctx, msk):
    atoms = specimen()
    aZ, aY = np.zeros(4), np.deg2rad([0.0, 20.0, 40.0, 60.0])
    defoci = [0.0, 150.0]
    ref, _ = ctx.tilt_series(series(msk), *atoms, aZ, aY, defoci)
    planes = [[(d, 0.0, 0.0, 0.0) for d in defoci]] * 4
    imgs, _ = ctx.tilt_series_planes(series(msk), *atoms, aZ, aY, planes)
    assert np.array_equal(imgs.reshape(ref.shape), ref)


def test_frozen_phonon_with_planes(ctx, msk):
    spec = sp.random_specimen(300, 48.0, 8.0, 40.0, 1032)
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    disp = sp.phonon_displacements(spec, 3, 0.08, 1032)
    aZ, aY = np.zeros(2), np.deg2rad([15.0, 75.0])
    planes = [[(0.0, 0.0, 0.0, 0.0)], [(120.0, 0.2, 10.0, 0.5), (0.0, 0.0, 0.0, 0.0)]]
    s = series(msk)
    s.max_batch = 2  # configurations of one orientation split over batches
    imgs, _ = ctx.tilt_series_planes(s, *atoms, aZ, aY, planes, nconfig=3, displacements=disp)
    k = 0
    for a in range(2):
        for q in planes[a]:
            ref = single(ctx, msk, atoms, aZ[a], aY[a], q, (0.0, 0.0), nconfig=3, disp=disp)
            assert np.allclose(imgs[k], ref, rtol=1e-6, atol=1e-7), (a, q)
            k += 1


def test_run_from_orientation_file(ctx, msk, tmp_path):
    atoms = specimen()
    p = tmp_path / "orient.txt"
    p.write_text("// Z Y' Z''1 defocus1 Z''2 defocus2\n"
                 "10 30 0 0 25 150\n"
                 "-20 100 5 60\n")
    imgs, _ = ctx.tilt_series_from_file(series(msk), *atoms, p)
    rad = np.pi / 180
    assert imgs.shape[0] == 3
    ref = single(ctx, msk, atoms, 10 * rad, 30 * rad, (150.0, 25 * rad, 0.0, 0.0), (0.0, 0.0))
    assert np.array_equal(imgs[1], ref)
    ref = single(ctx, msk, atoms, -20 * rad, 100 * rad, (60.0, 5 * rad, 0.0, 0.0), (0.0, 0.0))
    assert np.array_equal(imgs[2], ref)


def test_plane_list_errors(ctx, msk):
    atoms = specimen()
    s = series(msk)
    import ctypes as C
    off = np.array([0, 2, 1], np.int32)  # decreasing
    arr = (msk.Plane * 2)()
    st = ctx.L.msk_tilt_series_planes(ctx.h, C.byref(s), len(atoms[1]),
                                      *[a.ctypes.data for a in (np.ascontiguousarray(atoms[0], np.int32),) +
                                        tuple(np.ascontiguousarray(v, np.float32) for v in atoms[1:])],
                                      2, np.zeros(2), np.zeros(2), off.ctypes.data,
                                      C.addressof(arr), None, 1, None,
                                      np.zeros((2, 64, 64), np.float32).ctypes.data, None, None)
    assert st == msk.MSK_EINVAL


def test_run_from_reference_orientation_file(ctx, msk, oracle):
    """A tilt series driven by the orientation file the reference ships beside
    MsctKirkland (tests/golden/DefocusRand108_2_NEW2.txt: 108 random Z / Y'
    orientations, two detector planes each with their own Z'' rotation and
    defocus), read by msk_read_orientations in place of MultisliceT.cpp:264-277
    and run by msk_tilt_series_planes at 128^2 (MsctKirkland.txt's 200 keV and
    1.25 A slices): all 216 images against the FP64 oracle within 1e-5, kept
    atom counts equal.  The oracle's orientations run on host threads."""
    import concurrent.futures as cf
    import os
    from conftest import GOLDEN, rel_l2
    from oracle.oracle import SeriesParams
    path = os.path.join(GOLDEN, "DefocusRand108_2_NEW2.txt")
    spec = sp.random_specimen(300, 48.0, 8.0, 40.0, 1108)
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    s = msk.Series()
    s.nx = s.ny = 128
    s.ctblength = s.ctblengthz = 48.0
    s.v0, s.deltaz = 200.0, 1.25
    imgs, kept = ctx.tilt_series_from_file(s, *atoms, path)
    angles, planes, _ = msk.read_orientations(path)
    assert imgs.shape == (216, 128, 128)
    p = SeriesParams()
    p.ax, p.ctblengthz, p.nx, p.ny, p.v0, p.deltaz = 48.0, 48.0, 128, 128, 200.0, 1.25
    p.max_slices, p.min_slice = -1, 0
    lam, rad = oracle.wavelength(200.0), np.pi / 180.0

    def ref(a):
        _, ew64, k = oracle.orientation(p, *atoms, angles[a, 0] * rad, angles[a, 1] * rad,
                                        np.zeros(0), fp64=True, want_exit=True)
        return k, [oracle.image_plane(ew64, 48.0, lam, q[1] - 24.0, q[0] * rad, 24.0, 24.0, 0, 0)
                   for q in planes[a]]

    with cf.ThreadPoolExecutor(8) as ex:
        refs = list(ex.map(ref, range(108)))
    worst = 0.0
    for a, (k, r) in enumerate(refs):
        assert kept[a] == k, a
        for j in range(2):
            worst = max(worst, rel_l2(imgs[2 * a + j], r[j]))
    assert worst < 1e-5, worst


def test_file_run_to_page_locked_images(ctx, msk):
    """The shipped orientation file (108 orientations, two planes each, Z''
    rotations and shifts) into page-locked host images: each batch's planes
    staged on the device and written out beside the next batch (batches of 8,
    92 and 8 orientations), equal bit for bit to device images."""
    import os
    from conftest import GOLDEN
    torch = pytest.importorskip("torch")
    path = os.path.join(GOLDEN, "DefocusRand108_2_NEW2.txt")
    spec = sp.random_specimen(300, 48.0, 8.0, 40.0, 1109)
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    s = msk.Series()
    s.nx = s.ny = 64
    s.ctblength = s.ctblengthz = 48.0
    s.v0, s.deltaz = 200.0, 1.25
    dev = torch.zeros((216, 64, 64), dtype=torch.float32, device="cuda")
    ctx.tilt_series_from_file(s, *atoms, path, images=dev)
    pin = torch.full((216, 64, 64), -1.0, dtype=torch.float32).pin_memory()
    ctx.tilt_series_from_file(s, *atoms, path, images=pin)
    torch.cuda.synchronize()
    assert torch.equal(pin, dev.cpu())
