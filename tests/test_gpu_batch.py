"""msk_tilt_series_batch: specimens of different atom counts, boxes, grids and
orientation counts in one call (concurrent streams, optionally one CUDA
graph).  Each specimen's images must equal msk_tilt_series on that specimen
alone, bit for bit: the same kernels run on the same data, only the order of
independent launches differs."""
import numpy as np
import pytest

from utr_public_gb300 import specimen as sp

pytestmark = pytest.mark.gpu


def series(msk, aobj=0.0, cs3=0.0):
    s = msk.Series()
    s.v0, s.deltaz, s.aobj, s.cs3 = 300.0, 1.0, aobj, cs3
    return s


def batch_case():
    out = []
    for i, (natom, fov, n, nang) in enumerate([(400, 32.0, 64, 3), (600, 48.0, 128, 1),
                                               (300, 40.0, 64, 2), (900, 64.0, 256, 5),
                                               (0, 32.0, 32, 2)]):
        edge = fov / np.sqrt(2.0)
        lo = 0.5 * (fov - edge)
        spec = sp.random_specimen(natom, fov, lo, lo + edge, 2000 + i)
        aY = np.deg2rad(np.linspace(0.0, 170.0, nang))
        aZ = np.full(nang, 0.05 * i)
        out.append((spec, n, aZ, aY))
    return out


@pytest.mark.parametrize("graph", [True, False])
def test_batch_equals_single_specimen_calls(ctx, msk, graph):
    cases = batch_case()
    defoci = [0.0, 300.0]
    s = series(msk, aobj=0.015, cs3=1e6)
    imgs, kept = ctx.tilt_series_batch(s, cases, defoci, graph=graph)
    for (spec, n, aZ, aY), im, k in zip(cases, imgs, kept):
        s1 = series(msk, aobj=0.015, cs3=1e6)
        s1.nx = s1.ny = n
        s1.ctblength = s1.ctblengthz = spec.fov
        ref, k1 = ctx.tilt_series(s1, spec.Znum, spec.x, spec.y, spec.z, spec.occ, aZ, aY,
                                  defoci)
        assert np.array_equal(k, k1)
        assert np.array_equal(im, ref)


def test_batch_device_images_and_repeat(ctx, msk):
    torch = pytest.importorskip("torch")
    cases = batch_case()
    defoci = [50.0]
    s = series(msk)
    host, _ = ctx.tilt_series_batch(s, cases, defoci)
    dev = [torch.zeros((len(aZ), 1, n, n), dtype=torch.float32, device="cuda")
           for _, n, aZ, _ in cases]
    ctx.tilt_series_batch(s, cases, defoci, images=dev)
    for h, d in zip(host, dev):
        assert np.array_equal(h, d.cpu().numpy())
    again, _ = ctx.tilt_series_batch(s, cases, defoci)  # the arena is reused
    for h, a in zip(host, again):
        assert np.array_equal(h, a)


@pytest.mark.parametrize("graph", [True, False])
def test_batch_pinned_host_images(ctx, msk, graph):
    """Page-locked host images are copied on each specimen's lane (inside the
    graph when there is one); they equal the pageable and device results."""
    torch = pytest.importorskip("torch")
    cases = batch_case()
    defoci = [0.0, 120.0]
    s = series(msk, aobj=0.02)
    ref, _ = ctx.tilt_series_batch(s, cases, defoci, graph=graph)
    pinned = [torch.full((len(aZ), 2, n, n), -1.0, dtype=torch.float32).pin_memory()
              for _, n, aZ, _ in cases]
    for _ in range(2):  # a second call reuses the arena
        ctx.tilt_series_batch(s, cases, defoci, graph=graph, images=pinned)
        for r, h in zip(ref, pinned):
            assert np.array_equal(r, h.numpy())


@pytest.mark.parametrize("graph", [True, False])
def test_batch_spherical_wave_and_image_plane(ctx, msk, graph):
    """A spherical incident wave and a rotated, shifted image plane: each
    specimen's images equal msk_tilt_series on that specimen, bit for bit."""
    cases = batch_case()
    defoci = [0.0, 200.0]
    rot = np.array([0.0, 0.3])
    s = series(msk, aobj=0.02)
    s.R1 = 4000.0
    s.rotation = rot.ctypes.data
    s.xshift, s.yshift = 1.1, -0.6
    imgs, _ = ctx.tilt_series_batch(s, cases, defoci, graph=graph)
    for spec, n, aZ, aY in cases:
        s1 = series(msk, aobj=0.02)
        s1.R1 = 4000.0
        s1.rotation = rot.ctypes.data
        s1.xshift, s1.yshift = 1.1, -0.6
        s1.nx = s1.ny = n
        s1.ctblength = s1.ctblengthz = spec.fov
        ref, _ = ctx.tilt_series(s1, spec.Znum, spec.x, spec.y, spec.z, spec.occ, aZ, aY,
                                 defoci)
        im = imgs.pop(0)
        assert np.array_equal(im, ref)


def test_batch_debye_waller(ctx, msk):
    """lwobble = 1 (one configuration: the Debye-Waller branch) with each
    specimen's wobble: images equal msk_tilt_series on that specimen."""
    cases = batch_case()
    for i, (spec, _, _, _) in enumerate(cases):
        spec.wobble = (0.03 + 0.02 * ((np.arange(spec.natom) + i) % 5)).astype(np.float32)
    defoci = [0.0, 150.0]
    s = series(msk)
    s.lwobble, s.temperature = 1, 290.0
    imgs, _ = ctx.tilt_series_batch(s, cases, defoci)
    for (spec, n, aZ, aY), im in zip(cases, imgs):
        s1 = series(msk)
        s1.lwobble, s1.temperature = 1, 290.0
        s1.wobble = spec.wobble.ctypes.data
        s1.nx = s1.ny = n
        s1.ctblength = s1.ctblengthz = spec.fov
        ref, _ = ctx.tilt_series(s1, spec.Znum, spec.x, spec.y, spec.z, spec.occ, aZ, aY,
                                 defoci)
        assert np.array_equal(im, ref)


def test_batch_thermal_configurations(ctx, msk):
    """lwobble = 1 with three configurations per orientation (random
    displacements from seed - orientation, images averaged): each specimen
    equals msk_tilt_series with nconfig = 3, bit for bit."""
    cases = batch_case()
    for i, (spec, _, _, _) in enumerate(cases):
        spec.wobble = (0.04 + 0.02 * ((np.arange(spec.natom) + i) % 3)).astype(np.float32)
    defoci = [0.0, 150.0]
    s = series(msk)
    s.lwobble, s.temperature, s.seed = 1, 300.0, 4711
    imgs, kept = ctx.tilt_series_batch(s, cases, defoci, nconfig=3)
    for (spec, n, aZ, aY), im, k in zip(cases, imgs, kept):
        s1 = series(msk)
        s1.lwobble, s1.temperature, s1.seed = 1, 300.0, 4711
        s1.wobble = spec.wobble.ctypes.data
        s1.nx = s1.ny = n
        s1.ctblength = s1.ctblengthz = spec.fov
        ref, k1 = ctx.tilt_series(s1, spec.Znum, spec.x, spec.y, spec.z, spec.occ, aZ, aY,
                                  defoci, nconfig=3)
        assert np.array_equal(k, k1)
        assert np.array_equal(im, ref)


def test_batch_given_displacements(ctx, msk):
    """Two configurations per orientation from caller-given displacements:
    each specimen equals msk_tilt_series with the same displacements."""
    cases = batch_case()
    rng = np.random.default_rng(77)
    disp = [(0.05 * rng.standard_normal((2, 3, spec.natom))).astype(np.float32)
            for spec, _, _, _ in cases]
    defoci = [0.0, 150.0]
    s = series(msk, aobj=0.02)
    imgs, _ = ctx.tilt_series_batch(s, cases, defoci, nconfig=2, displacements=disp)
    for (spec, n, aZ, aY), im, dd in zip(cases, imgs, disp):
        s1 = series(msk, aobj=0.02)
        s1.nx = s1.ny = n
        s1.ctblength = s1.ctblengthz = spec.fov
        ref, _ = ctx.tilt_series(s1, spec.Znum, spec.x, spec.y, spec.z, spec.occ, aZ, aY,
                                 defoci, nconfig=2, displacements=dd)
        assert np.array_equal(im, ref)


@pytest.mark.parametrize("pinned", [False, True])
def test_batch_exit_waves(ctx, msk, pinned):
    """Exit waves out of the batch (pageable or page-locked host memory,
    graph capture): equal to msk_tilt_series's, bit for bit."""
    torch = pytest.importorskip("torch")
    cases = batch_case()
    defoci = [0.0]
    s = series(msk, aobj=0.02)
    ews = None
    if pinned:
        ews = [torch.zeros((len(aZ), 1, n, n, 2), dtype=torch.float32).pin_memory()
               for _, n, aZ, _ in cases]
    imgs, _, ew = ctx.tilt_series_batch(s, cases, defoci, exitwaves=ews, want_exit=True)
    for (spec, n, aZ, aY), e in zip(cases, ew):
        s1 = series(msk, aobj=0.02)
        s1.nx = s1.ny = n
        s1.ctblength = s1.ctblengthz = spec.fov
        _, ref, _ = ctx.tilt_series(s1, spec.Znum, spec.x, spec.y, spec.z, spec.occ, aZ, aY,
                                    defoci, want_exit=True)
        e = e.numpy() if pinned else e
        assert np.array_equal(e.reshape(ref.shape), ref)


@pytest.mark.parametrize("graph", [True, False])
def test_batch_features_together(ctx, msk, graph):
    """Spherical incident wave, three thermal configurations drawn in the engine,
    a rotated and shifted image plane and exit waves in one batch: each specimen
    equals msk_tilt_series on it, bit for bit."""
    cases = batch_case()
    for i, (spec, _, _, _) in enumerate(cases):
        spec.wobble = (0.03 + 0.01 * ((np.arange(spec.natom) + i) % 4)).astype(np.float32)
    defoci = [0.0, 220.0]
    rot = np.array([0.25, 0.0])

    def setup(s):
        s.R1 = 3500.0
        s.rotation = rot.ctypes.data
        s.xshift, s.yshift = -0.8, 0.5
        s.lwobble, s.temperature, s.seed = 1, 300.0, 99
        return s

    s = setup(series(msk, aobj=0.02, cs3=5e5))
    imgs, kept, ews = ctx.tilt_series_batch(s, cases, defoci, graph=graph, nconfig=3,
                                            want_exit=True)
    for (spec, n, aZ, aY), im, k, ew in zip(cases, imgs, kept, ews):
        s1 = setup(series(msk, aobj=0.02, cs3=5e5))
        s1.wobble = spec.wobble.ctypes.data
        s1.nx = s1.ny = n
        s1.ctblength = s1.ctblengthz = spec.fov
        ref, ref_ew, k1 = ctx.tilt_series(s1, spec.Znum, spec.x, spec.y, spec.z, spec.occ, aZ,
                                          aY, defoci, nconfig=3, want_exit=True)
        assert np.array_equal(k, k1)
        assert np.array_equal(im, ref)
        assert np.array_equal(ew.reshape(ref_ew.shape), ref_ew)


@pytest.mark.parametrize("graph", [True, False])
def test_batch_per_orientation_planes(ctx, msk, graph):
    """Specimens with their own detector planes per orientation (as orientation
    files give them: defocus, rotation, astigmatism and an image shift per
    orientation; a plane every orientation shares, planes only some have, an
    orientation without planes) beside a specimen on the call's common defoci:
    each equals msk_tilt_series_planes (msk_tilt_series) on it alone, bit for
    bit."""
    cases = batch_case()
    defoci = [0.0, 150.0]
    planes, shifts = [], []
    for i, (spec, n, aZ, aY) in enumerate(cases):
        if i == 1:
            planes.append(None)
            shifts.append(None)
            continue
        pa = []
        for a in range(len(aZ)):
            rows = [(0.0, 0.0, 0.0, 0.0)]
            if (a + i) % 3 != 2:
                rows.append((100.0 + 40.0 * (a % 2), 0.3 * (a % 2), 25.0 * (i % 2), 0.4))
            if a == 0:
                rows.append((-60.0, 0.0, 0.0, 0.0))
            pa.append(rows)
        if i == 2:
            pa[1] = []
        planes.append(pa)
        shifts.append(np.array([[0.7 * (a % 2), -0.4 * a] for a in range(len(aZ))]))
    s = series(msk, aobj=0.015, cs3=1e6)
    imgs, kept = ctx.tilt_series_batch(s, cases, defoci, graph=graph, planes=planes,
                                       shifts=shifts)
    for (spec, n, aZ, aY), pa, sh, im, k in zip(cases, planes, shifts, imgs, kept):
        s1 = series(msk, aobj=0.015, cs3=1e6)
        s1.nx = s1.ny = n
        s1.ctblength = s1.ctblengthz = spec.fov
        if pa is None:
            ref, k1 = ctx.tilt_series(s1, spec.Znum, spec.x, spec.y, spec.z, spec.occ, aZ, aY,
                                      defoci)
        else:
            ref, k1 = ctx.tilt_series_planes(s1, spec.Znum, spec.x, spec.y, spec.z, spec.occ,
                                             aZ, aY, pa, shifts=sh)
        assert np.array_equal(k, k1)
        assert im.shape == ref.shape
        assert np.array_equal(im, ref)


def test_batch_errors(ctx, msk):
    cases = batch_case()[:2]
    s = series(msk)
    bad = [(cases[0][0], 48, cases[0][2], cases[0][3])]
    with pytest.raises(msk.MskError) as e:
        ctx.tilt_series_batch(s, bad, [0.0])
    assert e.value.status == msk.MSK_EUNSUPPORTED
    sw = series(msk)
    sw.lwobble = 1  # the Debye-Waller branch needs each specimen's wobble
    for spec, _, _, _ in cases:
        spec.wobble = None
    with pytest.raises(msk.MskError) as e:
        ctx.tilt_series_batch(sw, cases, [0.0])
    assert e.value.status == msk.MSK_EINVAL
    # several configurations need displacements: drawn (lwobble) or given
    with pytest.raises(msk.MskError) as e:
        ctx.tilt_series_batch(s, cases, [0.0], nconfig=2)
    assert e.value.status == msk.MSK_EINVAL
    spec = sp.random_specimen(10, 32.0, 8.0, 24.0, 7)
    spec.Znum[3] = 104
    with pytest.raises(msk.MskError) as e:
        ctx.tilt_series_batch(s, [cases[1], (spec, 64, [0.0], [0.0])], [0.0])
    assert e.value.status == msk.MSK_EZNUM
    # a specimen's plane offsets must start at 0 and not decrease (checked on the host)
    good = msk._plane_arrays

    def bad_offsets(planes, na):
        off, arr, total = good(planes, na)
        off[1] = off[2] + 1
        return off, arr, total

    with pytest.MonkeyPatch.context() as mp:
        mp.setattr(msk, "_plane_arrays", bad_offsets)
        with pytest.raises(msk.MskError) as e:
            ctx.tilt_series_batch(s, cases[:1], [0.0], planes=[[[(0.0, 0, 0, 0)]] * 3])
    assert e.value.status == msk.MSK_EINVAL
    # the context stays usable
    imgs, _ = ctx.tilt_series_batch(s, cases, [0.0])
    assert all(np.isfinite(i).all() for i in imgs)
