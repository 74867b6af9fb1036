"""Parity of the CUDA path (through the C ABI) with the reference and the
oracle.  Tolerances (relative L2 over the whole grid):
  * exit wave vs the reference's FP32 CPU result (golden):  2e-5
  * exit wave and images vs the FP64 oracle:                1e-5 at these sizes
    (the path's accuracy target is 1e-4)
Bit-exact where the arithmetic is exact (plane wave through an empty box).
"""
import numpy as np
import pytest

from conftest import golden, rel_l2
from utr_public_gb300 import specimen as sp

pytestmark = pytest.mark.gpu

EXIT_CASES = ["c1_128", "c1_256", "rect_64x128", "proj_64"]


def golden_case(name):
    g = golden("ref_exit_%s.npz" % name)
    s = sp.plain_specimen(int(g["seed"]))
    n = int(g["natom"])
    atoms = (s.Znum[:n], s.x[:n], s.y[:n], s.z[:n], s.occ[:n])
    return g, atoms


@pytest.mark.parametrize("name", EXIT_CASES)
def test_calculate_matches_reference_golden(ctx, msk, oracle, name):
    g, atoms = golden_case(name)
    fov, nx, ny = float(g["fov"]), int(g["nx"]), int(g["ny"])
    param = msk.make_param(fov, fov, nx, ny, float(g["v0"]), float(g["deltaz"]))
    pix = ctx.calculate(param, *atoms, fov, fov, nmode=int(g["nmode"]))
    assert rel_l2(pix, g["pix"]) < 2e-5
    ref64 = oracle.calculate(param, *atoms, fov, fov, nmode=int(g["nmode"]), fp64=True)
    assert rel_l2(pix, ref64) < 1e-5


@pytest.mark.parametrize("nx,ny,fov,dz", [(16, 16, 8.0, 2.0), (32, 32, 16.0, 2.0),
                                          (32, 64, 20.0, 1.0), (64, 32, 20.0, 1.0),
                                          (512, 512, 64.0, 2.0), (128, 2048, 64.0, 4.0),
                                          (2048, 64, 64.0, 4.0), (4096, 32, 64.0, 8.0),
                                          (32, 4096, 64.0, 8.0)])
def test_calculate_grid_sizes(ctx, msk, oracle, nx, ny, fov, dz):
    s = sp.random_specimen(120, fov, 0.1 * fov, 0.9 * fov, 4242 + nx + ny)
    atoms = (s.Znum, s.x, s.y, s.z, s.occ)
    param = msk.make_param(fov, fov, nx, ny, 300.0, dz)
    pix = ctx.calculate(param, *atoms, fov, fov)
    ref64 = oracle.calculate(param, *atoms, fov, fov, fp64=True)
    assert rel_l2(pix, ref64) < 1e-5


def test_calculate_with_tilt_and_incident_wave(ctx, msk, oracle):
    s = sp.random_specimen(200, 32.0, 4.0, 28.0, 99)
    atoms = (s.Znum, s.x, s.y, s.z, s.occ)
    param = msk.make_param(32.0, 32.0, 128, 128, 200.0, 1.0, ctiltx=0.004, ctilty=-0.003)
    rng = np.random.default_rng(5)
    ph = rng.uniform(0, 2 * np.pi, (128, 128))
    w0 = np.stack([np.cos(ph), np.sin(ph)], -1).astype(np.float32)
    pix = ctx.calculate(param, *atoms, 32.0, 32.0, wave0=w0)
    ref64 = oracle.calculate(param, *atoms, 32.0, 32.0, wave0=w0.astype(np.float64), fp64=True)
    assert rel_l2(pix, ref64) < 1e-5


@pytest.mark.parametrize("n", [64, 4096])
def test_empty_box_keeps_plane_wave_exactly(ctx, msk, n):
    """An empty box at the smallest test grid and at the largest grid in both
    dimensions: every transform of the plane wave is exact, so it stays 1."""
    param = msk.make_param(32.0, 32.0, n, n, 200.0, 8.0 if n > 1024 else 2.0)
    e = np.zeros(0, np.float32)
    pix = ctx.calculate(param, e.astype(np.int32), e, e, e, e, 32.0, 32.0)
    assert np.all(pix[..., 0] == 1.0) and np.all(pix[..., 1] == 0.0)


def test_deterministic(ctx, msk):
    g, atoms = golden_case("c1_256")
    param = msk.make_param(64.0, 64.0, 256, 256, 200.0, 2.0)
    a = ctx.calculate(param, *atoms, 64.0, 64.0)
    b = ctx.calculate(param, *atoms, 64.0, 64.0)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_error_statuses(ctx, msk):
    s = sp.random_specimen(50, 32.0, 4.0, 28.0, 3)
    atoms = [s.Znum, s.x, s.y, s.z, s.occ]
    param = msk.make_param(32.0, 32.0, 64, 64, 200.0, 2.0)
    bad = [a.copy() for a in atoms]
    bad[1][7] = 40.0
    with pytest.raises(msk.MskError) as e:
        ctx.calculate(param, *bad, 32.0, 32.0)
    assert e.value.status == msk.MSK_EBOX
    bad = [a.copy() for a in atoms]
    bad[0][3] = 104
    with pytest.raises(msk.MskError) as e:
        ctx.calculate(param, *bad, 32.0, 32.0)
    assert e.value.status == msk.MSK_EZNUM
    with pytest.raises(msk.MskError) as e:
        ctx.calculate(msk.make_param(32.0, 32.0, 100, 64, 200.0, 2.0), *atoms, 32.0, 32.0)
    assert e.value.status == msk.MSK_EUNSUPPORTED
    p2 = param.copy()
    p2[msk.pNWOBBLE] = 2  # random displacements need a seed
    with pytest.raises(msk.MskError) as e:
        ctx.calculate(p2, *atoms, 32.0, 32.0, lwobble=1)
    assert e.value.status == msk.MSK_EINVAL
    # the context stays usable after every failure
    pix = ctx.calculate(param, *atoms, 32.0, 32.0)
    assert np.isfinite(pix).all()


def series(msk, nx, fov, v0, dz, aobj=0.0, cs3=0.0, max_batch=0):
    s = msk.Series()
    s.nx = s.ny = nx
    s.ctblength = s.ctblengthz = fov
    s.v0, s.deltaz, s.aobj, s.cs3 = v0, dz, aobj, cs3
    s.max_batch = max_batch
    return s


def oracle_series(oracle, nx, fov, v0, dz, aobj=0.0, cs3=0.0):
    from oracle.oracle import SeriesParams
    p = SeriesParams()
    p.ax, p.ctblengthz, p.nx, p.ny, p.v0, p.deltaz = fov, fov, nx, nx, v0, dz
    p.aobj, p.cs3, p.max_slices = aobj, cs3, -1
    return p


@pytest.mark.parametrize("aobj,cs3", [(0.0, 0.0), (0.02, 1.2e7)])
def test_tilt_series_matches_oracle(ctx, msk, oracle, aobj, cs3):
    spec = sp.random_specimen(800, 64.0, 10.0, 54.0, 1010)
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    angY = np.deg2rad([0.0, 30.0, 45.0, 90.0, 137.0])
    angZ = np.array([0.0, 0.0, 0.3, 0.0, 1.1])
    defoci = np.array([0.0, 500.0, -120.0])
    imgs, ew, kept = ctx.tilt_series(series(msk, 128, 64.0, 300.0, 1.0, aobj, cs3), *atoms, angZ,
                                     angY, defoci, want_exit=True)
    sp64 = oracle_series(oracle, 128, 64.0, 300.0, 1.0, aobj, cs3)
    for a in range(len(angY)):
        ref, ref_ew, k = oracle.orientation(sp64, *atoms, angZ[a], angY[a], defoci, fp64=True,
                                            want_exit=True)
        assert kept[a] == k
        assert rel_l2(ew[a, 0], ref_ew) < 1e-5
        for d in range(len(defoci)):
            assert rel_l2(imgs[a, d], ref[d]) < 1e-5, (a, d)


def test_tilt_series_angle_zero_equals_calculate(ctx, msk):
    spec = sp.random_specimen(600, 64.0, 10.0, 54.0, 1011)
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    _, ew, _ = ctx.tilt_series(series(msk, 128, 64.0, 200.0, 2.0), *atoms, [0.0], [0.0], [0.0],
                               want_exit=True)
    x, y, z = msk.rotate(64.0, 0.0, 0.0, spec.x, spec.y, spec.z)
    param = msk.make_param(64.0, 64.0, 128, 128, 200.0, 2.0)
    pix = ctx.calculate(param, spec.Znum, x, y, z, spec.occ, 64.0, 64.0)
    assert np.array_equal(ew[0, 0].view(np.uint32), pix.view(np.uint32))


@pytest.mark.parametrize("max_batch", [0, 3, 4])
def test_frozen_phonon_average(ctx, msk, oracle, max_batch):
    spec = sp.random_specimen(400, 64.0, 10.0, 54.0, 1003)
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    nconf = 4
    disp = sp.phonon_displacements(spec, nconf, 0.08, 1003)
    angY = np.deg2rad([0.0, 40.0, 95.0])
    angZ = np.zeros(3)
    defoci = np.array([0.0, 300.0])
    imgs, kept = ctx.tilt_series(series(msk, 64, 64.0, 200.0, 1.0, max_batch=max_batch), *atoms,
                                 angZ, angY, defoci, nconfig=nconf, displacements=disp)
    sp64 = oracle_series(oracle, 64, 64.0, 200.0, 1.0)
    for a in range(3):
        acc = np.zeros((len(defoci), 64, 64))
        for c in range(nconf):
            ref, _ = oracle.orientation(sp64, *atoms, angZ[a], angY[a], defoci, fp64=True,
                                        disp=disp[c])
            acc += ref
        acc /= nconf
        for d in range(len(defoci)):
            assert rel_l2(imgs[a, d], acc[d]) < 1e-5


def test_tilt_series_device_output(ctx, msk):
    torch = pytest.importorskip("torch")
    spec = sp.random_specimen(300, 64.0, 10.0, 54.0, 1012)
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    s = series(msk, 64, 64.0, 200.0, 2.0)
    host, _ = ctx.tilt_series(s, *atoms, [0.0, 0.5], [0.2, 1.0], [0.0, 100.0])
    dev = torch.zeros((2, 2, 64, 64), dtype=torch.float32, device="cuda")
    ctx.tilt_series(s, *atoms, [0.0, 0.5], [0.2, 1.0], [0.0, 100.0], images=dev)
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy(), host)


def test_full_grid_thin_slab(ctx, msk, oracle):
    """The tilt-series grid (1024^2 over 160 A, 300 keV, 1 A slices) on a
    thin slab that the FP64 oracle finishes in seconds."""
    spec = sp.random_specimen(400, 160.0, 20.0, 140.0, 1013)
    spec.z[:] = np.float32(2.0) + (spec.z - 20.0) * np.float32(4.0 / 120.0)
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    param = msk.make_param(160.0, 160.0, 1024, 1024, 300.0, 1.0)
    pix = ctx.calculate(param, *atoms, 160.0, 8.0)
    ref64 = oracle.calculate(param, *atoms, 160.0, 8.0, fp64=True)
    assert rel_l2(pix, ref64) < 1e-5


@pytest.mark.parametrize("n,fov", [(2048, 200.0), (4096, 256.0)])
def test_large_grid_thin_slab(ctx, msk, oracle, n, fov):
    """The uneven batch's largest grid (2048^2) and the largest supported grid
    (4096^2), both with atoms, on a slab of five 1 A slices that the FP64 oracle
    finishes in seconds: every line length of the row and column passes at
    full width in both dimensions."""
    spec = sp.random_specimen(600, fov, 0.1 * fov, 0.9 * fov, 777 + n)
    spec.z[:] = np.float32(1.0) + (spec.z - np.float32(0.1 * fov)) * np.float32(3.0 / (0.8 * fov))
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    param = msk.make_param(fov, fov, n, n, 300.0, 1.0)
    pix = ctx.calculate(param, *atoms, fov, 5.0)
    ref64 = oracle.calculate(param, *atoms, fov, 5.0, fp64=True)
    assert rel_l2(pix, ref64) < 1e-5


def test_per_angle_form_matches_batched(ctx, msk, oracle):
    """The per-orientation comparison form computes the same images."""
    spec = sp.random_specimen(500, 64.0, 10.0, 54.0, 1014)
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    angY = np.deg2rad([0.0, 33.0, 71.0])
    angZ = np.array([0.0, 0.2, 0.0])
    defoci = np.array([0.0, 250.0])
    s = series(msk, 128, 64.0, 300.0, 1.0, 0.02, 0.0)
    imgs, _ = ctx.tilt_series(s, *atoms, angZ, angY, defoci)
    pa, _ = ctx.tilt_series_per_angle(s, *atoms, angZ, angY, defoci)
    sp64 = oracle_series(oracle, 128, 64.0, 300.0, 1.0, 0.02, 0.0)
    for a in range(3):
        ref, _ = oracle.orientation(sp64, *atoms, angZ[a], angY[a], defoci, fp64=True)
        for d in range(2):
            assert rel_l2(pa[a, d], ref[d]) < 1e-5
            assert rel_l2(imgs[a, d], pa[a, d]) < 1e-5


def test_full_size_tilt_series(ctx, msk, oracle):
    """The tilt-series workload at its full size (20000 atoms, 1024^2, 160 slices of
    1 A, 300 keV, defoci 0 and 500 A): the 45-, 90- and 135-degree orientations of a
    four-orientation call against the FP64 oracle (exit waves and images within 1e-5;
    at 45 and 135 degrees the box rule drops the cube's corner atoms, and the kept
    counts must agree), and the 45-degree orientation computed alone equal to it bit
    for bit (units are independent).  The oracle's orientations run on host threads
    (its calls release the interpreter lock)."""
    import concurrent.futures as cf
    from oracle.oracle import SeriesParams
    spec = sp.tilt_specimen(1002)
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    s = msk.Series()
    s.nx = s.ny = 1024
    s.ctblength = s.ctblengthz = 160.0
    s.v0, s.deltaz = 300.0, 1.0
    angY = np.deg2rad([0.0, 45.0, 90.0, 135.0])
    defoci = [0.0, 500.0]
    imgs, ew, kept = ctx.tilt_series(s, *atoms, np.zeros(4), angY, defoci, want_exit=True)
    one, ew1, _ = ctx.tilt_series(s, *atoms, [0.0], angY[1:2], defoci, want_exit=True)
    assert np.array_equal(one[0], imgs[1]) and np.array_equal(ew1[0], ew[1])
    sr = SeriesParams()
    sr.ax, sr.ctblengthz, sr.nx, sr.ny, sr.v0, sr.deltaz = 160.0, 160.0, 1024, 1024, 300.0, 1.0
    sr.max_slices, sr.min_slice = -1, 0

    def ref(a):
        return oracle.orientation(sr, *atoms, 0.0, angY[a], np.array(defoci), fp64=True,
                                  want_exit=True)

    with cf.ThreadPoolExecutor(3) as ex:
        refs = dict(zip((1, 2, 3), ex.map(ref, (1, 2, 3))))
    for a, (ref_img, ref_ew, k) in refs.items():
        assert kept[a] == k, a
        assert rel_l2(ew[a, 0], ref_ew) < 1e-5, a
        for d in range(2):
            assert rel_l2(imgs[a, d], ref_img[d]) < 1e-5, (a, d)
    assert kept[1] < 20000 and kept[3] < 20000 and kept[2] == 20000


@pytest.mark.parametrize("nconf,max_batch,nang", [(1, 0, 3), (3, 2, 3), (1, 0, 40), (2, 0, 20)])
def test_tilt_series_pinned_host_output(ctx, msk, nconf, max_batch, nang):
    """Page-locked host images: each batch's images made in a device buffer and
    copied out on the library's third stream beside the next batch (40 units:
    batches of 8, 24 and 8 units, the copies waiting on one another), or, when a
    configuration average spans batches, written in place by the image pass
    (the GPU addresses them directly) adding onto partial sums already in host
    memory: equal bit for bit to device images."""
    torch = pytest.importorskip("torch")
    spec = sp.random_specimen(300, 64.0, 10.0, 54.0, 1015)
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    s = series(msk, 64, 64.0, 200.0, 2.0, max_batch=max_batch)
    disp = sp.phonon_displacements(spec, nconf, 0.08, 1015) if nconf > 1 else None
    angZ = np.linspace(0.0, 0.5, nang)
    angY = np.linspace(0.2, 2.0, nang)
    df = [0.0, 100.0]
    dev = torch.zeros((nang, 2, 64, 64), dtype=torch.float32, device="cuda")
    ctx.tilt_series(s, *atoms, angZ, angY, df, nconfig=nconf, displacements=disp, images=dev)
    pin = torch.full((nang, 2, 64, 64), -1.0, dtype=torch.float32, pin_memory=True)
    ctx.tilt_series(s, *atoms, angZ, angY, df, nconfig=nconf, displacements=disp, images=pin)
    torch.cuda.synchronize()
    assert torch.equal(pin, dev.cpu())


def test_calculate_reuses_its_grid(ctx, msk, oracle):
    """Calls on one grid reuse the grid tables of the previous call; a call with
    other atomic numbers, another grid in between, or a tilt series (which
    uploads tables of its own) must not leave stale tables behind: every call
    equals the same call in a fresh context bit for bit."""
    a = sp.random_specimen(200, 32.0, 4.0, 28.0, 71)
    b = sp.random_specimen(200, 32.0, 4.0, 28.0, 72)
    b.Znum[:] = 79  # gold only: another table of potentials
    p = msk.make_param(32.0, 32.0, 128, 128, 200.0, 1.0)
    q = msk.make_param(32.0, 32.0, 64, 64, 300.0, 2.0)
    atoms = lambda s: (s.Znum, s.x, s.y, s.z, s.occ)
    seq = [(p, a), (p, a), (p, b), (q, a), (p, a), (p, b)]
    got = []
    for param, s in seq:
        got.append(ctx.calculate(param, *atoms(s), 32.0, 32.0))
        if len(got) == 4:
            ctx.tilt_series(series(msk, 64, 32.0, 300.0, 2.0), *atoms(a), [0.0], [0.3], [0.0])
    fresh = msk.Context(0)
    try:
        for (param, s), g in zip(seq, got):
            ref = fresh.calculate(param, *atoms(s), 32.0, 32.0)
            assert np.array_equal(g.view(np.uint32), ref.view(np.uint32))
            fresh.close()
            fresh = msk.Context(0)
    finally:
        fresh.close()
    ref64 = oracle.calculate(p, *atoms(b), 32.0, 32.0, fp64=True)
    assert rel_l2(got[-1], ref64) < 1e-5


def test_tilt_series_reuses_its_grid(ctx, msk):
    """Tilt series, calculate() and potential stacks share the grid tables of
    the previous call when the grid parameters match (the same tables either
    way); other atomic numbers or another grid in between must not leave stale
    tables behind: every call equals the same call in a fresh context bit for
    bit."""
    a = sp.random_specimen(300, 32.0, 4.0, 28.0, 73)
    b = sp.random_specimen(300, 32.0, 4.0, 28.0, 74)
    b.Znum[:] = 79
    atoms = lambda s: (s.Znum, s.x, s.y, s.z, s.occ)
    sa = series(msk, 128, 32.0, 200.0, 1.0)
    sb = series(msk, 64, 32.0, 300.0, 2.0)
    p = msk.make_param(32.0, 32.0, 128, 128, 200.0, 1.0)  # sa's grid
    st = msk.Stack()  # sa's grid too, no atoms (potential stacks)
    st.nx = st.ny = 128
    st.ax = st.by = 32.0
    st.v0, st.deltaz, st.nslices = 200.0, 1.0, 6
    v = np.random.default_rng(75).uniform(0.0, 2.0, (2, 6, 128, 128)).astype(np.float32)
    seq = [("t", sa, a), ("t", sa, a), ("t", sa, b), ("c", p, a), ("t", sa, a), ("t", sb, a),
           ("t", sa, b), ("s", st, None), ("t", sa, b), ("c", p, b), ("s", st, None)]

    def run(c, kind, g, s):
        if kind == "c":
            return c.calculate(g, *atoms(s), 32.0, 32.0)
        if kind == "s":
            return c.stack_images(g, v, [0.0])
        return c.tilt_series(g, *atoms(s), [0.0, 0.4], [0.3, 1.1], [0.0, 150.0])[0]
    got = [run(ctx, *x) for x in seq]
    for x, g in zip(seq, got):
        fresh = msk.Context(0)
        try:
            ref = run(fresh, *x)
        finally:
            fresh.close()
        assert np.array_equal(g.view(np.uint32), ref.view(np.uint32)), x[0]


def test_calculate_into_out_buffer(ctx, msk):
    """calculate(out=...) writes the exit wave into the caller's array (reused
    across calls) and equals the returned array bit for bit; the default plane
    wave the wrapper keeps per grid size is left as it was."""
    a = sp.random_specimen(200, 32.0, 4.0, 28.0, 76)
    atoms = (a.Znum, a.x, a.y, a.z, a.occ)
    p = msk.make_param(32.0, 32.0, 128, 128, 200.0, 1.0)
    ref = ctx.calculate(p, *atoms, 32.0, 32.0)
    out = np.full((128, 128, 2), np.nan, np.float32)
    for _ in range(2):
        got = ctx.calculate(p, *atoms, 32.0, 32.0, out=out)
        assert got is out
        assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
    w0 = ctx._plane_waves[(128, 128)]
    assert np.all(w0[..., 0] == 1.0) and np.all(w0[..., 1] == 0.0)
    with pytest.raises(ValueError):
        ctx.calculate(p, *atoms, 32.0, 32.0, out=np.zeros((64, 64, 2), np.float32))


def test_calculate_keeps_an_unchanged_incident_wave(ctx, msk):
    """calculate() uploads its incident wave only when it differs from the
    previous call's (compared on the host); a new wave, the same wave again
    after another, and a spherical-wave tilt series in between (which writes
    the same device buffer) must each give the fresh-context result."""
    a = sp.random_specimen(200, 32.0, 4.0, 28.0, 77)
    atoms = (a.Znum, a.x, a.y, a.z, a.occ)
    p = msk.make_param(32.0, 32.0, 128, 128, 200.0, 1.0)
    rng = np.random.default_rng(78)
    w1 = rng.normal(size=(128, 128, 2)).astype(np.float32)
    w2 = rng.normal(size=(128, 128, 2)).astype(np.float32)
    sph = series(msk, 128, 32.0, 200.0, 1.0)
    sph.R1 = 500.0
    seq = ["w1", "w1", "w2", "w1", "sph", "w1"]
    got = []
    for k in seq:
        if k == "sph":
            ctx.tilt_series(sph, *atoms, [0.0], [0.2], [0.0])
            continue
        w = w1 if k == "w1" else w2
        got.append((w, ctx.calculate(p, *atoms, 32.0, 32.0, wave0=w)))
    for w, g in got:
        fresh = msk.Context(0)
        try:
            ref = fresh.calculate(p, *atoms, 32.0, 32.0, wave0=w)
        finally:
            fresh.close()
        assert np.array_equal(g.view(np.uint32), ref.view(np.uint32))
