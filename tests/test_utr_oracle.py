"""The UTR reconstruction's oracle (no GPU): its float restatement of the
reference's UTR.h templates pinned bit for bit to their own outputs
(tests/golden/ref_utr.npz, and the live build where the reference tree
exists), its geometry, its centred DFT, and the equivalence that the GPU
path rests on (the Hermitian step plus a complex-to-real inverse = factors
on the x-Nyquist plane plus the real part of a complex inverse)."""
import numpy as np
import pytest

from conftest import golden, rel_l2
from oracle import oracle as orc
import utr_cases as uc

WL = 0.0196875
XST = 0.5


def geometry(nx, ny, nz):
    xlo, ylo, zlo = -0.5 * XST * nx, -0.5 * XST * ny, -0.5 * XST * nz
    fxst, fyst, fzst = 1 / (XST * nx), 1 / (XST * ny), 1 / (XST * nz)
    fx = tuple(np.float32(v) for v in (-fxst * (nx // 2), fxst, -fyst * (ny // 2), fyst,
                                       -fzst * (nz // 2), fzst))
    return fx, (zlo, zlo + XST * nz, ylo, ylo + XST * ny, xlo, xlo + XST * nx)


GRID = {"flat": (16, [(0.0, 17.0), (0.0, 71.0)], 0, (0.0, 0.0, 0.0)),
        "escc_shift": (8, [(12.0, 33.0), (-40.0, 95.0), (5.0, 150.0)], 1, (0.4, -0.3, 0.2))}
CTF = {"plain": (120.0, 0.0, 0.0, 0.0, 0.05, 1e-3, 0),
       "escc_cs_auto_eps": (-80.0, 2.0, 1.2e7, 3e9, 0.1, 0.0, 1)}


@pytest.mark.parametrize("name", sorted(GRID))
def test_gridding_mirror_matches_reference_golden(oracle, name):
    G = golden("ref_utr.npz")
    nz, angles, escc, shift = GRID[name]
    k2 = G["grid_%s_k2" % name]
    fcs = G["grid_%s_fc" % name]
    ny, nx = k2.shape[1:3]
    fx, _ = geometry(nx, ny, nz)
    v3 = np.zeros((nz, ny, nx, 2), np.float32)
    s3 = np.zeros((nz, ny, nx), np.float32)
    for a, (az, ay) in enumerate(angles):
        oracle.utr_grid(k2[a], nz, np.deg2rad(ay), np.deg2rad(az), fx, fcs[a], WL, any(shift),
                        escc, v3=v3, samp3=s3)
    assert np.array_equal(v3.view(np.uint32), G["grid_%s_v3" % name].view(np.uint32))
    assert np.array_equal(s3.view(np.uint32), G["grid_%s_samp3" % name].view(np.uint32))
    assert (s3 > 0).sum() > 100


@pytest.mark.parametrize("name", sorted(CTF))
def test_ctf3d_mirror_matches_reference_golden(oracle, name):
    G = golden("ref_utr.npz")
    df, q2, cs3, cs5, sig, eps, escc = CTF[name]
    _, box = geometry(16, 16, 16)
    got = oracle.utr_ctf3d(G["vol_in"].copy(), WL, box, df, q2, cs3, cs5, sig, eps, escc)
    assert np.array_equal(got.view(np.uint32), G["ctf_%s" % name].view(np.uint32))


def test_invlap3d_mirror_matches_reference_golden(oracle):
    G = golden("ref_utr.npz")
    got = oracle.utr_invlap3d(G["vol_in"].copy(), 8.0, 8.0, 8.3, 0.7, 1.3)
    assert np.array_equal(got.view(np.uint32), G["invlap"].view(np.uint32))


@pytest.mark.skipif(not orc.utr_reference_available(), reason="reference UTR build absent")
def test_mirrors_match_live_reference(oracle):
    ref = orc.UtrReference()
    rng = np.random.default_rng(77)
    for trial in range(4):
        nx, ny, nz = 32, 16, 16
        fx, box = geometry(nx, ny, nz)
        k2 = rng.standard_normal((ny, nx, 2)).astype(np.float32)
        fc = np.zeros(6, np.float32)
        fc[1::2] = rng.uniform(-1, 1, 3)
        angY, angZ = rng.uniform(0, np.pi), rng.uniform(-np.pi, np.pi)
        a = oracle.utr_grid(k2, nz, angY, angZ, fx, fc, WL, trial % 2, trial // 2)
        b = ref.grid(k2, nz, angY, angZ, fx, fc, WL, trial % 2, trial // 2)
        assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32))
        assert np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))
        v = rng.standard_normal((nz, ny, nx, 2)).astype(np.float32)
        args = (WL, box, rng.uniform(-200, 200), rng.uniform(0, 3), 1e7 * trial, 0.0,
                rng.uniform(0, 0.3), [0.0, 1e-3][trial % 2], trial // 2)
        assert np.array_equal(oracle.utr_ctf3d(v.copy(), *args).view(np.uint32),
                              ref.ctf3d(v.copy(), *args).view(np.uint32))


def test_geometry(oracle):
    p = uc.params(nx=64, ny=32, nz=16, xst=0.457, wl=0.02507934)
    p.zlo, p.zhi = 3.6, -3.7  # swapped and not a multiple of the pixel size
    g = oracle.utr_geom(p, [[0, 0], [0, 10], [0, 20]], [10.0, 20.0, 30.0])
    assert g.nz == int((7.3) / 0.457 + 0.5) and g.zlo == -3.7 and g.zhi == 3.6
    assert abs(g.ee / 1e3 - 200.0) < 0.01  # 0.02507934 A <-> 200 keV (the readme's pair)
    assert g.zout_aver == 20.0 and g.rot_y_only and not g.rot_z_only
    assert g.fxst == pytest.approx(1 / (64 * 0.457)) and g.fxlo == -32 * g.fxst
    # the flags are set from the second orientation on (UTR.cpp:214-222)
    g = oracle.utr_geom(p, [[30, 0], [0, 10]], [0.0, 0.0])
    assert g.rot_y_only
    x = uc.params(modality=1, asigma=-0.01, zlo=0.0, zhi=0.0, nx=32, ny=32, xst=0.5)
    gx = oracle.utr_geom(x, [[0, 0]], [0.0])
    assert gx.nz == 32 and gx.zlo == gx.xlo


def test_centred_spectrum_definition(oracle):
    img = uc.images(uc.params(nx=32, ny=16), 1, seed=3)[0]
    got = oracle.utr_k2four(img)
    lg = np.log(img.astype(np.float64))
    want = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(lg)))
    assert rel_l2(got[..., 0] + 1j * got[..., 1], want) < 1e-12


@pytest.mark.parametrize("case", ["ctf_nsr0", "none_nsr_invlap", "tiehom", "ctf_shift_xray"])
def test_complex_inverse_plan_equals_c2r(oracle, case):
    rng = np.random.default_rng(3)
    nx, ny, nz = 32, 16, 16
    kw = {"ctf_nsr0": dict(ctf_mode=4, escc=1),
          "none_nsr_invlap": dict(ctf_mode=0, nsr=0.05, inv_laplace=1),
          "tiehom": dict(ctf_mode=2, asigma=-0.1),
          "ctf_shift_xray": dict(ctf_mode=4, modality=1, asigma=-0.2, dxc=0.3, cs3=1.0)}[case]
    p = uc.params(nx=nx, ny=ny, nz=nz, **kw)
    az = 10.0 if case == "ctf_shift_xray" else 0.0
    ang = np.array([[az * a / 3, a * 10.0] for a in range(18)])
    df = np.full(18, 60.0)
    v3 = rng.standard_normal((nz, ny, nx, 2))
    samp = rng.uniform(0, 3, (nz, ny, nx))
    samp[samp < 0.5] = 0
    vol = oracle.utr_finish(p, ang, df, v3, samp)
    model = uc.complex_inverse_model(oracle, p, ang, df, v3, samp)
    assert (vol != 0).sum() > 500
    assert rel_l2(model, vol) < 1e-12


def test_reconstruction_linear_in_log_images(oracle):
    # with no SNR filter every stage after the log is linear
    p = uc.params(nx=32, ny=32, nz=16, ctf_mode=4)
    ang = uc.tilt_angles(12)
    df = np.full(12, 80.0)
    g = np.log(uc.images(p, 12, seed=5).astype(np.float64))
    v1 = oracle.utr_reconstruct(p, ang, df, np.exp(g).astype(np.float32), nthreads=4)
    v2 = oracle.utr_reconstruct(p, ang, df, np.exp(2.0 * g).astype(np.float32), nthreads=2)
    assert np.abs(v1).max() > 0
    assert rel_l2(v2, 2.0 * v1) < 1e-5  # the images are rounded to float
    # flat images reconstruct to zero
    assert not oracle.utr_reconstruct(p, ang, df, np.ones_like(g, np.float32)).any()


def test_library_depth_matches_oracle(msk, oracle):
    # msk_utr_depth is host code: no GPU needed
    L = msk.load()
    for kw in (dict(nx=64, ny=32, xst=0.457, zlo=3.6, zhi=-3.7), dict(nx=32, ny=32, xst=0.5),
               dict(modality=1, asigma=-0.01, zlo=0.0, zhi=0.0, nx=32, ny=32, xst=0.5)):
        p = uc.params(**kw)
        u = msk.Utr()
        for name, _ in p._fields_:
            setattr(u, name, getattr(p, name))
        assert L.msk_utr_depth(u) == oracle.utr_geom(p, [[0, 0]], [0.0]).nz
    bad = msk.Utr(nx=32, ny=32, xst=0.0, zlo=-1.0, zhi=1.0, wl=0.02)
    assert L.msk_utr_depth(bad) == -8


def test_image_plane_definitions(oracle):
    L = oracle.L
    import ctypes as C
    L.mo_utr_image_plane_f64.argtypes = [np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS"),
                                         C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                         C.c_long, C.c_long]
    rng = np.random.default_rng(4)
    img = 1.0 + 0.1 * rng.standard_normal((24, 32))
    edge = np.ones_like(img, bool)
    edge[5:-5, 5:-5] = False
    f = img[edge].mean()
    # a pure shift: whole pixels, the edge mean coming in
    a = img.copy()
    L.mo_utr_image_plane_f64(a, 32, 24, 16.0, 12.0, 0.0, 3, -2)
    assert np.array_equal(a[:22, 3:], img[2:, :29])
    assert np.allclose(a[:, :3], f, rtol=1e-14) and np.allclose(a[22:], f, rtol=1e-14)
    # a rotation by t then -t about the same centre: a smooth interior comes back
    y, x = np.mgrid[0:24, 0:32]
    sm = 1.0 + 0.2 * np.exp(-((x - 14.0) ** 2 + (y - 11.0) ** 2) / 18.0)
    b = sm.copy()
    L.mo_utr_image_plane_f64(b, 32, 24, 16.0, 12.0, 0.3, 0, 0)
    assert np.abs(b - sm).max() > 1e-2
    L.mo_utr_image_plane_f64(b, 32, 24, 16.0, 12.0, -0.3, 0, 0)
    assert np.abs(b - sm)[8:16, 10:22].max() < 0.05 * np.abs(sm - 1).max()
    # a quarter turn of the sample grid is exact away from the edges
    sq = 1.0 + 0.1 * rng.standard_normal((32, 32))
    c = sq.copy()
    L.mo_utr_image_plane_f64(c, 32, 32, 16.0, 16.0, np.pi / 2, 0, 0)
    # out(i, j) = in(c + R(-t)(p - c)): for t = pi/2, x' = cx + (j - cy), y' = cy - (i - cx)
    j, i = 20, 10
    assert abs(c[j, i] - sq[int(16 - (i - 16)), int(16 + (j - 16))]) < 1e-9


def test_zero_planes_equal_plain_reconstruction(oracle):
    p = uc.params(nx=32, ny=32, nz=16)
    ang = uc.tilt_angles(8)
    df = np.full(8, 40.0)
    imgs = uc.images(p, 8, seed=9)
    a = oracle.utr_reconstruct(p, ang, df, imgs)
    b = oracle.utr_reconstruct(p, ang, df, imgs, zrot=np.zeros(8), shifts=np.zeros((8, 2)))
    assert np.array_equal(a, b)
    c = oracle.utr_reconstruct(p, ang, df, imgs, zrot=np.linspace(0, 20, 8))
    assert rel_l2(c, a) > 1e-3
