"""UTR reconstruction on the GPU (msk_utr_*) against the oracle: the
gridding sums, the 3D corrections (against the float restatement that equals
the reference's UTR.h templates bit for bit) and the whole reconstruction
against the FP64 restatement of UTR.cpp (relative L2 <= 1e-4)."""
import numpy as np
import pytest

from conftest import rel_l2
import utr_cases as uc

pytestmark = pytest.mark.gpu

WL = 0.0196875


def as_msk(msk, p):
    u = msk.Utr()
    for name, _ in p._fields_:
        setattr(u, name, getattr(p, name))
    return u


def test_gridding_sums_match_oracle(ctx, msk, oracle):
    p = uc.params(nx=32, ny=32, nz=16, escc=1, dxc=0.4, dyc=-0.3, dzc=0.2)
    ang = np.array([[15.0, 20.0], [-30.0, 80.0], [5.0, 140.0]])
    rng = np.random.default_rng(11)
    k2 = rng.standard_normal((3, 32, 32, 2)).astype(np.float32)
    v3, s3 = ctx.utr_grid(as_msk(msk, p), ang, k2)
    g = oracle.utr_geom(p, ang, np.zeros(3))
    fx = tuple(np.float32(v) for v in (g.fxlo, g.fxst, g.fylo, g.fyst, g.fzlo, g.fzst))
    V = np.zeros((g.nz, 32, 32, 2))
    S = np.zeros((g.nz, 32, 32))
    tpi = 2 * np.pi
    for a, (az, ay) in enumerate(ang):
        Z, Y = np.deg2rad(az), np.deg2rad(ay)
        cy, sy, cz, sz = np.cos(Y), np.sin(Y), np.cos(Z), np.sin(Z)
        fa = np.float32([tpi * (p.dxc * (1 - cy * cz) - p.dyc * sz + p.dzc * sy * cz),
                         tpi * (p.dxc * cy * sz + p.dyc * (1 - cz) - p.dzc * sy * sz),
                         tpi * (-p.dxc * sy + p.dzc * (1 - cy))])
        fc = np.zeros(6, np.float32)
        fc[1::2] = -fa
        oracle.utr_grid(k2[a], g.nz, Y, Z, fx, fc, WL, 1, 1, mode="acc64", v3=V, samp3=S)
    assert (S > 0).sum() > 1000
    assert rel_l2(s3, S) < 1e-6
    assert rel_l2(v3, V) < 1e-6
    assert np.abs(s3 - S).max() < 1e-5 * S.max()


@pytest.mark.parametrize("escc", [0, 1])
def test_tilt_series_gridding_matches_oracle(ctx, msk, oracle, escc):
    # tilts about Y' alone take the per-plane tile form
    p = uc.params(nx=128, ny=32, nz=64, escc=escc, dxc=0.3 * escc)
    ang = uc.tilt_angles(37, span=185.0)
    rng = np.random.default_rng(12 + escc)
    k2 = rng.standard_normal((37, 32, 128, 2)).astype(np.float32)
    v3, s3 = ctx.utr_grid(as_msk(msk, p), ang, k2)
    g = oracle.utr_geom(p, ang, np.zeros(37))
    fx = tuple(np.float32(v) for v in (g.fxlo, g.fxst, g.fylo, g.fyst, g.fzlo, g.fzst))
    V = np.zeros((g.nz, 32, 128, 2))
    S = np.zeros((g.nz, 32, 128))
    for a, (az, ay) in enumerate(ang):
        Y = np.deg2rad(ay)
        fa = np.float32([2 * np.pi * p.dxc * (1 - np.cos(Y)), 0.0, -2 * np.pi * p.dxc * np.sin(Y)])
        fc = np.zeros(6, np.float32)
        fc[1::2] = -fa
        oracle.utr_grid(k2[a], g.nz, Y, 0.0, fx, fc, WL, escc, escc, mode="acc64", v3=V, samp3=S)
    assert (S > 0).sum() > 10000
    assert rel_l2(s3, S) < 1e-6
    assert rel_l2(v3, V) < 1e-6


def test_ctf_and_laplacian_match_reference_restatement(ctx, oracle):
    rng = np.random.default_rng(5)
    v = rng.standard_normal((16, 32, 64, 2)).astype(np.float32)
    box = (-4.0, 4.0, -8.0, 8.0, -16.0, 16.0)
    for args in ((WL, box, 120.0, 0.0, 0.0, 0.0, 0.05, 1e-3, 0),
                 (WL, box, -80.0, 2.0, 1.2e7, 3e9, 0.1, 0.0, 1)):
        want = oracle.utr_ctf3d(v.copy(), *args)
        got = ctx.utr_ctf_correction3d(v.copy(), *args)
        assert rel_l2(got, want) < 2e-5
    want = oracle.utr_invlap3d(v.copy(), 8.0, 16.0, 32.3, 0.7, 1.3)
    got = ctx.utr_inverse_mlaplacian3d(v.copy(), 8.0, 16.0, 32.3, 0.7, 1.3)
    assert rel_l2(got, want) < 1e-6


CASES = {
    # name: (nx, ny, nz, nangles, param overrides, angle Z step)
    "ctf3d": (32, 32, 16, 24, dict(ctf_mode=4), 0.0),
    "ctf3d_escc_cs_aperture": (64, 64, 32, 36, dict(ctf_mode=4, escc=1, cs3=1.2, aobj=30.0), 0.0),
    "none_nsr_invlap": (64, 32, 32, 30, dict(ctf_mode=0, nsr=0.02, inv_laplace=1), 0.0),
    "tiehom_xray_shift": (32, 64, 16, 20,
                          dict(ctf_mode=2, modality=1, asigma=-0.05, dxc=0.5, dzc=-0.25,
                               wl=1.2e-4, xst=0.7), 3.0),
    "ctf3d_double_tilt": (32, 32, 32, 30, dict(ctf_mode=4, epsilon=0.0, f1=2.0, f2=0.1), 7.0),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_reconstruction_matches_fp64_oracle(ctx, msk, oracle, name):
    nx, ny, nz, na, kw, azstep = CASES[name]
    p = uc.params(nx=nx, ny=ny, nz=nz, **kw)
    ang = uc.tilt_angles(na)
    ang[:, 0] = azstep * np.arange(na)
    df = np.full(na, 60.0) + np.linspace(0.0, 10.0, na)
    imgs = uc.images(p, na, seed=na)
    want = oracle.utr_reconstruct(p, ang, df, imgs, nthreads=8)
    got = ctx.utr_reconstruct(as_msk(msk, p), ang, df, imgs)
    assert got.shape == (nz, ny, nx)
    assert np.abs(want).max() > 0
    assert rel_l2(got, want) <= 1e-4, name


def test_reconstruction_repeatable_and_device_pointers(ctx, msk):
    # the gridding sums are float atomics (as the reference's threaded float
    # sums): repeated runs agree to rounding, not bit for bit
    torch = pytest.importorskip("torch")
    p = as_msk(msk, uc.params(nx=64, ny=64, nz=32, ctf_mode=4, escc=1, nsr=0.01))
    ang = uc.tilt_angles(40)
    df = np.full(40, 50.0)
    imgs = uc.images(p, 40, seed=2)
    a = ctx.utr_reconstruct(p, ang, df, imgs)
    b = ctx.utr_reconstruct(p, ang, df, imgs)
    assert rel_l2(b, a) < 1e-6
    timgs = torch.from_numpy(imgs).cuda()
    vol = torch.empty((32, 64, 64), dtype=torch.float32, device="cuda")
    ctx.utr_reconstruct(p, ang, df, timgs, volume=vol)
    torch.cuda.synchronize()
    assert rel_l2(vol.cpu().numpy(), a) < 1e-6


def test_reconstruction_errors(ctx, msk):
    p = as_msk(msk, uc.params(nx=32, ny=32, nz=16))
    ang, df, imgs = uc.tilt_angles(4), np.full(4, 10.0), np.ones((4, 32, 32), np.float32)
    for kw, status in ((dict(ctf_mode=3), -6), (dict(ctf_mode=1), -6), (dict(zhi=4.3), -6),
                       (dict(epsilon=0.0, asigma=0.0), -8), (dict(f1=0.0), -8),
                       (dict(modality=1, asigma=0.1), -8), (dict(ctf_mode=2, asigma=0.1), -8)):
        q = as_msk(msk, uc.params(nx=32, ny=32, nz=16, **kw))
        with pytest.raises(msk.MskError) as e:
            ctx.utr_reconstruct(q, ang, df, imgs)
        assert e.value.status == status, kw
    # flat images: log 1 = 0 everywhere
    assert not ctx.utr_reconstruct(p, ang, df, imgs).any()


def test_reconstruction_with_image_planes_matches_oracle(ctx, msk, oracle):
    # Z'' rotations and shifts of the input images, undone before the spectra
    p = uc.params(nx=64, ny=64, nz=32, ctf_mode=4, escc=1, dxc=0.4, dyc=-0.3)
    na = 24
    ang = uc.tilt_angles(na)
    df = np.full(na, 70.0)
    imgs = uc.images(p, na, seed=31)
    zrot = np.linspace(-25.0, 25.0, na)
    shifts = np.stack([np.linspace(-1.6, 1.6, na), np.linspace(0.9, -0.9, na)], axis=1)
    want = oracle.utr_reconstruct(p, ang, df, imgs, nthreads=8, zrot=zrot, shifts=shifts)
    got = ctx.utr_reconstruct(as_msk(msk, p), ang, df, imgs, zrot=zrot, shifts=shifts)
    assert rel_l2(got, want) <= 1e-4
    plain = ctx.utr_reconstruct(as_msk(msk, p), ang, df, imgs)
    assert rel_l2(plain, want) > 1e-3  # the planes change the reconstruction
    # shifts alone (no rotation) take the whole-pixel path
    want_s = oracle.utr_reconstruct(p, ang, df, imgs, nthreads=8, shifts=shifts)
    got_s = ctx.utr_reconstruct(as_msk(msk, p), ang, df, imgs, shifts=shifts)
    assert rel_l2(got_s, want_s) <= 1e-4
