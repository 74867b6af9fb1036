"""Thermal branches of calculate() (lwobble = 1) and the spherical incident
wave on the GPU.

  * Debye-Waller (nwobble 1) and random displacements (nwobble 3) against the
    reference's own FP32 build (tests/golden/ref_thermal_*.npz): relative L2
    <= 2e-5, and the advanced gasdev seed equal;
  * against the FP64 oracle: <= 1e-5;
  * through msk_tilt_series: the angle-zero orientation equals msk_calculate on
    the same atoms bit for bit (Debye-Waller; displacements drawn from the
    seed, configuration by configuration), and a spherical incident wave equals
    msk_calculate started from the same wave.
"""
import numpy as np
import pytest

from conftest import golden, rel_l2
from utr_public_gb300 import specimen as sp

pytestmark = pytest.mark.gpu


def thermal_case(msk, name):
    g = golden("ref_thermal_%s.npz" % name)
    n, nx = int(g["natom"]), int(g["nx"])
    s = sp.plain_specimen(1001)
    wob = (0.05 + 0.025 * (np.arange(n) % 3)).astype(np.float32)
    param = msk.make_param(64.0, 64.0, nx, nx, 200.0, 2.0)
    param[msk.pNWOBBLE], param[msk.pTEMPER] = float(g["nwobble"]), float(g["temperature"])
    atoms = (s.Znum[:n], s.x[:n], s.y[:n], s.z[:n], s.occ[:n])
    return g, param, atoms, wob


@pytest.mark.parametrize("name", ["dw_128", "wobble_128"])
def test_thermal_calculate_matches_reference(ctx, msk, oracle, name):
    g, param, atoms, wob = thermal_case(msk, name)
    pix, seed = ctx.calculate(param, *atoms, 64.0, 64.0, wobble=wob, lwobble=1,
                              iseed=int(g["iseed0"]))
    assert rel_l2(pix, g["pix"]) < 2e-5
    assert seed == int(g["iseed1"])
    ref64, _ = oracle.calculate_thermal(param, *atoms, wob, 64.0, 64.0, iseed=int(g["iseed0"]),
                                        fp64=True)
    assert rel_l2(pix, ref64) < 1e-5


def test_thermal_needs_wobble_and_seed(ctx, msk):
    g, param, atoms, wob = thermal_case(msk, "wobble_128")
    with pytest.raises(msk.MskError) as e:  # nwobble > 1 without a seed
        ctx.calculate(param, *atoms, 64.0, 64.0, wobble=wob, lwobble=1)
    assert e.value.status == msk.MSK_EINVAL


def series(msk, n, fov):
    s = msk.Series()
    s.nx = s.ny = n
    s.ctblength = s.ctblengthz = fov
    s.v0, s.deltaz = 200.0, 2.0
    return s


def test_tilt_series_debye_waller_equals_calculate(ctx, msk):
    spec = sp.random_specimen(500, 64.0, 10.0, 54.0, 1021)
    wob = (0.04 + 0.03 * (np.arange(spec.natom) % 4)).astype(np.float32)
    s = series(msk, 128, 64.0)
    s.lwobble, s.temperature = 1, 280.0
    s.wobble = wob.ctypes.data
    _, ew, _ = ctx.tilt_series(s, spec.Znum, spec.x, spec.y, spec.z, spec.occ, [0.0], [0.0],
                               [0.0], want_exit=True)
    x, y, z = msk.rotate(64.0, 0.0, 0.0, spec.x, spec.y, spec.z)
    param = msk.make_param(64.0, 64.0, 128, 128, 200.0, 2.0)
    param[msk.pNWOBBLE], param[msk.pTEMPER] = 1.0, 280.0
    pix = ctx.calculate(param, spec.Znum, x, y, z, spec.occ, 64.0, 64.0, wobble=wob, lwobble=1)
    assert np.array_equal(ew[0, 0].view(np.uint32), pix.view(np.uint32))
    plain = ctx.calculate(msk.make_param(64.0, 64.0, 128, 128, 200.0, 2.0), spec.Znum, x, y, z,
                          spec.occ, 64.0, 64.0)
    assert rel_l2(pix, plain) > 1e-4  # the damping acts


def test_tilt_series_random_displacements_equal_calculate(ctx, msk):
    spec = sp.random_specimen(400, 64.0, 10.0, 54.0, 1022)
    wob = np.full(spec.natom, 0.08, np.float32)
    s = series(msk, 64, 64.0)
    s.lwobble, s.temperature, s.seed = 1, 300.0, -4242
    s.wobble = wob.ctypes.data
    _, ew, _ = ctx.tilt_series(s, spec.Znum, spec.x, spec.y, spec.z, spec.occ, [0.0], [0.0],
                               [0.0], nconfig=3, displacements=None, want_exit=True)
    x, y, z = msk.rotate(64.0, 0.0, 0.0, spec.x, spec.y, spec.z)
    param = msk.make_param(64.0, 64.0, 64, 64, 200.0, 2.0)
    param[msk.pNWOBBLE], param[msk.pTEMPER] = 3.0, 300.0
    seed = -4242  # orientation 0 draws from the seed itself, configurations in order
    for c in range(3):
        pix, seed = ctx.calculate(param, spec.Znum, x, y, z, spec.occ, 64.0, 64.0, wobble=wob,
                                  lwobble=1, iseed=seed)
        assert np.array_equal(ew[0, c].view(np.uint32), pix.view(np.uint32)), c


def test_spherical_incident_wave(ctx, msk, oracle):
    spec = sp.random_specimen(300, 64.0, 10.0, 54.0, 1023)
    s = series(msk, 128, 64.0)
    s.R1 = 5000.0
    _, ew, _ = ctx.tilt_series(s, spec.Znum, spec.x, spec.y, spec.z, spec.occ, [0.0], [0.0],
                               [0.0], want_exit=True)
    # MsctKirkland's wave (autosliccmd.cpp:650-689), built here in numpy
    n, fov, R1in = 128, 64.0, 5000.0 - 32.0
    lam = oracle.wavelength(200.0)
    st = np.float32(fov) / np.float32(n)
    i = np.arange(n) - n // 2
    xx = (i * float(st)) ** 2
    r2 = xx[:, None] + xx[None, :]
    amp = (1.0 / np.sqrt(1.0 + r2 / R1in ** 2)).astype(np.float32)
    phamax = 2 * np.pi / lam * np.sqrt(2 * float(st) ** 2 * (n // 2) ** 2 + R1in ** 2)
    pha = (2 * np.pi / lam * np.sqrt(r2 + R1in ** 2) - phamax).astype(np.float32)
    w0 = np.stack([amp * np.cos(pha.astype(np.float64)), amp * np.sin(pha.astype(np.float64))],
                  axis=-1).astype(np.float32)
    x, y, z = msk.rotate(64.0, 0.0, 0.0, spec.x, spec.y, spec.z)
    pix = ctx.calculate(msk.make_param(64.0, 64.0, 128, 128, 200.0, 2.0), spec.Znum, x, y, z,
                        spec.occ, 64.0, 64.0, wave0=w0)
    assert rel_l2(ew[0, 0], pix) < 1e-6
    _, plane, _ = ctx.tilt_series(series(msk, 128, 64.0), spec.Znum, spec.x, spec.y, spec.z,
                                  spec.occ, [0.0], [0.0], [0.0], want_exit=True)
    assert rel_l2(ew[0, 0], plane[0, 0]) > 1e-3


def test_image_plane_rotation_and_shift(ctx, msk, oracle):
    """Rotation about the optic axis and a whole-pixel shift of the propagated
    amplitude (autosliccmd.cpp:1119-1143, this library's definitions) against
    the FP64 oracle, per detector plane; planes without them are unchanged."""
    from oracle.oracle import SeriesParams
    spec = sp.random_specimen(500, 64.0, 10.0, 54.0, 1024)
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    s = series(msk, 128, 64.0)
    s.dxc, s.dyc = 1.5, -2.0
    rot = np.array([0.3, 0.0, -1.1])
    s.rotation = rot.ctypes.data
    s.xshift, s.yshift = 1.3, -0.7
    defoci = np.array([0.0, 150.0, 40.0])
    angY, angZ = np.deg2rad([25.0]), np.array([0.2])
    imgs, ew, _ = ctx.tilt_series(s, *atoms, angZ, angY, defoci, want_exit=True)
    p = SeriesParams()
    p.ax, p.ctblengthz, p.nx, p.ny, p.v0, p.deltaz = 64.0, 64.0, 128, 128, 200.0, 2.0
    p.dxc, p.dyc, p.max_slices = 1.5, -2.0, -1
    _, ew64, _ = oracle.orientation(p, *atoms, angZ[0], angY[0], defoci, fp64=True,
                                    want_exit=True)
    st = float(np.float32(64.0) / np.float32(128))
    lam = oracle.wavelength(200.0)
    sx, sy = int(np.floor(1.3 / st + 0.5)), int(np.floor(-0.7 / st + 0.5))
    for d in range(3):
        ref = oracle.image_plane(ew64, 64.0, lam, defoci[d] - 32.0, rot[d], 32.0 + 1.5,
                                 32.0 - 2.0, sx, sy)
        assert rel_l2(imgs[0, d], ref) < 1e-5, d
    plain, _ = ctx.tilt_series(series(msk, 128, 64.0), *atoms, angZ, angY, defoci)
    assert rel_l2(imgs[0, 1], plain[0, 1]) > 1e-3  # the shift acts on every plane
