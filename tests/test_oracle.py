"""The oracle pinned against the reference's own outputs (tests/golden, made
by tests/golden/make_golden.py from the reference compiled unmodified).

The FP32 restatement mirrors the reference operation by operation and uses
the same CPU FFT as the reference build, so on the machine that made the
fixtures (x86-64) it reproduces them bit for bit; elsewhere libm may round a
last bit differently, so the bound there is 1e-6 relative L2.
"""
import platform

import numpy as np
import pytest

from conftest import golden, rel_l2
from utr_public_gb300 import specimen as sp

EXIT_CASES = ["c1_128", "c1_256", "rect_64x128", "proj_64"]
SAME_MACHINE = platform.machine() == "x86_64"


def case(g):
    s = sp.plain_specimen(int(g["seed"]))
    n = int(g["natom"])
    return s.Znum[:n], s.x[:n], s.y[:n], s.z[:n], s.occ[:n]


def test_physics_matches_reference(oracle):
    g = golden("ref_physics.npz")
    for k, w, s in zip(g["kev"], g["wavelength"], g["sigma"]):
        assert oracle.wavelength(k) == w
        assert oracle.sigma(k) == s
    for xv, k0, i0 in zip(g["bessk0_x"], g["bessk0"], g["bessi0"]):
        assert oracle.L.mo_bessk0(xv) == pytest.approx(k0, rel=1e-15, abs=0)
        assert oracle.L.mo_bessi0(xv) == pytest.approx(i0, rel=1e-15, abs=0)
    for zi, Z in enumerate(g["lut_Z"]):
        for ri, r2 in enumerate(g["lut_rsq"]):
            assert oracle.L.mo_vzatomLUT(int(Z), float(r2)) == pytest.approx(
                g["lut"][zi, ri], rel=1e-14, abs=1e-300)
            assert oracle.L.mo_vzatom(int(Z), float(np.sqrt(r2))) == pytest.approx(
                g["vzatom"][zi, ri], rel=1e-14, abs=1e-300)


@pytest.mark.parametrize("n,a", [(64, 64.0), (128, 64.0), (256, 64.0), (1024, 160.0), (100, 37.5)])
def test_freqn_bit_exact(oracle, n, a):
    g = golden("ref_physics.npz")
    k, k2, xp = oracle.freqn(n, a)
    assert np.array_equal(k, g["freqn_%d_k" % n])
    assert np.array_equal(k2, g["freqn_%d_k2" % n])
    assert np.array_equal(xp, g["freqn_%d_x" % n])


def test_sort_permutation_bit_exact(oracle):
    g = golden("ref_sort.npz")
    s = sp.plain_specimen(1001)
    idx = np.arange(s.natom, dtype=np.float32)
    _, _, _, zs, perm = oracle.sort_by_z(s.Znum, s.x, s.y, s.z, idx)
    assert np.array_equal(perm.astype(np.int32), g["perm"])
    assert np.array_equal(zs, g["zsorted"])
    assert np.all(np.diff(zs) >= 0)


@pytest.mark.parametrize("name", EXIT_CASES)
def test_fp32_restatement_matches_reference(oracle, name):
    g = golden("ref_exit_%s.npz" % name)
    from oracle.oracle import make_param
    fov, nx, ny = float(g["fov"]), int(g["nx"]), int(g["ny"])
    param = make_param(fov, fov, nx, ny, float(g["v0"]), float(g["deltaz"]))
    pix = oracle.calculate(param, *case(g), fov, fov, nmode=int(g["nmode"]))
    if SAME_MACHINE:
        assert np.array_equal(pix.view(np.uint32), g["pix"].view(np.uint32))
    else:
        assert rel_l2(pix, g["pix"]) < 1e-6


@pytest.mark.parametrize("name", EXIT_CASES)
def test_fp64_oracle_close_to_reference(oracle, name):
    g = golden("ref_exit_%s.npz" % name)
    from oracle.oracle import make_param
    fov, nx, ny = float(g["fov"]), int(g["nx"]), int(g["ny"])
    param = make_param(fov, fov, nx, ny, float(g["v0"]), float(g["deltaz"]))
    pix = oracle.calculate(param, *case(g), fov, fov, nmode=int(g["nmode"]), fp64=True)
    # the reference's own FP32 rounding error, well inside the 1e-4 budget
    assert rel_l2(g["pix"], pix) < 1e-5


def test_slice_counts(oracle):
    # C1: 64 A box in 2 A slices; C2: 160 A box in 1 A slices (autoslic.cpp:756)
    assert oracle.slice_count(2.0, 64.0) == 32
    assert oracle.slice_count(1.0, 160.0) == 160
    assert oracle.slice_count(1.25, 100.0) == 80


def test_slice_assign_consistent(oracle):
    s = sp.plain_specimen(1001)
    _, _, _, zs, _ = oracle.sort_by_z(s.Znum, s.x, s.y, s.z, s.occ)
    sl, n = oracle.slice_assign(2.0, 64.0, zs)
    assert n == 32
    assert np.all(np.diff(sl) >= 0)
    # slice k holds (k*dz, (k+1)*dz] in double arithmetic
    for k in range(n):
        zk = zs[sl == k].astype(np.float64)
        if zk.size:
            assert zk.max() < (k + 1) * 2.0 and (k == 0 or zk.min() >= k * 2.0)


def test_empty_specimen_plane_wave_is_exact(oracle):
    from oracle.oracle import make_param
    param = make_param(32.0, 32.0, 64, 64, 200.0, 2.0)
    e = np.zeros(0)
    pix = oracle.calculate(param, e.astype(np.int32), e, e, e, e, 32.0, 32.0)
    assert np.all(pix[..., 0] == 1.0) and np.all(pix[..., 1] == 0.0)


def test_defocus_properties(oracle):
    from oracle.oracle import make_param
    s = sp.plain_specimen(1001)
    param = make_param(64.0, 64.0, 128, 128, 200.0, 2.0)
    pix = oracle.calculate(param, s.Znum[:300], s.x[:300], s.y[:300], s.z[:300], s.occ[:300],
                           64.0, 64.0, fp64=True)
    lam = oracle.wavelength(200.0)
    # R = 0, no aperture: the intensity of the exit wave itself
    i0 = oracle.defocus(pix, 64.0, 64.0, lam, 0.0, fp64=True)
    assert rel_l2(i0, pix[..., 0] ** 2 + pix[..., 1] ** 2) < 1e-12
    # free-space propagation is unitary: total intensity is kept
    i1 = oracle.defocus(pix, 64.0, 64.0, lam, 250.0, fp64=True)
    assert abs(i1.sum() / i0.sum() - 1.0) < 1e-12
    assert rel_l2(i1, i0) > 1e-3  # and it does change the image


def stack_params(nx, ny, S, ax=16.0, aobj=0.0, cs3=0.0):
    from oracle.oracle import StackParams
    p = StackParams()
    p.nx, p.ny, p.ax, p.by, p.v0, p.deltaz, p.nslices = nx, ny, ax, ax * ny / nx, 200.0, 1.0, S
    p.aobj, p.cs3 = aobj, cs3
    return p


def test_stack_adjoint_matches_central_differences(oracle):
    """The FP64 adjoint of the potential-stack multislice against central
    finite differences of its own loss (relative error <= 1e-6 per voxel)."""
    p = stack_params(32, 32, 6, aobj=0.02, cs3=1e6)
    v = sp.potential_stack(1, 6, 32, 32, seed=7)[0].astype(np.float64)
    rp = np.array([5.0, 40.0])
    T = oracle.stack_images(p, sp.perturbed(v, seed=8), rp).astype(np.float32)
    g, L = oracle.stack_adjoint(p, v, rp, T)
    assert abs(L / oracle.stack_loss(p, v, rp, T) - 1.0) < 1e-12
    rng = np.random.default_rng(9)
    gmax = np.abs(g).max()
    vox, fds = [], []
    for _ in range(12):
        k, i, j = rng.integers(0, 6), rng.integers(0, 32), rng.integers(0, 32)
        h = 1e-3 * max(1.0, abs(v[k, i, j]))
        vp = v.copy()
        vp[k, i, j] += h
        vm = v.copy()
        vm[k, i, j] -= h
        fd = (oracle.stack_loss(p, vp, rp, T) - oracle.stack_loss(p, vm, rp, T)) / (2 * h)
        assert abs(fd - g[k, i, j]) <= 1e-6 * max(abs(fd), 1e-3 * gmax)
        vox.append((k, i, j))
        fds.append(fd)
    # the incremental finite differences (base waves reused, threads) agree
    fast = oracle.stack_fd(p, v, rp, T, vox, nthreads=3)
    assert np.allclose(fast, fds, rtol=1e-6, atol=1e-9 * gmax)  # FD rounding ~1e-8


def test_stack_images_free_space_is_unitary(oracle):
    p = stack_params(32, 64, 4)
    v = sp.potential_stack(1, 4, 32, 64, seed=3)[0]
    im = oracle.stack_images(p, v, [0.0, 300.0])
    # no aperture: the propagator and the free-space step keep the total intensity
    # once the band limit has acted (the transmission is not unitary after it)
    assert abs(im[1].sum() / im[0].sum() - 1.0) < 1e-12
    assert rel_l2(im[1], im[0]) > 1e-4


def test_stack_of_atom_potentials_reproduces_orientation_images(oracle):
    """The potential-stack model fed with the atom path's own per-slice
    potentials gives that path's images (FP64 both; defocus measured from the
    box centre there, from the exit face here)."""
    from oracle.oracle import SeriesParams, StackParams
    spec = sp.random_specimen(300, 32.0, 6.0, 26.0, 1012)
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    sr = SeriesParams()
    sr.ax, sr.ctblengthz, sr.nx, sr.ny, sr.v0, sr.deltaz = 32.0, 32.0, 64, 64, 300.0, 2.0
    sr.aobj, sr.cs3, sr.max_slices = 0.02, 1e6, -1
    defoci = np.array([0.0, 250.0])
    for angY in (0.0, 0.6):
        v, kept = oracle.orientation_potential(sr, *atoms, 0.2, angY)
        ref, k = oracle.orientation(sr, *atoms, 0.2, angY, defoci, fp64=True)
        assert kept == k
        p = StackParams()
        p.nx, p.ny, p.ax, p.by, p.v0, p.deltaz = 64, 64, 32.0, 32.0, 300.0, 2.0
        p.nslices, p.aobj, p.cs3 = v.shape[0], 0.02, 1e6
        im = oracle.stack_images(p, v, defoci - 0.5 * 32.0)
        assert rel_l2(im, ref) < 1e-12


@pytest.mark.parametrize("name", ["dw_128", "wobble_128"])
def test_thermal_branches_match_reference_bit_for_bit(oracle, name):
    """The oracle's thermal calculate() against the reference's own build:
    Debye-Waller (nwobble 1) and random displacements (nwobble 3)."""
    from oracle.oracle import make_param, pNWOBBLE, pTEMPER
    g = golden("ref_thermal_%s.npz" % name)
    n, nx = int(g["natom"]), int(g["nx"])
    s = sp.plain_specimen(1001)
    wob = (0.05 + 0.025 * (np.arange(n) % 3)).astype(np.float32)
    param = make_param(64.0, 64.0, nx, nx, 200.0, 2.0)
    param[pNWOBBLE], param[pTEMPER] = float(g["nwobble"]), float(g["temperature"])
    atoms = (s.Znum[:n], s.x[:n], s.y[:n], s.z[:n], s.occ[:n])
    pix, seed = oracle.calculate_thermal(param, *atoms, wob, 64.0, 64.0, iseed=int(g["iseed0"]))
    assert np.array_equal(pix, g["pix"])
    assert seed == int(g["iseed1"])
    pix64, _ = oracle.calculate_thermal(param, *atoms, wob, 64.0, 64.0, iseed=int(g["iseed0"]),
                                        fp64=True)
    assert rel_l2(g["pix"], pix64) < 1e-5
    # the thermal branch changes the result
    plain = oracle.calculate(param, *atoms, 64.0, 64.0)
    assert rel_l2(plain, pix64) > 1e-4


def test_image_plane_rotation_and_shift_definitions(oracle):
    """The oracle's image-plane operations: a whole-pixel shift moves the field
    exactly, a quarter turn about a pixel centre permutes pixels, zero does
    nothing."""
    import ctypes as C
    n = 32
    rng = np.random.default_rng(5)
    amp = rng.standard_normal((n, n, 2))
    L = oracle.L
    L.mo_image_plane_f64.argtypes = [np.ctypeslib.ndpointer(np.float64), C.c_int, C.c_int,
                                     C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.c_int, C.c_int]
    a = amp.copy()
    L.mo_image_plane_f64(a.reshape(-1), n, n, 0.5, 0.5, 8.0, 8.0, 0.0, 0, 0)
    assert np.array_equal(a, amp)
    a = amp.copy()
    L.mo_image_plane_f64(a.reshape(-1), n, n, 0.5, 0.5, 8.0, 8.0, 0.0, 3, -2)
    assert np.array_equal(a[3:, :n - 2], amp[:n - 3, 2:])
    edge = np.ones((n, n), bool)
    edge[5:n - 5, 5:n - 5] = False
    assert np.allclose(a[0, 0], amp[edge].mean(axis=0))
    a = amp.copy()
    L.mo_image_plane_f64(a.reshape(-1), n, n, 0.5, 0.5, 8.0, 8.0, np.pi / 2, 0, 0)
    # out(ix, iy) = in(c + R(-90)(p - c)): in pixels (cx = cy = 16) -> (16 + (iy-16), 16 - (ix-16))
    ix, iy = 20, 9
    assert np.allclose(a[ix, iy], amp[16 + (iy - 16), 16 - (ix - 16)], atol=1e-12)
