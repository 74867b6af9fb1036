"""Potential-stack multislice and its adjoint on the GPU (msk_stack_images,
msk_adjoint) against the FP64 oracle and central finite differences.

Tolerances (relative L2):
  * images vs the FP64 oracle:                          1e-5
  * dL/dv vs the FP64 oracle adjoint:                   1e-3
  * dL/dv vs central finite differences of the FP64
    oracle loss, over the sampled voxels:               1e-3
  * loss vs the FP64 oracle loss:                       1e-4
dL/dv is linear in the residuals I - T.  A 1% perturbation of the potential
moves the images by only ~1e-4..1e-3 of their value, so the residuals carry
the forward pass's error in I magnified by 1e3..1e4.  The stack path keeps
its waves in the scattered form (psi = 1 + phi), which leaves ~1e-7 relative
error in I instead of the ~1e-6 of FP32 waves psi; dL/dv then stays within
1e-3 of the FP64 adjoint and of central differences.
"""
import numpy as np
import pytest

from conftest import rel_l2
from utr_public_gb300 import specimen as sp

pytestmark = pytest.mark.gpu


def make_stack(msk, nx, ny, S, ax=16.0, aobj=0.0, cs3=0.0, checkpoint=0, max_batch=0,
               ctilt=(0.0, 0.0)):
    s = msk.Stack()
    s.nx, s.ny, s.ax, s.by, s.v0, s.deltaz = nx, ny, ax, ax * ny / nx, 200.0, 1.0
    s.ctiltx, s.ctilty = ctilt
    s.aobj, s.cs3, s.cs5 = aobj, cs3, 0.0
    s.nslices, s.checkpoint, s.max_batch = S, checkpoint, max_batch
    return s


def oracle_params(s):
    from oracle.oracle import StackParams
    p = StackParams()
    p.nx, p.ny, p.ax, p.by, p.v0, p.deltaz = s.nx, s.ny, s.ax, s.by, s.v0, s.deltaz
    p.ctiltx, p.ctilty, p.nslices, p.aobj, p.cs3, p.cs5 = (s.ctiltx, s.ctilty, s.nslices, s.aobj,
                                                           s.cs3, s.cs5)
    return p


def case(nx, ny, S, nunits, seed):
    v = sp.potential_stack(nunits, S, nx, ny, blobs=4, peak=300.0, seed=seed)
    vt = sp.perturbed(v, seed=seed + 1)
    return v, vt


@pytest.mark.parametrize("nx,ny,S,aobj,cs3,ctilt", [
    (64, 64, 10, 0.0, 0.0, (0.0, 0.0)),
    (64, 128, 7, 0.02, 1e6, (0.0, 0.0)),
    (128, 64, 5, 0.0, 0.0, (0.01, -0.02)),
    (32, 4096, 3, 0.0, 0.0, (0.0, 0.0)),
])
def test_stack_images_match_oracle(ctx, msk, oracle, nx, ny, S, aobj, cs3, ctilt):
    s = make_stack(msk, nx, ny, S, aobj=aobj, cs3=cs3, ctilt=ctilt)
    v, _ = case(nx, ny, S, 3, 11)
    rp = [0.0, 120.0]
    im = ctx.stack_images(s, v, rp)
    p = oracle_params(s)
    for u in range(3):
        ref = oracle.stack_images(p, v[u], rp)
        assert rel_l2(im[u], ref) < 1e-5


@pytest.mark.parametrize("S,checkpoint", [(10, 0), (10, 4), (9, 3), (5, 1), (6, 6)])
def test_adjoint_matches_oracle(ctx, msk, oracle, S, checkpoint):
    nx = ny = 64
    s = make_stack(msk, nx, ny, S, aobj=0.03, checkpoint=checkpoint)
    v, vt = case(nx, ny, S, 2, 21)
    rp = [10.0, 200.0]
    p = oracle_params(s)
    target = np.stack([oracle.stack_images(p, vt[u], rp) for u in range(2)]).astype(np.float32)
    loss, g = ctx.adjoint(s, v, rp, target)
    L64 = 0.0
    for u in range(2):
        gref, Lu = oracle.stack_adjoint(p, v[u], rp, target[u])
        L64 += Lu
        assert rel_l2(g[u], gref) < 1e-3
    assert abs(loss / L64 - 1.0) < 1e-4


def test_adjoint_matches_finite_differences(ctx, msk, oracle):
    """Central differences of the FP64 oracle loss on random voxels."""
    nx = ny = 64
    S = 12
    s = make_stack(msk, nx, ny, S, aobj=0.02, checkpoint=4)
    v, vt = case(nx, ny, S, 1, 31)
    rp = [0.0, 150.0]
    p = oracle_params(s)
    target = oracle.stack_images(p, vt[0], rp).astype(np.float32)[None]
    _, g = ctx.adjoint(s, v, rp, target)
    v64 = v[0].astype(np.float64)
    rng = np.random.default_rng(32)
    # voxels where the gradient is not negligible: on and near the potential peaks
    cand = np.argwhere(np.abs(g[0]) > 0.05 * np.abs(g[0]).max())
    pick = cand[rng.choice(len(cand), size=24, replace=False)]
    fd = []
    for k, i, j in pick:
        h = 1e-3 * max(1.0, abs(v64[k, i, j]))
        vp = v64.copy()
        vp[k, i, j] += h
        vm = v64.copy()
        vm[k, i, j] -= h
        fd.append((oracle.stack_loss(p, vp, rp, target[0]) -
                   oracle.stack_loss(p, vm, rp, target[0])) / (2 * h))
    ours = np.array([g[0][k, i, j] for k, i, j in pick])
    assert rel_l2(ours, np.array(fd)) < 1e-3


def test_adjoint_splatted_specimen_finite_differences(ctx, msk, oracle):
    """The adjoint workload's setting at 128^2: potentials splatted from a
    random specimen, the target from v (1 + 0.01 N(0, 1)), one detector plane;
    dL/dv against the FP64 adjoint and central differences on 128 random
    voxels (within 1e-3 of both)."""
    import os
    spec = sp.random_specimen(600, 32.0, 4.0, 28.0, 1021)
    s = msk.Series()
    s.nx = s.ny = 128
    s.ctblength = s.ctblengthz = 32.0
    s.v0, s.deltaz = 200.0, 1.0
    v, _ = ctx.potential_stack(s, spec.Znum, spec.x, spec.y, spec.z, spec.occ,
                               np.array([0.0, 0.3]), np.array([0.0, 0.7]))
    S = v.shape[1]
    vt = sp.perturbed(v, seed=1022)
    st = make_stack(msk, 128, 128, S, ax=32.0, checkpoint=8)
    rp = [-16.0]
    target = ctx.stack_images(st, vt, rp)
    _, g = ctx.adjoint(st, v, rp, target)
    p = oracle_params(st)
    rng = np.random.default_rng(1023)
    for u in range(2):
        gref, _ = oracle.stack_adjoint(p, v[u], rp, target[u])
        assert rel_l2(g[u], gref) < 1e-3
        vox = np.stack([rng.integers(0, S, 128), rng.integers(0, 128, 128),
                        rng.integers(0, 128, 128)], axis=1)
        fd = oracle.stack_fd(p, v[u], rp, target[u], vox, nthreads=os.cpu_count() or 1)
        ours = np.array([g[u][k, i, j] for k, i, j in vox])
        assert rel_l2(ours, fd) < 1e-3


def test_adjoint_batching_and_device_pointers(ctx, msk, oracle):
    torch = pytest.importorskip("torch")
    nx = ny = 64
    S = 8
    v, vt = case(nx, ny, S, 5, 41)
    rp = [0.0]
    s = make_stack(msk, nx, ny, S, checkpoint=3)
    target = ctx.stack_images(s, vt, rp)
    loss_a, ga = ctx.adjoint(s, v, rp, target)
    s1 = make_stack(msk, nx, ny, S, checkpoint=3, max_batch=2)
    loss_b, gb = ctx.adjoint(s1, v, rp, target)
    assert np.array_equal(ga, gb)  # units are independent: bit-equal in any batch
    assert abs(loss_b / loss_a - 1.0) < 1e-12
    dv = torch.from_numpy(v).cuda()
    dt = torch.from_numpy(target).cuda()
    dg = torch.zeros_like(dv)
    loss_c, _ = ctx.adjoint(s, dv, rp, dt, grad=dg)
    assert np.array_equal(dg.cpu().numpy(), ga)
    assert loss_c == loss_a
    di = torch.zeros((5, 1, nx, ny), dtype=torch.float32, device="cuda")
    ctx.stack_images(s, torch.from_numpy(vt).cuda(), rp, images=di)
    assert np.array_equal(di.cpu().numpy(), target)
    # page-locked host stacks: their slices move through the mapped addresses
    # (one batch, and two batches sharing two staging slots)
    hv = torch.from_numpy(v).pin_memory()
    ht = torch.from_numpy(target).pin_memory()
    for st in (s, s1):
        hg = torch.full(v.shape, -1.0, dtype=torch.float32).pin_memory()
        loss_d, _ = ctx.adjoint(st, hv, rp, ht, grad=hg)
        assert np.array_equal(hg.numpy(), ga)
        assert abs(loss_d / loss_a - 1.0) < 1e-12
    hi = torch.zeros((5, 1, nx, ny), dtype=torch.float32).pin_memory()
    ctx.stack_images(s1, torch.from_numpy(vt).pin_memory(), rp, images=hi)
    assert np.array_equal(hi.numpy(), target)


def test_stack_zero_potential_is_plane_wave(ctx, msk):
    """v = 0: every transmission is 1 and the image exactly 1 (the scattered
    parts tau and phi are exactly zero throughout)."""
    s = make_stack(msk, 32, 32, 4)
    im = ctx.stack_images(s, np.zeros((2, 4, 32, 32), np.float32), [0.0, 50.0])
    assert np.all(im == 1.0)


def test_stack_errors(ctx, msk):
    v = np.zeros((1, 2, 32, 32), np.float32)
    s = make_stack(msk, 32, 32, 0)
    with pytest.raises(msk.MskError) as e:
        ctx.stack_images(s, v, [0.0])
    assert e.value.status == msk.MSK_EINVAL
    s = make_stack(msk, 48, 32, 2)
    with pytest.raises(msk.MskError) as e:
        ctx.stack_images(s, v, [0.0])
    assert e.value.status == msk.MSK_EUNSUPPORTED
    s = make_stack(msk, 32, 32, 2)
    with pytest.raises(msk.MskError) as e:  # the adjoint needs a detector plane
        ctx.adjoint(s, v, [], np.zeros((1, 0, 32, 32), np.float32))
    assert e.value.status == msk.MSK_EINVAL


def test_potential_stack_matches_oracle_and_atom_path(ctx, msk, oracle):
    """msk_potential_stack against the oracle's FP64 slice potentials, and the
    potential-stack images of those potentials against msk_tilt_series."""
    from oracle.oracle import SeriesParams
    spec = sp.random_specimen(800, 64.0, 10.0, 54.0, 1013)
    atoms = (spec.Znum, spec.x, spec.y, spec.z, spec.occ)
    s = msk.Series()
    s.nx = s.ny = 128
    s.ctblength = s.ctblengthz = 64.0
    s.v0, s.deltaz, s.aobj = 300.0, 1.0, 0.02
    angY = np.deg2rad([0.0, 35.0, 120.0])
    angZ = np.array([0.0, 0.4, 0.0])
    v, kept = ctx.potential_stack(s, *atoms, angZ, angY)
    sr = SeriesParams()
    sr.ax, sr.ctblengthz, sr.nx, sr.ny, sr.v0, sr.deltaz = 64.0, 64.0, 128, 128, 300.0, 1.0
    sr.aobj, sr.max_slices = 0.02, -1
    for a in range(3):
        ref, k = oracle.orientation_potential(sr, *atoms, angZ[a], angY[a])
        assert kept[a] == k
        assert rel_l2(v[a], ref) < 1e-5
    defoci = np.array([0.0, 400.0])
    imgs, _ = ctx.tilt_series(s, *atoms, angZ, angY, defoci)
    st = make_stack(msk, 128, 128, v.shape[1], ax=64.0, aobj=0.02)
    st.v0 = 300.0
    im2 = ctx.stack_images(st, v, defoci - 32.0)
    assert rel_l2(im2, imgs) < 1e-5
