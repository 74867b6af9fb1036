"""Generate the golden fixtures in tests/golden/ from the reference's own code.

The reference (timg021/UTR_public) ships no tests or golden vectors, so the
fixtures come from its TemsimLibrary sources compiled here unmodified
(oracle/_ref, built by `make -C oracle ref`, linked with the oracle's
FFTW-API shim).  The reference tree and that build exist only where this
script runs; the fixtures travel with the repository.

    python tests/golden/make_golden.py

Fixtures (seeded synthetic specimens, see utr_public_gb300/specimen.py):
  ref_physics.npz   wavelength/sigma, freqn grids, vzatomLUT samples, bessk0
  ref_sort.npz      sortByZ permutation of the 2000-atom specimen
  ref_exit_*.npz    exit waves of autoslic::calculate (coherent branch)
  ref_thermal_*.npz exit waves of its thermal branches (lwobble = 1)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from utr_public_gb300 import specimen as sp  # noqa: E402

CASES = {
    # name: (natom subset, fov, nx, ny, v0, deltaz, nmode, seed)
    "c1_128": (600, 64.0, 128, 128, 200.0, 2.0, 0, 1001),
    "c1_256": (2000, 64.0, 256, 256, 200.0, 2.0, 0, 1001),
    "rect_64x128": (300, 64.0, 64, 128, 300.0, 1.5, 0, 1007),
    "proj_64": (200, 64.0, 64, 64, 200.0, 2.0, 1, 1008),
}


THERMAL = {
    # name: (natom subset of the 64 A plain specimen, grid, nwobble, temperature K, iseed)
    "dw_128": (600, 128, 1, 300.0, -1),
    "wobble_128": (400, 128, 3, 250.0, -12345),
}


def thermal_wobble(natom):
    """Per-atom rms displacement at 300 K (A): 0.05, 0.075, 0.1 cycling, so that
    the slice averages of the Debye-Waller branch depend on which entries count."""
    return (0.05 + 0.025 * (np.arange(natom) % 3)).astype(np.float32)


def case_specimen(natom, seed):
    s = sp.plain_specimen(seed)
    return s.Znum[:natom], s.x[:natom], s.y[:natom], s.z[:natom], s.occ[:natom]


def main():
    orc.build(with_ref=True)
    R = orc.Reference()
    out = {}
    # physics
    kevs = np.array([80.0, 100.0, 200.0, 300.0])
    out["kev"] = kevs
    out["wavelength"] = np.array([R.L.ref_wavelength(k) for k in kevs])
    out["sigma"] = np.array([R.L.ref_sigma(k) for k in kevs])
    xs = np.linspace(1e-3, 25.0, 101)
    out["bessk0_x"] = xs
    out["bessk0"] = np.array([R.L.ref_bessk0(v) for v in xs])
    out["bessi0"] = np.array([R.L.ref_bessi0(v) for v in xs])
    zs = np.array([1, 6, 7, 8, 16, 29, 79, 103], np.int32)
    rsq = np.concatenate([np.geomspace(1e-5, 30.0, 61), [0.0016, 0.5, 9.0]])
    out["lut_Z"] = zs
    out["lut_rsq"] = rsq
    out["lut"] = np.array([[R.vzatomLUT(int(z), float(r)) for r in rsq] for z in zs])
    out["vzatom"] = np.array([[R.L.ref_vzatom(int(z), float(np.sqrt(r))) for r in rsq] for z in zs])
    for n, a in ((64, 64.0), (128, 64.0), (256, 64.0), (1024, 160.0), (100, 37.5)):
        k, k2, xp = R.freqn(n, a)
        out["freqn_%d_k" % n], out["freqn_%d_k2" % n], out["freqn_%d_x" % n] = k, k2, xp
    np.savez_compressed(os.path.join(HERE, "ref_physics.npz"), **out)

    # sort permutation (occ carries the original index, exact in float)
    s = sp.plain_specimen(1001)
    idx = np.arange(s.natom, dtype=np.float32)
    Zs, xs_, ys_, zs_, perm = R.sort_by_z(s.Znum, s.x, s.y, s.z, idx)
    np.savez_compressed(os.path.join(HERE, "ref_sort.npz"), perm=perm.astype(np.int32),
                        zsorted=zs_)

    # exit waves
    for name, (natom, fov, nx, ny, v0, dz, nmode, seed) in CASES.items():
        Z, x, y, z, occ = case_specimen(natom, seed)
        param = orc.make_param(fov, fov, nx, ny, v0, dz)
        pix = R.calculate(param, Z, x, y, z, occ, fov, fov, nmode=nmode)
        np.savez_compressed(os.path.join(HERE, "ref_exit_%s.npz" % name), pix=pix,
                            natom=natom, fov=fov, nx=nx, ny=ny, v0=v0, deltaz=dz, nmode=nmode,
                            seed=seed)
        print("wrote", name, pix.shape)

    # thermal branches of calculate (lwobble = 1): Debye-Waller (nwobble 1) and
    # random displacements (nwobble > 1, the build's gasdev)
    for name, (natom, nx, nwob, temp, seed0) in THERMAL.items():
        Z, x, y, z, occ = case_specimen(natom, 1001)
        wob = thermal_wobble(natom)
        param = orc.make_param(64.0, 64.0, nx, nx, 200.0, 2.0)
        param[orc.pNWOBBLE], param[orc.pTEMPER] = nwob, temp
        pix, seed1 = R.calculate(param, Z, x, y, z, occ, 64.0, 64.0, wobble=wob, lwobble=1,
                                 iseed=seed0)
        np.savez_compressed(os.path.join(HERE, "ref_thermal_%s.npz" % name), pix=pix,
                            natom=natom, nx=nx, nwobble=nwob, temperature=temp, iseed0=seed0,
                            iseed1=seed1)
        print("wrote thermal", name, pix.shape)


if __name__ == "__main__":
    main()
