"""Synthetic specimens and Kirkland XYZ files.

The workloads are seeded synthetic specimens with the shapes the
MsctKirkland tilt-series configurations use: atoms drawn uniformly in a cube
centred in the field of view, atomic numbers C:N:O:S = 0.50:0.17:0.30:0.03,
occupancy 1, no thermal displacement.  ``write_xyz``/``read_xyz`` use
Kirkland's XYZ layout as read by the reference's ReadXYZcoord
(TemsimLibrary/slicelib.cpp:2242-2374): a description line, a line
``ax by cz``, then ``Z x y z occ wobble`` per atom, ended by ``-1``.
"""
from dataclasses import dataclass

import numpy as np

Z_MIX = ((6, 0.50), (7, 0.17), (8, 0.30), (16, 0.03))


@dataclass
class Specimen:
    Znum: np.ndarray   # int32 [natom]
    x: np.ndarray      # float32 [natom], Angstrom
    y: np.ndarray
    z: np.ndarray
    occ: np.ndarray
    wobble: np.ndarray
    fov: float         # field of view = box edge (ctblength), Angstrom

    @property
    def natom(self):
        return int(self.x.shape[0])


def random_specimen(natom, fov, lo, hi, seed):
    """natom atoms uniform in [lo, hi]^3 inside a fov^3 box (seeded)."""
    rng = np.random.default_rng(seed)
    zs = np.array([z for z, _ in Z_MIX], np.int32)
    ps = np.array([p for _, p in Z_MIX])
    Znum = rng.choice(zs, size=natom, p=ps / ps.sum()).astype(np.int32)
    xyz = rng.uniform(lo, hi, size=(3, natom)).astype(np.float32)
    ones = np.ones(natom, np.float32)
    return Specimen(Znum, xyz[0].copy(), xyz[1].copy(), xyz[2].copy(), ones,
                    np.zeros(natom, np.float32), float(fov))


def plain_specimen(seed=1001):
    """2000 atoms in [7, 57]^3 inside a 64 Angstrom box (single orientation case)."""
    return random_specimen(2000, 64.0, 7.0, 57.0, seed)


def tilt_specimen(seed=1002):
    """20000 atoms in [20, 140]^3 inside a 160 Angstrom box (tilt-series case)."""
    return random_specimen(20000, 160.0, 20.0, 140.0, seed)


def phonon_displacements(spec, nconfig, rms=0.08, seed=1003):
    """Per-configuration isotropic Gaussian displacements [nconfig, 3, natom]."""
    out = np.empty((nconfig, 3, spec.natom), np.float32)
    for c in range(nconfig):
        rng = np.random.default_rng((seed, c))
        out[c] = rng.normal(0.0, rms, size=(3, spec.natom)).astype(np.float32)
    return out


def uneven_batch(nspec=64, seed=1004):
    """Specimens of log-uniform atom count (5e3..2e5) at 0.1 atoms/A^3, field of
    view sqrt(2)*edge, grids drawn from {256,512,1024,2048}, 1..90 angles."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(nspec):
        natom = int(round(np.exp(rng.uniform(np.log(5e3), np.log(2e5)))))
        edge = (natom / 0.1) ** (1.0 / 3.0)
        fov = float(np.float32(np.sqrt(2.0) * edge))
        n = int(rng.choice([256, 512, 1024, 2048]))
        nang = int(rng.integers(1, 91))
        lo = 0.5 * (fov - edge)
        spec = random_specimen(natom, fov, lo, lo + edge, seed * 1000 + i)
        out.append((spec, n, nang))
    return out


def write_xyz(path, spec, description="synthetic specimen"):
    with open(path, "w") as f:
        f.write(description + "\n")
        f.write("%.6f %.6f %.6f\n" % (spec.fov, spec.fov, spec.fov))
        for i in range(spec.natom):
            f.write("%d %.7g %.7g %.7g %.7g %.7g\n" % (spec.Znum[i], spec.x[i], spec.y[i],
                                                      spec.z[i], spec.occ[i], spec.wobble[i]))
        f.write("-1\n")


def read_xyz(path):
    with open(path) as f:
        f.readline()
        ax, by, cz = (float(v) for v in f.readline().split()[:3])
        rows = []
        for line in f:
            parts = line.split()
            if not parts:
                continue
            z = int(parts[0])
            if z <= 0:
                break
            vals = [float(v) for v in parts[1:6]] + [0.0] * (5 - len(parts[1:6]))
            rows.append((z, *vals))
    a = np.array(rows, dtype=np.float64).reshape(-1, 6)
    f32 = lambda c: a[:, c].astype(np.float32)
    return Specimen(a[:, 0].astype(np.int32), f32(1), f32(2), f32(3), f32(4), f32(5),
                    float(max(ax, by, cz)))


def potential_stack(nunits, nslices, nx, ny, blobs=3, peak=60.0, width=2.0, seed=1005):
    """Synthetic per-slice projected potentials v[nunits, nslices, nx, ny]
    (V*Angstrom, float32): `blobs` periodic Gaussian peaks per slice, the
    shape a splatted atom gives, for the potential-stack and adjoint paths."""
    rng = np.random.default_rng(seed)
    X, Y = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    v = np.zeros((nunits, nslices, nx, ny), np.float64)
    for u in range(nunits):
        for k in range(nslices):
            for _ in range(blobs):
                cx, cy = rng.uniform(0, nx), rng.uniform(0, ny)
                dx = (X - cx + nx / 2) % nx - nx / 2
                dy = (Y - cy + ny / 2) % ny - ny / 2
                v[u, k] += peak * np.exp(-(dx * dx + dy * dy) / (2 * width * width))
    return v.astype(np.float32)


def perturbed(v, rel=0.01, seed=1005):
    """v * (1 + rel N(0, 1)): the potential whose images are the adjoint's target."""
    rng = np.random.default_rng(seed)
    return (v * (1.0 + rel * rng.standard_normal(v.shape))).astype(np.float32)
