"""Generate tests/golden/ref_utr.npz from the reference's own UTR.h templates.

The reference ships no tests or golden vectors for its UTR reconstruction, so
the fixtures come from PhaseRetrieval/UTR.h (CT_3Dgridding, CTFcorrection3D,
InverseMLaplacian3D) compiled here unmodified against the XArray stand-ins
of oracle/utr_include (oracle/_ref/libutr_ref.so, `make -C oracle ref`).
The reference tree exists only where this script runs; the fixture travels
with the repository.

    python tests/golden/make_golden_utr.py

Every case stores its seeded inputs and the reference's float outputs.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402

# gridding: (images, nx, ny, nz, angles deg (Z, Y'), escc, centre shift)
GRID = {
    "flat": (2, 16, 16, 16, [(0.0, 17.0), (0.0, 71.0)], 0, (0.0, 0.0, 0.0)),
    "escc_shift": (3, 16, 16, 8, [(12.0, 33.0), (-40.0, 95.0), (5.0, 150.0)], 1, (0.4, -0.3, 0.2)),
}
# CTF: (defocus, q2max, cs3, cs5 (length units), sigma, epsilon, escc)
CTF = {
    "plain": (120.0, 0.0, 0.0, 0.0, 0.05, 1e-3, 0),
    "escc_cs_auto_eps": (-80.0, 2.0, 1.2e7, 3e9, 0.1, 0.0, 1),
}
WL = 0.0196875
XST = 0.5


def geometry(nx, ny, nz):
    xlo, ylo = -0.5 * XST * nx, -0.5 * XST * ny
    zlo = -0.5 * XST * nz
    fxst, fyst, fzst = 1 / (XST * nx), 1 / (XST * ny), 1 / (XST * nz)
    fx = tuple(np.float32(v) for v in (-fxst * (nx // 2), fxst, -fyst * (ny // 2), fyst,
                                       -fzst * (nz // 2), fzst))
    box = (zlo, zlo + XST * nz, ylo, ylo + XST * ny, xlo, xlo + XST * nx)
    return fx, box


def main():
    ref = orc.UtrReference()
    out = {}
    rng = np.random.default_rng(2024)
    for name, (nimg, nx, ny, nz, angles, escc, shift) in GRID.items():
        fx, _ = geometry(nx, ny, nz)
        k2 = rng.standard_normal((nimg, ny, nx, 2)).astype(np.float32)
        v3 = np.zeros((nz, ny, nx, 2), np.float32)
        s3 = np.zeros((nz, ny, nx), np.float32)
        fcs = []
        for a, (az, ay) in enumerate(angles):
            angZ, angY = np.deg2rad(az), np.deg2rad(ay)
            dxc, dyc, dzc = shift
            tpi = 2 * np.pi
            cy, sy, cz, sz = np.cos(angY), np.sin(angY), np.cos(angZ), np.sin(angZ)
            fa = np.float32([tpi * (dxc * (1 - cy * cz) - dyc * sz + dzc * sy * cz),
                             tpi * (dxc * cy * sz + dyc * (1 - cz) - dzc * sy * sz),
                             tpi * (-dxc * sy + dzc * (1 - cy))])
            fc = np.zeros(6, np.float32)
            fc[1::2] = -fa
            fcs.append(fc)
            ref.grid(k2[a], nz, angY, angZ, fx, fc, WL, any(shift), escc, v3, s3)
        out["grid_%s_k2" % name] = k2
        out["grid_%s_fc" % name] = np.array(fcs)
        out["grid_%s_v3" % name] = v3
        out["grid_%s_samp3" % name] = s3
    nz, ny, nx = 16, 16, 16
    _, box = geometry(nx, ny, nz)
    vin = rng.standard_normal((nz, ny, nx, 2)).astype(np.float32)
    out["vol_in"] = vin
    for name, (df, q2, cs3, cs5, sig, eps, escc) in CTF.items():
        out["ctf_%s" % name] = ref.ctf3d(vin.copy(), WL, box, df, q2, cs3, cs5, sig, eps, escc)
    out["invlap"] = ref.invlap3d(vin.copy(), 8.0, 8.0, 8.3, 0.7, 1.3)
    np.savez_compressed(os.path.join(HERE, "ref_utr.npz"), **out)
    print("wrote ref_utr.npz:", ", ".join(sorted(out)))


if __name__ == "__main__":
    main()
