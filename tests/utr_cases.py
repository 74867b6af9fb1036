"""Shared inputs and a numpy model for the UTR reconstruction tests.

``complex_inverse_model`` is the GPU path's plan written in numpy: the
Fourier-space stages of the oracle, the x-Nyquist-plane factors that stand
for the Hermitian step, and a centred complex inverse 3D FFT whose real part
is taken -- the tests check it against the oracle's literal restatement
(in-place Hermitian step, then FFTW-style complex-to-real transform).
"""
import numpy as np

from oracle import oracle as orc


def params(nx=32, ny=32, nz=16, xst=0.5, **kw):
    """UTR parameters for a volume of nx x ny x nz voxels of edge xst (TEM,
    300 keV, CTF-3D, no noise filter unless overridden)."""
    p = orc.UtrParams(modality=0, f1=1.0, f2=0.0, nx=nx, ny=ny, xst=xst,
                      zlo=-0.5 * xst * nz, zhi=0.5 * xst * nz, wl=0.0196875, ctf_mode=4,
                      asigma=0.1, epsilon=1e-3, nsr=0.0)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def tilt_angles(n, span=180.0, az=0.0):
    return np.array([[az, span * a / n] for a in range(n)], np.float64)


def images(p, nangles, seed=0, contrast=0.05):
    """Positive flat-field-like images [nangles, ny, nx]: 1 + smooth structure."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:p.ny, 0:p.nx]
    out = np.empty((nangles, p.ny, p.nx), np.float32)
    for a in range(nangles):
        g = np.zeros((p.ny, p.nx))
        for _ in range(6):
            cx, cy = rng.uniform(0.3, 0.7, 2) * (p.nx, p.ny)
            s = rng.uniform(1.0, 3.0)
            g += rng.uniform(-1, 1) * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * s * s))
        out[a] = 1.0 + contrast * g + 0.002 * rng.standard_normal(g.shape)
    return out


def complex_inverse_model(o, p, angles, defocus, v3, samp3):
    g = o.utr_geom(p, angles, defocus)
    nz, ny, nx = g.nz, p.ny, p.nx
    V = np.array(v3, np.float64)
    x = np.asarray(samp3, np.float64)
    nsr = p.nsr * np.sqrt(nx * ny)
    with np.errstate(divide="ignore", invalid="ignore"):
        s = np.where(x == 0, 0.0, 1.0 / x)
        if nsr:
            y = np.hypot(V[..., 0], V[..., 1]) / (nsr * np.sqrt(x))
            s = np.where(x == 0, 0.0, s * (0.5 + np.arctan(100 * (y - 1.414213562373)) / np.pi))
    V = V * s[..., None]
    box = (g.zlo, g.zhi, g.ylo, g.yhi, g.xlo, g.xhi)
    if g.zout_aver != 0 and p.ctf_mode == 4:
        o.utr_ctf3d(V, g.wl, box, g.zout_aver, g.k2maxo, g.cs3, g.cs5, p.asigma, p.epsilon, p.escc)
    if g.zout_aver != 0 and p.ctf_mode == 2:
        alpha = -4 * np.pi * p.asigma / (g.zout_aver * g.wl)
        norm = -alpha * np.sqrt(1 + p.asigma ** 2) / p.asigma
        o.utr_invlap3d(V, g.zhi - g.zlo, g.yhi - g.ylo, g.xhi - g.ylo, alpha, norm)
    if p.inv_laplace and p.ctf_mode not in (1, 2):
        o.utr_invlap3d(V, g.zhi - g.zlo, g.yhi - g.ylo, g.xhi - g.ylo, p.epsilon, p.epsilon)
    Z = V[..., 0] + 1j * V[..., 1]
    P = Z[:, :, 0].copy()
    for k in range(nz):
        ka = 0 if k == 0 else nz - k
        for j in range(ny):
            ja = 0 if j == 0 else ny - j
            f = 1.0 if (k, j) == (ka, ja) else (0.75 if (k, j) < (ka, ja) else 1.25)
            Z[k, j, 0] = P[k, j] * f
    sg = lambda n: (-1.0) ** np.arange(n)  # noqa: E731
    M = sg(nz)[:, None, None] * sg(ny)[None, :, None] * sg(nx)[None, None, :]
    R = (np.fft.ifftn(Z * M) * M).real
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    kk2 = 0 if (g.rot_z_only or g.rot_z2_only) else (k - g.kc) ** 2
    jj2 = kk2 if g.rot_y_only else (j - g.jc) ** 2 + kk2
    ii2 = (i - g.ic) ** 2 + jj2
    r2 = lambda c, n: c * c if c <= n // 2 else (n - c) ** 2  # noqa: E731
    nxR2, nyR2, nzR2 = r2(g.ic, nx), r2(g.jc, ny), r2(g.kc, nz)
    if g.rot_y_only:
        nR2 = min(nxR2, nzR2)
    elif g.rot_z_only or g.rot_z2_only:
        nR2 = min(nxR2, nyR2)
    else:
        nR2 = min(nxR2, nyR2, nzR2)
    dtemp = 2.0 / (g.kc ** 2 + g.jc ** 2 + g.ic ** 2)
    if p.modality == 0:
        fnorm = g.ee * g.wl / (2 * np.pi * np.sqrt(1 + p.asigma ** 2) * g.xst)
    else:
        fnorm = p.asigma * g.wl / (4 * np.pi * np.sqrt(1 + p.asigma ** 2) * g.xst)
    return np.where(ii2 > nR2, 0.0, R * np.exp(dtemp * ii2) * fnorm)
