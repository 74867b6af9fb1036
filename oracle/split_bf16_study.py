"""Would split-BF16 tensor-core DFT stages keep the multislice accurate enough?
TEST INFRASTRUCTURE ONLY (an accuracy study run by tests/test_split_bf16_study.py).

The optional tensor-core form of the line transforms evaluates each DFT stage
as a matrix product D X on the tensor cores: D (the complex DFT matrix of the
stage) and X (the data) in BF16, products exact, sums in FP32.  BF16 keeps 8
significant bits, so the operands are split -- x = x_hi + x_lo (+ x_lo2) with
each part rounded to BF16 -- and the product is the sum of the partial
products that matter:
  3-term:  D_hi X_hi + D_hi X_lo + D_lo X_hi               (~16 bits)
  6-term:  the same with a third part of each, every pair whose weight is
           above 2^-24 (hi.hi, hi.lo, lo.hi, hi.lo2, lo.lo, lo2.hi)
This module emulates that arithmetic on the host -- BF16 rounding of every
operand part, products and sums in float64, each product rounded to FP32 as
the accumulator holds it -- inside the slice loop of the multislice (the FP64
oracle's per-slice potentials, t = exp(i sigma v), 2/3 band limit, Fresnel
propagator; TemsimLibrary/autoslic.cpp:756-830), with every 2D FFT done as
row and column transforms of two DFT stages (32 x n/32, the twiddles between
them in FP32), and reports the exit wave's relative L2 distance from the same
loop in float64.  The FP32 form (every stage in FP32) is reported beside it.
"""
import numpy as np


def bf16(x):
    """x (float32 array) rounded to the nearest BF16 value (ties to even),
    returned as float32."""
    x = np.ascontiguousarray(x, np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    lsb = (b >> 16) & 1
    b = ((b + 0x7FFF + lsb) >> 16) << 16
    return b.astype(np.uint32).view(np.float32)


def split(x, parts):
    """x (float32) as `parts` BF16 pieces whose sum approximates x."""
    out, r = [], np.asarray(x, np.float32)
    for _ in range(parts):
        p = bf16(r)
        out.append(p)
        r = (r - p).astype(np.float32)
    return out


# partial products kept by each form (indices into the operand splits)
TERMS = {3: ((0, 0), (0, 1), (1, 0)),
         6: ((0, 0), (0, 1), (1, 0), (0, 2), (1, 1), (2, 0))}


def real_matmul(A, B, form):
    """A @ B (real float32 matrices) in the emulated arithmetic."""
    if form == "fp32":
        return (A.astype(np.float64) @ B.astype(np.float64)).astype(np.float32)
    terms = TERMS[form]
    parts = 1 + max(max(i, j) for i, j in terms)
    As, Bs = split(A, parts), split(B, parts)
    acc = np.zeros((A.shape[0], B.shape[1]), np.float64)
    for i, j in terms:
        acc += (As[i].astype(np.float64) @ Bs[j].astype(np.float64))
    return acc.astype(np.float32)


def complex_matmul(Dr, Di, Xr, Xi, form):
    """(Dr + i Di) @ (Xr + i Xi) as one real product of the stacked operands."""
    A = np.block([[Dr, -Di], [Di, Dr]]).astype(np.float32)
    Y = real_matmul(A, np.vstack([Xr, Xi]).astype(np.float32), form)
    n = Dr.shape[0]
    return Y[:n], Y[n:]


def dft_matrix(n, sign):
    k = np.arange(n)
    a = sign * 2.0 * np.pi * np.outer(k, k) / n
    return np.cos(a).astype(np.float32), np.sin(a).astype(np.float32)


def line_dft(x, sign, form):
    """DFT along axis 1 of x (complex64 [lines, n]) as two stages: 32-point DFTs
    of the strided sub-sequences, FP32 twiddles, n/32-point DFTs."""
    lines, n = x.shape
    r1 = min(32, n)
    r2 = n // r1
    # x[j1 + r2 j2] -> stage 1 over j2 (r1 points) for each j1
    xs = x.reshape(lines, r1, r2)  # [line, j2, j1]
    Dr, Di = dft_matrix(r1, sign)
    Xr = np.transpose(xs.real, (1, 0, 2)).reshape(r1, -1)
    Xi = np.transpose(xs.imag, (1, 0, 2)).reshape(r1, -1)
    Yr, Yi = complex_matmul(Dr, Di, Xr, Xi, form)  # [k1, line*j1]
    Y = (Yr + 1j * Yi).reshape(r1, lines, r2).astype(np.complex64)
    # twiddles exp(sign 2 pi i j1 k1 / n), FP32
    k1 = np.arange(r1)[:, None, None]
    j1 = np.arange(r2)[None, None, :]
    tw = np.exp(sign * 2j * np.pi * k1 * j1 / n).astype(np.complex64)
    Y = (Y * tw).astype(np.complex64)
    if r2 == 1:
        return np.transpose(Y[:, :, 0], (1, 0))
    # stage 2 over j1 (r2 points): X[k1 + r1 k2]
    D2r, D2i = dft_matrix(r2, sign)
    Zr = np.transpose(Y.real, (2, 1, 0)).reshape(r2, -1)
    Zi = np.transpose(Y.imag, (2, 1, 0)).reshape(r2, -1)
    Or, Oi = complex_matmul(D2r, D2i, Zr, Zi, form)  # [k2, line*k1]
    O = (Or + 1j * Oi).reshape(r2, lines, r1)
    return np.transpose(O, (1, 0, 2)).reshape(lines, r2 * r1).astype(np.complex64)


def fft2(x, sign, form):
    """Unnormalised 2D DFT (sign +1: the reference's forward cfpix::fft)."""
    if form == "fp64":
        f = np.fft.ifft2 if sign > 0 else np.fft.fft2
        y = f(x)
        return y * (x.size if sign > 0 else 1.0)
    y = line_dft(x.astype(np.complex64), sign, form)
    return line_dft(y.T.copy(), sign, form).T.copy()


def multislice(v, sigma, kx2, ky2, k2max, prop_x, prop_y, form):
    """Exit wave of the slice loop on per-slice potentials v[S, nx, ny]: in the
    given arithmetic ('fp64', 'fp32' or the split-BF16 forms 3 and 6)."""
    nx, ny = v.shape[1], v.shape[2]
    cdt = np.complex128 if form == "fp64" else np.complex64
    mask = (kx2[:, None] + ky2[None, :]) < k2max
    prop = (prop_x[:, None] * prop_y[None, :]) * mask
    psi = np.ones((nx, ny), cdt)
    inv = 1.0 / (nx * ny)
    for k in range(v.shape[0]):
        if np.any(v[k] != 0):
            t = np.exp(1j * sigma * v[k]).astype(cdt)
            t = (fft2(mask * fft2(t, +1, form), -1, form) * inv).astype(cdt)
            psi = (psi * t).astype(cdt)
        psi = (fft2((prop * fft2(psi, +1, form)).astype(cdt), -1, form) * inv).astype(cdt)
    return psi


def study(oracle, n=128, fov=64.0, v0=200.0, dz=2.0, natom=600, seed=1001, forms=("fp32", 3, 6)):
    """Relative L2 exit-wave error of each arithmetic form against float64, on
    the plain specimen (its first `natom` atoms) at angle 0."""
    from oracle.oracle import SeriesParams
    from utr_public_gb300 import specimen as sp
    s = sp.plain_specimen(seed)
    atoms = (s.Znum[:natom], s.x[:natom], s.y[:natom], s.z[:natom], s.occ[:natom])
    p = SeriesParams()
    p.ax, p.ctblengthz, p.nx, p.ny, p.v0, p.deltaz = fov, fov, n, n, v0, dz
    p.max_slices, p.min_slice = -1, 0
    v, _ = oracle.orientation_potential(p, *atoms, 0.0, 0.0)
    lam = oracle.wavelength(v0)
    sigma = oracle.sigma(v0) / 1000.0
    k, k2, _ = oracle.freqn(n, fov)
    kmax = 0.5 * n / fov
    k2max = (2.0 / 3.0 * kmax) ** 2
    ph = np.pi * dz * lam * k2.astype(np.float64)
    px = np.exp(-1j * ph)
    ref = multislice(v, sigma, k2, k2, k2max, px, px, "fp64")
    out = {}
    for f in forms:
        got = multislice(v, sigma, k2, k2, k2max, px, px, f)
        out[str(f)] = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    out["slices"] = int(v.shape[0])
    out["grid"] = n
    return out
