"""ctypes access to the test oracle.  TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only as the reference the GPU results are compared with (or
the timed CPU baseline).  The
shipped package never imports it.

* ``Oracle`` wraps ``oracle/liboracle.so``, the C restatement of the
  reference's hot path (msk_oracle.c): FP32 mirror and FP64 oracle.
* ``Reference`` wraps ``oracle/_ref/libautoslic_ref.so``, the reference's own
  TemsimLibrary sources compiled here (only where the reference tree exists).
* ``UtrReference`` wraps ``oracle/_ref/libutr_ref.so``, the reference's own
  PhaseRetrieval/UTR.h templates compiled here.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_ORACLE = os.path.join(HERE, "liboracle.so")
LIB_REF = os.path.join(HERE, "_ref", "libautoslic_ref.so")
LIB_UTR_REF = os.path.join(HERE, "_ref", "libutr_ref.so")
# The reference tree (timg021/UTR_public sources) for the recipe that compiles
# its own code: MSK_REFERENCE_TREE, or the tree a previous build recorded.
REF_RECORD = os.path.join(HERE, "_ref", "tree.txt")

# param[] offsets (slicelib.hpp:142-240)
pXCTILT, pYCTILT, pDEFOCUS, pENERGY, pOAPERT = 9, 10, 11, 16, 17
pDELTAZ, pAX, pBY, pNX, pNY = 30, 101, 102, 104, 105
pNWOBBLE, pTEMPER = 111, 120
NPARAM = 200

_fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def reference_tree(tree=None):
    """The reference source tree to compile from, or None: `tree`, else the
    MSK_REFERENCE_TREE environment variable, else the tree recorded by the last
    build of oracle/_ref; only a tree that holds TemsimLibrary counts."""
    cands = [tree, os.environ.get("MSK_REFERENCE_TREE")]
    if os.path.exists(REF_RECORD):
        with open(REF_RECORD) as f:
            cands.append(f.read().strip())
    for t in cands:
        if t and os.path.isdir(os.path.join(t, "TemsimLibrary")):
            return t
    return None


def build(with_ref=None, tree=None):
    """Compile liboracle.so, and oracle/_ref from the reference tree (see
    reference_tree) when there is one; with_ref=True requires it."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    ref = reference_tree(tree)
    if with_ref and ref is None:
        raise RuntimeError("the reference tree is needed: set MSK_REFERENCE_TREE")
    if ref is not None and with_ref is not False:
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + ref], check=True)
        with open(REF_RECORD, "w") as f:
            f.write(ref + "\n")


class SeriesParams(C.Structure):
    _fields_ = [("ax", C.c_float), ("ctblengthz", C.c_float), ("nx", C.c_int), ("ny", C.c_int),
                ("v0", C.c_float), ("deltaz", C.c_float), ("aobj", C.c_float),
                ("cs3", C.c_double), ("cs5", C.c_double), ("dxc", C.c_double),
                ("dyc", C.c_double), ("dzc", C.c_double), ("nmode", C.c_int),
                ("max_slices", C.c_int), ("min_slice", C.c_int)]


def make_param(ax, by, nx, ny, v0, deltaz, ctiltx=0.0, ctilty=0.0, aobj=0.0):
    p = np.zeros(NPARAM, np.float32)
    p[pAX], p[pBY], p[pNX], p[pNY] = ax, by, nx, ny
    p[pENERGY], p[pDELTAZ], p[pXCTILT], p[pYCTILT], p[pOAPERT] = v0, deltaz, ctiltx, ctilty, aobj
    return p


def _atoms(Znum, x, y, z, occ):
    return (np.ascontiguousarray(Znum, np.int32), np.ascontiguousarray(x, np.float32),
            np.ascontiguousarray(y, np.float32), np.ascontiguousarray(z, np.float32),
            np.ascontiguousarray(occ, np.float32))


class StackParams(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("ax", C.c_float), ("by", C.c_float),
                ("v0", C.c_float), ("deltaz", C.c_float), ("ctiltx", C.c_float),
                ("ctilty", C.c_float), ("nslices", C.c_int), ("aobj", C.c_float),
                ("cs3", C.c_double), ("cs5", C.c_double)]


class UtrParams(C.Structure):
    """msk_utr (include/msk_utr.h): UTR.exe's reconstruction parameters."""
    _fields_ = [("modality", C.c_int), ("f1", C.c_double), ("f2", C.c_double),
                ("nx", C.c_int), ("ny", C.c_int), ("xst", C.c_double), ("zlo", C.c_double),
                ("zhi", C.c_double), ("dzextra", C.c_double), ("dxc", C.c_double),
                ("dyc", C.c_double), ("dzc", C.c_double), ("wl", C.c_double),
                ("aobj", C.c_double), ("cs3", C.c_double), ("cs5", C.c_double),
                ("ctf_mode", C.c_int), ("escc", C.c_int), ("asigma", C.c_double),
                ("nsr", C.c_double), ("epsilon", C.c_double), ("inv_laplace", C.c_int)]


class UtrGeom(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int)] + \
        [(n, C.c_double) for n in ("xst", "xlo", "xhi", "ylo", "yhi", "zlo", "zhi", "fxst", "fyst",
                                   "fzst", "fxlo", "fylo", "fzlo", "xc", "yc", "zc")] + \
        [("ic", C.c_long), ("jc", C.c_long), ("kc", C.c_long)] + \
        [(n, C.c_double) for n in ("wl", "ee", "k2maxo", "cs3", "cs5", "zout_aver")] + \
        [("rot_y_only", C.c_int), ("rot_z_only", C.c_int), ("rot_z2_only", C.c_int)]


_GRID_ARGS = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double] + [C.c_float] * 6


class Oracle:
    def __init__(self, path=LIB_ORACLE):
        if not os.path.exists(path):
            build(with_ref=False)
        L = C.CDLL(path)
        self.L = L
        L.mo_wavelength.restype = C.c_double
        L.mo_wavelength.argtypes = [C.c_double]
        L.mo_sigma.restype = C.c_double
        L.mo_sigma.argtypes = [C.c_double]
        L.mo_vzatom.restype = C.c_double
        L.mo_vzatom.argtypes = [C.c_int, C.c_double]
        L.mo_vzatomLUT.restype = C.c_double
        L.mo_vzatomLUT.argtypes = [C.c_int, C.c_double]
        L.mo_bessk0.restype = C.c_double
        L.mo_bessk0.argtypes = [C.c_double]
        L.mo_bessi0.restype = C.c_double
        L.mo_bessi0.argtypes = [C.c_double]
        L.mo_freqn.argtypes = [_fp, _fp, _fp, C.c_int, C.c_double]
        L.mo_lut_table.argtypes = [C.c_int, _dp, _dp, _dp, _dp, _dp]
        L.mo_sortByZ.argtypes = [_fp, _fp, _fp, _fp, _ip, C.c_int]
        L.mo_rotate.argtypes = [C.c_float, C.c_double, C.c_double, C.c_double, C.c_double,
                                C.c_double, C.c_int, _fp, _fp, _fp]
        L.mo_drop_outside.argtypes = [C.c_float, C.c_float, C.c_int, _fp, _fp, _fp, _fp, _ip]
        L.mo_slice_count.argtypes = [C.c_float, C.c_float]
        L.mo_slice_assign.argtypes = [C.c_float, C.c_float, C.c_int, _fp, _ip]
        for nm, T in (("mo_calculate_f32", _fp), ("mo_calculate_f64", _dp)):
            getattr(L, nm).argtypes = [T, T, _fp, C.c_int, _ip, _fp, _fp, _fp, _fp, C.c_float,
                                       C.c_float, C.c_int, C.c_int]
        for nm, T in (("mo_defocus_f32", _fp), ("mo_defocus_f64", _dp)):
            getattr(L, nm).argtypes = [T, C.c_int, C.c_int, C.c_float, C.c_float, C.c_double,
                                       C.c_double, C.c_float, C.c_double, C.c_double, C.c_double,
                                       C.c_double, T]
        L.mo_orientation_potential_f64.argtypes = [C.POINTER(SeriesParams), C.c_int, _ip, _fp,
                                                   _fp, _fp, _fp, C.c_double, C.c_double, _dp]
        for nm, T in (("mo_orientation_f32", _fp), ("mo_orientation_f64", _dp)):
            getattr(L, nm).argtypes = [C.POINTER(SeriesParams), C.c_int, _ip, _fp, _fp, _fp, _fp,
                                       C.c_double, C.c_double, C.c_void_p, C.c_int, _dp, T,
                                       C.c_void_p]
        L.mo_stack_images_f64.argtypes = [C.POINTER(StackParams), _dp, C.c_int, _dp, _dp]
        L.mo_stack_loss_f64.argtypes = [C.POINTER(StackParams), _dp, C.c_int, _dp, _fp]
        L.mo_stack_loss_f64.restype = C.c_double
        L.mo_stack_adjoint_f64.argtypes = [C.POINTER(StackParams), _dp, C.c_int, _dp, _fp, _dp,
                                           C.POINTER(C.c_double)]
        L.mo_orientations_f32.argtypes = [C.POINTER(SeriesParams), C.c_int, C.c_int, C.c_int,
                                          C.c_long, _ip, _fp, _fp, _fp, _fp, _dp, _dp, C.c_int,
                                          _dp, _fp]
        # UTR reconstruction
        L.mo_utr_geom_make.argtypes = [C.POINTER(UtrParams), C.c_int, _dp, _dp,
                                       C.POINTER(UtrGeom)]
        L.mo_utr_k2four_f32.argtypes = [_fp, C.c_int, C.c_int, C.c_double, C.c_double, _fp]
        L.mo_utr_k2four_f64.argtypes = [_fp, C.c_int, C.c_int, C.c_double, C.c_double, _dp]
        L.mo_utr_grid_f32.argtypes = [_fp] + _GRID_ARGS + [_fp, C.c_double, C.c_int, C.c_int,
                                                            _fp, _fp]
        L.mo_utr_grid_acc64.argtypes = [_fp] + _GRID_ARGS + [_fp, C.c_double, C.c_int, C.c_int,
                                                              _dp, _dp]
        L.mo_utr_grid_f64.argtypes = [_dp] + _GRID_ARGS + [_dp, C.c_double, C.c_int, C.c_int,
                                                            _dp, _dp]
        for nm, T in (("mo_utr_ctf3d_f32", _fp), ("mo_utr_ctf3d_f64", _dp)):
            getattr(L, nm).argtypes = [T, C.c_int, C.c_int, C.c_int] + [C.c_double] * 13 + \
                [C.c_int]
        for nm, T in (("mo_utr_invlap3d_f32", _fp), ("mo_utr_invlap3d_f64", _dp)):
            getattr(L, nm).argtypes = [T, C.c_int, C.c_int, C.c_int] + [C.c_double] * 5
        L.mo_utr_reconstruct_f64.argtypes = [C.POINTER(UtrParams), C.c_int, _dp, _dp, C.c_void_p,
                                             C.c_void_p, _fp, _dp, C.c_int]
        L.mo_utr_finish_f64.argtypes = [C.POINTER(UtrParams), C.c_int, _dp, _dp, _dp, _dp, _dp]

    # -- physics
    def wavelength(self, kev):
        return self.L.mo_wavelength(kev)

    def sigma(self, kev):
        return self.L.mo_sigma(kev)

    def freqn(self, n, a):
        k, k2, xp = (np.zeros(n, np.float32) for _ in range(3))
        self.L.mo_freqn(k, k2, xp, n, a)
        return k, k2, xp

    def lut_table(self, Z):
        arrs = [np.zeros(100) for _ in range(5)]
        st = self.L.mo_lut_table(Z, *arrs)
        if st:
            raise ValueError("bad atomic number %d" % Z)
        return arrs

    # -- host prep
    def sort_by_z(self, Znum, x, y, z, occ):
        Znum, x, y, z, occ = (a.copy() for a in _atoms(Znum, x, y, z, occ))
        self.L.mo_sortByZ(x, y, z, occ, Znum, len(x))
        return Znum, x, y, z, occ

    def rotate(self, ctblength, angleZ, angleY, x, y, z, dxc=0.0, dyc=0.0, dzc=0.0):
        x, y, z = (np.array(a, np.float32) for a in (x, y, z))
        self.L.mo_rotate(ctblength, dxc, dyc, dzc, angleZ, angleY, len(x), x, y, z)
        return x, y, z

    def drop_outside(self, ctblength, ctblengthz, Znum, x, y, z, occ):
        Znum, x, y, z, occ = (a.copy() for a in _atoms(Znum, x, y, z, occ))
        n = self.L.mo_drop_outside(ctblength, ctblengthz, len(x), x, y, z, occ, Znum)
        return Znum[:n], x[:n], y[:n], z[:n], occ[:n]

    def slice_count(self, deltaz, zmax):
        return self.L.mo_slice_count(deltaz, zmax)

    def slice_assign(self, deltaz, zmax, zsorted):
        zs = np.ascontiguousarray(zsorted, np.float32)
        out = np.zeros(len(zs), np.int32)
        n = self.L.mo_slice_assign(deltaz, zmax, len(zs), zs, out)
        return out, n

    # -- multislice
    def calculate(self, param, Znum, x, y, z, occ, ctblength, ctblengthz, nmode=0,
                  wave0=None, fp64=False, max_slices=-1):
        nx, ny = int(param[pNX] + 0.1), int(param[pNY] + 0.1)
        T = np.float64 if fp64 else np.float32
        if wave0 is None:
            wave0 = np.zeros((nx, ny, 2), T)
            wave0[..., 0] = 1
        wave0 = np.ascontiguousarray(wave0, T).reshape(-1)
        pix = np.zeros(2 * nx * ny, T)
        fn = self.L.mo_calculate_f64 if fp64 else self.L.mo_calculate_f32
        st = fn(pix, wave0, np.ascontiguousarray(param, np.float32), len(x),
                *_atoms(Znum, x, y, z, occ), ctblength, ctblengthz, nmode, max_slices)
        if st:
            raise RuntimeError("oracle calculate failed: %d" % st)
        return pix.reshape(nx, ny, 2)

    def calculate_thermal(self, param, Znum, x, y, z, occ, wobble, ctblength, ctblengthz,
                          nmode=0, lwobble=1, iseed=-1, wave0=None, fp64=False):
        """calculate() with its thermal branches; returns (pix, advanced iseed)."""
        nx, ny = int(param[pNX] + 0.1), int(param[pNY] + 0.1)
        T = np.float64 if fp64 else np.float32
        if wave0 is None:
            wave0 = np.zeros((nx, ny, 2), T)
            wave0[..., 0] = 1
        wave0 = np.ascontiguousarray(wave0, T).reshape(-1)
        pix = np.zeros(2 * nx * ny, T)
        seed = C.c_long(iseed)
        fn = self.L.mo_calculate_thermal_f64 if fp64 else self.L.mo_calculate_thermal_f32
        fn.argtypes = [_dp if fp64 else _fp, _dp if fp64 else _fp, _fp, C.c_int, _ip, _fp, _fp,
                       _fp, _fp, _fp, C.c_float, C.c_float, C.c_int, C.c_int,
                       C.POINTER(C.c_long)]
        st = fn(pix, wave0, np.ascontiguousarray(param, np.float32), len(x),
                *_atoms(Znum, x, y, z, occ), np.ascontiguousarray(wobble, np.float32),
                ctblength, ctblengthz, nmode, lwobble, C.byref(seed))
        if st:
            raise RuntimeError("oracle calculate failed: %d" % st)
        return pix.reshape(nx, ny, 2), seed.value

    def image_plane(self, pix64, ax, wavlen, rprime, theta, xc, yc, sx, sy, k2maxo=0.0,
                    cs3=0.0, cs5=0.0):
        """FP64 image of a detector plane with the image-plane rotation and shift."""
        nx, ny = pix64.shape[0], pix64.shape[1]
        amp = np.zeros(2 * nx * ny)
        self.L.mo_defocus_amp_f64.argtypes = [_dp, C.c_int, C.c_int, C.c_float, C.c_float,
                                              C.c_double, C.c_double, C.c_float, C.c_double,
                                              C.c_double, _dp]
        self.L.mo_image_plane_f64.argtypes = [_dp, C.c_int, C.c_int, C.c_double, C.c_double,
                                              C.c_double, C.c_double, C.c_double, C.c_int,
                                              C.c_int]
        self.L.mo_defocus_amp_f64(np.ascontiguousarray(pix64, np.float64).reshape(-1), nx, ny, ax,
                                  ax, wavlen, rprime, k2maxo, cs3, cs5, amp)
        st = np.float64(np.float32(ax) / np.float32(nx))
        self.L.mo_image_plane_f64(amp, nx, ny, st, st, xc, yc, theta, sx, sy)
        a = amp.reshape(nx, ny, 2)
        return a[..., 0] ** 2 + a[..., 1] ** 2

    def defocus(self, pix, ax, by, wavlen, rprime, k2maxo=0.0, cs3=0.0, cs5=0.0, astig=0.0,
                astig_angle=0.0, fp64=False):
        nx, ny = pix.shape[0], pix.shape[1]
        T = np.float64 if fp64 else np.float32
        out = np.zeros(nx * ny, T)
        fn = self.L.mo_defocus_f64 if fp64 else self.L.mo_defocus_f32
        fn(np.ascontiguousarray(pix, T).reshape(-1), nx, ny, ax, by, wavlen, rprime, k2maxo,
           cs3, cs5, astig, astig_angle, out)
        return out.reshape(nx, ny)

    def orientation(self, sp, Znum, x, y, z, occ, angleZ, angleY, defoci, fp64=False,
                    want_exit=False, disp=None):
        T = np.float64 if fp64 else np.float32
        n = sp.nx * sp.ny
        imgs = np.zeros(len(defoci) * n, T)
        ew = np.zeros(2 * n, T) if want_exit else None
        fn = self.L.mo_orientation_f64 if fp64 else self.L.mo_orientation_f32
        d = None if disp is None else np.ascontiguousarray(disp, np.float32)
        kept = fn(C.byref(sp), len(x), *_atoms(Znum, x, y, z, occ), angleZ, angleY,
                  None if d is None else d.ctypes.data, len(defoci),
                  np.ascontiguousarray(defoci, np.float64), imgs,
                  ew.ctypes.data if want_exit else None)
        if kept < 0:
            raise RuntimeError("oracle orientation failed: %d" % kept)
        imgs = imgs.reshape(len(defoci), sp.nx, sp.ny)
        return (imgs, ew.reshape(sp.nx, sp.ny, 2), kept) if want_exit else (imgs, kept)

    # -- potential stacks (FP64)
    def stack_images(self, sp, v, rprime):
        v = np.ascontiguousarray(v, np.float64)
        rp = np.ascontiguousarray(rprime, np.float64)
        out = np.zeros(len(rp) * sp.nx * sp.ny)
        st = self.L.mo_stack_images_f64(C.byref(sp), v.reshape(-1), len(rp), rp, out)
        if st:
            raise RuntimeError("oracle stack images failed: %d" % st)
        return out.reshape(len(rp), sp.nx, sp.ny)

    def stack_loss(self, sp, v, rprime, target):
        return self.L.mo_stack_loss_f64(C.byref(sp), np.ascontiguousarray(v, np.float64).reshape(-1),
                                        len(rprime), np.ascontiguousarray(rprime, np.float64),
                                        np.ascontiguousarray(target, np.float32).reshape(-1))

    def stack_adjoint(self, sp, v, rprime, target):
        v = np.ascontiguousarray(v, np.float64)
        g = np.zeros(v.size)
        loss = C.c_double()
        st = self.L.mo_stack_adjoint_f64(C.byref(sp), v.reshape(-1), len(rprime),
                                         np.ascontiguousarray(rprime, np.float64),
                                         np.ascontiguousarray(target, np.float32).reshape(-1), g,
                                         C.byref(loss))
        if st:
            raise RuntimeError("oracle stack adjoint failed: %d" % st)
        return g.reshape(v.shape), loss.value

    def stack_fd(self, sp, v, rprime, target, voxels, h_rel=1e-3, nthreads=1):
        """Central differences dL/dv at voxels [(k, ix, iy), ...] (FP64)."""
        v = np.ascontiguousarray(v, np.float64)
        vox = np.ascontiguousarray(voxels, np.int32).reshape(-1)
        fd = np.zeros(len(vox) // 3)
        fn = self.L.mo_stack_fd_f64
        fn.argtypes = [C.POINTER(StackParams), _dp, C.c_int, _dp, _fp, C.c_int, _ip, C.c_double,
                       C.c_int, _dp]
        st = fn(C.byref(sp), v.reshape(-1), len(rprime), np.ascontiguousarray(rprime, np.float64),
                np.ascontiguousarray(target, np.float32).reshape(-1), len(fd), vox, h_rel,
                nthreads, fd)
        if st:
            raise RuntimeError("oracle finite differences failed: %d" % st)
        return fd

    def orientation_potential(self, sp, Znum, x, y, z, occ, angleZ, angleY):
        """FP64 per-slice projected potentials [nslices, nx, ny] of one
        orientation and the number of atoms kept."""
        ns = self.slice_count(sp.deltaz, sp.ctblengthz)
        v = np.zeros(ns * sp.nx * sp.ny)
        kept = self.L.mo_orientation_potential_f64(C.byref(sp), len(x), *_atoms(Znum, x, y, z, occ),
                                                   angleZ, angleY, v)
        if kept < 0:
            raise RuntimeError("oracle potential failed: %d" % kept)
        return v.reshape(ns, sp.nx, sp.ny), kept

    def orientations_f32(self, sp, Znum, x, y, z, occ, angZ, angY, defoci, nthreads,
                         coord_stride=0):
        nunits = len(angZ)
        imgs = np.zeros(nunits * len(defoci) * sp.nx * sp.ny, np.float32)
        natom = len(Znum) if coord_stride == 0 else coord_stride
        st = self.L.mo_orientations_f32(C.byref(sp), nunits, nthreads, natom, coord_stride,
                                         *_atoms(Znum, x, y, z, occ),
                                         np.ascontiguousarray(angZ, np.float64),
                                         np.ascontiguousarray(angY, np.float64), len(defoci),
                                         np.ascontiguousarray(defoci, np.float64), imgs)
        if st:
            raise RuntimeError("oracle orientations failed: %d" % st)
        return imgs.reshape(nunits, len(defoci), sp.nx, sp.ny)


    # -- UTR reconstruction
    def utr_geom(self, p, angles, defocus):
        g = UtrGeom()
        ang = np.ascontiguousarray(angles, np.float64).reshape(-1)
        st = self.L.mo_utr_geom_make(C.byref(p), len(ang) // 2, ang,
                                     np.ascontiguousarray(defocus, np.float64), C.byref(g))
        if st:
            raise ValueError("bad UTR parameters")
        return g

    def utr_k2four(self, img, f1=1.0, f2=0.0, f64=True):
        img = np.ascontiguousarray(img, np.float32)
        ny, nx = img.shape
        if f64:
            out = np.zeros((ny, nx, 2), np.float64)
            self.L.mo_utr_k2four_f64(img, nx, ny, f1, f2, out)
        else:
            out = np.zeros((ny, nx, 2), np.float32)
            self.L.mo_utr_k2four_f32(img, nx, ny, f1, f2, out)
        return out

    def utr_grid(self, k2four, nz, angleY, angleZ, fx, fc, wl, rotshift, escc, mode="f32",
                 v3=None, samp3=None):
        """One image into (v3, samp3); fx = (fxlo, fxst, fylo, fyst, fzlo, fzst) as floats;
        mode "f32" (float sums), "acc64" (float products, double sums) or "f64"
        (double spectrum and phase; fc = the three imaginary parts)."""
        ny, nx = k2four.shape[:2]
        T = np.float32 if mode == "f32" else np.float64
        if v3 is None:
            v3 = np.zeros((nz, ny, nx, 2), T)
            samp3 = np.zeros((nz, ny, nx), T)
        fn = {"f32": self.L.mo_utr_grid_f32, "acc64": self.L.mo_utr_grid_acc64,
              "f64": self.L.mo_utr_grid_f64}[mode]
        kt = np.float64 if mode == "f64" else np.float32
        fn(np.ascontiguousarray(k2four, kt), nx, ny, nz, angleY, angleZ, *[float(v) for v in fx],
           np.ascontiguousarray(fc, kt), wl, int(rotshift), int(escc), v3, samp3)
        return v3, samp3

    def utr_ctf3d(self, v3, wl, box, defocdist, q2max, cs3, cs5, sigma, epsilon, escc):
        """box = (zlo, zhi, ylo, yhi, xlo, xhi); v3 [nz][ny][nx][2], changed in place."""
        nz, ny, nx = v3.shape[:3]
        fn = self.L.mo_utr_ctf3d_f32 if v3.dtype == np.float32 else self.L.mo_utr_ctf3d_f64
        if fn(v3, nx, ny, nz, wl, *box, defocdist, q2max, cs3, cs5, sigma, epsilon, int(escc)):
            raise ValueError("CTFcorrection3D: bad sizes or evanescent waves")
        return v3

    def utr_invlap3d(self, v3, zaper, yaper, xaper, alpha, norm):
        nz, ny, nx = v3.shape[:3]
        fn = self.L.mo_utr_invlap3d_f32 if v3.dtype == np.float32 else self.L.mo_utr_invlap3d_f64
        if fn(v3, nx, ny, nz, zaper, yaper, xaper, alpha, norm):
            raise ValueError("InverseMLaplacian3D: bad arguments")
        return v3

    def utr_reconstruct(self, p, angles, defocus, images, nthreads=1, zrot=None, shifts=None):
        g = self.utr_geom(p, angles, defocus)
        vol = np.zeros((g.nz, p.ny, p.nx), np.float64)
        ang = np.ascontiguousarray(angles, np.float64).reshape(-1)
        zr = None if zrot is None else np.ascontiguousarray(zrot, np.float64)
        sh = None if shifts is None else np.ascontiguousarray(shifts, np.float64).reshape(-1)
        st = self.L.mo_utr_reconstruct_f64(C.byref(p), len(ang) // 2, ang,
                                           np.ascontiguousarray(defocus, np.float64),
                                           None if zr is None else zr.ctypes.data,
                                           None if sh is None else sh.ctypes.data,
                                           np.ascontiguousarray(images, np.float32), vol,
                                           nthreads)
        if st:
            raise ValueError("oracle reconstruction failed")
        return vol

    def utr_finish(self, p, angles, defocus, v3, samp3):
        g = self.utr_geom(p, angles, defocus)
        vol = np.zeros((g.nz, p.ny, p.nx), np.float64)
        ang = np.ascontiguousarray(angles, np.float64).reshape(-1)
        v = np.array(v3, np.float64)
        if self.L.mo_utr_finish_f64(C.byref(p), len(ang) // 2, ang,
                                    np.ascontiguousarray(defocus, np.float64), v,
                                    np.ascontiguousarray(samp3, np.float64), vol):
            raise ValueError("oracle finish failed")
        return vol


class UtrReference:
    """The reference's own PhaseRetrieval/UTR.h templates compiled here (oracle/_ref)."""

    def __init__(self, path=LIB_UTR_REF):
        L = C.CDLL(path)
        self.L = L
        L.ref_utr_grid_f.argtypes = [_fp] + _GRID_ARGS + [_fp, C.c_double, C.c_int, C.c_int,
                                                           _fp, _fp]
        L.ref_utr_ctf3d_f.argtypes = [_fp, C.c_int, C.c_int, C.c_int] + [C.c_double] * 13 + \
            [C.c_int]
        L.ref_utr_invlap3d_f.argtypes = [_fp, C.c_int, C.c_int, C.c_int] + [C.c_double] * 5

    def grid(self, k2four, nz, angleY, angleZ, fx, fc, wl, rotshift, escc, v3=None, samp3=None):
        ny, nx = k2four.shape[:2]
        if v3 is None:
            v3 = np.zeros((nz, ny, nx, 2), np.float32)
            samp3 = np.zeros((nz, ny, nx), np.float32)
        self.L.ref_utr_grid_f(np.ascontiguousarray(k2four, np.float32), nx, ny, nz, angleY,
                              angleZ, *[float(v) for v in fx],
                              np.ascontiguousarray(fc, np.float32), wl, int(rotshift),
                              int(escc), v3, samp3)
        return v3, samp3

    def ctf3d(self, v3, wl, box, defocdist, q2max, cs3, cs5, sigma, epsilon, escc):
        nz, ny, nx = v3.shape[:3]
        self.L.ref_utr_ctf3d_f(v3, nx, ny, nz, wl, *box, defocdist, q2max, cs3, cs5, sigma,
                               epsilon, int(escc))
        return v3

    def invlap3d(self, v3, zaper, yaper, xaper, alpha, norm):
        nz, ny, nx = v3.shape[:3]
        self.L.ref_utr_invlap3d_f(v3, nx, ny, nz, zaper, yaper, xaper, alpha, norm)
        return v3


class Reference:
    """The reference's own code compiled here (oracle/_ref)."""

    def __init__(self, path=LIB_REF):
        L = C.CDLL(path)
        self.L = L
        L.ref_calculate.argtypes = [_fp, _fp, _fp, C.c_int, _ip, _fp, _fp, _fp, _fp, _fp,
                                    C.c_float, C.c_float, C.c_int, C.c_int, C.c_void_p, C.c_int]
        L.ref_calculate_many.argtypes = [C.c_int, C.c_int, _fp, _fp, _fp,
                                         np.ctypeslib.ndpointer(dtype=np.int32),
                                         np.ctypeslib.ndpointer(dtype=np.int64),
                                         _ip, _fp, _fp, _fp, _fp, _fp, C.c_float, C.c_float,
                                         C.c_int]
        L.ref_sortByZ.argtypes = [_fp, _fp, _fp, _fp, _ip, C.c_int]
        for nm in ("ref_vzatomLUT", "ref_vzatom"):
            getattr(L, nm).restype = C.c_double
            getattr(L, nm).argtypes = [C.c_int, C.c_double]
        for nm in ("ref_wavelength", "ref_sigma", "ref_bessk0", "ref_bessi0"):
            getattr(L, nm).restype = C.c_double
            getattr(L, nm).argtypes = [C.c_double]
        L.ref_freqn.argtypes = [_fp, _fp, _fp, C.c_int, C.c_double]
        self._planned = None

    def calculate(self, param, Znum, x, y, z, occ, ctblength, ctblengthz, nmode=0, wave0=None,
                  wobble=None, lwobble=0, iseed=None):
        """autoslic::calculate; with lwobble = 1 its thermal branches (param[pNWOBBLE],
        param[pTEMPER]); iseed: the gasdev seed, returned advanced as the second
        value when given."""
        param = np.array(param, np.float32)
        nx, ny = int(param[pNX] + 0.1), int(param[pNY] + 0.1)
        if wave0 is None:
            wave0 = np.zeros((nx, ny, 2), np.float32)
            wave0[..., 0] = 1
        wave0 = np.ascontiguousarray(wave0, np.float32).reshape(-1)
        pix = np.zeros(2 * nx * ny, np.float32)
        Znum, x, y, z, occ = (a.copy() for a in _atoms(Znum, x, y, z, occ))
        wob = np.zeros(len(x), np.float32) if wobble is None else \
            np.ascontiguousarray(wobble, np.float32).copy()
        seed = C.c_long(-1 if iseed is None else iseed)
        self.L.ref_calculate(pix, wave0, param, len(x), Znum, x, y, z, occ, wob, ctblength,
                             ctblengthz, nmode, lwobble, C.addressof(seed), 1)
        pix = pix.reshape(nx, ny, 2)
        return pix if iseed is None else (pix, seed.value)

    def sort_by_z(self, Znum, x, y, z, occ):
        Znum, x, y, z, occ = (a.copy() for a in _atoms(Znum, x, y, z, occ))
        self.L.ref_sortByZ(x, y, z, occ, Znum, len(x))
        return Znum, x, y, z, occ

    def vzatomLUT(self, Z, rsq):
        return self.L.ref_vzatomLUT(Z, rsq)

    def freqn(self, n, a):
        k, k2, xp = (np.zeros(n, np.float32) for _ in range(3))
        self.L.ref_freqn(k, k2, xp, n, a)
        return k, k2, xp


def reference_available():
    return os.path.exists(LIB_REF)


def utr_reference_available():
    return os.path.exists(LIB_UTR_REF)
