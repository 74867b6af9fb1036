"""GB300 multislice: ctypes binding of libmsk.so (include/msk.h).

The library itself is C++/CUDA; this module is the Python plumbing used by
the tests and the benchmark.  It loads the in-tree libmsk.so and fails
loudly when it is missing -- there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

from . import specimen  # noqa: F401

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libmsk.so")

# status codes (include/msk.h)
MSK_OK, MSK_EBADSIZE, MSK_EBOX, MSK_EZSORT, MSK_EZNUM = 0, -1, -2, -3, -4
MSK_ENOMEM, MSK_EUNSUPPORTED, MSK_ECUDA, MSK_EINVAL, MSK_ETOOLARGE = -5, -6, -7, -8, -9

# param[] offsets (slicelib.hpp:142-240)
pXCTILT, pYCTILT, pENERGY, pOAPERT, pDELTAZ = 9, 10, 16, 17, 30
pAX, pBY, pNX, pNY, pNWOBBLE, pTEMPER = 101, 102, 104, 105, 111, 120
NPARAM = 200

EXPORTS = ("msk_create", "msk_destroy", "msk_last_error", "msk_status_string", "msk_calculate",
           "msk_tilt_series", "msk_slice_count", "msk_slice_assign", "msk_sort_by_z",
           "msk_rotate", "msk_potential_table", "msk_set_stream", "msk_profile",
           "msk_profile_read", "msk_calculate_static", "msk_tilt_series_per_angle",
           "msk_stack_images", "msk_adjoint", "msk_potential_stack", "msk_tilt_series_batch",
           "msk_write_grd", "msk_write_grc", "msk_write_tiff32", "msk_read_orientations",
           "msk_tilt_series_planes", "msk_utr_depth", "msk_utr_reconstruct",
           "msk_utr_reconstruct_planes", "msk_utr_grid",
           "msk_utr_ctf_correction3d", "msk_utr_inverse_mlaplacian3d",
           "msk_device_allocations", "msk_column_plan", "msk_row_plan")
MSK_BATCH_GRAPH = 1


class MskError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (status %d)" % (msg, status))
        self.status = status


class Series(C.Structure):
    """msk_series (include/msk.h)."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("ctblength", C.c_float),
                ("ctblengthz", C.c_float), ("v0", C.c_float), ("deltaz", C.c_float),
                ("aobj", C.c_float), ("cs3", C.c_double), ("cs5", C.c_double),
                ("astig", C.c_double), ("astig_angle", C.c_double), ("dxc", C.c_double),
                ("dyc", C.c_double), ("dzc", C.c_double), ("nmode", C.c_int),
                ("max_batch", C.c_int), ("lwobble", C.c_int), ("temperature", C.c_float),
                ("wobble", C.c_void_p), ("seed", C.c_long), ("R1", C.c_double),
                ("rotation", C.c_void_p), ("xshift", C.c_double), ("yshift", C.c_double)]


class Utr(C.Structure):
    """msk_utr (include/msk_utr.h): UTR.exe's reconstruction parameters, in the
    units of its ".txt" parameter file (ReadmeUTR.txt; bracketed: its lines).
    modality [1], f1 f2 [7], nx ny [8], xst [9], zlo zhi dzextra [10],
    dxc dyc dzc [11], wl [12], aobj (mrad) [13], cs3 cs5 (mm) [14],
    ctf_mode (0, 2 or 4) [15], escc [16], asigma [17], nsr [18], epsilon [19],
    inv_laplace [22]."""
    _fields_ = [("modality", C.c_int), ("f1", C.c_double), ("f2", C.c_double),
                ("nx", C.c_int), ("ny", C.c_int), ("xst", C.c_double), ("zlo", C.c_double),
                ("zhi", C.c_double), ("dzextra", C.c_double), ("dxc", C.c_double),
                ("dyc", C.c_double), ("dzc", C.c_double), ("wl", C.c_double),
                ("aobj", C.c_double), ("cs3", C.c_double), ("cs5", C.c_double),
                ("ctf_mode", C.c_int), ("escc", C.c_int), ("asigma", C.c_double),
                ("nsr", C.c_double), ("epsilon", C.c_double), ("inv_laplace", C.c_int)]

    def __init__(self, **kw):
        super().__init__()
        self.f1 = 1.0
        for k, v in kw.items():
            setattr(self, k, v)


class Stack(C.Structure):
    """msk_stack (include/msk.h): multislice from per-slice potentials."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("ax", C.c_float), ("by", C.c_float),
                ("v0", C.c_float), ("deltaz", C.c_float), ("ctiltx", C.c_float),
                ("ctilty", C.c_float), ("aobj", C.c_float), ("cs3", C.c_double),
                ("cs5", C.c_double), ("nslices", C.c_int), ("checkpoint", C.c_int),
                ("max_batch", C.c_int)]


class SpecimenDesc(C.Structure):
    """msk_specimen (include/msk.h): one specimen of a batch."""
    _fields_ = [("natom", C.c_int), ("Znum", C.c_void_p), ("x", C.c_void_p), ("y", C.c_void_p),
                ("z", C.c_void_p), ("occ", C.c_void_p), ("nx", C.c_int), ("ny", C.c_int),
                ("ctblength", C.c_float), ("ctblengthz", C.c_float), ("nangles", C.c_int),
                ("angleZ", C.c_void_p), ("angleY", C.c_void_p), ("images", C.c_void_p),
                ("kept", C.c_void_p), ("wobble", C.c_void_p), ("nconfig", C.c_int),
                ("displacements", C.c_void_p), ("exitwaves", C.c_void_p),
                ("plane_off", C.c_void_p), ("planes", C.c_void_p), ("shifts", C.c_void_p)]


class Plane(C.Structure):
    """msk_plane (include/msk.h): one detector plane of one orientation."""
    _fields_ = [("defocus", C.c_double), ("rotation", C.c_double), ("astig", C.c_double),
                ("astig_angle", C.c_double)]


def _plane_arrays(planes, na):
    """Per-orientation plane rows (defocus, rotation, astig, astig_angle) as
    the C arrays plane_off int32[na + 1] and msk_plane[total]."""
    off = np.zeros(na + 1, np.int32)
    rows = []
    for a in range(na):
        pa = np.asarray(planes[a], np.float64).reshape(-1, 4)
        rows.extend(pa)
        off[a + 1] = off[a] + len(pa)
    total = int(off[-1])
    arr = (Plane * max(total, 1))()
    for k, r in enumerate(rows):
        arr[k].defocus, arr[k].rotation, arr[k].astig, arr[k].astig_angle = map(float, r)
    return off, arr, total


class KernelStat(C.Structure):
    """msk_kernel_stat (include/msk.h)."""
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_longlong), ("ms", C.c_double),
                ("bytes", C.c_double)]


_lib = None
_fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def lib_path():
    return LIB_PATH


def load():
    """Load libmsk.so (built by utr_public_gb300._build); raise if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libmsk.so is not built: run `python -m utr_public_gb300._build` "
                           "(or __graft_entry__.build()); there is no CPU fallback")
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    L.msk_create.argtypes = [C.c_int, C.POINTER(vp)]
    L.msk_destroy.argtypes = [vp]
    L.msk_destroy.restype = None
    L.msk_last_error.argtypes = [vp]
    L.msk_last_error.restype = C.c_char_p
    L.msk_status_string.argtypes = [C.c_int]
    L.msk_status_string.restype = C.c_char_p
    L.msk_calculate.argtypes = [vp, vp, vp, _fp, C.c_int, vp, vp, vp, vp, vp, vp, C.c_float,
                                C.c_float, C.c_int, C.c_int, C.POINTER(C.c_long)]
    L.msk_tilt_series.argtypes = [vp, C.POINTER(Series), C.c_int, vp, vp, vp, vp, vp, C.c_int,
                                  _dp, _dp, C.c_int, vp, C.c_int, vp, vp, vp, vp]
    L.msk_slice_count.argtypes = [C.c_float, C.c_float]
    L.msk_slice_assign.argtypes = [C.c_float, C.c_float, C.c_int, _fp, _ip]
    L.msk_sort_by_z.argtypes = [_fp, _fp, _fp, _fp, _ip, C.c_int]
    L.msk_sort_by_z.restype = None
    L.msk_rotate.argtypes = [C.c_float, C.c_double, C.c_double, C.c_double, C.c_double,
                             C.c_double, C.c_int, _fp, _fp, _fp]
    L.msk_rotate.restype = None
    L.msk_potential_table.argtypes = [C.c_int, _dp, _dp]
    L.msk_set_stream.argtypes = [vp, vp]
    L.msk_profile.argtypes = [vp, C.c_int]
    L.msk_profile_read.argtypes = [vp, C.POINTER(KernelStat), C.c_int]
    L.msk_tilt_series_per_angle.argtypes = [vp, C.POINTER(Series), C.c_int, vp, vp, vp, vp, vp,
                                            C.c_int, _dp, _dp, C.c_int, vp, C.c_int, vp, vp, vp]
    L.msk_calculate_static.argtypes = [vp, vp, vp, _fp, C.c_int, vp, vp, vp, vp, vp, C.c_float,
                                       C.c_float, C.c_int]
    L.msk_column_plan.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]
    L.msk_row_plan.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]
    L.msk_device_allocations.argtypes = []
    L.msk_device_allocations.restype = C.c_longlong
    L.msk_stack_images.argtypes = [vp, C.POINTER(Stack), C.c_int, vp, C.c_int, vp, vp]
    L.msk_adjoint.argtypes = [vp, C.POINTER(Stack), C.c_int, vp, C.c_int, vp, vp, vp,
                                    C.POINTER(C.c_double)]
    L.msk_potential_stack.argtypes = [vp, C.POINTER(Series), C.c_int, vp, vp, vp, vp, vp,
                                      C.c_int, _dp, _dp, vp, vp]
    L.msk_tilt_series_batch.argtypes = [vp, C.POINTER(Series), C.c_int, C.POINTER(SpecimenDesc),
                                        C.c_int, vp, C.c_int]
    L.msk_tilt_series_planes.argtypes = [vp, C.POINTER(Series), C.c_int, vp, vp, vp, vp, vp,
                                         C.c_int, _dp, _dp, vp, vp, vp, C.c_int, vp, vp, vp, vp]
    L.msk_write_grd.argtypes = [C.c_char_p, _fp, C.c_int, C.c_int] + [C.c_double] * 4
    L.msk_write_grc.argtypes = [C.c_char_p, _fp, C.c_int, C.c_int] + [C.c_double] * 5
    L.msk_write_tiff32.argtypes = [C.c_char_p, _fp, C.c_int, C.c_int]
    L.msk_read_orientations.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), vp,
                                        vp, vp, vp]
    L.msk_utr_depth.argtypes = [C.POINTER(Utr)]
    L.msk_utr_reconstruct.argtypes = [vp, C.POINTER(Utr), C.c_int, _dp, _dp, vp, vp]
    L.msk_utr_reconstruct_planes.argtypes = [vp, C.POINTER(Utr), C.c_int, _dp, _dp, vp, vp, vp,
                                             vp]
    L.msk_utr_grid.argtypes = [vp, C.POINTER(Utr), C.c_int, _dp, vp, vp, vp]
    L.msk_utr_ctf_correction3d.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int] + \
        [C.c_double] * 13 + [C.c_int]
    L.msk_utr_inverse_mlaplacian3d.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int] + \
        [C.c_double] * 5
    _lib = L
    return L


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):  # torch tensor (device or host)
        return a.data_ptr()
    return a.ctypes.data


def _io_check(st, path):
    if st:
        raise MskError(st, "cannot write or read %s" % path)


def write_grd(path, img, xlo, xhi, ylo, yhi):
    """Image [nx, ny] to a binary GRD file (msk_write_grd)."""
    img = np.ascontiguousarray(img, np.float32)
    _io_check(load().msk_write_grd(os.fsencode(path), img.reshape(-1), img.shape[0],
                                   img.shape[1], xlo, xhi, ylo, yhi), path)


def write_grc(path, amp, wavelength, xlo, xhi, ylo, yhi):
    """Complex amplitude [nx, ny, 2] to a GRC file (msk_write_grc)."""
    amp = np.ascontiguousarray(amp, np.float32)
    _io_check(load().msk_write_grc(os.fsencode(path), amp.reshape(-1), amp.shape[0],
                                   amp.shape[1], wavelength, xlo, xhi, ylo, yhi), path)


def write_tiff32(path, img):
    """Image [nx, ny] to a 32-bit float TIFF (msk_write_tiff32)."""
    img = np.ascontiguousarray(img, np.float32)
    _io_check(load().msk_write_tiff32(os.fsencode(path), img.reshape(-1), img.shape[0],
                                      img.shape[1]), path)


def read_orientations(path):
    """(angles [n, 2] degrees, list of per-orientation plane arrays [k, 5], shifts
    [n, 2]) from a MsctKirkland orientation file (msk_read_orientations)."""
    L = load()
    na, npl = C.c_int(0), C.c_int(0)
    _io_check(L.msk_read_orientations(os.fsencode(path), C.byref(na), C.byref(npl), None, None,
                                      None, None), path)
    angles = np.zeros((na.value, 2))
    off = np.zeros(na.value + 1, np.int32)
    planes = np.zeros((max(npl.value, 1), 5))
    shifts = np.zeros((na.value, 2))
    _io_check(L.msk_read_orientations(os.fsencode(path), C.byref(na), C.byref(npl), _ptr(angles),
                                      _ptr(off), _ptr(planes), _ptr(shifts)), path)
    return angles, [planes[off[i]:off[i + 1]] for i in range(na.value)], shifts


def make_param(ax, by, nx, ny, v0, deltaz, ctiltx=0.0, ctilty=0.0):
    p = np.zeros(NPARAM, np.float32)
    p[pAX], p[pBY], p[pNX], p[pNY] = ax, by, nx, ny
    p[pENERGY], p[pDELTAZ], p[pXCTILT], p[pYCTILT] = v0, deltaz, ctiltx, ctilty
    return p


# ------------------------------------------------------------- host helpers

def slice_count(deltaz, ctblengthz):
    return load().msk_slice_count(deltaz, ctblengthz)


def slice_assign(deltaz, ctblengthz, zsorted):
    zs = np.ascontiguousarray(zsorted, np.float32)
    out = np.zeros(len(zs), np.int32)
    n = load().msk_slice_assign(deltaz, ctblengthz, len(zs), zs, out)
    return out, n


def sort_by_z(Znum, x, y, z, occ):
    Znum, x, y, z, occ = (np.array(a, dt) for a, dt in
                          ((Znum, np.int32), (x, np.float32), (y, np.float32), (z, np.float32),
                           (occ, np.float32)))
    load().msk_sort_by_z(x, y, z, occ, Znum, len(x))
    return Znum, x, y, z, occ


def rotate(ctblength, angleZ, angleY, x, y, z, dxc=0.0, dyc=0.0, dzc=0.0):
    x, y, z = (np.array(a, np.float32) for a in (x, y, z))
    load().msk_rotate(ctblength, dxc, dyc, dzc, angleZ, angleY, len(x), x, y, z)
    return x, y, z


def potential_table(Z):
    knots, coef = np.zeros(100), np.zeros(400)
    st = load().msk_potential_table(Z, knots, coef)
    if st:
        raise MskError(st, "bad atomic number")
    return knots, coef.reshape(100, 4)


def calculate_static(param, Znum, x, y, z, occ, ctblength, ctblengthz, nmode=0, wave0=None,
                     stream=None):
    """calculate() through msk_calculate_static, the entry point that allocates
    no device memory (for callers whose device memory is owned by someone
    else).  Its scratch is a fixed array inside libmsk.so, shared by every
    call: calls must not overlap.  Limits: nx*ny <= 512*512, 65536 atoms,
    4096 slices (MskError with MSK_ETOOLARGE beyond them)."""
    L = load()
    param = np.ascontiguousarray(param, np.float32)
    nx, ny = int(param[pNX] + 0.1), int(param[pNY] + 0.1)
    if wave0 is None:
        wave0 = np.zeros((nx, ny, 2), np.float32)
        wave0[..., 0] = 1.0
    wave0 = np.ascontiguousarray(wave0, np.float32)
    pix = np.zeros((nx, ny, 2), np.float32)
    arrs = [np.ascontiguousarray(a, dt) for a, dt in
            ((Znum, np.int32), (x, np.float32), (y, np.float32), (z, np.float32),
             (occ, np.float32))]
    st = L.msk_calculate_static(stream, _ptr(pix), _ptr(wave0), param, len(arrs[1]),
                                *[_ptr(a) for a in arrs], ctblength, ctblengthz, nmode)
    if st:
        raise MskError(st, L.msk_status_string(st).decode())
    return pix


COLUMN_PASSES = ("band_limit", "propagate", "free_space", "debye_waller")


def column_plan(device, nx, ny, pass_):
    """The column-pass schedule the tuner chose on `device` for an nx x ny grid:
    {"variant", "points_per_thread", "columns_per_cta"}, or None before the pass
    has run on that grid (msk_column_plan)."""
    info = (C.c_int * 3)()
    p = COLUMN_PASSES.index(pass_) if isinstance(pass_, str) else int(pass_)
    if load().msk_column_plan(device, nx, ny, p, info) != 0:
        return None
    return {"variant": info[0], "points_per_thread": info[1], "columns_per_cta": info[2]}


ROW_PASSES = ("transmit",)


def row_plan(device, nx, ny, pass_="transmit"):
    """The transmit schedule the row tuner chose on `device` for an nx x ny grid:
    {"variant", "points_per_thread", "rows_per_cta"}, or None before the
    transmit has run on that grid (msk_row_plan)."""
    info = (C.c_int * 3)()
    p = ROW_PASSES.index(pass_) if isinstance(pass_, str) else int(pass_)
    if load().msk_row_plan(device, nx, ny, p, info) != 0:
        return None
    return {"variant": info[0], "points_per_thread": info[1], "rows_per_cta": info[2]}


def device_allocations():
    """Device allocations libmsk has made in this process (msk_device_allocations)."""
    return int(load().msk_device_allocations())


# ------------------------------------------------------------------ context

class Context:
    """One libmsk context (device, stream and buffers)."""

    def __init__(self, device=0):
        L = load()
        h = C.c_void_p()
        st = L.msk_create(device, C.byref(h))
        if st:
            raise MskError(st, "msk_create failed: %s" % L.msk_status_string(st).decode())
        self.h = h
        self.L = L
        self._plane_waves = {}  # calculate()'s default incident wave per grid size

    def close(self):
        if self.h:
            self.L.msk_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st:
            msg = self.L.msk_last_error(self.h).decode() or self.L.msk_status_string(st).decode()
            raise MskError(st, msg)

    def set_stream(self, stream_handle):
        """Run on the caller's CUDA stream (an int cudaStream_t; 0/None: own stream)."""
        self._check(self.L.msk_set_stream(self.h, stream_handle or None))

    def profile(self, enable):
        self._check(self.L.msk_profile(self.h, 1 if enable else 0))

    def profile_read(self):
        """{kernel: (launches, total ms, algorithmic bytes)} since profile(True)."""
        buf = (KernelStat * 16)()
        n = self.L.msk_profile_read(self.h, buf, 16)
        if n < 0:
            self._check(n)
        return {buf[i].name.decode(): (int(buf[i].launches), float(buf[i].ms),
                                       float(buf[i].bytes)) for i in range(min(n, 16))}

    def calculate(self, param, Znum, x, y, z, occ, ctblength, ctblengthz, nmode=0, wave0=None,
                  wobble=None, lwobble=0, iseed=None, out=None):
        """autoslic::calculate coherent branch; returns the exit wave [nx, ny, 2] float32
        (into `out` when given: a C-contiguous float32 array of that shape).
        lwobble = 1 takes its thermal branches (param[pNWOBBLE], param[pTEMPER]); with
        iseed given (nwobble > 1) returns (exit wave, advanced seed)."""
        param = np.ascontiguousarray(param, np.float32)
        nx, ny = int(param[pNX] + 0.1), int(param[pNY] + 0.1)
        if wave0 is None:  # the unit plane wave, made once per grid size
            wave0 = self._plane_waves.get((nx, ny))
            if wave0 is None:
                wave0 = np.zeros((nx, ny, 2), np.float32)
                wave0[..., 0] = 1.0
                self._plane_waves[(nx, ny)] = wave0
        wave0 = np.ascontiguousarray(wave0, np.float32)
        if out is None:
            pix = np.empty((nx, ny, 2), np.float32)  # every element is written
        else:
            if (out.dtype != np.float32 or out.shape != (nx, ny, 2) or
                    not out.flags["C_CONTIGUOUS"]):
                raise ValueError("out must be a C-contiguous float32 array [nx, ny, 2]")
            pix = out
        arrs = [np.ascontiguousarray(a, dt) for a, dt in
                ((Znum, np.int32), (x, np.float32), (y, np.float32), (z, np.float32),
                 (occ, np.float32))]
        wob = None if wobble is None else np.ascontiguousarray(wobble, np.float32)
        if wob is None and lwobble:
            wob = np.zeros(len(arrs[1]), np.float32)
        seed = None if iseed is None else C.c_long(iseed)
        st = self.L.msk_calculate(self.h, _ptr(pix), _ptr(wave0), param, len(arrs[1]),
                                  *[_ptr(a) for a in arrs], _ptr(wob), ctblength, ctblengthz,
                                  nmode, lwobble, None if seed is None else C.byref(seed))
        self._check(st)
        return pix if seed is None else (pix, seed.value)

    def tilt_series(self, series, Znum, x, y, z, occ, angleZ, angleY, defocus, nconfig=1,
                    displacements=None, images=None, exitwaves=None, want_exit=False):
        """All orientations x configurations x defoci; returns images
        [nangles, ndef, nx, ny] (and exit waves [nangles, nconfig, nx, ny, 2]).
        images / exitwaves may be preallocated numpy arrays or torch CUDA tensors."""
        angleZ = np.ascontiguousarray(angleZ, np.float64)
        angleY = np.ascontiguousarray(angleY, np.float64)
        defocus = np.ascontiguousarray(defocus, np.float64)
        na, nd = len(angleZ), len(defocus)
        if images is None:
            images = np.zeros((na, nd, series.nx, series.ny), np.float32)
        if exitwaves is None and want_exit:
            exitwaves = np.zeros((na, nconfig, series.nx, series.ny, 2), np.float32)
        kept = np.zeros(na * nconfig, np.int32)
        arrs = [np.ascontiguousarray(a, dt) for a, dt in
                ((Znum, np.int32), (x, np.float32), (y, np.float32), (z, np.float32),
                 (occ, np.float32))]
        disp = None if displacements is None else np.ascontiguousarray(displacements, np.float32)
        st = self.L.msk_tilt_series(self.h, C.byref(series), len(arrs[1]), *[_ptr(a) for a in arrs],
                                    na, angleZ, angleY, nd, _ptr(defocus), nconfig, _ptr(disp),
                                    _ptr(images), _ptr(exitwaves), _ptr(kept))
        self._check(st)
        return (images, exitwaves, kept) if want_exit or exitwaves is not None else (images, kept)

    @staticmethod
    def _f32(a):
        if hasattr(a, "data_ptr"):
            return a
        return np.ascontiguousarray(a, np.float32)

    def tilt_series_batch(self, series, specimens, defocus, graph=True, images=None, nconfig=1,
                          displacements=None, exitwaves=None, want_exit=False, planes=None,
                          shifts=None):
        """Many specimens in one call (msk_tilt_series_batch).  specimens: list
        of (Specimen-like with Znum/x/y/z/occ/fov and, for series.lwobble = 1, a
        float32 `wobble` per atom, n, angleZ, angleY[, ctblengthz]);
        returns (images list [nangles, ndef, n, n] per specimen, kept list).
        nconfig > 1: thermal configurations per orientation, images averaged
        (kept then [nangles * nconfig]), drawn in the engine (series.lwobble =
        1) or given: displacements, per specimen float32 [nconfig, 3, natom].
        want_exit (or preallocated exitwaves, per specimen [nangles, nconfig, n,
        n, 2] float32 arrays or torch tensors): also returns the exit waves.
        images may be a list of preallocated arrays or torch CUDA tensors.
        planes (per specimen None or, per orientation, rows of (defocus,
        rotation, astig, astig_angle) as tilt_series_planes takes them) and
        shifts (per specimen None or [nangles, 2] Angstrom): that specimen's
        own detector planes; its images are then [total planes, n, n]."""
        defocus = np.ascontiguousarray(defocus, np.float64)
        nd = len(defocus)
        descs = (SpecimenDesc * len(specimens))()
        keep, outs, kepts, ews = [], [], [], []
        for i, item in enumerate(specimens):
            sp_, n, aZ, aY = item[:4]
            zc = item[4] if len(item) > 4 else sp_.fov
            arrs = [np.ascontiguousarray(a, dt) for a, dt in
                    ((sp_.Znum, np.int32), (sp_.x, np.float32), (sp_.y, np.float32),
                     (sp_.z, np.float32), (sp_.occ, np.float32))]
            aZ = np.ascontiguousarray(aZ, np.float64)
            aY = np.ascontiguousarray(aY, np.float64)
            pl_i = planes[i] if planes is not None else None
            if pl_i is not None:
                off, parr, total = _plane_arrays(pl_i, len(aZ))
                keep += [off, parr]
                shape = (total, n, n)
            else:
                shape = (len(aZ), nd, n, n)
            img = images[i] if images is not None else np.zeros(shape, np.float32)
            kp = np.zeros(len(aZ) * max(1, nconfig), np.int32)
            keep += arrs + [aZ, aY]
            outs.append(img)
            kepts.append(kp)
            d = descs[i]
            d.natom = len(arrs[1])
            d.Znum, d.x, d.y, d.z, d.occ = [_ptr(a) for a in arrs]
            d.nx = d.ny = n
            d.ctblength, d.ctblengthz = sp_.fov, zc
            d.nangles = len(aZ)
            d.angleZ, d.angleY = _ptr(aZ), _ptr(aY)
            d.images, d.kept = _ptr(img), _ptr(kp)
            d.nconfig = nconfig
            if pl_i is not None:
                d.plane_off, d.planes = _ptr(off), C.addressof(parr)
                if shifts is not None and shifts[i] is not None:
                    sh = np.ascontiguousarray(shifts[i], np.float64).reshape(-1)
                    keep.append(sh)
                    d.shifts = _ptr(sh)
            if exitwaves is not None or want_exit:
                ew = (exitwaves[i] if exitwaves is not None else
                      np.zeros((len(aZ), max(1, nconfig), n, n, 2), np.float32))
                ews.append(ew)
                d.exitwaves = _ptr(ew)
            if displacements is not None and displacements[i] is not None:
                disp = np.ascontiguousarray(displacements[i], np.float32)
                keep.append(disp)
                d.displacements = _ptr(disp)
            wob = getattr(sp_, "wobble", None)
            if wob is not None:
                wob = np.ascontiguousarray(wob, np.float32)
                keep.append(wob)
                d.wobble = _ptr(wob)
        st = self.L.msk_tilt_series_batch(self.h, C.byref(series), len(specimens), descs, nd,
                                          _ptr(defocus), MSK_BATCH_GRAPH if graph else 0)
        self._check(st)
        return (outs, kepts, ews) if ews else (outs, kepts)

    def potential_stack(self, series, Znum, x, y, z, occ, angleZ, angleY, v=None):
        """Per-slice projected potentials v [nangles, nslices, nx, ny] of a tilt
        series (msk_potential_stack); v may be a preallocated torch CUDA tensor."""
        angleZ = np.ascontiguousarray(angleZ, np.float64)
        angleY = np.ascontiguousarray(angleY, np.float64)
        na = len(angleZ)
        ns = slice_count(series.deltaz, series.ctblengthz)
        if v is None:
            v = np.zeros((na, ns, series.nx, series.ny), np.float32)
        kept = np.zeros(na, np.int32)
        arrs = [np.ascontiguousarray(a, dt) for a, dt in
                ((Znum, np.int32), (x, np.float32), (y, np.float32), (z, np.float32),
                 (occ, np.float32))]
        st = self.L.msk_potential_stack(self.h, C.byref(series), len(arrs[1]),
                                        *[_ptr(a) for a in arrs], na, angleZ, angleY, _ptr(v),
                                        _ptr(kept))
        self._check(st)
        return v, kept

    def stack_images(self, stack, v, defocus, images=None):
        """Images [nunits, ndef, nx, ny] of potential stacks v [nunits, nslices,
        nx, ny] (msk_stack_images); v / images may be torch CUDA tensors."""
        v = self._f32(v)
        defocus = np.ascontiguousarray(defocus, np.float64)
        nu = v.shape[0]
        if images is None:
            images = np.zeros((nu, len(defocus), stack.nx, stack.ny), np.float32)
        st = self.L.msk_stack_images(self.h, C.byref(stack), nu, _ptr(v), len(defocus),
                                     _ptr(defocus), _ptr(images))
        self._check(st)
        return images

    def adjoint(self, stack, v, defocus, target, grad=None):
        """(loss, dL/dv) for L = sum (I - target)^2 (msk_adjoint);
        grad has v's shape; v / target / grad may be torch CUDA tensors."""
        v = self._f32(v)
        target = self._f32(target)
        defocus = np.ascontiguousarray(defocus, np.float64)
        nu = v.shape[0]
        if grad is None:
            grad = np.zeros(tuple(v.shape), np.float32)
        loss = C.c_double(0.0)
        st = self.L.msk_adjoint(self.h, C.byref(stack), nu, _ptr(v), len(defocus),
                                      _ptr(defocus), _ptr(target), _ptr(grad), C.byref(loss))
        self._check(st)
        return loss.value, grad

    # -- UTR reconstruction (include/msk_utr.h)
    def utr_depth(self, utr):
        nz = self.L.msk_utr_depth(C.byref(utr))
        if nz < 0:
            raise MskError(nz, "bad UTR geometry")
        return nz

    def utr_reconstruct(self, utr, angles, defocus, images, volume=None, zrot=None, shifts=None):
        """3D potential (TEM) or beta (X-ray) [nz, ny, nx] from one defocused
        image per orientation (msk_utr_reconstruct, or msk_utr_reconstruct_planes
        with zrot / shifts).  angles [nangles, 2]: Z and Y' rotations in degrees;
        defocus [nangles]; zrot [nangles] Z'' angles in degrees and shifts
        [nangles, 2] x, y image shifts, undone first; images [nangles, ny, nx]
        (x fastest, flat-field corrected); images / volume may be torch CUDA
        tensors."""
        ang = np.ascontiguousarray(angles, np.float64).reshape(-1, 2)
        defocus = np.ascontiguousarray(defocus, np.float64)
        images = self._f32(images)
        if volume is None:
            volume = np.zeros((self.utr_depth(utr), utr.ny, utr.nx), np.float32)
        if zrot is None and shifts is None:
            st = self.L.msk_utr_reconstruct(self.h, C.byref(utr), len(ang), ang.reshape(-1),
                                            defocus, _ptr(images), _ptr(volume))
        else:
            zr = None if zrot is None else np.ascontiguousarray(zrot, np.float64)
            sh = None if shifts is None else np.ascontiguousarray(shifts, np.float64).reshape(-1)
            st = self.L.msk_utr_reconstruct_planes(self.h, C.byref(utr), len(ang),
                                                   ang.reshape(-1), defocus, _ptr(zr), _ptr(sh),
                                                   _ptr(images), _ptr(volume))
        self._check(st)
        return volume

    def utr_grid(self, utr, angles, k2four, v3=None, samp3=None):
        """CT_3Dgridding of centred spectra k2four [nangles, ny, nx, 2] into a
        zeroed volume (msk_utr_grid): (v3 [nz, ny, nx, 2], samp3 [nz, ny, nx])."""
        ang = np.ascontiguousarray(angles, np.float64).reshape(-1, 2)
        k2four = self._f32(k2four)
        nz = self.utr_depth(utr)
        if v3 is None:
            v3 = np.zeros((nz, utr.ny, utr.nx, 2), np.float32)
        if samp3 is None:
            samp3 = np.zeros((nz, utr.ny, utr.nx), np.float32)
        st = self.L.msk_utr_grid(self.h, C.byref(utr), len(ang), ang.reshape(-1), _ptr(k2four),
                                 _ptr(v3), _ptr(samp3))
        self._check(st)
        return v3, samp3

    def utr_ctf_correction3d(self, v3, wl, box, defocdist, q2max, cs3, cs5, sigma, epsilon,
                             escc):
        """CTFcorrection3D on a centred complex volume [nz, ny, nx, 2], in place;
        box = (zlo, zhi, ylo, yhi, xlo, xhi), cs in length units."""
        nz, ny, nx = v3.shape[:3]
        st = self.L.msk_utr_ctf_correction3d(self.h, _ptr(v3), nx, ny, nz, wl, *box, defocdist,
                                             q2max, cs3, cs5, sigma, epsilon, int(escc))
        self._check(st)
        return v3

    def utr_inverse_mlaplacian3d(self, v3, zaper, yaper, xaper, alpha, norm):
        """InverseMLaplacian3D on a centred complex volume [nz, ny, nx, 2], in place."""
        nz, ny, nx = v3.shape[:3]
        st = self.L.msk_utr_inverse_mlaplacian3d(self.h, _ptr(v3), nx, ny, nz, zaper, yaper,
                                                 xaper, alpha, norm)
        self._check(st)
        return v3

    def tilt_series_planes(self, series, Znum, x, y, z, occ, angleZ, angleY, planes,
                           shifts=None, nconfig=1, displacements=None, images=None,
                           want_exit=False):
        """Tilt series with per-orientation detector planes (msk_tilt_series_planes).
        planes: per orientation a sequence of (defocus, rotation, astig, astig_angle)
        rows (radians); shifts [nangles, 2] Angstrom.  Returns (images [total planes,
        nx, ny], kept) or (images, exit waves, kept) with want_exit."""
        angleZ = np.ascontiguousarray(angleZ, np.float64)
        angleY = np.ascontiguousarray(angleY, np.float64)
        na = len(angleZ)
        off, arr, total = _plane_arrays(planes, na)
        sh = None if shifts is None else np.ascontiguousarray(shifts, np.float64).reshape(-1)
        if images is None:
            images = np.zeros((total, series.nx, series.ny), np.float32)
        exitwaves = np.zeros((na, nconfig, series.nx, series.ny, 2), np.float32) \
            if want_exit else None
        kept = np.zeros(na * nconfig, np.int32)
        arrs = [np.ascontiguousarray(a, dt) for a, dt in
                ((Znum, np.int32), (x, np.float32), (y, np.float32), (z, np.float32),
                 (occ, np.float32))]
        disp = None if displacements is None else np.ascontiguousarray(displacements, np.float32)
        st = self.L.msk_tilt_series_planes(self.h, C.byref(series), len(arrs[1]),
                                           *[_ptr(a) for a in arrs], na, angleZ, angleY,
                                           _ptr(off), C.addressof(arr), _ptr(sh), nconfig,
                                           _ptr(disp), _ptr(images), _ptr(exitwaves),
                                           _ptr(kept))
        self._check(st)
        return (images, exitwaves, kept) if want_exit else (images, kept)

    def tilt_series_from_file(self, series, Znum, x, y, z, occ, path, **kw):
        """The tilt series a MsctKirkland orientation file (.txt or .relionnew)
        describes: its angles and Z'' rotations in degrees, defoci from the object
        centre, astigmatism and image shifts; images in file order."""
        angles, planes, shifts = read_orientations(path)
        rad = np.pi / 180.0
        pl = [np.stack([p[:, 1], p[:, 0] * rad, p[:, 2], p[:, 3] * rad], axis=1) for p in planes]
        return self.tilt_series_planes(series, Znum, x, y, z, occ, angles[:, 0] * rad,
                                       angles[:, 1] * rad, pl, shifts=shifts, **kw)

    def tilt_series_per_angle(self, series, Znum, x, y, z, occ, angleZ, angleY, defocus,
                              nconfig=1, displacements=None, images=None):
        """The same tilt series through msk_tilt_series_per_angle (orientation by
        orientation, cuFFT, unfused kernels): the comparison form."""
        angleZ = np.ascontiguousarray(angleZ, np.float64)
        angleY = np.ascontiguousarray(angleY, np.float64)
        defocus = np.ascontiguousarray(defocus, np.float64)
        na, nd = len(angleZ), len(defocus)
        if images is None:
            images = np.zeros((na, nd, series.nx, series.ny), np.float32)
        kept = np.zeros(na * nconfig, np.int32)
        arrs = [np.ascontiguousarray(a, dt) for a, dt in
                ((Znum, np.int32), (x, np.float32), (y, np.float32), (z, np.float32),
                 (occ, np.float32))]
        disp = None if displacements is None else np.ascontiguousarray(displacements, np.float32)
        st = self.L.msk_tilt_series_per_angle(self.h, C.byref(series), len(arrs[1]),
                                              *[_ptr(a) for a in arrs], na, angleZ, angleY, nd,
                                              _ptr(defocus), nconfig, _ptr(disp), _ptr(images),
                                              _ptr(kept))
        self._check(st)
        return images, kept
