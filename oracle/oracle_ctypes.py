"""ctypes access to the CPU oracle (oracle/libakaze_oracle.so).

Test infrastructure only: imported by tests/, by __graft_entry__.smoke() and by
the cpu_baseline / --impl reference legs of bench.py, always as the checker or
as the timed CPU baseline, never as the product path.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libakaze_oracle.so")
_REF_PATH = os.path.join(_HERE, "_ref", "libfed_ref.so")


class AkoOptions(ctypes.Structure):
    _fields_ = [
        ("omax", ctypes.c_int), ("nsublevels", ctypes.c_int),
        ("soffset", ctypes.c_float), ("derivative_factor", ctypes.c_float),
        ("sderivatives", ctypes.c_float), ("diffusivity", ctypes.c_int),
        ("dthreshold", ctypes.c_float), ("min_dthreshold", ctypes.c_float),
        ("descriptor", ctypes.c_int), ("descriptor_size", ctypes.c_int),
        ("descriptor_channels", ctypes.c_int), ("descriptor_pattern_size", ctypes.c_int),
        ("kcontrast_percentile", ctypes.c_float), ("kcontrast_nbins", ctypes.c_int),
        ("extrema_3d", ctypes.c_int),
    ]


class AkoLevel(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int), ("height", ctypes.c_int), ("octave", ctypes.c_int),
        ("sublevel", ctypes.c_int), ("esigma", ctypes.c_float), ("etime", ctypes.c_float),
        ("deriv_step", ctypes.c_int), ("size", ctypes.c_float), ("border", ctypes.c_float),
        ("nsteps", ctypes.c_int), ("kcontrast", ctypes.c_float),
    ]


KEYPOINT_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("size", "<f4"), ("angle", "<f4"),
                           ("response", "<f4"), ("octave", "<i4"), ("class_id", "<i4")])
DMATCH_DTYPE = np.dtype([("queryIdx", "<i4"), ("trainIdx", "<i4"), ("imgIdx", "<i4"), ("distance", "<f4")])
EXTREMUM_DTYPE = np.dtype([("x", "<i4"), ("y", "<i4"), ("level", "<i4"), ("octave", "<i4"),
                           ("response", "<f4"), ("size", "<f4"), ("octsub", "<f4"), ("dst1", "<f4")])

PLANES = {"Lt": 0, "Lsmooth": 1, "Lflow": 2, "Lx": 3, "Ly": 4, "Ldet": 5}


def reference_dir():
    """The reference source tree: $AKZ_REFERENCE_DIR, else a `reference`
    directory beside the repository (absent on machines without it)."""
    env = os.environ.get("AKZ_REFERENCE_DIR")
    if env:
        return env
    return os.path.normpath(os.path.join(_HERE, "..", "..", "reference"))


def build(quiet=True):
    """Compile the oracle (and oracle/_ref when the reference tree exists)."""
    out = subprocess.run(["make", "-C", _HERE, "all"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    ref_src = reference_dir()
    if os.path.isfile(os.path.join(ref_src, "src", "lib", "fed.cpp")):
        out = subprocess.run(["make", "-C", _HERE, "ref", "REF=" + ref_src], capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError("oracle/_ref build failed:\n" + out.stdout + out.stderr)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        L.ako_create.restype = P
        L.ako_create.argtypes = [ctypes.POINTER(AkoOptions), ctypes.c_int, ctypes.c_int]
        L.ako_destroy.argtypes = [P]
        L.ako_options_default.argtypes = [ctypes.POINTER(AkoOptions)]
        for name in ("ako_num_levels", "ako_num_extrema", "ako_num_keypoints", "ako_detect", "ako_describe"):
            getattr(L, name).argtypes = [P]
            getattr(L, name).restype = ctypes.c_int
        L.ako_get_level.argtypes = [P, ctypes.c_int, ctypes.POINTER(AkoLevel)]
        L.ako_get_tau.argtypes = [P, ctypes.c_int, P, ctypes.c_int]
        L.ako_fed_tau_by_process_time.argtypes = [ctypes.c_float, ctypes.c_int, ctypes.c_float, ctypes.c_int, P, ctypes.c_int]
        L.ako_gaussian_taps.argtypes = [ctypes.c_float, P, ctypes.c_int]
        L.ako_u8_to_unit.argtypes = [P, P, ctypes.c_long]
        L.ako_build.argtypes = [P, P]
        L.ako_build_f64.argtypes = [P, P]
        L.ako_kcontrast.argtypes = [P]
        L.ako_kcontrast.restype = ctypes.c_float
        L.ako_kcontrast_f64.argtypes = [P]
        L.ako_kcontrast_f64.restype = ctypes.c_double
        L.ako_get_plane.argtypes = [P, ctypes.c_int, ctypes.c_int, P]
        L.ako_get_plane_f64.argtypes = [P, ctypes.c_int, P]
        L.ako_get_extrema.argtypes = [P, P, ctypes.c_int]
        L.ako_get_level_offsets.argtypes = [P, P, ctypes.c_int]
        L.ako_get_nms_state.argtypes = [P, P, ctypes.c_int]
        L.ako_get_keypoints.argtypes = [P, P, ctypes.c_int]
        L.ako_get_descriptors.argtypes = [P, P, ctypes.c_int]
        L.ako_run_u8.argtypes = [P, P]
        L.ako_bfmatch.argtypes = [P, ctypes.c_int, P, ctypes.c_int, ctypes.c_int, P]
        L.ako_set_threads.argtypes = [ctypes.c_int]
        L.ako_descriptor_bytes.argtypes = [P]
        L.ako_mldb_table.argtypes = [ctypes.c_int, ctypes.c_int, P, P]
        L.ako_glibc_rand_sequence.argtypes = [ctypes.c_uint32, P, ctypes.c_int]
        _lib = L
    return _lib


def default_options(**kw):
    o = AkoOptions()
    lib().ako_options_default(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def set_threads(n):
    lib().ako_set_threads(int(n))


def u8_to_unit(img):
    img = np.ascontiguousarray(img, dtype=np.uint8)
    out = np.empty(img.shape, np.float32)
    lib().ako_u8_to_unit(img.ctypes.data, out.ctypes.data, img.size)
    return out


def fed_tau(T, M=1, tau_max=0.25, reordering=True, cap=4096):
    buf = np.zeros(cap, np.float32)
    n = lib().ako_fed_tau_by_process_time(float(T), int(M), float(tau_max), int(bool(reordering)), buf.ctypes.data, cap)
    return buf[:n].copy()


def fed_tau_reference(T, M=1, tau_max=0.25, reordering=True, cap=4096):
    """The reference's own fed.cpp (oracle/_ref/libfed_ref.so); None if not built."""
    if not os.path.exists(_REF_PATH):
        return None
    R = ctypes.CDLL(_REF_PATH)
    R.fedref_tau_by_process_time.argtypes = [ctypes.c_float, ctypes.c_int, ctypes.c_float, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    buf = np.zeros(cap, np.float32)
    n = R.fedref_tau_by_process_time(float(T), int(M), float(tau_max), int(bool(reordering)), buf.ctypes.data, cap)
    return buf[:n].copy()


_NLD_REF_PATH = os.path.join(_HERE, "_ref", "libnld_ref.so")
_nld_ref = None


def nld_ref():
    """The reference's own nldiffusion_functions.cpp and utils.cpp
    (oracle/_ref/libnld_ref.so, built where the reference tree is present);
    None if not built."""
    global _nld_ref
    if _nld_ref is None and os.path.exists(_NLD_REF_PATH):
        lib()  # the shim routes its filters to the oracle library, load it first
        R = ctypes.CDLL(_NLD_REF_PATH)
        P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        R.nldref_pm_g2.argtypes = [P, P, P, I, I, F]
        R.nldref_nld_step.argtypes = [P, P, I, I, F]
        R.nldref_k_percentile.argtypes = [P, I, I, F, F, I, P]
        R.nldref_k_percentile.restype = F
        R.nldref_gaussian.argtypes = [P, P, I, I, F, P]
        R.utilsref_save_keypoints.argtypes = [ctypes.c_char_p, P, I, P, I, I]
        R.utilsref_nndr_inliers.argtypes = [P, I, P, I, P, I, P, F, F, P, P, P]
        _nld_ref = R
    return _nld_ref


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def plane_conductance(lx, ly, k, kind=1):
    """The oracle's conductance (kind 1 = PM-g2) of (lx, ly) planes."""
    lx, ly = _f32(lx), _f32(ly)
    out = np.empty_like(lx)
    L = lib()
    L.ako_plane_conductance.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_long, ctypes.c_float, ctypes.c_int]
    L.ako_plane_conductance(lx.ctypes.data, ly.ctypes.data, out.ctypes.data, lx.size, float(k), int(kind))
    return out


def plane_nld_step(Ld, c, stepsize):
    """One oracle FED step of Ld (h x w) with conductance c."""
    out, c = _f32(Ld).copy(), _f32(c)
    L = lib()
    L.ako_plane_nld_step.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_float]
    L.ako_plane_nld_step(out.ctypes.data, c.ctypes.data, out.shape[1], out.shape[0], float(stepsize))
    return out


def plane_k_percentile(img, perc=0.7, nbins=300, gscale=1.0):
    img = _f32(img)
    L = lib()
    L.ako_plane_k_percentile.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_int,
                                         ctypes.c_float]
    L.ako_plane_k_percentile.restype = ctypes.c_float
    return np.float32(L.ako_plane_k_percentile(img.ctypes.data, img.shape[1], img.shape[0], float(perc), int(nbins),
                                               float(gscale)))


def plane_gaussian(img, sigma):
    """The oracle's Gaussian of sigma and the kernel size it used."""
    img = _f32(img)
    out = np.empty_like(img)
    ks = ctypes.c_int(0)
    L = lib()
    L.ako_plane_gaussian.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                     ctypes.c_void_p]
    if L.ako_plane_gaussian(img.ctypes.data, out.ctypes.data, img.shape[1], img.shape[0], float(sigma),
                            ctypes.byref(ks)) != 0:
        raise ValueError(sigma)
    return out, ks.value


def gaussian_taps(sigma):
    buf = np.zeros(129, np.float32)
    n = lib().ako_gaussian_taps(float(sigma), buf.ctypes.data, 129)
    return buf[:n].copy()


def mldb_table(channels=3, descriptor_size=0):
    """The oracle's M-LDB comparison table: (c1, c2) value indices 3*cell + channel."""
    c1 = np.zeros(512, np.int32)
    c2 = np.zeros(512, np.int32)
    n = lib().ako_mldb_table(int(channels), int(descriptor_size), c1.ctypes.data, c2.ctypes.data)
    return c1[:n].copy(), c2[:n].copy()


def glibc_rand_sequence(seed, n):
    out = np.zeros(n, np.int32)
    lib().ako_glibc_rand_sequence(int(seed), out.ctypes.data, int(n))
    return out


def bfmatch(q, t):
    q = np.ascontiguousarray(q, np.uint8)
    t = np.ascontiguousarray(t, np.uint8)
    nq, rb = q.shape
    out = np.zeros(2 * nq, DMATCH_DTYPE)
    r = lib().ako_bfmatch(q.ctypes.data, nq, t.ctypes.data if t.size else None, t.shape[0], rb, out.ctypes.data)
    if r != 0:
        raise ValueError("ako_bfmatch failed")
    return out.reshape(nq, 2) if nq else out.reshape(0, 2)


class Oracle:
    """One image through the oracle: scale space, detector, descriptors."""

    def __init__(self, width, height, options=None):
        self.opt = options if options is not None else default_options()
        self.ptr = lib().ako_create(ctypes.byref(self.opt), int(width), int(height))
        if not self.ptr:
            raise ValueError("oracle rejected the options or the image size")
        self.width, self.height = width, height

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().ako_destroy(self.ptr)
            self.ptr = None

    @property
    def nlevels(self):
        return lib().ako_num_levels(self.ptr)

    def level(self, i):
        L = AkoLevel()
        if lib().ako_get_level(self.ptr, i, ctypes.byref(L)) != 0:
            raise IndexError(i)
        return {f: getattr(L, f) for f, _ in AkoLevel._fields_}

    def tau(self, i):
        buf = np.zeros(4096, np.float32)
        n = lib().ako_get_tau(self.ptr, i, buf.ctypes.data, 4096)
        return buf[:n].copy()

    def build(self, img):
        img = np.ascontiguousarray(img)
        if img.dtype == np.uint8:
            img = u8_to_unit(img)
        img = np.ascontiguousarray(img, np.float32)
        assert img.shape == (self.height, self.width)
        if lib().ako_build(self.ptr, img.ctypes.data) != 0:
            raise RuntimeError("ako_build failed")

    def build_f64(self, img):
        img = np.ascontiguousarray(img)
        if img.dtype == np.uint8:
            img = u8_to_unit(img)
        img = np.ascontiguousarray(img, np.float32)
        if lib().ako_build_f64(self.ptr, img.ctypes.data) != 0:
            raise RuntimeError("ako_build_f64 failed")

    @property
    def kcontrast(self):
        return lib().ako_kcontrast(self.ptr)

    @property
    def kcontrast_f64(self):
        return lib().ako_kcontrast_f64(self.ptr)

    def plane(self, level, name="Lt"):
        L = self.level(level)
        out = np.empty((L["height"], L["width"]), np.float32)
        if lib().ako_get_plane(self.ptr, level, PLANES[name], out.ctypes.data) != 0:
            raise RuntimeError("ako_get_plane failed")
        return out

    def plane_f64(self, level):
        L = self.level(level)
        out = np.empty((L["height"], L["width"]), np.float64)
        if lib().ako_get_plane_f64(self.ptr, level, out.ctypes.data) != 0:
            raise RuntimeError("ako_get_plane_f64 failed")
        return out

    def detect(self):
        n = lib().ako_detect(self.ptr)
        if n < 0:
            raise RuntimeError("ako_detect failed")
        return n

    def extrema(self):
        n = lib().ako_num_extrema(self.ptr)
        out = np.zeros(max(n, 0), EXTREMUM_DTYPE)
        lib().ako_get_extrema(self.ptr, out.ctypes.data, n)
        return out

    def level_offsets(self):
        out = np.zeros(self.nlevels + 1, np.int32)
        lib().ako_get_level_offsets(self.ptr, out.ctypes.data, out.size)
        return out

    def nms_state(self):
        n = lib().ako_num_extrema(self.ptr)
        out = np.zeros(max(n, 0), np.int32)
        lib().ako_get_nms_state(self.ptr, out.ctypes.data, n)
        return out

    def keypoints(self):
        n = lib().ako_num_keypoints(self.ptr)
        out = np.zeros(max(n, 0), KEYPOINT_DTYPE)
        lib().ako_get_keypoints(self.ptr, out.ctypes.data, n)
        return out

    def describe(self):
        n = lib().ako_describe(self.ptr)
        if n < 0:
            raise RuntimeError("ako_describe failed")
        out = np.zeros((n, lib().ako_descriptor_bytes(self.ptr)), np.uint8)
        lib().ako_get_descriptors(self.ptr, out.ctypes.data, n)
        return out

    def run(self, img_u8):
        """Whole path on one u8 image; returns (keypoints, descriptors)."""
        img_u8 = np.ascontiguousarray(img_u8, np.uint8)
        n = lib().ako_run_u8(self.ptr, img_u8.ctypes.data)
        if n < 0:
            raise RuntimeError("ako_run_u8 failed")
        kp = self.keypoints()
        d = np.zeros((n, lib().ako_descriptor_bytes(self.ptr)), np.uint8)
        lib().ako_get_descriptors(self.ptr, d.ctypes.data, n)
        return kp, d
