"""akaze_gb300 - A-KAZE detect + M-LDB describe + 2-NN Hamming match on GB300.

Python face of libakaze_gb300.so, mirroring the reference's API
(libAKAZECU in src/lib/AKAZE.h and its Boost.Python module
python/python_bindings.cpp): AKAZEOptions, AKAZE with
Create_Nonlinear_Scale_Space / Feature_Detection / Compute_Descriptors, and
Matcher with bfmatch / BFMatch.  Every call runs the CUDA library; there is
no CPU fallback (loading fails loudly when the extension is missing).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import (AkazeError, DMATCH_DTYPE, EXTREMUM_DTYPE, KEYPOINT_DTYPE, AkzOptions, AkzTiming, check, load)

PM_G1, PM_G2, WEICKERT, CHARBONNIER = 0, 1, 2, 3
SURF_UPRIGHT, SURF, MSURF_UPRIGHT, MSURF, MLDB_UPRIGHT, MLDB = range(6)
PLANE_LT, PLANE_LSMOOTH, PLANE_LX, PLANE_LY = 0, 1, 3, 4
_PLANES = {"Lt": PLANE_LT, "Lsmooth": PLANE_LSMOOTH, "Lx": PLANE_LX, "Ly": PLANE_LY}


def compile_library(verbose=False, force=False):
    """Compile libakaze_gb300.so in-tree (akaze_gb300/build.py)."""
    import importlib
    return importlib.import_module(__name__ + ".build").build(verbose=verbose, force=force)


class AKAZEOptions(AkzOptions):
    """AKAZEOptions (AKAZEConfig.h:84-172) with the reference defaults."""

    def __init__(self, **kw):
        super().__init__()
        check(load().akz_options_default(ctypes.byref(self)))
        for k, v in kw.items():
            setattr(self, k, v)

    def setWidth(self, w):
        self.img_width = int(w)

    def setHeight(self, h):
        self.img_height = int(h)


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def plan(options, width, height):
    """Level plan of an image (host only, no GPU): list of dicts with size,
    octave, sublevel, esigma, deriv_step, border and the FED taus."""
    L = load()
    n = ctypes.c_int()
    check(L.akz_plan_info(ctypes.byref(options), width, height, -1, ctypes.byref(n), *([None] * 8), 0, None))
    out = []
    for i in range(n.value):
        lw, lh, o, s, ds, ns = (ctypes.c_int() for _ in range(6))
        es, bd = ctypes.c_float(), ctypes.c_float()
        tau = np.zeros(4096, np.float32)
        check(L.akz_plan_info(ctypes.byref(options), width, height, i, None, ctypes.byref(lw), ctypes.byref(lh),
                              ctypes.byref(o), ctypes.byref(s), ctypes.byref(es), ctypes.byref(ds), ctypes.byref(bd),
                              _ptr(tau), 4096, ctypes.byref(ns)))
        out.append({"width": lw.value, "height": lh.value, "octave": o.value, "sublevel": s.value, "esigma": es.value,
                    "deriv_step": ds.value, "border": bd.value, "nsteps": ns.value, "tau": tau[: ns.value].copy()})
    return out


def gaussian_taps(sigma):
    t = np.zeros(64, np.float32)
    n = ctypes.c_int()
    check(load().akz_gaussian_taps(float(sigma), _ptr(t), 64, ctypes.byref(n)))
    return t[: n.value].copy()


def descriptor_bytes(options):
    """Bytes of one descriptor row for the options (AKAZE.cpp:412-423)."""
    b = ctypes.c_int()
    check(load().akz_descriptor_bytes(ctypes.byref(options), ctypes.byref(b)))
    return b.value


class AKAZE:
    """libAKAZECU::AKAZE (AKAZE.h:58-143) over the C ABI."""

    def __init__(self, options):
        self._lib = load()
        self._h = ctypes.c_void_p()
        self.options = options
        check(self._lib.akz_create(ctypes.byref(options), ctypes.byref(self._h)))
        self.width, self.height = options.img_width, options.img_height
        self._n = 0

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.akz_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        self.close()

    def set_stream(self, stream_handle):
        check(self._lib.akz_set_stream(self._h, ctypes.c_void_p(int(stream_handle) if stream_handle else 0)))

    def Create_Nonlinear_Scale_Space(self, img):
        """img: HxW uint8 (0..255) or float32 (0..1), host numpy array."""
        img = np.ascontiguousarray(img)
        if img.dtype == np.uint8:
            dt = 0
        elif img.dtype == np.float32:
            dt = 1
        else:
            raise TypeError("image must be uint8 or float32")
        h, w = img.shape
        check(self._lib.akz_create_nonlinear_scale_space(self._h, _ptr(img), w, h, img.strides[0], dt, 0))
        return 0

    def create_from_device(self, dptr, pitch, dtype=0):
        check(self._lib.akz_create_nonlinear_scale_space(self._h, ctypes.c_void_p(dptr), self.width, self.height,
                                                         pitch, dtype, 1))

    def Feature_Detection(self):
        """Detector + suppression; returns the keypoint count (the reference
        fills the keypoint vector only in Compute_Descriptors)."""
        n = ctypes.c_int()
        check(self._lib.akz_feature_detection(self._h, ctypes.byref(n)))
        self._n = n.value
        return n.value

    def Compute_Descriptors(self):
        """Orientation + M-LDB; returns (descriptors n x row bytes uint8, keypoints)."""
        n = self._n
        kp = np.zeros(n, KEYPOINT_DTYPE)
        d = np.zeros((n, descriptor_bytes(self.options)), np.uint8)
        m = ctypes.c_int()
        check(self._lib.akz_compute_descriptors(self._h, _ptr(kp), _ptr(d), n, ctypes.byref(m)))
        return d[: m.value], kp[: m.value]

    def detect_and_compute(self, img):
        self.Create_Nonlinear_Scale_Space(img)
        self.Feature_Detection()
        d, kp = self.Compute_Descriptors()
        return kp, d

    def Get_Computation_Times(self):
        t = AkzTiming()
        check(self._lib.akz_get_timing(self._h, ctypes.byref(t)))
        return {f: getattr(t, f) for f, _ in AkzTiming._fields_}

    # inspection -------------------------------------------------------------
    @property
    def nlevels(self):
        n = ctypes.c_int()
        check(self._lib.akz_num_levels(self._h, ctypes.byref(n)))
        return n.value

    def level_info(self, level):
        w, h, o, s, n = (ctypes.c_int() for _ in range(5))
        e = ctypes.c_float()
        check(self._lib.akz_level_info(self._h, level, ctypes.byref(w), ctypes.byref(h), ctypes.byref(o),
                                       ctypes.byref(s), ctypes.byref(e), ctypes.byref(n)))
        return {"width": w.value, "height": h.value, "octave": o.value, "sublevel": s.value,
                "esigma": e.value, "nsteps": n.value}

    def plane(self, level, name="Lt"):
        info = self.level_info(level)
        out = np.empty((info["height"], info["width"]), np.float32)
        check(self._lib.akz_get_level_plane(self._h, level, _PLANES[name], _ptr(out)))
        return out

    @property
    def kcontrast(self):
        k = ctypes.c_float()
        check(self._lib.akz_get_kcontrast(self._h, ctypes.byref(k)))
        return k.value

    def extrema(self):
        n = ctypes.c_int()
        check(self._lib.akz_get_extrema(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, EXTREMUM_DTYPE)
        check(self._lib.akz_get_extrema(self._h, _ptr(out), n.value, ctypes.byref(n)))
        return out


class Matcher:
    """libAKAZECU::Matcher (AKAZE.h:29-55): brute-force 2-NN Hamming."""

    def __init__(self):
        self._lib = load()
        self._h = ctypes.c_void_p()
        check(self._lib.akz_matcher_create(ctypes.byref(self._h)))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.akz_matcher_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        self.close()

    def set_stream(self, stream_handle):
        check(self._lib.akz_matcher_set_stream(self._h, ctypes.c_void_p(int(stream_handle) if stream_handle else 0)))

    def bfmatch(self, desc_query, desc_train):
        """Matcher::bfmatch: (nq, 2) DMatch array, best then second best."""
        q = np.ascontiguousarray(desc_query, np.uint8)
        t = np.ascontiguousarray(desc_train, np.uint8)
        if q.ndim != 2 or t.ndim != 2 or (t.shape[0] and q.shape[1] != t.shape[1]):
            raise ValueError("descriptor matrices must be 2-D with equal row sizes")
        nq = q.shape[0]
        out = np.zeros(2 * nq, DMATCH_DTYPE)
        if nq:
            check(self._lib.akz_matcher_bfmatch(self._h, _ptr(q), nq, _ptr(t) if t.size else None, t.shape[0],
                                                q.shape[1], _ptr(out)))
        return out.reshape(nq, 2)

    def BFMatch(self, desc_query, desc_train):
        """Matcher::bfmatch_ (AKAZE.cpp:82-105): (nq, 8) float32 rows
        [queryIdx, trainIdx, 0, distance] for the best and second match."""
        m = self.bfmatch(desc_query, desc_train)
        out = np.zeros((m.shape[0], 8), np.float32)
        for k in range(2):
            out[:, 4 * k + 0] = m[:, k]["queryIdx"]
            out[:, 4 * k + 1] = m[:, k]["trainIdx"]
            out[:, 4 * k + 3] = m[:, k]["distance"]
        return out

    def bfmatch_device(self, q64_ptr, nq, t64_ptr, nt, out_ptr):
        check(self._lib.akz_matcher_bfmatch_device(self._h, ctypes.c_void_p(q64_ptr), nq, ctypes.c_void_p(t64_ptr), nt,
                                                   ctypes.c_void_p(out_ptr)))


class Batch:
    """Many images of uneven sizes, one launch per stage (graph-replayed)."""

    def __init__(self, options, sizes):
        self._lib = load()
        self.sizes = [(int(w), int(h)) for w, h in sizes]
        ws = np.array([w for w, _ in self.sizes], np.int32)
        hs = np.array([h for _, h in self.sizes], np.int32)
        self._h = ctypes.c_void_p()
        check(self._lib.akz_batch_create(ctypes.byref(options), len(self.sizes), _ptr(ws), _ptr(hs), ctypes.byref(self._h)))
        self.n = len(self.sizes)
        self.options = options

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.akz_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        self.close()

    def set_stream(self, stream_handle):
        check(self._lib.akz_batch_set_stream(self._h, ctypes.c_void_p(int(stream_handle) if stream_handle else 0)))

    def upload(self, images):
        imgs = [np.ascontiguousarray(im, np.uint8) for im in images]
        for im, (w, h) in zip(imgs, self.sizes):
            assert im.shape == (h, w)
        ptrs = (ctypes.c_void_p * self.n)(*[im.ctypes.data for im in imgs])
        strides = (ctypes.c_size_t * self.n)(*[im.strides[0] for im in imgs])
        self._keep = imgs
        check(self._lib.akz_batch_upload(self._h, ptrs, strides, 0))

    def input_ptr(self, i):
        p = ctypes.c_void_p()
        pitch = ctypes.c_size_t()
        check(self._lib.akz_batch_input(self._h, i, ctypes.byref(p), ctypes.byref(pitch)))
        return p.value, pitch.value

    def run(self):
        check(self._lib.akz_batch_run(self._h))

    def counts(self):
        c = np.zeros(self.n, np.int32)
        check(self._lib.akz_batch_counts(self._h, _ptr(c)))
        return c

    def results(self, i):
        n = ctypes.c_int()
        check(self._lib.akz_batch_results(self._h, i, None, None, 0, ctypes.byref(n)))
        kp = np.zeros(n.value, KEYPOINT_DTYPE)
        d = np.zeros((n.value, descriptor_bytes(self.options)), np.uint8)
        check(self._lib.akz_batch_results(self._h, i, _ptr(kp), _ptr(d), n.value, ctypes.byref(n)))
        return kp, d

    def device_results(self, i):
        kp = ctypes.c_void_p()
        d = ctypes.c_void_p()
        check(self._lib.akz_batch_device_results(self._h, i, ctypes.byref(kp), ctypes.byref(d)))
        return kp.value, d.value

    def kernel_count(self):
        n = ctypes.c_int()
        check(self._lib.akz_batch_kernel_count(self._h, ctypes.byref(n)))
        return n.value

    def set_surrogate(self, params=None, first_octave=1, check_tol=0.0, s_out=None):
        """Use the learned FED surrogate (FP32 params of akaze_gb300.surrogate,
        or None to switch it off) for the levels of octave >= first_octave."""
        if params is None:
            check(self._lib.akz_batch_set_surrogate(self._h, None, None, ctypes.c_float(0), 1, ctypes.c_float(0)))
            return
        from . import surrogate
        blob, biases = surrogate.pack_inference(params)
        blob = np.ascontiguousarray(blob, np.uint16)
        biases = np.ascontiguousarray(biases, np.float32)
        check(self._lib.akz_batch_set_surrogate(self._h, _ptr(blob), _ptr(biases),
                                                ctypes.c_float(surrogate.S_OUT if s_out is None else s_out),
                                                int(first_octave), ctypes.c_float(check_tol)))

    def autotune(self):
        """Pick the FED blocking depth (4..8) of every level by timing the
        uploaded batch; returns (depth per level from 1, {depth: stage ms
        with every level at that depth})."""
        ms = np.zeros(5, np.float32)
        dl = np.full(64, -1, np.int32)
        check(self._lib.akz_batch_autotune(self._h, _ptr(ms), 5, _ptr(dl), 64))
        return [int(x) for x in dl[1:] if x > 0], {4 + k: float(v) for k, v in enumerate(ms)}

    def set_fed_depth(self, depth):
        check(self._lib.akz_batch_set_fed_depth(self._h, int(depth)))

    def surrogate_errors(self):
        n = ctypes.c_int()
        check(self._lib.akz_batch_surrogate_errors(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, np.float32)
        check(self._lib.akz_batch_surrogate_errors(self._h, _ptr(out), n.value, ctypes.byref(n)))
        return out

    def profile(self):
        """Per-stage device ms of one run (contrast, level 0, levels, detector,
        scan+extract, suppression, orientation+M-LDB)."""
        ms = np.zeros(7, np.float32)
        check(self._lib.akz_batch_profile(self._h, _ptr(ms), 7))
        return ms

    def detect_describe(self, images, capacity=None):
        """Whole job through the C ABI: host u8 in, host keypoints/descriptors out."""
        imgs = [np.ascontiguousarray(im, np.uint8) for im in images]
        cap = capacity or self.options.maxkeypoints
        if not hasattr(self, "_out") or self._out[0] != cap:
            kps = [np.zeros(cap, KEYPOINT_DTYPE) for _ in range(self.n)]
            ds = [np.zeros((cap, descriptor_bytes(self.options)), np.uint8) for _ in range(self.n)]
            self._out = (cap, kps, ds)
        _, kps, ds = self._out
        return self.detect_describe_into(imgs, kps, ds)

    def detect_describe_into(self, imgs, kps, ds):
        ptrs = (ctypes.c_void_p * self.n)(*[im.ctypes.data for im in imgs])
        strides = (ctypes.c_size_t * self.n)(*[im.strides[0] for im in imgs])
        kp_p = (ctypes.c_void_p * self.n)(*[k.ctypes.data for k in kps])
        d_p = (ctypes.c_void_p * self.n)(*[d.ctypes.data for d in ds])
        caps = np.array([len(k) for k in kps], np.int32)
        counts = np.zeros(self.n, np.int32)
        check(self._lib.akz_batch_detect_describe(self._h, ptrs, strides, kp_p, d_p, _ptr(caps), _ptr(counts)))
        return counts

    def detect_describe_packed(self, imgs, kp_out, d_out):
        """Whole job with packed output: kp_out (capacity records) and d_out
        (capacity x descriptor_bytes(options)) receive all images' results back to back; returns
        the per-image counts."""
        ptrs = (ctypes.c_void_p * self.n)(*[im.ctypes.data for im in imgs])
        strides = (ctypes.c_size_t * self.n)(*[im.strides[0] for im in imgs])
        counts = np.zeros(self.n, np.int32)
        total = ctypes.c_int()
        check(self._lib.akz_batch_detect_describe_packed(self._h, ptrs, strides, _ptr(kp_out), _ptr(d_out), len(kp_out),
                                                         _ptr(counts), ctypes.byref(total)))
        return counts

    def image_info(self, i):
        """(raw extrema, keypoints, suppression rounds, contrast factor) of image i."""
        nraw, nkp, rounds = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        kc = ctypes.c_float()
        check(self._lib.akz_batch_image_info(self._h, int(i), ctypes.byref(nraw), ctypes.byref(nkp),
                                             ctypes.byref(rounds), ctypes.byref(kc)))
        return nraw.value, nkp.value, rounds.value, kc.value

    def set_nms_round_cap(self, cap):
        """Suppression rounds before an image reports AKZ_ERR_TIMEOUT (default 2^20)."""
        check(self._lib.akz_batch_set_nms_round_cap(self._h, int(cap)))

    def submit(self, imgs):
        """First half of detect_describe_packed: enqueues the upload, the
        graph, the device-side packing and the count read-back, and returns
        at once.  Up to two runs may be outstanding; the images of a run must
        stay unchanged until it is collected."""
        sub = [np.ascontiguousarray(im, np.uint8) for im in imgs]
        ptrs = (ctypes.c_void_p * self.n)(*[im.ctypes.data for im in sub])
        strides = (ctypes.c_size_t * self.n)(*[im.strides[0] for im in sub])
        check(self._lib.akz_batch_submit(self._h, ptrs, strides))
        self._subs = getattr(self, "_subs", []) + [sub]  # kept until collected

    def discard_outstanding(self):
        """Waits for and drops every submitted run not yet collected (after
        an error part way through a pipeline)."""
        kp = np.zeros(0, KEYPOINT_DTYPE)
        d = np.zeros((0, max(descriptor_bytes(self.options), 1)), np.uint8)
        while getattr(self, "_subs", []):
            try:
                self.collect_packed(kp, d)
            except AkazeError:
                pass  # the run is dropped whatever the collect reports

    def collect_packed(self, kp_out, d_out):
        """Second half: waits for the oldest submitted run of this batch,
        writes its results packed into kp_out / d_out; returns (per-image
        counts, total)."""
        counts = np.zeros(self.n, np.int32)
        total = ctypes.c_int()
        try:
            check(self._lib.akz_batch_collect_packed(self._h, _ptr(kp_out), _ptr(d_out), len(kp_out), _ptr(counts),
                                                     ctypes.byref(total)))
        finally:
            self._subs = getattr(self, "_subs", [])[1:]
        return counts, total.value

    def plane(self, i, level, name="Lt", shape=None):
        out = np.empty(shape, np.float32)
        check(self._lib.akz_batch_level_plane(self._h, i, level, _PLANES[name], _ptr(out)))
        return out


class BatchGroup:
    """A batch split into `groups` native batches of consecutive images, each
    with its own CUDA stream and captured graph, so that the stages of one
    group overlap those of the others on the GPU (suppression is one CTA per
    image, the small FED levels leave SMs idle, and host<->device copies of
    one group overlap the kernels of another).  Results equal those of one
    Batch over the same images; image i keeps its index."""

    def __init__(self, options, sizes, groups=2):
        sizes = [(int(w), int(h)) for w, h in sizes]
        groups = max(1, min(int(groups), len(sizes)))
        bounds = [len(sizes) * g // groups for g in range(groups + 1)]
        self.parts = [Batch(options, sizes[bounds[g]:bounds[g + 1]]) for g in range(groups)]
        self.bounds = bounds
        self.sizes = sizes
        self.n = len(sizes)
        self.options = options

    def _locate(self, i):
        for g, b in enumerate(self.parts):
            if i < self.bounds[g + 1]:
                return b, i - self.bounds[g]
        raise IndexError(i)

    def close(self):
        for b in self.parts:
            b.close()

    def set_streams(self, handles):
        for b, h in zip(self.parts, handles):
            b.set_stream(h)

    def set_fed_depth(self, depth):
        for b in self.parts:
            b.set_fed_depth(depth)

    def autotune(self):
        return [b.autotune() for b in self.parts]

    def upload(self, images):
        for g, b in enumerate(self.parts):
            b.upload(images[self.bounds[g]:self.bounds[g + 1]])

    def run(self):
        """Launches every group (asynchronous, each on its own stream)."""
        for b in self.parts:
            b.run()

    def counts(self):
        return np.concatenate([b.counts() for b in self.parts])

    def results(self, i):
        b, k = self._locate(i)
        return b.results(k)

    def plane(self, i, level, name="Lt", shape=None):
        b, k = self._locate(i)
        return b.plane(k, level, name, shape)

    def detect_describe_packed(self, imgs, kp_out, d_out):
        """Whole job with host buffers: every group is submitted (upload,
        graph, count read-back, all asynchronous on its own stream), then
        collected in order, each into kp_out / d_out right after the groups
        before it, so a group's copies overlap the others' kernels.  Returns
        the per-image counts."""
        return self.detect_describe_packed_steps([imgs], kp_out, d_out)

    def detect_describe_packed_steps(self, steps, kp_out, d_out, on_step=None):
        """Several whole-job calls in a row (`steps`: one image list per
        step), pipelined two deep: every group has its next step submitted
        while its current one computes, and a step is collected (packed
        results copied out beside the next step's graph) before the step
        after the next is submitted.  Each step's results are packed into
        kp_out / d_out (overwritten by the next step); on_step(step_index,
        counts), if given, runs after a step is collected.  Returns the last
        step's per-image counts."""
        part = lambda si, g: steps[si][self.bounds[g]:self.bounds[g + 1]]
        counts = None
        try:
            for si in range(min(2, len(steps))):
                for g, b in enumerate(self.parts):
                    b.submit(part(si, g))
            for si in range(len(steps)):
                at, parts = 0, []
                for g, b in enumerate(self.parts):
                    c, n = b.collect_packed(kp_out[at:], d_out[at:])
                    parts.append(c)
                    at += n
                    if si + 2 < len(steps):
                        b.submit(part(si + 2, g))
                counts = np.concatenate(parts)
                if on_step:
                    on_step(si, counts)
        except BaseException:
            for b in self.parts:  # leave every group usable
                b.discard_outstanding()
            raise
        return counts


def save_keypoints(path, kpts, desc=None, save_desc=None):
    """save_keypoints (utils.cpp:97-152): Mikolajczyk text format.  save_desc
    (default: desc given) only sets the header's descriptor length; as in
    the reference, rows carry desc's bytes whenever desc is given."""
    kp = np.ascontiguousarray(kpts, KEYPOINT_DTYPE)
    d = None if desc is None else np.ascontiguousarray(desc, np.uint8)
    if save_desc is None:
        save_desc = d is not None
    check(load().akz_save_keypoints(str(path).encode(), _ptr(kp) if kp.size else None, len(kp),
                                    _ptr(d) if d is not None and d.size else None,
                                    0 if d is None else d.shape[1], int(bool(save_desc))))
