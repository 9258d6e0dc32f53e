"""Loads libakaze_gb300.so (built in-tree by akaze_gb300/build.py) and
declares the C ABI of include/akaze_gb300.h for ctypes."""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libakaze_gb300.so")

AKZ_OK, AKZ_ERR_INVALID_ARG, AKZ_ERR_OOM, AKZ_ERR_CUDA, AKZ_ERR_OVERFLOW, AKZ_ERR_TIMEOUT, AKZ_ERR_UNSUPPORTED, AKZ_ERR_STATE = range(8)
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA_ERROR", 4: "OVERFLOW", 5: "TIMEOUT", 6: "UNSUPPORTED", 7: "STATE"}

KEYPOINT_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("size", "<f4"), ("angle", "<f4"),
                           ("response", "<f4"), ("octave", "<i4"), ("class_id", "<i4")])
DMATCH_DTYPE = np.dtype([("queryIdx", "<i4"), ("trainIdx", "<i4"), ("imgIdx", "<i4"), ("distance", "<f4")])
EXTREMUM_DTYPE = np.dtype([("x", "<i4"), ("y", "<i4"), ("level", "<i4"), ("octave", "<i4"),
                           ("response", "<f4"), ("size", "<f4"), ("octsub", "<f4"), ("dst1", "<f4")])

# every symbol include/akaze_gb300.h declares
EXPORTS = [
    "akz_version", "akz_last_error", "akz_options_default", "akz_plan_info", "akz_gaussian_taps", "akz_create", "akz_destroy", "akz_set_stream",
    "akz_create_nonlinear_scale_space", "akz_feature_detection", "akz_compute_descriptors", "akz_get_timing",
    "akz_num_levels", "akz_level_info", "akz_get_level_plane", "akz_get_kcontrast", "akz_get_extrema",
    "akz_batch_create", "akz_batch_destroy", "akz_batch_set_stream", "akz_batch_upload", "akz_batch_input",
    "akz_batch_run", "akz_batch_counts", "akz_batch_results", "akz_batch_device_results",
    "akz_batch_detect_describe", "akz_batch_level_plane", "akz_batch_kernel_count", "akz_batch_profile",
    "akz_matcher_create", "akz_matcher_destroy", "akz_matcher_set_stream", "akz_matcher_bfmatch",
    "akz_matcher_bfmatch_device", "akz_matcher_bfmatch_noalloc", "akz_measure_popc_rate",
    "akz_sg_conv_forward", "akz_sg_conv_backward_data", "akz_sg_conv_backward_weights", "akz_sg_adam",
    "akz_sg_weight_elems", "akz_sg_infer_level", "akz_sg_mse_grad", "akz_batch_set_surrogate",
    "akz_batch_surrogate_errors", "akz_nndr_homography_inliers", "akz_save_keypoints",
    "akz_batch_detect_describe_packed", "akz_sg_set_tcgen05", "akz_sg_tcgen05_status", "akz_selfcheck_pm_g2",
    "akz_batch_autotune", "akz_batch_set_fed_depth", "akz_batch_submit", "akz_batch_collect_packed",
    "akz_batch_image_info", "akz_batch_set_nms_round_cap", "akz_selfcheck_bounded_wait", "akz_selfcheck_matcher_timeout", "akz_descriptor_bytes",
    "akz_matcher_set_tensor_cores", "akz_matcher_tensor_status",
]


class AkzOptions(ctypes.Structure):
    _fields_ = [
        ("omin", ctypes.c_int), ("omax", ctypes.c_int), ("nsublevels", ctypes.c_int),
        ("img_width", ctypes.c_int), ("img_height", ctypes.c_int),
        ("soffset", ctypes.c_float), ("derivative_factor", ctypes.c_float), ("sderivatives", ctypes.c_float),
        ("diffusivity", ctypes.c_int), ("dthreshold", ctypes.c_float), ("min_dthreshold", ctypes.c_float),
        ("descriptor", ctypes.c_int), ("descriptor_size", ctypes.c_int), ("descriptor_channels", ctypes.c_int),
        ("descriptor_pattern_size", ctypes.c_int), ("kcontrast", ctypes.c_float),
        ("kcontrast_percentile", ctypes.c_float), ("kcontrast_nbins", ctypes.c_size_t),
        ("save_scale_space", ctypes.c_int), ("save_keypoints", ctypes.c_int), ("verbosity", ctypes.c_int),
        ("ncudaimages", ctypes.c_int), ("maxkeypoints", ctypes.c_int), ("extrema_3d", ctypes.c_int), ("fast_math", ctypes.c_int),
    ]


class AkzTiming(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("kcontrast", "scale", "derivatives", "detector", "extrema", "subpixel", "descriptor")]


class AkazeError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


_lib = None


def load():
    """The loaded library; raises if the CUDA extension has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with python -m akaze_gb300.build "
                          "(the library has no CPU fallback)")
    L = ctypes.CDLL(LIB_PATH)
    P, I, S = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
    IP = ctypes.POINTER(ctypes.c_int)
    sig = {
        "akz_version": ([], ctypes.c_char_p), "akz_last_error": ([], ctypes.c_char_p),
        "akz_options_default": ([ctypes.POINTER(AkzOptions)], I),
        "akz_descriptor_bytes": ([ctypes.POINTER(AkzOptions), IP], I),
        "akz_matcher_set_tensor_cores": ([I], I), "akz_matcher_tensor_status": ([IP], I),
        "akz_plan_info": ([ctypes.POINTER(AkzOptions), I, I, I, IP, IP, IP, IP, IP, ctypes.POINTER(ctypes.c_float), IP,
                           ctypes.POINTER(ctypes.c_float), P, I, IP], I),
        "akz_gaussian_taps": ([ctypes.c_float, P, I, IP], I),
        "akz_create": ([ctypes.POINTER(AkzOptions), ctypes.POINTER(P)], I),
        "akz_destroy": ([P], I), "akz_set_stream": ([P, P], I),
        "akz_create_nonlinear_scale_space": ([P, P, I, I, S, I, I], I),
        "akz_feature_detection": ([P, IP], I),
        "akz_compute_descriptors": ([P, P, P, I, IP], I),
        "akz_get_timing": ([P, ctypes.POINTER(AkzTiming)], I),
        "akz_num_levels": ([P, IP], I),
        "akz_level_info": ([P, I, IP, IP, IP, IP, ctypes.POINTER(ctypes.c_float), IP], I),
        "akz_get_level_plane": ([P, I, I, P], I),
        "akz_get_kcontrast": ([P, ctypes.POINTER(ctypes.c_float)], I),
        "akz_get_extrema": ([P, P, I, IP], I),
        "akz_batch_create": ([ctypes.POINTER(AkzOptions), I, P, P, ctypes.POINTER(P)], I),
        "akz_batch_destroy": ([P], I), "akz_batch_set_stream": ([P, P], I),
        "akz_batch_upload": ([P, P, P, I], I),
        "akz_batch_input": ([P, I, ctypes.POINTER(P), ctypes.POINTER(S)], I),
        "akz_batch_run": ([P], I), "akz_batch_counts": ([P, P], I),
        "akz_batch_results": ([P, I, P, P, I, IP], I),
        "akz_batch_device_results": ([P, I, ctypes.POINTER(P), ctypes.POINTER(P)], I),
        "akz_batch_detect_describe": ([P, P, P, P, P, P, P], I),
        "akz_batch_level_plane": ([P, I, I, I, P], I),
        "akz_batch_kernel_count": ([P, IP], I),
        "akz_batch_profile": ([P, P, I], I),
        "akz_matcher_create": ([ctypes.POINTER(P)], I), "akz_matcher_destroy": ([P], I),
        "akz_matcher_set_stream": ([P, P], I),
        "akz_matcher_bfmatch": ([P, P, I, P, I, I, P], I),
        "akz_matcher_bfmatch_device": ([P, P, I, P, I, P], I),
        "akz_matcher_bfmatch_noalloc": ([P, I, P, I, P, P], I),
        "akz_measure_popc_rate": ([I, ctypes.POINTER(ctypes.c_double), P], I),
        "akz_sg_conv_forward": ([P, P, P, P, I, I, I, I, I, I, P], I),
        "akz_sg_conv_backward_data": ([P, P, P, P, I, I, I, I, I, P], I),
        "akz_sg_conv_backward_weights": ([P, P, P, P, I, I, I, I, I, P], I),
        "akz_sg_adam": ([P, P, P, P, I, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, I, P], I),
        "akz_sg_weight_elems": ([], ctypes.c_size_t),
        "akz_sg_mse_grad": ([P, P, P, I, ctypes.c_float, P, I, P], I),
        "akz_batch_set_surrogate": ([P, P, P, ctypes.c_float, I, ctypes.c_float], I),
        "akz_batch_surrogate_errors": ([P, P, I, IP], I),
        "akz_nndr_homography_inliers": ([P, I, P, P, P, ctypes.c_float, ctypes.c_float, P, P, P], I),
        "akz_save_keypoints": ([ctypes.c_char_p, P, I, P, I, I], I),
        "akz_batch_detect_describe_packed": ([P, P, P, P, P, I, P, IP], I),
        "akz_sg_set_tcgen05": ([I], I),
        "akz_sg_tcgen05_status": ([IP], I),
        "akz_selfcheck_pm_g2": ([P, P, I, I, P], I),
        "akz_batch_autotune": ([P, P, I, P, I], I),
        "akz_batch_set_fed_depth": ([P, I], I),
        "akz_batch_submit": ([P, P, P], I),
        "akz_batch_image_info": ([P, I, IP, IP, IP, ctypes.POINTER(ctypes.c_float)], I),
        "akz_batch_set_nms_round_cap": ([P, I], I),
        "akz_selfcheck_bounded_wait": ([I, I, IP], I),
        "akz_selfcheck_matcher_timeout": ([I, IP], I),
        "akz_batch_collect_packed": ([P, P, P, I, P, IP], I),
        "akz_sg_infer_level": ([P, P, ctypes.c_size_t, I, I, ctypes.c_float, ctypes.c_float, P, P, P, P, P], I),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def check(status):
    if status != AKZ_OK:
        raise AkazeError(status, load().akz_last_error().decode(errors="replace"))
