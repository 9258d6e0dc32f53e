"""NNDR matches and homography inliers on the device against the output of
the reference's own utils.cpp (golden vectors) and against its arithmetic
(utils.cpp:154-243) restated in numpy: float NNDR and projection, the
distance in double."""
import ctypes

import numpy as np
import pytest

from akaze_gb300 import synth

pytestmark = pytest.mark.gpu


from eval_reference import reference_status as _reference_status
from eval_reference import status_from_point_lists


def _device_status(gpu_lib, torch, m, k1, k2, Hm):
    lib = gpu_lib.load()
    dm = torch.from_numpy(m.reshape(-1).view(np.uint8).copy()).cuda()
    dk1 = torch.from_numpy(k1.view(np.uint8).copy()).cuda()
    dk2 = torch.from_numpy(k2.view(np.uint8).copy()).cuda()
    st = torch.zeros(len(m), dtype=torch.int8, device="cuda")
    cnt = torch.zeros(2, dtype=torch.int32, device="cuda")
    Hf = np.ascontiguousarray(Hm, np.float32)
    r = lib.akz_nndr_homography_inliers(ctypes.c_void_p(dm.data_ptr()), len(m), ctypes.c_void_p(dk1.data_ptr()),
                                        ctypes.c_void_p(dk2.data_ptr()), Hf.ctypes.data_as(ctypes.c_void_p),
                                        ctypes.c_float(0.8), ctypes.c_float(2.5), ctypes.c_void_p(st.data_ptr()),
                                        ctypes.c_void_p(cnt.data_ptr()), None)
    assert r == 0, lib.akz_last_error()
    torch.cuda.synchronize()
    return st.cpu().numpy(), cnt.cpu().numpy()


def test_nndr_homography_inliers_match_reference_output(gpu_lib):
    """Against the output of the reference's own utils.cpp, recorded in
    tests/golden/nld_ref.npz by tests/golden/make_golden_ref.py."""
    import os
    torch = pytest.importorskip("torch")
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "nld_ref.npz"))
    m = g["nn_m"].reshape(-1).view(gpu_lib.DMATCH_DTYPE).reshape(-1, 2)
    kq = g["nn_kq"].reshape(-1).view(gpu_lib.KEYPOINT_DTYPE)
    kt = g["nn_kt"].reshape(-1).view(gpu_lib.KEYPOINT_DTYPE)
    want = status_from_point_lists(m, kq, kt, g["nn_pts"], g["nn_inl"])
    got, cnt = _device_status(gpu_lib, torch, m, kq, kt, g["nn_H"])
    assert np.array_equal(got, want)
    assert cnt[0] == len(g["nn_pts"]) and cnt[1] == len(g["nn_inl"])


def test_nndr_homography_inliers_match_reference_arithmetic(gpu_lib):
    torch = pytest.importorskip("torch")
    W, H = 640, 480
    img1, img2, Hm = synth.synth_pair(31, W, H)
    o = gpu_lib.AKAZEOptions()
    o.setWidth(W)
    o.setHeight(H)
    ak = gpu_lib.AKAZE(o)
    k1, d1 = ak.detect_and_compute(img1)
    k2, d2 = ak.detect_and_compute(img2)
    m = gpu_lib.Matcher().bfmatch(d1, d2)
    want = _reference_status(m, k1, k2, Hm)
    got, c = _device_status(gpu_lib, torch, m, k1, k2, Hm)
    assert np.array_equal(got, want)
    assert c[0] == int((want > 0).sum()) and c[1] == int((want == 2).sum())
    assert c[1] > 0.5 * c[0]  # a synthetic homography pair: most NNDR matches are inliers
