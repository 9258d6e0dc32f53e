"""NNDR matches and homography inliers on the device against the
reference's arithmetic (utils.cpp:154-243) restated in numpy: float NNDR
and projection, the distance in double."""
import ctypes

import numpy as np
import pytest

from akaze_gb300 import synth

pytestmark = pytest.mark.gpu


def _reference_status(m, kq, kt, H, nndr=np.float32(0.8), err=np.float32(2.5)):
    f = np.float32
    d1, d2 = m[:, 0]["distance"].astype(f), m[:, 1]["distance"].astype(f)
    st = np.zeros(len(m), np.int8)
    good = d1 < nndr * d2
    st[good] = 1
    qi, ti = m[good, 0]["queryIdx"], m[good, 0]["trainIdx"]
    x1, y1 = kq["x"][qi].astype(f), kq["y"][qi].astype(f)
    x2, y2 = kt["x"][ti].astype(f), kt["y"][ti].astype(f)
    h = H.astype(f).reshape(-1)
    s = (h[6] * x1 + h[7] * y1) + h[8]
    x2m = ((h[0] * x1 + h[1] * y1) + h[2]) / s
    y2m = ((h[3] * x1 + h[4] * y1) + h[5]) / s
    dx, dy = (x2m - x2).astype(np.float64), (y2m - y2).astype(np.float64)
    dist = np.sqrt(dx * dx + dy * dy).astype(f)
    idx = np.nonzero(good)[0]
    st[idx[dist <= err]] = 2
    return st


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
    got = st.cpu().numpy()
    assert np.array_equal(got, want)
    c = cnt.cpu().numpy()
    assert c[0] == int((want > 0).sum()) and c[1] == int((want == 2).sum())
    assert c[1] > 0.5 * c[0]  # a synthetic homography pair: most NNDR matches are inliers
