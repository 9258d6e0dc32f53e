"""matches2points_nndr + compute_inliers_homography (utils.cpp:155-243), as
akaze_match.cpp:161-168 chains them, restated in numpy as a per-query
status: 0 (no NNDR match), 1 (match), 2 (match and inlier).  The arithmetic
is the reference's: float NNDR and projection, the distance in double.
tests/test_oracle_vs_reference_cpu.py pins it to the reference's own
utils.cpp."""
import numpy as np


def reference_status(m, kq, kt, H, nndr=np.float32(0.8), err=np.float32(2.5)):
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


def status_from_point_lists(m, kq, kt, pts, inl):
    """Per-query status from the reference's output lists: the putative
    pairs (x1, y1, x2, y2) in query order, and the inlier pairs among them."""
    st = np.zeros(len(m), np.int8)
    good = []
    k = 0
    for i in range(len(m)):
        if k < len(pts):
            q, t = m[i, 0]["queryIdx"], m[i, 0]["trainIdx"]
            if (np.float32(kq["x"][q]), np.float32(kq["y"][q]), np.float32(kt["x"][t]), np.float32(kt["y"][t])) == tuple(pts[k]):
                st[i] = 1
                good.append(i)
                k += 1
    assert k == len(pts), "the putative pairs are not in query order"
    j = 0
    for i in good:
        if j < len(inl) and tuple(inl[j]) == tuple(pts[good.index(i)]):
            st[i] = 2
            j += 1
    assert j == len(inl), "the inliers are not an ordered subset of the putative pairs"
    return st
