"""Writes tests/golden/nld_ref.npz from the reference's own code.

Run in a tree where the reference sources are present: oracle/Makefile
target "ref" compiles the reference's src/lib/nldiffusion_functions.cpp and
src/lib/utils.cpp (over the OpenCV-shaped headers of oracle/ref_shim/) into
oracle/_ref/libnld_ref.so, and this script records what those functions
compute on small seeded inputs:

  pm_g2            nldiffusion_functions.cpp:72-83
  nld_step_scalar  nldiffusion_functions.cpp:213-317 (three steps)
  compute_k_percentile and gaussian_2D_convolution's kernel-size rule
                   nldiffusion_functions.cpp:29-47, :121-201
  save_keypoints   utils.cpp:97-152 (the file text)
  matches2points_nndr + compute_inliers_homography  utils.cpp:155-243

tests/test_oracle_vs_reference_cpu.py checks the oracle (and the library's
host and device code) against these vectors on any machine.

  python tests/golden/make_golden_ref.py
"""
import ctypes
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from akaze_gb300 import synth  # noqa: E402
from oracle import oracle_ctypes as oc  # noqa: E402

KEYPOINT = oc.KEYPOINT_DTYPE
DMATCH = oc.DMATCH_DTYPE
SIGMAS = np.array([0.7, 1.0, 1.6, 2.0, 2.26, 3.2, 4.52, 6.4, 9.05], np.float32)


def nndr_case(rng, nq=400, nt=380, W=640, H=480):
    """Keypoints of two images related by a homography, 2-NN matches in
    which most true pairs come first, and the homography."""
    Hm = synth.random_homography(77, W, H).astype(np.float32)
    kq = np.zeros(nq, KEYPOINT)
    kq["x"] = rng.uniform(0, W, nq)
    kq["y"] = rng.uniform(0, H, nq)
    kq["size"] = rng.uniform(4, 40, nq)
    kt = np.zeros(nt, KEYPOINT)
    kt["x"] = rng.uniform(0, W, nt)
    kt["y"] = rng.uniform(0, H, nt)
    m = np.zeros((nq, 2), DMATCH)
    m["queryIdx"] = np.arange(nq)[:, None]
    for i in range(nq):
        j = int(rng.integers(0, nt))
        if rng.random() < 0.6:  # a true correspondence, perturbed by up to ~4 px
            x, y = float(kq["x"][i]), float(kq["y"][i])
            d = Hm[2, 0] * x + Hm[2, 1] * y + Hm[2, 2]
            kt["x"][j] = (Hm[0, 0] * x + Hm[0, 1] * y + Hm[0, 2]) / d + rng.normal(0, 1.5)
            kt["y"][j] = (Hm[1, 0] * x + Hm[1, 1] * y + Hm[1, 2]) / d + rng.normal(0, 1.5)
        d1 = int(rng.integers(0, 200))
        m[i, 0]["trainIdx"], m[i, 0]["distance"] = j, d1
        m[i, 1]["trainIdx"], m[i, 1]["distance"] = int(rng.integers(0, nt)), d1 + int(rng.integers(0, 120))
    return m, kq, kt, Hm


def reference_nndr(R, m, kq, kt, Hm, nndr=0.8, err=2.5):
    nq = len(m)
    pts = np.zeros(4 * nq, np.float32)
    inl = np.zeros(4 * nq, np.float32)
    ninl = ctypes.c_int(0)
    mm = np.ascontiguousarray(m.reshape(-1))
    n = R.utilsref_nndr_inliers(mm.ctypes.data, nq, kq.ctypes.data, len(kq), kt.ctypes.data, len(kt),
                                np.ascontiguousarray(Hm, np.float32).ctypes.data, nndr, err, pts.ctypes.data,
                                inl.ctypes.data, ctypes.byref(ninl))
    assert n >= 0
    return pts[:4 * n].reshape(n, 4), inl[:4 * ninl.value].reshape(ninl.value, 4)


def reference_save_keypoints(R, kp, desc):
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "k.txt")
        if desc is None:
            st = R.utilsref_save_keypoints(p.encode(), kp.ctypes.data, len(kp), None, 0, 0)
        else:
            st = R.utilsref_save_keypoints(p.encode(), kp.ctypes.data, len(kp), desc.ctypes.data, desc.shape[1], 1)
        assert st == 0
        return open(p, "rb").read()


def main():
    oc.build()
    R = oc.nld_ref()
    if R is None:
        sys.exit("oracle/_ref/libnld_ref.so is missing: build oracle/Makefile target ref with the reference tree")
    rng = np.random.default_rng(2024)
    h, w = 64, 96
    out = {}
    lx = rng.normal(0, 0.05, (h, w)).astype(np.float32)
    ly = rng.normal(0, 0.05, (h, w)).astype(np.float32)
    lx[::5, ::7] = 0
    ly[::5, ::7] = 0
    g = np.zeros_like(lx)
    R.nldref_pm_g2(lx.ctypes.data, ly.ctypes.data, g.ctypes.data, w, h, 0.0123)
    out.update(pm_lx=lx, pm_ly=ly, pm_k=np.float32(0.0123), pm_out=g)

    L = oc.u8_to_unit(synth.synth_image(5, w, h))
    taus = np.array([0.41, 1.27, 2.93], np.float32)
    c = np.clip(g, 1e-3, 1).astype(np.float32)
    Ld = L.copy()
    for t in taus:
        R.nldref_nld_step(Ld.ctypes.data, c.ctypes.data, w, h, float(t))
    out.update(nld_L=L, nld_c=c, nld_tau=taus, nld_out=Ld)

    kimgs, kvals, kks = [], [], []
    for seed in (6, 7, 8):
        img = oc.u8_to_unit(synth.synth_image(seed, w, h))
        ks = ctypes.c_int(0)
        kvals.append(R.nldref_k_percentile(img.ctypes.data, w, h, 0.7, 1.0, 300, ctypes.byref(ks)))
        kks.append(ks.value)
        kimgs.append(img)
    out.update(kp_imgs=np.stack(kimgs), kp_vals=np.array(kvals, np.float32), kp_ksize=np.array(kks, np.int32))

    gk = []
    for s in SIGMAS:
        o = np.zeros_like(L)
        ks = ctypes.c_int(0)
        assert R.nldref_gaussian(L.ctypes.data, o.ctypes.data, w, h, float(s), ctypes.byref(ks)) == 0
        gk.append(ks.value)
    out.update(gauss_sigma=SIGMAS, gauss_ksize=np.array(gk, np.int32))

    kp = np.zeros(6, KEYPOINT)
    kp["x"] = rng.uniform(0, 1920, 6)
    kp["y"] = rng.uniform(0, 1080, 6)
    kp["size"] = rng.uniform(3, 60, 6)
    desc = rng.integers(0, 256, (6, 61)).astype(np.uint8)
    out.update(sk_kp=kp.view(np.uint8).reshape(6, -1), sk_desc=desc,
               sk_text_desc=np.frombuffer(reference_save_keypoints(R, kp, desc), np.uint8),
               sk_text_nodesc=np.frombuffer(reference_save_keypoints(R, kp, None), np.uint8))

    m, kq, kt, Hm = nndr_case(rng)
    pts, inl = reference_nndr(R, m, kq, kt, Hm)
    out.update(nn_m=m.view(np.uint8).reshape(len(m), -1), nn_kq=kq.view(np.uint8).reshape(len(kq), -1),
               nn_kt=kt.view(np.uint8).reshape(len(kt), -1), nn_H=Hm, nn_pts=pts, nn_inl=inl)

    path = os.path.join(HERE, "nld_ref.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes;", len(pts), "NNDR matches,", len(inl), "inliers")


if __name__ == "__main__":
    main()
