"""The oracle against the reference's own code.

The reference's src/lib/nldiffusion_functions.cpp and src/lib/utils.cpp are
compiled unchanged from the reference tree over the OpenCV-shaped headers of
oracle/ref_shim/ (oracle/Makefile, target "ref"; the shim's GaussianBlur,
Scharr and resize are the oracle's own filters).  Two kinds of checks:

- golden vectors that tests/golden/make_golden_ref.py recorded from that
  build (tests/golden/nld_ref.npz), on every machine;
- the live build on larger seeded inputs where the reference tree is
  present (skipped elsewhere).

Pinned, bit for bit: PM-g2 (nldiffusion_functions.cpp:72-83), the FED step
with its border formulas (:213-317), the contrast percentile's histogram and
threshold (:121-201), the Gaussian kernel-size rule (:29-47), the
Mikolajczyk keypoint file (utils.cpp:97-152) as the library writes it, and
the NNDR + homography-inlier chain (utils.cpp:155-243) as the tests restate
it.
"""
import ctypes
import os

import numpy as np
import pytest

import akaze_gb300 as akz
from akaze_gb300 import synth
from eval_reference import reference_status, status_from_point_lists

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "nld_ref.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="module")
def ref(oracle):
    R = oracle.nld_ref()
    if R is None:
        pytest.skip("the reference tree is not present (oracle/_ref/libnld_ref.so not built)")
    return R


# ---- golden vectors (every machine) ----------------------------------------

def test_pm_g2_golden(oracle, golden):
    g = oracle.plane_conductance(golden["pm_lx"], golden["pm_ly"], golden["pm_k"])
    assert np.array_equal(g, golden["pm_out"])


def test_nld_step_golden(oracle, golden):
    L = golden["nld_L"]
    for t in golden["nld_tau"]:
        L = oracle.plane_nld_step(L, golden["nld_c"], t)
    assert np.array_equal(L, golden["nld_out"])


def test_k_percentile_golden(oracle, golden):
    for img, v in zip(golden["kp_imgs"], golden["kp_vals"]):
        assert oracle.plane_k_percentile(img) == v
    assert list(golden["kp_ksize"]) == [5, 5, 5]


def test_gaussian_kernel_size_rule_golden(oracle, golden):
    img = golden["nld_L"]
    for s, ks in zip(golden["gauss_sigma"], golden["gauss_ksize"]):
        assert oracle.plane_gaussian(img, s)[1] == ks, s
        if s <= 5.5:  # the library's level-0 range (soffset <= 5.5) uses the same rule
            assert len(akz.gaussian_taps(float(s))) == ks, s


def test_save_keypoints_golden(golden, tmp_path):
    kp = golden["sk_kp"].reshape(-1).view(akz.KEYPOINT_DTYPE)
    p1, p2 = tmp_path / "a.txt", tmp_path / "b.txt"
    akz.save_keypoints(p1, kp, golden["sk_desc"])
    akz.save_keypoints(p2, kp)
    assert p1.read_bytes() == golden["sk_text_desc"].tobytes()
    assert p2.read_bytes() == golden["sk_text_nodesc"].tobytes()


def test_nndr_inliers_golden(golden):
    m = golden["nn_m"].reshape(-1).view(akz.DMATCH_DTYPE).reshape(-1, 2)
    kq = golden["nn_kq"].reshape(-1).view(akz.KEYPOINT_DTYPE)
    kt = golden["nn_kt"].reshape(-1).view(akz.KEYPOINT_DTYPE)
    want = status_from_point_lists(m, kq, kt, golden["nn_pts"], golden["nn_inl"])
    assert np.array_equal(reference_status(m, kq, kt, golden["nn_H"]), want)
    assert 0 < (want == 2).sum() < (want > 0).sum() < len(m)


# ---- the live reference build ------------------------------------------------

SIZES = [(640, 480, 1), (331, 257, 2), (97, 61, 3)]


def _gradients(rng, h, w, scale):
    lx = rng.normal(0, scale, (h, w)).astype(np.float32)
    ly = rng.normal(0, scale, (h, w)).astype(np.float32)
    lx[::7, ::5] = 0
    ly[::7, ::5] = 0
    lx[3, :] = np.float32(1e-20)  # tiny and huge arguments
    ly[4, :] = np.float32(3e3)
    return lx, ly


@pytest.mark.parametrize("w,h,seed", SIZES)
def test_pm_g2_equals_reference(oracle, ref, w, h, seed):
    rng = np.random.default_rng(seed)
    for k in (0.0123, 0.3, 1e-4):
        lx, ly = _gradients(rng, h, w, 0.05)
        want = np.zeros_like(lx)
        assert ref.nldref_pm_g2(lx.ctypes.data, ly.ctypes.data, want.ctypes.data, w, h, k) == 0
        assert np.array_equal(oracle.plane_conductance(lx, ly, k), want), k


@pytest.mark.parametrize("w,h,seed", SIZES)
def test_nld_step_equals_reference(oracle, ref, w, h, seed):
    rng = np.random.default_rng(seed)
    L = oracle.u8_to_unit(synth.synth_image(seed, w, h))
    lx, ly = _gradients(rng, h, w, 0.02)
    c = oracle.plane_conductance(lx, ly, 0.01)
    taus = oracle.fed_tau(7.3)  # a real FED cycle: growing, reordered steps
    want = L.copy()
    got = L.copy()
    for t in taus:
        assert ref.nldref_nld_step(want.ctypes.data, c.ctypes.data, w, h, float(t)) == 0
        got = oracle.plane_nld_step(got, c, t)
        assert np.array_equal(got, want), t


@pytest.mark.parametrize("w,h,seed", SIZES + [(1920, 1080, 4)])
def test_k_percentile_equals_reference(oracle, ref, w, h, seed):
    img = oracle.u8_to_unit(synth.synth_image(seed, w, h))
    for perc, nbins in ((0.7, 300), (0.5, 77), (0.95, 1000)):
        ks = ctypes.c_int(0)
        want = ref.nldref_k_percentile(img.ctypes.data, w, h, perc, 1.0, nbins, ctypes.byref(ks))
        assert want >= 0 and ks.value == 5
        assert oracle.plane_k_percentile(img, perc, nbins) == np.float32(want), (perc, nbins)
    flat = np.full((h, w), 0.3, np.float32)  # no gradient: the reference returns 0
    want = ref.nldref_k_percentile(flat.ctypes.data, w, h, 0.7, 1.0, 300, None)
    assert oracle.plane_k_percentile(flat) == np.float32(want) == 0.0


def test_oracle_contrast_factor_equals_reference(oracle, ref):
    """The oracle's level-0 contrast factor (what the GPU path is checked
    against) is the reference's compute_k_percentile of the input image."""
    for w, h, seed in SIZES:
        img = synth.synth_image(seed, w, h)
        orc = oracle.Oracle(w, h)
        orc.build(img)
        f = oracle.u8_to_unit(img)
        want = ref.nldref_k_percentile(f.ctypes.data, w, h, 0.7, 1.0, 300, None)
        assert orc.kcontrast == np.float32(want)


def test_gaussian_kernel_size_rule_equals_reference(oracle, ref):
    img = oracle.u8_to_unit(synth.synth_image(9, 120, 90))
    for s in np.concatenate([np.linspace(0.5, 12.0, 47), [1.6 * 2 ** (k / 4) for k in range(13)]]).astype(np.float32):
        out = np.zeros_like(img)
        ks = ctypes.c_int(0)
        assert ref.nldref_gaussian(img.ctypes.data, out.ctypes.data, 120, 90, float(s), ctypes.byref(ks)) == 0
        g, k2 = oracle.plane_gaussian(img, s)
        assert ks.value == k2 and np.array_equal(out, g), s


def test_save_keypoints_equals_reference(ref, tmp_path):
    rng = np.random.default_rng(5)
    for n, cols in ((0, 61), (1, 61), (40, 61), (17, 21)):
        kp = np.zeros(n, akz.KEYPOINT_DTYPE)
        kp["x"] = rng.uniform(0, 4000, n)
        kp["y"] = rng.uniform(0, 3000, n)
        kp["size"] = rng.uniform(-60, 60, n)  # weak points carry a negative size
        desc = rng.integers(0, 256, (n, cols)).astype(np.uint8)
        for save_desc in (0, 1):
            a, b = tmp_path / "lib.txt", tmp_path / "ref.txt"
            akz.save_keypoints(a, kp, desc, save_desc=bool(save_desc))
            st = ref.utilsref_save_keypoints(str(b).encode(), kp.ctypes.data, n, desc.ctypes.data, cols, save_desc)
            assert st == 0
            assert a.read_bytes() == b.read_bytes(), (n, cols, save_desc)


def test_nndr_inliers_restatement_equals_reference(ref):
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden_ref", os.path.join(os.path.dirname(GOLDEN), "make_golden_ref.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    for seed in range(4):
        m, kq, kt, Hm = mg.nndr_case(np.random.default_rng(100 + seed), nq=700, nt=650)
        pts, inl = mg.reference_nndr(ref, m, kq, kt, Hm)
        want = status_from_point_lists(m, kq, kt, pts, inl)
        assert np.array_equal(reference_status(m, kq, kt, Hm), want), seed
