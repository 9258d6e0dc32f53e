"""Known-answer tests of the CPU oracle: hand-derived values from the
reference's code, an independent numpy restatement of its CPU scale-space
functions, its suppression rule against a literal emulation of the
reference's round-based kernels, and the matcher against brute force."""
import ctypes

import numpy as np
import pytest

import fork_nms_emulation as fe
import numpy_reference as nr
from akaze_gb300 import synth


def test_gaussian_kernel_sizes_and_taps(oracle):
    # nldiffusion_functions.cpp:33-43: ksize = ceil(2(1+(sigma-0.8)/0.3)) made odd
    assert len(oracle.gaussian_taps(1.0)) == 5
    assert len(oracle.gaussian_taps(1.6)) == 9
    for s in (1.0, 1.6, 2.3):
        t = oracle.gaussian_taps(s)
        assert np.array_equal(t, t[::-1])
        assert abs(float(t.sum()) - 1.0) < 1e-6
        want, _ = nr.gauss_taps(s)
        assert np.array_equal(t, want)


def test_level_geometry_known_answers(oracle):
    o = oracle.Oracle(640, 480)
    sizes = [(o.level(i)["width"], o.level(i)["height"]) for i in range(o.nlevels)]
    assert sizes == [(640, 480)] * 4 + [(320, 240)] * 4 + [(160, 120)] * 4 + [(80, 60)] * 4
    L = o.level(5)
    assert L["octave"] == 1 and L["sublevel"] == 1
    assert np.float32(L["esigma"]) == np.float32(np.float32(1.6) * np.float32(2.0 ** 1.25))
    # detector step fRound(esigma*1.5/2^o) and border 10*sqrt(2)*fRound(size/2^o) (AKAZE.cpp:328-363)
    assert [o.level(i)["deriv_step"] for i in range(4)] == [2, 3, 3, 4]
    assert abs(o.level(0)["border"] - 10 * np.sqrt(2) * 2) < 1e-4


@pytest.mark.parametrize("w,h,seed", [(96, 64, 1), (160, 120, 2), (97, 45, 3)])
def test_scale_space_equals_numpy_restatement(oracle, w, h, seed):
    img = synth.synth_image(seed, w, h)
    o = oracle.Oracle(w, h)
    o.build(img)
    levels = [o.level(i) for i in range(o.nlevels)]
    taus = [o.tau(i) for i in range(o.nlevels)]
    if any(levels[i]["octave"] > levels[i - 1]["octave"] and
           (levels[i - 1]["width"] != 2 * levels[i]["width"] or levels[i - 1]["height"] != 2 * levels[i]["height"])
           for i in range(1, len(levels))):
        pytest.skip("odd-size half-sample is exercised against the GPU, not restated in numpy")
    k, Lt, Ls = nr.scale_space(oracle.u8_to_unit(img), levels, taus)
    assert np.float32(o.kcontrast) == k
    for i in range(o.nlevels):
        assert np.array_equal(o.plane(i, "Lt"), Lt[i]), i
        assert np.array_equal(o.plane(i, "Lsmooth"), Ls[i]), i


def test_contrast_factor_of_a_flat_image_is_zero(oracle):
    # compute_k_percentile skips zero gradients: a constant image has no
    # points, nthreshold = 0 and k = hmax * 0/nbins = 0 (:175-197)
    o = oracle.Oracle(64, 48)
    o.build(np.full((48, 64), 100, np.uint8))
    assert o.kcontrast == 0.0


def test_single_blob_gives_a_keypoint_at_its_centre(oracle):
    w, h = 200, 160
    yy, xx = np.mgrid[0:h, 0:w]
    img = (60 + 150 * np.exp(-((xx - 101.3) ** 2 + (yy - 77.6) ** 2) / (2 * 6.0 ** 2))).astype(np.uint8)
    o = oracle.Oracle(w, h)
    o.build(img)
    n = o.detect()
    kp = o.keypoints()
    assert n >= 1
    d = np.hypot(kp["x"] - 101.3, kp["y"] - 77.6)
    assert d.min() < 1.5


@pytest.mark.parametrize("seed,w,h", [(1, 640, 480), (2, 320, 240), (3, 500, 333), (6, 400, 300)])
def test_suppression_equals_round_based_emulation(oracle, seed, w, h):
    a, b, _ = synth.synth_pair(seed, w, h)
    for img in (a, b):
        o = oracle.Oracle(w, h)
        o.build(img)
        n = o.detect()
        mem, emitted = fe.suppress(o.extrema(), o.level_offsets())
        assert np.array_equal(mem, o.nms_state())
        assert len(emitted) == n


def test_descriptor_comparison_pairs(oracle):
    i1 = (ctypes.c_int * 486)()
    i2 = (ctypes.c_int * 486)()
    assert oracle.lib().ako_descriptor_pairs(i1, i2) == 486
    pairs = list(zip(i1, i2))
    # InitCompareIndices (cuda_akaze.cu:2034-2111): per grid, channel-major
    # pairs (3j+ch, 3i+ch), j < i, over cells 0-3, 4-12 and 13-28
    assert pairs[:6] == [(0, 3), (0, 6), (0, 9), (3, 6), (3, 9), (6, 9)]
    assert pairs[6:12] == [(1, 4), (1, 7), (1, 10), (4, 7), (4, 10), (7, 10)]
    assert pairs[18] == (12, 15) and pairs[18 + 36] == (13, 16)
    assert pairs[126] == (39, 42) and pairs[-1] == (83, 86)


def _brute(q, t):
    qb = np.unpackbits(q, axis=1)
    tb = np.unpackbits(t, axis=1)
    d = (qb[:, None, :] != tb[None, :, :]).sum(2) if len(t) else np.zeros((len(q), 0), int)
    out = []
    for i in range(len(q)):
        order = sorted(range(len(t)), key=lambda j: (d[i, j], j))
        best = [(j, d[i, j]) for j in order[:2]]
        while len(best) < 2:
            best.append((0, 512))
        out.append(best)
    return out


@pytest.mark.parametrize("nq,nt", [(50, 80), (7, 1), (5, 0), (64, 64)])
def test_matcher_equals_brute_force_with_tie_rule(oracle, nq, nt):
    q, t = synth.matcher_rows(nq * 100 + nt, nq, nt)
    if nt >= 4:
        t[3] = t[1]  # duplicate rows: equal distances, lower index first
        q[0] = t[1]
    m = oracle.bfmatch(q, t)
    for i, best in enumerate(_brute(q, t)):
        for k in range(2):
            assert m[i, k]["queryIdx"] == i
            assert (m[i, k]["trainIdx"], m[i, k]["distance"]) == (best[k][0], float(best[k][1])), (i, k)


def test_shared_float_routines_against_numpy(oracle):
    L = oracle.lib()
    L.ako_atan2f.restype = ctypes.c_float
    L.ako_atan2f.argtypes = [ctypes.c_float, ctypes.c_float]
    L.ako_expf.restype = ctypes.c_float
    L.ako_expf.argtypes = [ctypes.c_float]
    L.ako_recip1pf.restype = ctypes.c_float
    L.ako_recip1pf.argtypes = [ctypes.c_float]
    L.ako_sincosf.argtypes = [ctypes.c_float, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
    rng = np.random.default_rng(3)
    ulp = lambda v: np.spacing(np.abs(np.float32(v)))  # noqa: E731
    for y, x in rng.normal(size=(3000, 2)).astype(np.float32):
        r = L.ako_atan2f(float(y), float(x))
        assert abs(r - np.arctan2(np.float64(y), np.float64(x))) <= 3 * ulp(r) + 1e-12
    assert L.ako_atan2f(0.0, 0.0) == 0.0 and L.ako_atan2f(0.0, -0.0) == np.float32(np.pi)
    s, c = ctypes.c_float(), ctypes.c_float()
    for a in rng.uniform(0, 2 * np.pi, 3000).astype(np.float32):
        L.ako_sincosf(float(a), ctypes.byref(s), ctypes.byref(c))
        assert abs(s.value - np.sin(np.float64(a))) <= 3 * ulp(1.0)
        assert abs(c.value - np.cos(np.float64(a))) <= 3 * ulp(1.0)
    for v in rng.uniform(-30, 5, 3000).astype(np.float32):
        e = L.ako_expf(float(v))
        assert abs(e - np.exp(np.float64(v))) <= 2 * ulp(e)
    fs = np.concatenate([rng.uniform(0, 4, 20000), 10.0 ** rng.uniform(-12, 12, 20000)]).astype(np.float32)
    fs = np.concatenate([fs, np.float32([float.fromhex(h) for h in ('0x1.e691c6p-12', '0x1.f0001ep-21', '0x1.084208p-4', '0x1.5124ccp+38')])])
    for f in fs:
        assert L.ako_recip1pf(float(f)) == np.float32(1.0 / (1.0 + np.float64(f))), f
