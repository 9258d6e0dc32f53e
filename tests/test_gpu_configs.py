"""The benchmark configurations that the stage tests leave out, on the GPU
against the oracle, through the C ABI:

- 3840x2160 with 6 octaves x 4 sublevels (24 levels, past the fork's fixed
  4x4 limit).  The reference's float FED diverges at octave 5 on this size
  (levels reach |L| ~ 1e12 and can overflow), so planes are compared with
  NaN equal to NaN; extrema, keypoints and descriptors must be identical;
- the Hamming 2-NN matcher sweep: 486-bit rows with 30 % of the queries
  planted as Binomial(486, 0.05) copies of train rows, plus duplicated train
  rows that force equal distances (the lower train index must win), exact at
  N = M = 8192 and 32768, and on 4096 sampled queries at N = M = 131072;
- the full batch of 64 uneven sizes (W ~ U[320, 1920], H ~ U[240, 1080],
  multiples of 8), image by image;
- the upright M-LDB descriptor (MLDB_UPRIGHT) at 640x480.
"""
import numpy as np
import pytest

from akaze_gb300 import synth

pytestmark = pytest.mark.gpu


def _ak(gpu_lib, w, h, **kw):
    o = gpu_lib.AKAZEOptions(**kw)
    o.setWidth(w)
    o.setHeight(h)
    return gpu_lib.AKAZE(o)


def _oracle(oracle, w, h, **kw):
    return oracle.Oracle(w, h, oracle.default_options(**kw))


def test_4k_six_octaves_matches_oracle(gpu_lib, oracle):
    W, H = 3840, 2160
    img = synth.synth_image(4006, W, H)
    ak = _ak(gpu_lib, W, H, omax=6)
    kp, d = ak.detect_and_compute(img)
    orc = _oracle(oracle, W, H, omax=6)
    okp, od = orc.run(img)
    assert ak.nlevels == orc.nlevels == 24
    assert ak.kcontrast == orc.kcontrast
    for lv in range(orc.nlevels):
        for name in ("Lt", "Lsmooth", "Lx", "Ly"):
            g, c = ak.plane(lv, name), orc.plane(lv, name)
            assert g.shape == c.shape
            assert np.array_equal(g, c, equal_nan=True), (lv, name)
    ext, oext = ak.extrema(), orc.extrema()
    assert ext.tobytes() == oext.tobytes(), (len(ext), len(oext))
    assert len(kp) == len(okp) and len(kp) > 100
    assert kp.tobytes() == okp.tobytes()
    assert np.array_equal(d, od)
    # the first 16 levels have the default 4-octave plan's geometry
    four = _oracle(oracle, W, H)
    geo = ("width", "height", "octave", "sublevel", "esigma", "etime", "deriv_step", "nsteps")
    for lv in range(16):
        assert [four.level(lv)[k] for k in geo] == [orc.level(lv)[k] for k in geo], lv


def _rows_with_ties(seed, n, m, dup_frac=0.05):
    q, t = synth.matcher_rows(seed, n, m)
    rng = np.random.default_rng(seed + 1)
    k = int(dup_frac * m)
    src = rng.integers(0, m, k)
    dst = rng.integers(0, m, k)
    t[dst] = t[src]  # equal rows at different indices: equal distances for every query
    return q, t


@pytest.mark.parametrize("n", [8192, 32768])
def test_matcher_sweep_exact(gpu_lib, oracle, n):
    q, t = _rows_with_ties(5000 + n, n, n)
    got = gpu_lib.Matcher().bfmatch(q, t)
    want = oracle.bfmatch(q, t)
    assert got.tobytes() == want.tobytes()
    best = want[:, 0]["distance"]
    assert np.mean(best < 100) > 0.25  # the planted near-duplicates are found
    # ties were forced: some queries have equal best and second-best distances
    assert np.any(want[:, 0]["distance"] == want[:, 1]["distance"])


def test_matcher_sweep_largest_sampled(gpu_lib, oracle):
    n = 131072
    q, t = _rows_with_ties(5131, n, n)
    got = gpu_lib.Matcher().bfmatch(q, t)
    rng = np.random.default_rng(7)
    idx = np.sort(rng.choice(n, 4096, replace=False))
    want = oracle.bfmatch(q[idx], t)
    want["queryIdx"] = idx[:, None]
    assert got[idx].tobytes() == want.tobytes()


def test_uneven_batch_of_64_matches_oracle(gpu_lib, oracle):
    sizes = synth.uneven_sizes(2024, 64)
    imgs = [synth.synth_image(6400 + i, w, h) for i, (w, h) in enumerate(sizes)]
    b = gpu_lib.Batch(gpu_lib.AKAZEOptions(), sizes)
    b.upload(imgs)
    b.run()
    total = 0
    for i, ((w, h), img) in enumerate(zip(sizes, imgs)):
        kp, d = b.results(i)
        okp, od = oracle.Oracle(w, h).run(img)
        assert kp.tobytes() == okp.tobytes(), (i, w, h, len(kp), len(okp))
        assert np.array_equal(d, od), (i, w, h)
        total += len(kp)
    assert total > 64 * 50


def test_upright_mldb_matches_oracle(gpu_lib, oracle):
    img = synth.synth_image(4040, 640, 480)
    ak = _ak(gpu_lib, 640, 480, descriptor=4)
    kp, d = ak.detect_and_compute(img)
    orc = _oracle(oracle, 640, 480, descriptor=4)
    okp, od = orc.run(img)
    assert len(kp) > 50
    assert kp.tobytes() == okp.tobytes()
    assert np.array_equal(d, od)
    assert np.all(kp["angle"] == 0.0)  # upright: no orientation
    # the rotation-invariant descriptor of the same keypoints differs
    rot = _ak(gpu_lib, 640, 480)
    rkp, rd = rot.detect_and_compute(img)
    for f in ("x", "y", "size", "response", "octave", "class_id"):
        assert np.array_equal(rkp[f], kp[f]), f
    assert not np.array_equal(rd, d)
