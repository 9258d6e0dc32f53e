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


@pytest.mark.parametrize("w,h,seed,dfac", [(640, 480, 4041, 1.5), (1920, 1080, 4042, 1.5), (331, 257, 4043, 1.5),
                                           (640, 480, 4044, 0.8), (640, 480, 4045, 2.0)])
def test_extrema_3d_matches_oracle(gpu_lib, oracle, w, h, seed, dfac):
    """The 3 x 3 x 3 extrema option (akz_options.extrema_3d): candidates must
    also exceed the adjacent levels of their octave.  derivative_factor 0.8
    and 2.0 run the tile detector (steps 1 and 5) as well as the strip one."""
    img = synth.synth_image(seed, w, h)
    ak = _ak(gpu_lib, w, h, extrema_3d=1, derivative_factor=dfac)
    kp, d = ak.detect_and_compute(img)
    orc = _oracle(oracle, w, h, extrema_3d=1, derivative_factor=dfac)
    okp, od = orc.run(img)
    ext, oext = ak.extrema(), orc.extrema()
    assert ext.tobytes() == oext.tobytes(), (len(ext), len(oext))
    assert kp.tobytes() == okp.tobytes() and np.array_equal(d, od)
    plain = _oracle(oracle, w, h, derivative_factor=dfac)
    plain.run(img)
    assert 0 < len(oext) < len(plain.extrema())  # the rule removes candidates, never adds


def test_extrema_3d_uneven_batch(gpu_lib, oracle):
    sizes = synth.uneven_sizes(77, 5)
    imgs = [synth.synth_image(7700 + i, w, h) for i, (w, h) in enumerate(sizes)]
    b = gpu_lib.Batch(gpu_lib.AKAZEOptions(extrema_3d=1), sizes)
    b.upload(imgs)
    b.run()
    for i, ((w, h), img) in enumerate(zip(sizes, imgs)):
        kp, d = b.results(i)
        okp, od = _oracle(oracle, w, h, extrema_3d=1).run(img)
        assert kp.tobytes() == okp.tobytes() and np.array_equal(d, od), (i, w, h)


@pytest.mark.parametrize("desc,channels,size", [(5, 1, 0), (5, 2, 0), (5, 3, 256), (5, 1, 64), (5, 2, 100),
                                                (4, 3, 128), (4, 2, 0), (5, 3, 486)])
def test_descriptor_modes_match_oracle(gpu_lib, oracle, desc, channels, size):
    """descriptor_channels 1 and 2 (rows of ceil(162 c / 8) bytes; the second
    channel of 2 is the gradient magnitude) and the random-bit subsets of
    descriptor_size bits (generateDescriptorSubsample, AKAZE.cpp:498-603),
    rotation-invariant and upright, against the oracle bit for bit; the
    matcher on those rows too."""
    w, h = 640, 480
    img = synth.synth_image(4100 + channels + size, w, h)
    kw = dict(descriptor=desc, descriptor_channels=channels, descriptor_size=size)
    ak = _ak(gpu_lib, w, h, **kw)
    kp, d = ak.detect_and_compute(img)
    okp, od = _oracle(oracle, w, h, **kw).run(img)
    rb = (size if size else 162 * channels) + 7 >> 3
    assert d.shape == od.shape == (len(okp), rb)
    assert kp.tobytes() == okp.tobytes()
    assert np.array_equal(d, od)
    bits = size if size else 162 * channels
    if bits % 8:  # the pad bits of the last byte stay zero
        assert not np.any(d[:, -1] >> (bits % 8))
    m = gpu_lib.Matcher().bfmatch(d, d[::-1].copy())
    assert m.tobytes() == oracle.bfmatch(od, od[::-1].copy()).tobytes()


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
