"""Edge cases of the GPU path against the oracle: a flat image (contrast
factor 0, as compute_k_percentile gives it, so the PM-g2 conductance is
0/0 and the levels are NaN on both sides; no keypoints), an image small
enough to keep only octave 0, the largest benchmark size, the raw-extrema
capacity overflow, and the matcher with an empty or one-row train set.
Failure detection without a GPU fault: a bounded device wait that nothing
completes gives up and reports it, and a suppression round cap that an image
exceeds is reported as AKZ_ERR_TIMEOUT; the context stays usable after both."""
import ctypes

import numpy as np
import pytest

from akaze_gb300 import synth

pytestmark = pytest.mark.gpu


def _ak(gpu_lib, w, h, **kw):
    o = gpu_lib.AKAZEOptions(**kw)
    o.setWidth(w)
    o.setHeight(h)
    return gpu_lib.AKAZE(o)


def test_flat_image(gpu_lib, oracle):
    img = np.full((120, 160), 77, np.uint8)
    ak = _ak(gpu_lib, 160, 120)
    kp, d = ak.detect_and_compute(img)
    orc = oracle.Oracle(160, 120)
    okp, od = orc.run(img)
    assert len(kp) == 0 and len(okp) == 0 and d.shape == (0, 61)
    assert ak.kcontrast == 0.0 and orc.kcontrast == 0.0
    for lv in range(ak.nlevels):
        assert np.array_equal(ak.plane(lv), orc.plane(lv), equal_nan=True), lv


@pytest.mark.parametrize("w,h,seed", [(24, 20, 55), (120, 90, 55), (159, 81, 57)])
def test_small_images(gpu_lib, oracle, w, h, seed):
    img = synth.synth_image(seed, w, h)
    ak = _ak(gpu_lib, w, h)
    kp, d = ak.detect_and_compute(img)
    orc = oracle.Oracle(w, h)
    okp, od = orc.run(img)
    assert ak.nlevels == orc.nlevels
    for lv in range(ak.nlevels):  # a tiny image can also get a zero contrast factor (NaN levels on both sides)
        assert np.array_equal(ak.plane(lv), orc.plane(lv), equal_nan=True), lv
    assert kp.tobytes() == okp.tobytes() and np.array_equal(d, od)


def test_largest_benchmark_size(gpu_lib, oracle):
    W, H = 3840, 2160
    img = synth.synth_image(56, W, H)
    ak = _ak(gpu_lib, W, H)
    kp, d = ak.detect_and_compute(img)
    orc = oracle.Oracle(W, H)
    okp, od = orc.run(img)
    assert kp.tobytes() == okp.tobytes() and np.array_equal(d, od)
    assert len(kp) > 50


def test_raw_extrema_overflow_is_an_error(gpu_lib):
    img = synth.synth_image(57, 640, 480)
    ak = _ak(gpu_lib, 640, 480, maxkeypoints=16)
    ak.Create_Nonlinear_Scale_Space(img)
    with pytest.raises(gpu_lib.AkazeError) as e:
        ak.Feature_Detection()
    assert "maxkeypoints" in str(e.value)


def test_matcher_with_empty_and_single_row_train(gpu_lib, oracle):
    q, t = synth.matcher_rows(58, 300, 1)
    m = gpu_lib.Matcher()
    got = m.bfmatch(q, t)
    want = oracle.bfmatch(q, t)
    assert got.tobytes() == want.tobytes()
    assert np.all(got[:, 1]["distance"] == 512) and np.all(got[:, 1]["trainIdx"] == 0)
    empty = m.bfmatch(q, t[:0])
    assert np.all(empty["distance"] == 512) and np.all(empty["trainIdx"] == 0)
    assert empty.tobytes() == oracle.bfmatch(q, t[:0]).tobytes()


def test_bounded_wait_gives_up_and_reports(gpu_lib):
    lib = gpu_lib.load()
    t = ctypes.c_int(-1)
    assert lib.akz_selfcheck_bounded_wait(0, 1 << 14, ctypes.byref(t)) == 0
    assert t.value == 1  # nothing completed the barrier: the wait gave up
    assert lib.akz_selfcheck_bounded_wait(1, 1 << 24, ctypes.byref(t)) == 0
    assert t.value == 0  # completed: the wait succeeded
    # the context is still usable
    img = synth.synth_image(3, 320, 240)
    ak = _ak(gpu_lib, 320, 240)
    ak.Create_Nonlinear_Scale_Space(img)
    ak.Feature_Detection()
    desc, kp = ak.Compute_Descriptors()
    assert len(kp) > 0


def test_suppression_round_cap_reports_timeout(gpu_lib):
    img = synth.synth_image(7, 640, 480)
    b = gpu_lib.Batch(gpu_lib.AKAZEOptions(), [(640, 480)])
    b.upload([img])
    b.run()
    _, nkp, rounds, _ = b.image_info(0)
    kp0, d0 = b.results(0)
    assert rounds >= 2, rounds
    b.set_nms_round_cap(1)
    b.run()
    with pytest.raises(gpu_lib.AkazeError) as e:
        b.counts()
    assert e.value.status == 5  # AKZ_ERR_TIMEOUT
    b.set_nms_round_cap(1 << 20)
    b.run()
    kp1, d1 = b.results(0)
    assert np.array_equal(kp0.view(np.uint8), kp1.view(np.uint8)) and np.array_equal(d0, d1)


TINY = [(16, 16, 61), (17, 16, 62), (33, 29, 63), (64, 48, 64), (97, 61, 65), (101, 77, 66)]


@pytest.mark.parametrize("w,h,seed", TINY)
@pytest.mark.parametrize("fast_math", [0, 1])
def test_tiny_and_odd_sizes(gpu_lib, oracle, w, h, seed, fast_math):
    """Every stage at sizes where tiles, strips, halos and level geometry
    are mostly border (the bounds checks of the sanitizer, which is closed
    on this hardware, stand on these cases and the oracle): exact mode
    equals the oracle at every level, with NaN where both are NaN; fused
    mode stays within 1e-4 of each level's largest magnitude."""
    img = synth.synth_image(seed, w, h)
    ak = _ak(gpu_lib, w, h, fast_math=fast_math)
    kp, d = ak.detect_and_compute(img)
    orc = oracle.Oracle(w, h)
    okp, od = orc.run(img)
    assert ak.nlevels == orc.nlevels
    for lv in range(ak.nlevels):
        for name in ("Lt", "Lsmooth", "Lx", "Ly"):
            g, c = ak.plane(lv, name), orc.plane(lv, name)
            if fast_math == 0:
                assert np.array_equal(g, c, equal_nan=True), (lv, name)
            elif np.isfinite(c).all():
                rel = np.max(np.abs(g - c)) / max(float(np.max(np.abs(c))), 1e-30)
                assert rel <= 1e-4, (lv, name, rel)
    if fast_math == 0:
        assert kp.tobytes() == okp.tobytes() and np.array_equal(d, od)


def test_sizes_outside_the_supported_range_are_rejected(gpu_lib):
    """Images narrower or lower than 16 pixels (or above 32768) are refused
    before any device work with AKZ_ERR_INVALID_ARG; the context is not
    created."""
    for w, h in [(15, 16), (16, 15), (9, 7), (32769, 16)]:
        with pytest.raises(gpu_lib.AkazeError):
            _ak(gpu_lib, w, h)
