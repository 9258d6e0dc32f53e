"""Edge cases of the GPU path against the oracle: a flat image (contrast
factor 0, as compute_k_percentile gives it, so the PM-g2 conductance is
0/0 and the levels are NaN on both sides; no keypoints), an image small
enough to keep only octave 0, the largest benchmark size, the raw-extrema
capacity overflow, and the matcher with an empty or one-row train set."""
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
