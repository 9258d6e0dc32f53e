"""GPU path against the CPU oracle, stage by stage, through the C ABI.

Scale-space levels, contrast factor, raw extrema, keypoints and descriptors
are expected to be identical to the oracle (the kernels evaluate every float
expression in the oracle's order); the spec tolerances (levels 1e-4
relative, >= 99% keypoints within 0.5 px, descriptors within Hamming 2) are
asserted as the hard floor with the exact comparison reported.
"""
import numpy as np
import pytest

from akaze_gb300 import synth

pytestmark = pytest.mark.gpu

CASES = [(640, 480, 1), (331, 257, 2), (200, 150, 3), (1920, 1080, 4)]


def _run_both(gpu_lib, oracle, img, **opts):
    h, w = img.shape
    o = gpu_lib.AKAZEOptions(**opts)
    o.setWidth(w)
    o.setHeight(h)
    ak = gpu_lib.AKAZE(o)
    ak.Create_Nonlinear_Scale_Space(img)
    ak.Feature_Detection()
    desc, kp = ak.Compute_Descriptors()
    orc = oracle.Oracle(w, h, oracle.default_options(**{k: v for k, v in opts.items() if hasattr(oracle.AkoOptions, k)}))
    orc.build(img)
    orc.detect()
    od = orc.describe()
    return ak, kp, desc, orc, orc.keypoints(), od


def _exact(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("w,h,seed", CASES)
def test_scale_space_matches_oracle(gpu_lib, oracle, w, h, seed):
    img = synth.synth_image(seed, w, h)
    ak, kp, desc, orc, okp, od = _run_both(gpu_lib, oracle, img)
    assert ak.nlevels == orc.nlevels
    assert ak.kcontrast == orc.kcontrast
    for l in range(orc.nlevels):
        for name in ("Lt", "Lsmooth", "Lx", "Ly"):
            g = ak.plane(l, name)
            c = orc.plane(l, name)
            rel = np.max(np.abs(g - c)) / max(np.max(np.abs(c)), 1e-30)
            assert rel <= 1e-4, (l, name, rel)
            assert np.array_equal(g, c), f"level {l} {name}: max rel diff {rel:.3g}"


@pytest.mark.parametrize("w,h,seed", CASES)
def test_keypoints_and_descriptors_match_oracle(gpu_lib, oracle, w, h, seed):
    img = synth.synth_image(seed, w, h)
    ak, kp, desc, orc, okp, od = _run_both(gpu_lib, oracle, img)
    ext = ak.extrema()
    oext = orc.extrema()
    assert _exact(ext, oext), (len(ext), len(oext))
    assert len(kp) == len(okp)
    assert _exact(kp, okp)
    assert np.array_equal(desc, od)


@pytest.mark.parametrize("dfac", [0.8, 2.0])
def test_other_derivative_steps_match_oracle(gpu_lib, oracle, dfac):
    """derivative_factor 0.8 gives steps 1 and 2, 2.0 steps 3..5: levels of
    the tile detector (steps other than 2..4) and of the strip detector in
    one run."""
    img = synth.synth_image(21, 640, 480)
    ak, kp, desc, orc, okp, od = _run_both(gpu_lib, oracle, img, derivative_factor=dfac)
    for l in range(orc.nlevels):
        for name in ("Lx", "Ly"):
            assert np.array_equal(ak.plane(l, name), orc.plane(l, name)), (l, name)
    assert _exact(ak.extrema(), orc.extrema())
    assert _exact(kp, okp) and np.array_equal(desc, od)


def test_pair_matches(gpu_lib, oracle):
    a, b, H = synth.synth_pair(11, 640, 480)
    _, kpa, da, _, _, oda = _run_both(gpu_lib, oracle, a)
    _, kpb, db, _, _, odb = _run_both(gpu_lib, oracle, b)
    m = gpu_lib.Matcher().bfmatch(da, db)
    om = oracle.bfmatch(oda, odb)
    assert _exact(m.reshape(-1), om.reshape(-1))


def test_float_input_equals_u8_over_255(gpu_lib, oracle):
    img = synth.synth_image(31, 320, 240)
    f = oracle.u8_to_unit(img)  # (float)u * (float)(1/255), as the demos' convertTo
    res = []
    for im in (img, f):
        o = gpu_lib.AKAZEOptions()
        o.setWidth(320)
        o.setHeight(240)
        ak = gpu_lib.AKAZE(o)
        ak.Create_Nonlinear_Scale_Space(im)
        ak.Feature_Detection()
        res.append(ak.Compute_Descriptors())
    assert np.array_equal(res[0][0], res[1][0])
    assert np.array_equal(res[0][1].view(np.uint8), res[1][1].view(np.uint8))


def test_uneven_batch_equals_single_images(gpu_lib, oracle):
    sizes = synth.uneven_sizes(5, 6)
    imgs = [synth.synth_image(700 + i, w, h) for i, (w, h) in enumerate(sizes)]
    b = gpu_lib.Batch(gpu_lib.AKAZEOptions(), sizes)
    b.upload(imgs)
    b.run()
    counts = b.counts()
    b.run()  # graph replay gives the same results
    assert np.array_equal(counts, b.counts())
    for i, ((w, h), img) in enumerate(zip(sizes, imgs)):
        kp, d = b.results(i)
        orc = oracle.Oracle(w, h)
        okp, od = orc.run(img)
        assert _exact(kp, okp), (i, w, h)
        assert np.array_equal(d, od), (i, w, h)


@pytest.mark.parametrize("opts,rb", [({}, 61), ({"descriptor_channels": 1}, 21), ({"descriptor_size": 100}, 13),
                                     ({"descriptor_size": 64}, 8)])
def test_packed_output_equals_per_image_results(gpu_lib, opts, rb):
    """Packed rows of every width: word stores of the packed byte stream,
    images meeting inside a word."""
    sizes = synth.uneven_sizes(9, 5)
    imgs = [synth.synth_image(900 + i, w, h) for i, (w, h) in enumerate(sizes)]
    o = gpu_lib.AKAZEOptions(**opts)
    assert gpu_lib.descriptor_bytes(o) == rb
    b = gpu_lib.Batch(o, sizes)
    b.upload(imgs)
    b.run()
    per = [b.results(i) for i in range(len(sizes))]
    total = sum(len(k) for k, _ in per)
    kp = np.zeros(total, gpu_lib.KEYPOINT_DTYPE)
    d = np.zeros((total, rb), np.uint8)
    counts = b.detect_describe_packed(imgs, kp, d)
    assert list(counts) == [len(k) for k, _ in per]
    off = 0
    for k, dd in per:
        assert kp[off:off + len(k)].tobytes() == k.tobytes()
        assert np.array_equal(d[off:off + len(k)], dd)
        off += len(k)
    with pytest.raises(gpu_lib.AkazeError):
        b.detect_describe_packed(imgs, kp[: total - 1], d[: total - 1])


def test_fed_blocking_depths_give_identical_results(gpu_lib):
    """Every FED blocking depth (steps per level-kernel launch) computes the
    same arithmetic; the autotuner only picks the fastest."""
    sizes = synth.uneven_sizes(11, 6)
    imgs = [synth.synth_image(1100 + i, w, h) for i, (w, h) in enumerate(sizes)]
    b = gpu_lib.Batch(gpu_lib.AKAZEOptions(), sizes)
    b.upload(imgs)
    b.run()
    want = [b.results(i) for i in range(len(sizes))]
    for depth in (4, 5, 6, 7, 8):
        b.set_fed_depth(depth)
        b.run()
        for i, (k, d) in enumerate(want):
            kk, dd = b.results(i)
            assert kk.tobytes() == k.tobytes() and np.array_equal(dd, d), (depth, i)
    depths, ms = b.autotune()
    assert depths and all(4 <= x <= 8 for x in depths)
    assert sorted(ms) == [4, 5, 6, 7, 8] and all(v > 0 for v in ms.values())
    b.upload(imgs)
    b.run()
    assert all(b.results(i)[0].tobytes() == want[i][0].tobytes() for i in range(len(sizes)))
    with pytest.raises(gpu_lib.AkazeError):
        b.set_fed_depth(3)


def test_batch_group_equals_one_batch(gpu_lib):
    """Groups on their own streams (overlapping on the GPU, packed output
    from one host thread per group) give the single batch's results."""
    sizes = synth.uneven_sizes(13, 7)
    imgs = [synth.synth_image(1300 + i, w, h) for i, (w, h) in enumerate(sizes)]
    one = gpu_lib.Batch(gpu_lib.AKAZEOptions(), sizes)
    one.upload(imgs)
    one.run()
    want = [one.results(i) for i in range(len(sizes))]
    grp = gpu_lib.BatchGroup(gpu_lib.AKAZEOptions(), sizes, groups=3)
    assert [len(b.sizes) for b in grp.parts] == [2, 2, 3]
    grp.upload(imgs)
    grp.run()
    grp.run()
    assert list(grp.counts()) == [len(k) for k, _ in want]
    for i, (k, d) in enumerate(want):
        kk, dd = grp.results(i)
        assert kk.tobytes() == k.tobytes() and np.array_equal(dd, d), i
    total = sum(len(k) for k, _ in want)
    kp = np.zeros(total + 300, gpu_lib.KEYPOINT_DTYPE)
    d = np.zeros((total + 300, 61), np.uint8)
    counts = grp.detect_describe_packed(imgs, kp, d)
    assert list(counts) == [len(k) for k, _ in want]
    off = 0
    for k, dd in want:
        assert kp[off:off + len(k)].tobytes() == k.tobytes() and np.array_equal(d[off:off + len(k)], dd)
        off += len(k)
    with pytest.raises(gpu_lib.AkazeError):  # nothing submitted
        grp.parts[0].collect_packed(kp, d)


def test_batch_group_pipelined_steps(gpu_lib):
    """Pipelined whole-job steps give each step the results of a single call."""
    sizes = synth.uneven_sizes(17, 6)
    a = [synth.synth_image(1700 + i, w, h) for i, (w, h) in enumerate(sizes)]
    b = [synth.synth_image(1800 + i, w, h) for i, (w, h) in enumerate(sizes)]
    grp = gpu_lib.BatchGroup(gpu_lib.AKAZEOptions(), sizes, groups=2)
    cap = 200000
    kp = np.zeros(cap, gpu_lib.KEYPOINT_DTYPE)
    d = np.zeros((cap, 61), np.uint8)
    want = []
    for imgs in (a, b):
        c = grp.detect_describe_packed(imgs, kp, d)
        n = int(c.sum())
        want.append((c.copy(), kp[:n].tobytes(), d[:n].copy()))
    got = []

    def keep(si, c):
        n = int(c.sum())
        got.append((c.copy(), kp[:n].tobytes(), d[:n].copy()))

    grp.detect_describe_packed_steps([a, b, a], kp, d, on_step=keep)
    for (wc, wk, wd), (gc, gk, gd) in zip(want + [want[0]], got):
        assert np.array_equal(wc, gc) and wk == gk and np.array_equal(wd, gd)


def test_two_runs_outstanding(gpu_lib):
    """submit, submit, collect, collect: each collect returns its own run's
    results, in order; a third submit, a whole-job call with a run
    outstanding and a collect with none are refused."""
    sizes = synth.uneven_sizes(19, 3)
    a = [synth.synth_image(1900 + i, w, h) for i, (w, h) in enumerate(sizes)]
    b = [synth.synth_image(1950 + i, w, h) for i, (w, h) in enumerate(sizes)]
    bt = gpu_lib.Batch(gpu_lib.AKAZEOptions(), sizes)
    cap = 200000
    kp = np.zeros(cap, gpu_lib.KEYPOINT_DTYPE)
    d = np.zeros((cap, 61), np.uint8)
    want = []
    for imgs in (a, b):
        c = bt.detect_describe_packed(imgs, kp, d)
        n = int(c.sum())
        want.append((c.copy(), kp[:n].tobytes(), d[:n].copy()))
    assert want[0][1] != want[1][1]
    bt.submit(a)
    bt.submit(b)
    with pytest.raises(gpu_lib.AkazeError):
        bt.submit(a)
    with pytest.raises(gpu_lib.AkazeError):
        bt.detect_describe_packed(a, kp, d)
    for wc, wk, wd in want:
        c, n = bt.collect_packed(kp, d)
        assert np.array_equal(c, wc) and kp[:n].tobytes() == wk and np.array_equal(d[:n], wd)
    with pytest.raises(gpu_lib.AkazeError):
        bt.collect_packed(kp, d)
    c = bt.detect_describe_packed(b, kp, d)  # usable again
    assert np.array_equal(c, want[1][0])


def test_pipelined_steps_recover_from_a_failed_collect(gpu_lib):
    """An output buffer too small for a step raises; the runs still in
    flight are dropped, and the group then works as before."""
    sizes = synth.uneven_sizes(23, 4)
    a = [synth.synth_image(2300 + i, w, h) for i, (w, h) in enumerate(sizes)]
    grp = gpu_lib.BatchGroup(gpu_lib.AKAZEOptions(), sizes, groups=2)
    cap = 200000
    kp = np.zeros(cap, gpu_lib.KEYPOINT_DTYPE)
    d = np.zeros((cap, 61), np.uint8)
    want = grp.detect_describe_packed(a, kp, d).copy()
    assert want.sum() > 2
    with pytest.raises(gpu_lib.AkazeError):
        grp.detect_describe_packed_steps([a, a, a], kp[:1], d[:1])
    assert all(not getattr(b, "_subs", []) for b in grp.parts)
    assert np.array_equal(grp.detect_describe_packed(a, kp, d), want)
