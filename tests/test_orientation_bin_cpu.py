"""The orientation bin shortcut of k_describe (akaze_gb300/csrc/akz_describe.cu).

The reference computes the bin of an angle a (a float from atan2, |a| <= pi)
as (int)((double)a * (21 / pi)) (cuda_akaze.cu:2114-2167).  The kernel
forms the float product tf = a * (float)(21 / pi) and keeps (int)tf unless
tf lies within 2^-17 of an integer; only then does it evaluate the double
product.  The float product is within a few 1e-6 of the double one, so
away from integers the two truncations agree.  This test checks that on every
float in a dense sweep of [-pi, pi], on random floats, and on the floats
next to every bin edge."""
import numpy as np

C64 = 21.0 / np.pi
C32 = np.float32(C64)
EPS = np.float32(2.0 ** -17)


def kernel_bin(a):
    tf = (a * C32).astype(np.float32)
    near = np.abs(tf - np.rint(tf)) <= EPS
    fast = np.trunc(tf).astype(np.int64)
    slow = np.trunc(a.astype(np.float64) * C64).astype(np.int64)
    return np.where(near, slow, fast)


def reference_bin(a):
    return np.trunc(a.astype(np.float64) * C64).astype(np.int64)


def test_float_product_shortcut_equals_double_truncation():
    pi32 = np.float32(np.pi)
    sweep = np.linspace(-pi32, pi32, 1 << 22, dtype=np.float32)
    rnd = np.random.default_rng(9).uniform(-np.pi, np.pi, 1 << 22).astype(np.float32)
    # the floats next to each bin edge k * pi / 21 (k = -21 .. 21), 64 ulps either side
    edges = (np.arange(-21, 22) / C64).astype(np.float32)
    near = [edges]
    lo, hi = edges.copy(), edges.copy()
    for _ in range(64):
        lo = np.nextafter(lo, np.float32(-np.inf))
        hi = np.nextafter(hi, np.float32(np.inf))
        near += [lo, hi]
    a = np.concatenate([sweep, rnd, np.concatenate(near)])
    a = a[np.abs(a) <= pi32]
    assert np.array_equal(kernel_bin(a), reference_bin(a))
    # the margin: the float product never strays by more than 2^-17 from the double one
    err = np.abs((a * C32).astype(np.float64) - a.astype(np.float64) * C64)
    assert err.max() < 2.0 ** -17
