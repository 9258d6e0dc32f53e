"""The level kernel's exact PM-g2 reciprocal (akz_pm_g2_pair in
akaze_gb300/csrc/akz_scale.cu), replayed in exact rational arithmetic.

The reference evaluates g = (float)(1.0 / (1.0 + (double)f))
(nldiffusion_functions.cpp:81).  The kernel forms s = fl(1 + f) and its
exact error lo (TwoSum), takes an approximate reciprocal q of s (relative
error below 2^-22), one Newton step r = 1 - q (s + lo) with FMAs, and rounds
v = q + q r twice, at v - q 2^-41 and v + q 2^-41.  Where both roundings
agree it returns that float, else it evaluates the reference's double
expression.  This test emulates every float32 operation with correct
rounding (an FMA rounds once) and the approximate reciprocal by a random
relative error of up to 2^-22.  It checks that TwoSum is exact, that
r -/+ 2^-41 is exact in float32, and that every non-fallback result equals
the reference's double-then-float rounding.  That covers random arguments
and arguments whose quotient lies next to a float rounding midpoint.  The
device routine itself is checked against double division on the GPU
(tests/test_device_math_gpu.py)."""
from fractions import Fraction as F
import math
import random

import numpy as np


def _rn(x, mant_bits):
    """Round the rational x to the nearest binary float with mant_bits
    significand bits (ties to even); normal range only."""
    if x == 0:
        return F(0)
    sign = -1 if x < 0 else 1
    a = abs(x)
    e = math.floor(math.log2(a.numerator) - math.log2(a.denominator))
    # fix e so that 2^e <= a < 2^(e+1)
    while F(2) ** e > a:
        e -= 1
    while F(2) ** (e + 1) <= a:
        e += 1
    scale = F(2) ** (e - (mant_bits - 1))
    n = a / scale
    fl = n.numerator // n.denominator
    rem = n - fl
    if rem > F(1, 2) or (rem == F(1, 2) and fl % 2 == 1):
        fl += 1
    return sign * fl * scale


def rn32(x):
    return _rn(x, 24)


def rn64(x):
    return _rn(x, 53)


BAND = F(1, 2 ** 41)


def kernel_g(f, rel_err):
    one = F(1)
    s = rn32(one + f)
    bb = rn32(s - one)
    lo = rn32(rn32(one - rn32(s - bb)) + rn32(f - bb))
    assert lo == one + f - s  # TwoSum is exact
    q = rn32((one / s) * (one + rel_err))  # the approximate reciprocal
    t = rn32(one - q * s)  # fma(-q, s, 1)
    r = rn32(t - q * lo)  # fma(-q, lo, t)
    assert abs(r) < F(1, 2 ** 21)
    rm, rp = rn32(r - BAND), rn32(r + BAND)
    assert rm == r - BAND and rp == r + BAND  # exact, so each FMA below rounds once
    lo_r = rn32(q * rm + q)
    hi_r = rn32(q * rp + q)
    return lo_r if lo_r == hi_r else None


def reference_g(f):
    return rn32(rn64(F(1) / (F(1) + f)))


def _arguments(n_random, n_near):
    rng = np.random.default_rng(21)
    a = np.exp(rng.uniform(np.log(1e-8), np.log(1e6), n_random)).astype(np.float32)
    e = rng.integers(-12, 0, n_near)
    k = rng.integers(1 << 23, 1 << 24, n_near)
    y = (k + 0.5) * np.exp2(e - 24.0)
    near = (1.0 / y - 1.0).astype(np.float32)
    near = near[near > 0]
    return [F(float(v)) for v in np.concatenate([a, near, np.nextafter(near, np.float32(np.inf))])]


def test_two_rounding_decision_is_exact():
    random.seed(3)
    args = _arguments(1500, 1000)
    fallback = 0
    for f in args:
        for rel in (F(0), F(random.uniform(-1, 1)) * F(1, 2 ** 22)):
            g = kernel_g(f, rel)
            if g is None:
                fallback += 1
                continue
            assert g == reference_g(f), (float(f), float(rel))
    # the midpoint-adjacent arguments are the ones that fall back; random ones almost never do
    assert fallback < len(args)
