"""Fits the polynomial coefficients of akz_fmath.h and checks the header.

Each routine of akz_fmath.h evaluates a short polynomial after an argument
reduction.  The coefficients come from this script: a weighted minimax fit
by Lawson's algorithm (iteratively reweighted least squares) on Chebyshev
nodes of the reduced interval, weighted so that the error is relative to the
function value, then rounded to the nearest float32.

  atan(a)  = a + a^3 * P(a^2),  a in [0, 1],         P of degree 7
  sin(r)   = r + r^3 * S(r^2),  r in [0, pi/4],      S of degree 3
  cos(r)   = 1 + r^2 * C(r^2),  r in [0, pi/4],      C of degree 3
  exp(r)   = 1 + r + r^2 * E(r), r in [-ln2/2, ln2/2], E of degree 4

  python fit_fmath.py          prints the coefficients as C hex floats
  python fit_fmath.py --check  exits 1 unless akz_fmath.h holds exactly them

Only numpy (float64) is used; the reduced functions are evaluated with
series where float64 cancellation would otherwise lose digits.
"""
import os
import re
import sys

import numpy as np

HEADER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "akz_fmath.h")
NODES = 4000
ITERS = 300


def _cheb(lo, hi, n=NODES):
    k = np.arange(n)
    return 0.5 * (lo + hi) + 0.5 * (hi - lo) * np.cos(np.pi * (k + 0.5) / n)


def _series(x, terms):
    """sum_k c_k x^k for the given (power, coefficient) list, Horner-free."""
    out = np.zeros_like(x)
    for p, c in terms:
        out += c * x ** p
    return out


def _atan_reduced(s):
    # (atan(a) - a) / a^3 with s = a^2; the series -1/3 + s/5 - s^2/7 ... for small s
    a = np.sqrt(s)
    direct = (np.arctan(a) - a) / (a * s)
    small = _series(s, [(k, (-1) ** (k + 1) / (2 * k + 3)) for k in range(40)])
    return np.where(s < 0.04, small, direct)


def _sin_reduced(s):
    r = np.sqrt(s)
    direct = (np.sin(r) - r) / (r * s)
    fact = [1.0]
    for k in range(1, 40):
        fact.append(fact[-1] * k)
    small = _series(s, [(k, (-1) ** (k + 1) / fact[2 * k + 3]) for k in range(12)])
    return np.where(s < 0.05, small, direct)


def _cos_reduced(s):
    r = np.sqrt(s)
    direct = (np.cos(r) - 1.0) / s
    fact = [1.0]
    for k in range(1, 40):
        fact.append(fact[-1] * k)
    small = _series(s, [(k, (-1) ** (k + 1) / fact[2 * k + 2]) for k in range(12)])
    return np.where(s < 0.05, small, direct)


def _exp_reduced(r):
    direct = (np.exp(r) - 1.0 - r) / (r * r)
    fact = [1.0]
    for k in range(1, 40):
        fact.append(fact[-1] * k)
    small = _series(r, [(k, 1.0 / fact[k + 2]) for k in range(16)])
    return np.where(np.abs(r) < 0.1, small, direct)


def lawson(x, f, w, deg):
    """Coefficients (lowest power first) of the degree-deg polynomial that
    minimises max |w * (p(x) - f)| over the nodes x (Lawson's algorithm)."""
    V = np.vander(x, deg + 1, increasing=True)
    lam = np.full(len(x), 1.0 / len(x))
    c = None
    for _ in range(ITERS):
        sw = np.sqrt(lam) * w
        c, *_ = np.linalg.lstsq(V * sw[:, None], f * sw, rcond=None)
        e = np.abs(w * (V @ c - f))
        lam = lam * e
        s = lam.sum()
        if not s > 0:
            break
        lam /= s
    return c


def fit():
    out = {}
    s = _cheb(0.0, 1.0)  # a^2 for a in [0, 1]
    a = np.sqrt(s)
    out["atan"] = lawson(s, _atan_reduced(s), a ** 3 / np.arctan(np.maximum(a, 1e-300)), 7)
    r = _cheb(0.0, np.pi / 4)
    s = r * r
    out["sin"] = lawson(s, _sin_reduced(s), r ** 3 / np.sin(np.maximum(r, 1e-300)), 3)
    out["cos"] = lawson(s, _cos_reduced(s), s / np.cos(r), 3)
    r = _cheb(-np.log(2) / 2, np.log(2) / 2)
    out["exp"] = lawson(r, _exp_reduced(r), r * r / np.exp(r), 4)
    return {k: [float(np.float32(v)) for v in c] for k, c in out.items()}


def c_hex(v):
    """C99 hex literal of a float32 value, e.g. -0x1.5554dcp-2f."""
    f = np.float32(v)
    if f == 0:
        return "0x0p+0f"
    m, e = np.frexp(np.float64(f))  # f = m * 2^e, 0.5 <= |m| < 1
    mant = int(round(abs(m) * 2 ** 24))  # 24 significant bits, leading bit at 2^23
    frac = (mant - (1 << 23)) << 1  # 23 fraction bits, padded to 24 = 6 hex digits
    return f"{'-' if f < 0 else ''}0x1.{frac:06x}p{e - 1:+d}f"


def header_coefficients(text):
    """The literals of each polynomial in the header, highest power first."""
    lit = r"(-?0x1\.[0-9a-f]{6}p[+-]\d+f)"
    spans = {
        "atan": ("float p = 0x", "r = AKZ_FMA(AKZ_MUL(a, s), p, a)"),
        "sin": ("float ps =", "const float sr"),
        "cos": ("float pc =", "const float cr"),
        "exp": ("p = AKZ_FMA(p, r, 0x", "const float e ="),
    }
    res = {}
    for key, (a, b) in spans.items():
        i = text.index(a)
        if key == "exp":  # the exp polynomial starts one line above its first FMA
            i = text.rindex("float p =", 0, i)
        res[key] = re.findall(lit, text[i:text.index(b, i)])
    return res


def main():
    coef = fit()
    want = {k: [c_hex(v) for v in reversed(c)] for k, c in coef.items()}  # highest power first, as evaluated
    if "--check" in sys.argv:
        have = header_coefficients(open(HEADER).read())
        ok = all(have[k] == want[k] for k in want)
        for k in want:
            print(k, "ok" if have[k] == want[k] else f"differs: header {have[k]} fit {want[k]}")
        sys.exit(0 if ok else 1)
    for k, v in want.items():
        print(k, ", ".join(v))


if __name__ == "__main__":
    main()
