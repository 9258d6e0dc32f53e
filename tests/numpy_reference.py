"""Independent numpy restatement of the reference's CPU scale-space functions
(src/lib/nldiffusion_functions.cpp), used to cross-check the C oracle on
small images.  Same operation order as the oracle (float32 arithmetic, the
reference's double-precision intermediates where it has them)."""
import numpy as np

f32 = np.float32


def gauss_R(sigma):
    ks = int(np.ceil(2.0 * (1.0 + (float(np.float32(sigma)) - 0.8) / 0.3)))
    if ks % 2 == 0:
        ks += 1
    return ks // 2


def gauss_taps(sigma):
    R = gauss_R(sigma)
    x = np.arange(-R, R + 1, dtype=np.float64)
    s = float(np.float32(sigma))
    t = np.exp((-0.5 / (s * s)) * x * x)
    return (t / t.sum()).astype(np.float32), R


def _sym_conv(get, k, R):
    """acc = k0*(v[-R]+v[R]); acc += k[R-d]*(v[-d]+v[d]) for d=R-1..1; acc += k[R]*v[0]"""
    if R == 0:
        return k[0] * get(0)
    acc = k[0] * (get(-R) + get(R))
    for d in range(R - 1, 0, -1):
        acc = acc + k[R - d] * (get(-d) + get(d))
    return acc + k[R] * get(0)


def gaussian(img, sigma):
    k, R = gauss_taps(sigma)
    h, w = img.shape
    xs = np.arange(w)
    ys = np.arange(h)
    tmp = _sym_conv(lambda d: img[:, np.clip(xs + d, 0, w - 1)], k, R).astype(np.float32)
    return _sym_conv(lambda d: tmp[np.clip(ys + d, 0, h - 1), :], k, R).astype(np.float32)


def refl101(i, n):
    i = np.where(i < 0, -i, i)
    return np.where(i >= n, 2 * n - 2 - i, i)


def scharr(s):
    h, w = s.shape
    xs, ys = np.arange(w), np.arange(h)
    xm, xp = refl101(xs - 1, w), refl101(xs + 1, w)
    ym, yp = refl101(ys - 1, h), refl101(ys + 1, h)
    rx = s[:, xp] - s[:, xm]
    lx = f32(3) * (rx[ym, :] + rx[yp, :]) + f32(10) * rx
    sy = f32(3) * (s[:, xm] + s[:, xp]) + f32(10) * s
    ly = sy[yp, :] - sy[ym, :]
    return lx.astype(np.float32), ly.astype(np.float32)


def k_percentile(img, perc=0.7, nbins=300):
    g = gaussian(img, 1.0)
    lx, ly = scharr(g)
    lx, ly = lx[1:-1, 1:-1], ly[1:-1, 1:-1]
    m2 = (lx * lx + ly * ly).astype(np.float32)
    hmax = np.float32(np.sqrt(np.float32(m2.max())))
    modg = np.sqrt(m2).astype(np.float32)
    nz = modg != 0
    nbin = np.floor(np.float32(nbins) * (modg[nz] / hmax)).astype(np.int64)
    nbin[nbin == nbins] = nbins - 1
    hist = np.bincount(nbin, minlength=nbins).astype(np.float32)
    npoints = np.float32(nz.sum())
    nthreshold = int(np.float32(npoints * np.float32(perc)))
    nel, k = 0, 0
    while nel < nthreshold and k < nbins:
        nel = int(np.float32(np.float32(nel) + hist[k]))
        k += 1
    if nel < nthreshold:
        return np.float32(0.03)
    return np.float32(hmax * (np.float32(k) / np.float32(nbins)))


def pm_g2(lx, ly, k):
    inv_k = np.float32(1.0 / float(np.float32(k * k)))
    m = (inv_k * (lx * lx + ly * ly)).astype(np.float32)
    return (1.0 / (1.0 + m.astype(np.float64))).astype(np.float32)


def nld_step(L, c, tau):
    """nld_step_scalar with the reference's border formulas."""
    h, w = L.shape
    st = np.zeros_like(L)
    half = 0.5 * float(np.float32(tau))

    def flux(cy, cx, dy, dx):
        # (c[p] + c[p+d]) * (L[p+d] - L[p]) on the slice (cy, cx)
        return (c[cy, cx] + c[cy + dy, cx + dx]) * (L[cy + dy, cx + dx] - L[cy, cx])

    I, J = slice(1, h - 1), slice(1, w - 1)
    ys, xs = np.arange(1, h - 1)[:, None], np.arange(1, w - 1)[None, :]
    xpos = (c[ys, xs] + c[ys, xs + 1]) * (L[ys, xs + 1] - L[ys, xs])
    xneg = (c[ys, xs - 1] + c[ys, xs]) * (L[ys, xs] - L[ys, xs - 1])
    ypos = (c[ys, xs] + c[ys + 1, xs]) * (L[ys + 1, xs] - L[ys, xs])
    yneg = (c[ys - 1, xs] + c[ys, xs]) * (L[ys, xs] - L[ys - 1, xs])
    st[I, J] = (half * (xpos - xneg + ypos - yneg).astype(np.float64)).astype(np.float32)
    for r, rp in ((0, 1), (h - 1, h - 2)):
        x = np.arange(1, w - 1)
        xpos = (c[r, x] + c[r, x + 1]) * (L[r, x + 1] - L[r, x])
        xneg = (c[r, x - 1] + c[r, x]) * (L[r, x] - L[r, x - 1])
        ypos = (c[r, x] + c[rp, x]) * (L[rp, x] - L[r, x])
        st[r, 1:w - 1] = (half * (xpos - xneg + ypos).astype(np.float64)).astype(np.float32)
        xpos = (c[r, 0] + c[r, 1]) * (L[r, 1] - L[r, 0])
        ypos = (c[r, 0] + c[rp, 0]) * (L[rp, 0] - L[r, 0])
        st[r, 0] = np.float32(half * float(xpos + ypos))
        x = w - 1
        xneg = (c[r, x - 1] + c[r, x]) * (L[r, x] - L[r, x - 1])
        ypos = (c[r, x] + c[rp, x]) * (L[rp, x] - L[r, x])
        st[r, x] = np.float32(half * float(-xneg + ypos))
    i = np.arange(1, h - 1)
    xpos = (c[i, 0] + c[i, 1]) * (L[i, 1] - L[i, 0])
    ypos = (c[i, 0] + c[i + 1, 0]) * (L[i + 1, 0] - L[i, 0])
    yneg = (c[i - 1, 0] + c[i, 0]) * (L[i, 0] - L[i - 1, 0])
    st[1:h - 1, 0] = (half * (xpos + ypos - yneg).astype(np.float64)).astype(np.float32)
    x = w - 1
    xneg = (c[i, x - 1] + c[i, x]) * (L[i, x] - L[i, x - 1])
    ypos = (c[i, x] + c[i + 1, x]) * (L[i + 1, x] - L[i, x])
    yneg = (c[i - 1, x] + c[i, x]) * (L[i, x] - L[i - 1, x])
    st[1:h - 1, x] = (half * (-xneg + ypos - yneg).astype(np.float64)).astype(np.float32)
    return (L + st).astype(np.float32)


def halfsample2(L):
    a, b = L[0::2, 0::2], L[0::2, 1::2]
    c, d = L[1::2, 0::2], L[1::2, 1::2]
    return (np.float32(0.25) * (((a + b) + c) + d)).astype(np.float32)


def scale_space(img01, levels, taus, soffset=1.6):
    """levels: list of dicts (width, height, octave); taus: per level.
    Returns (k, [Lt], [Lsmooth])."""
    k = k_percentile(img01)
    Lt = [gaussian(img01, soffset)]
    Ls = [Lt[0].copy()]
    kc = k
    for i in range(1, len(levels)):
        if levels[i]["octave"] > levels[i - 1]["octave"]:
            L = halfsample2(Lt[-1])
            kc = np.float32(float(kc) * 0.75)
        else:
            L = Lt[-1].copy()
        s = gaussian(L, 1.0)
        lx, ly = scharr(s)
        g = pm_g2(lx, ly, kc)
        for t in taus[i]:
            L = nld_step(L, g, t)
        Lt.append(L)
        Ls.append(s)
    return k, Lt, Ls
