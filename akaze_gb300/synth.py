"""Seeded synthetic test scenes for the A-KAZE path (numpy).

The scene is analytic, so a homography-warped partner image is rendered by
evaluating the scene at inverse-mapped coordinates (no resampling):

  value(u, v) = 128
              + sum of 40 isotropic Gaussian blobs: centre uniform in the frame,
                sigma ~ U[3, 40] px, amplitude ~ U[30, 120], sign +-1
              + 3 oriented sinusoid gratings: period ~ U[8, 64] px,
                angle ~ U[0, pi), phase ~ U[0, 2 pi), amplitude ~ U[6, 20]
              + uniform noise in [-8, 8] (fresh per image)
  clipped to [0, 255] and rounded to uint8.

The partner homography is a rotation ~ U[-30, 30] deg about the centre, an
isotropic scale ~ U[0.7, 1.3] and perspective terms ~ U[-1e-4, 1e-4].
"""
import numpy as np


def scene_params(seed, width, height, nblobs=40, ngratings=3):
    rng = np.random.default_rng(seed)
    blobs = np.stack([
        rng.uniform(0, width, nblobs), rng.uniform(0, height, nblobs),
        rng.uniform(3, 40, nblobs), rng.uniform(30, 120, nblobs) * (rng.integers(0, 2, nblobs) * 2 - 1),
    ], 1)
    gratings = np.stack([
        rng.uniform(8, 64, ngratings), rng.uniform(0, np.pi, ngratings),
        rng.uniform(0, 2 * np.pi, ngratings), rng.uniform(6, 20, ngratings),
    ], 1)
    return {"blobs": blobs, "gratings": gratings, "width": width, "height": height}


def random_homography(seed, width, height):
    rng = np.random.default_rng(seed)
    ang = np.deg2rad(rng.uniform(-30, 30))
    s = rng.uniform(0.7, 1.3)
    p1, p2 = rng.uniform(-1e-4, 1e-4, 2)
    cx, cy = width / 2.0, height / 2.0
    T = np.array([[1, 0, cx], [0, 1, cy], [0, 0, 1]], np.float64)
    Ti = np.array([[1, 0, -cx], [0, 1, -cy], [0, 0, 1]], np.float64)
    A = np.array([[s * np.cos(ang), -s * np.sin(ang), 0], [s * np.sin(ang), s * np.cos(ang), 0], [p1, p2, 1]], np.float64)
    Hm = T @ A @ Ti
    return Hm / Hm[2, 2]


def _apply(Hm, x, y):
    d = Hm[2, 0] * x + Hm[2, 1] * y + Hm[2, 2]
    return (Hm[0, 0] * x + Hm[0, 1] * y + Hm[0, 2]) / d, (Hm[1, 0] * x + Hm[1, 1] * y + Hm[1, 2]) / d


def render(params, noise_seed, Hm=None, width=None, height=None):
    """Render the scene (optionally warped by Hm: out(x) = scene(Hm^-1 x))."""
    W = width or params["width"]
    H = height or params["height"]
    Hi = None if Hm is None else np.linalg.inv(Hm)
    img = np.full((H, W), 128.0, np.float64)
    ys, xs = np.mgrid[0:H, 0:W].astype(np.float64)
    if Hi is None:
        u, v = xs, ys
    else:
        u, v = _apply(Hi, xs, ys)
    for per, ang, ph, amp in params["gratings"]:
        img += amp * np.sin(2 * np.pi * (u * np.cos(ang) + v * np.sin(ang)) / per + ph)
    for cx, cy, sg, amp in params["blobs"]:
        r = 4.0 * sg
        if Hm is None:
            x0, x1, y0, y1 = cx - r, cx + r, cy - r, cy + r
        else:
            cxs, cys = _apply(Hm, np.array([cx - r, cx + r, cx - r, cx + r]), np.array([cy - r, cy - r, cy + r, cy + r]))
            x0, x1, y0, y1 = cxs.min() - 2, cxs.max() + 2, cys.min() - 2, cys.max() + 2
        xa, xb = max(int(np.floor(x0)), 0), min(int(np.ceil(x1)) + 1, W)
        ya, yb = max(int(np.floor(y0)), 0), min(int(np.ceil(y1)) + 1, H)
        if xa >= xb or ya >= yb:
            continue
        uu, vv = u[ya:yb, xa:xb], v[ya:yb, xa:xb]
        img[ya:yb, xa:xb] += amp * np.exp(-((uu - cx) ** 2 + (vv - cy) ** 2) / (2 * sg * sg))
    rng = np.random.default_rng(noise_seed)
    img += rng.uniform(-8, 8, img.shape)
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)


def synth_image(seed, width, height):
    return render(scene_params(seed, width, height), noise_seed=seed * 7919 + 1)


def synth_pair(seed, width, height):
    """(image, partner warped by H, H) for one seed."""
    p = scene_params(seed, width, height)
    Hm = random_homography(seed + 104729, width, height)
    return render(p, seed * 7919 + 1), render(p, seed * 7919 + 2, Hm), Hm


def uneven_sizes(seed, n, wmin=320, wmax=1920, hmin=240, hmax=1080):
    """n (width, height) pairs drawn uniformly and rounded to multiples of 8."""
    rng = np.random.default_rng(seed)
    w = (np.rint(rng.uniform(wmin, wmax, n) / 8) * 8).astype(int)
    h = (np.rint(rng.uniform(hmin, hmax, n) / 8) * 8).astype(int)
    return list(zip(w.tolist(), h.tolist()))


def matcher_rows(seed, n, m, planted=0.3, flip_p=0.05):
    """Query (n x 61) and train (m x 61) M-LDB-shaped rows: 486 Bernoulli(0.5)
    bits packed LSB-first (pad bits zero); a fraction of the queries are
    copies of a random train row with Binomial(486, flip_p) bits flipped."""
    rng = np.random.default_rng(seed)

    def rows(k):
        bits = rng.integers(0, 2, (k, 488), dtype=np.uint8)
        bits[:, 486:] = 0
        return np.packbits(bits, axis=1, bitorder="little")

    t = rows(m)
    q = rows(n)
    npl = int(round(planted * n))
    if npl and m:
        qi = rng.choice(n, npl, replace=False)
        ti = rng.integers(0, m, npl)
        bits = np.unpackbits(t[ti], axis=1, bitorder="little")[:, :488]
        flips = rng.random((npl, 486)) < flip_p
        bits[:, :486] ^= flips.astype(np.uint8)
        q[qi] = np.packbits(bits, axis=1, bitorder="little")
    return q, t
