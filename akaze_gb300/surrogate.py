"""Learned FED surrogate: training and inference driver.

The net (3 -> 32 -> 32 -> 32 -> 32 -> 1, 3x3 convolutions, ReLU) maps a
level's starting image L_start, its conductance g and a feature of the
level's FED time span dt to (L_end - L_start) / S_OUT, where L_end is the
level after its whole FED cycle (AKAZE.cpp:244-270).  Every arithmetic step
of training and inference runs in this package's CUDA kernels (akz_sg_* in
libakaze_gb300.so); torch tensors only hold device memory.

Training data are (L_start, g, dt, L_end) quadruples taken from the plain
FED path of this library on seeded synthetic images: L_end is the level's
Lt, L_start its predecessor's Lt (exactly half-sampled at an octave start),
g the PM-g2 conductance of the level's Lsmooth with the level's contrast
factor.  Crops of 48 x 48 inputs train 38 x 38 valid outputs.

    python -m akaze_gb300.surrogate train --out weights.npz
"""
import argparse
import ctypes
import time

import numpy as np

from . import _lib

LAYERS = [(3, 32), (32, 32), (32, 32), (32, 32), (32, 1)]
S_OUT = 0.05
CROP_IN = 48  # small enough for the 67-pixel-high levels of octave 5 at 3840x2160
CROP_OUT = CROP_IN - 2 * len(LAYERS)


def dt_feature(dt):
    return float(0.25 * np.log2(max(dt, 1e-12)))


def to_bf16_bits(a):
    """float32 -> bf16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def from_bf16_bits(b):
    return (np.asarray(b, np.uint32) << 16).view(np.float32)


def pack_inference(params):
    """FP32 training weights -> (bf16 blob, biases) in the layout of
    akz_sg_infer_level."""
    w1, b1 = params[0]
    blocks = []
    W1 = np.zeros((32, 32), np.float32)
    for co in range(32):
        for ky in range(3):
            for kx in range(3):
                for ch in range(3):
                    W1[co, (ky * 3 + kx) * 3 + ch] = w1[co, ch, ky, kx]
    blocks.append(W1)
    for li in (1, 2, 3):
        w = params[li][0]
        blocks.append(np.transpose(w, (0, 2, 3, 1)).reshape(32, 288))  # k = (ky*3+kx)*32 + ci
    w5 = params[4][0]
    W5 = np.zeros((8, 288), np.float32)
    W5[0] = np.transpose(w5, (0, 2, 3, 1)).reshape(1, 288)[0]
    blocks.append(W5)
    blob = to_bf16_bits(np.concatenate([b.reshape(-1) for b in blocks]))
    biases = np.zeros(4 * 32 + 8, np.float32)
    for li in range(4):
        biases[32 * li:32 * li + 32] = params[li][1]
    biases[128] = params[4][1][0]
    return blob, biases


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class SurrogateNet:
    """FP32 parameters and Adam state on the current CUDA device."""

    def __init__(self, seed=0, params=None):
        import torch
        self.torch = torch
        self.L = _lib.load()
        rng = np.random.default_rng(seed)
        if params is None:
            params = []
            for i, (cin, cout) in enumerate(LAYERS):
                w = rng.normal(0.0, np.sqrt(2.0 / (cin * 9)), (cout, cin, 3, 3)).astype(np.float32)
                if i == len(LAYERS) - 1:
                    w *= 0.1
                params.append((w, np.zeros(cout, np.float32)))
        self.w = [torch.from_numpy(np.ascontiguousarray(w, np.float32)).cuda() for w, _ in params]
        self.b = [torch.from_numpy(np.ascontiguousarray(b, np.float32)).cuda() for _, b in params]
        self.gw = [torch.zeros_like(t) for t in self.w]
        self.gb = [torch.zeros_like(t) for t in self.b]
        self.m = [torch.zeros_like(t) for t in self.w + self.b]
        self.v = [torch.zeros_like(t) for t in self.w + self.b]
        self.step_no = 0
        self.stream = torch.cuda.current_stream().cuda_stream

    def params_numpy(self):
        return [(w.cpu().numpy(), b.cpu().numpy()) for w, b in zip(self.w, self.b)]

    def forward(self, x):
        """x: (B, 3, H, W) float32 CUDA tensor -> activations [x, a1, .., out]."""
        torch = self.torch
        acts = [x]
        for i, (cin, cout) in enumerate(LAYERS):
            B, _, H, W = acts[-1].shape
            out = torch.empty((B, cout, H - 2, W - 2), dtype=torch.float32, device="cuda")
            _lib.check(self.L.akz_sg_conv_forward(_ptr(acts[-1]), _ptr(self.w[i]), _ptr(self.b[i]), _ptr(out), B, cin, cout,
                                                  H, W, int(i < len(LAYERS) - 1), ctypes.c_void_p(self.stream)))
            acts.append(out)
        return acts

    def backward(self, acts, dout):
        torch = self.torch
        g = dout
        for i in range(len(LAYERS) - 1, -1, -1):
            cin, cout = LAYERS[i]
            x = acts[i]
            B, _, H, W = x.shape
            _lib.check(self.L.akz_sg_conv_backward_weights(_ptr(x), _ptr(g), _ptr(self.gw[i]), _ptr(self.gb[i]), B, cin, cout,
                                                           H, W, ctypes.c_void_p(self.stream)))
            if i > 0:
                dx = torch.empty_like(x)
                _lib.check(self.L.akz_sg_conv_backward_data(_ptr(g), _ptr(self.w[i]), _ptr(x), _ptr(dx), B, cin, cout, H, W,
                                                            ctypes.c_void_p(self.stream)))
                g = dx

    def loss_grad(self, out, target):
        """dL/dout for L = mean((out - target)^2) and the loss itself."""
        torch = self.torch
        n = out.numel()
        dout = torch.empty_like(out)
        parts = torch.empty(256, dtype=torch.float32, device="cuda")
        _lib.check(self.L.akz_sg_mse_grad(_ptr(out), _ptr(target), _ptr(dout), n, ctypes.c_float(2.0 / n), _ptr(parts), 256,
                                          ctypes.c_void_p(self.stream)))
        return dout, float(parts.cpu().numpy().astype(np.float64).sum() / n)

    def adam(self, lr, b1=0.9, b2=0.999, eps=1e-8):
        self.step_no += 1
        for p, g, m, v in zip(self.w + self.b, self.gw + self.gb, self.m, self.v):
            _lib.check(self.L.akz_sg_adam(_ptr(p), _ptr(g), _ptr(m), _ptr(v), p.numel(), ctypes.c_float(lr),
                                          ctypes.c_float(b1), ctypes.c_float(b2), ctypes.c_float(eps), self.step_no,
                                          ctypes.c_void_p(self.stream)))

    def train_step(self, x, target, lr):
        acts = self.forward(x)
        dout, loss = self.loss_grad(acts[-1], target)
        self.backward(acts, dout)
        self.adam(lr)
        return loss


# ---------------------------------------------------------------------------
# training data from the plain FED path

def scharr_pm_g2(ls, k):
    """PM-g2 conductance of the Scharr gradient of Lsmooth (reflect-101),
    nldiffusion_functions.cpp:50-83, in float64."""
    p = np.pad(ls.astype(np.float64), 1, mode="reflect")
    h = p[:, 2:] - p[:, :-2]
    gx = 3.0 * (h[:-2] + h[2:]) + 10.0 * h[1:-1]
    s = 3.0 * (p[:, :-2] + p[:, 2:]) + 10.0 * p[:, 1:-1]
    gy = s[2:] - s[:-2]
    return (1.0 / (1.0 + (gx * gx + gy * gy) / (k * k))).astype(np.float32)


def half_sample(img):
    h, w = img.shape[0] // 2, img.shape[1] // 2
    a = img[:2 * h:2, :2 * w:2] + img[:2 * h:2, 1:2 * w:2]
    return (0.25 * ((a + img[1:2 * h:2, :2 * w:2]) + img[1:2 * h:2, 1:2 * w:2])).astype(np.float32)


def level_quads(ak, first_octave=1):
    """(level, octave, L_start, g, dt, L_end) for every level of octave >=
    first_octave of the context's last image."""
    kc = ak.kcontrast
    out = []
    prev = None
    for lv in range(ak.nlevels):
        info = ak.level_info(lv)
        lt = ak.plane(lv, "Lt")
        # a level whose plain FED result left the image range is not a
        # target: the reference's single long FED cycle in float32 diverges at
        # octave 5 of a 6-octave 3840x2160 stack (96 steps, largest step 467)
        sane = bool(np.isfinite(lt).all() and np.abs(lt).max() <= 2.0)
        if info["octave"] >= first_octave and prev is not None and sane:
            pinfo, plt = prev
            start = plt if pinfo["octave"] == info["octave"] else half_sample(plt)
            if start.shape == lt.shape:
                k = kc
                for _ in range(info["octave"]):
                    k = float(np.float32(k * 0.75))
                g = scharr_pm_g2(ak.plane(lv, "Lsmooth"), k)
                dt = 0.5 * (info["esigma"] ** 2 - pinfo["esigma"] ** 2)
                out.append((lv, info["octave"], start, g, dt, lt))
        prev = (info, lt)
    return out


def make_crops(quads, n_per_level, rng):
    xs, ys = [], []
    for (_, _, l0, g, dt, l1) in quads:
        H, W = l0.shape
        if H < CROP_IN or W < CROP_IN:
            continue
        f = dt_feature(dt)
        for _ in range(n_per_level):
            y0 = int(rng.integers(0, H - CROP_IN + 1))
            x0 = int(rng.integers(0, W - CROP_IN + 1))
            sl = (slice(y0, y0 + CROP_IN), slice(x0, x0 + CROP_IN))
            x = np.stack([l0[sl], g[sl], np.full((CROP_IN, CROP_IN), f, np.float32)])
            m = (CROP_IN - CROP_OUT) // 2
            t = (l1[sl] - l0[sl])[m:m + CROP_OUT, m:m + CROP_OUT] / S_OUT
            xs.append(x)
            ys.append(t[None])
    return np.stack(xs).astype(np.float32), np.stack(ys).astype(np.float32)


def build_dataset(nimages, width, height, omax, n_per_level, seed=0):
    from . import AKAZE, AKAZEOptions, synth
    rng = np.random.default_rng(seed)
    o = AKAZEOptions(omax=omax)
    o.setWidth(width)
    o.setHeight(height)
    ak = AKAZE(o)
    X, Y = [], []
    for i in range(nimages):
        ak.detect_and_compute(synth.synth_image(7000 + i, width, height))
        x, y = make_crops(level_quads(ak), n_per_level, rng)
        X.append(x)
        Y.append(y)
    ak.close()
    return np.concatenate(X), np.concatenate(Y)


def train(nimages=4, width=1920, height=1080, omax=6, n_per_level=96, iters=3000, batch=32, lr=1e-3, seed=0, log=print,
          max_seconds=None):
    import torch
    t0 = time.time()
    X, Y = build_dataset(nimages, width, height, omax, n_per_level, seed)
    log(f"dataset: {len(X)} crops of {CROP_IN}x{CROP_IN} from {nimages} images ({time.time() - t0:.1f} s)")
    Xd, Yd = torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda()
    n = len(X)
    nval = max(1, n // 10)
    net = SurrogateNet(seed)
    rng = np.random.default_rng(seed + 1)
    hist = []
    t1 = time.time()
    for it in range(iters):
        if max_seconds is not None and time.time() - t1 > max_seconds:
            iters = it
            break
        idx = torch.from_numpy(rng.integers(nval, n, batch)).cuda()
        cur_lr = lr * (0.1 if it > 0.8 * iters else 1.0)
        loss = net.train_step(Xd[idx].contiguous(), Yd[idx].contiguous(), cur_lr)
        if it % 200 == 0 or it == iters - 1:
            hist.append((it, loss))
            log(f"iter {it} loss {loss:.5f}")
    torch.cuda.synchronize()
    tt = time.time() - t1
    # held-out loss against the zero-residual baseline (plain identity)
    vl, base = 0.0, 0.0
    for s in range(0, nval, batch):
        xv, yv = Xd[s:s + batch].contiguous(), Yd[s:s + batch].contiguous()
        out = net.forward(xv)[-1]
        _, l = net.loss_grad(out, yv)
        vl += l * len(xv)
        base += float((yv.double() ** 2).mean().cpu()) * len(xv)
    return net, {"crops": n, "val_crops": nval, "iters": iters, "train_s": tt, "val_mse": vl / nval,
                 "val_mse_zero_residual": base / nval, "loss_curve": hist}


def save(path, net, meta):
    arrs = {}
    for i, (w, b) in enumerate(net.params_numpy()):
        arrs[f"w{i}"] = w
        arrs[f"b{i}"] = b
    np.savez(path, meta=np.array(repr(meta)), **arrs)


def load_params(path):
    d = np.load(path)
    return [(d[f"w{i}"], d[f"b{i}"]) for i in range(len(LAYERS))]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train"])
    ap.add_argument("--out", default="surrogate_weights.npz")
    ap.add_argument("--images", type=int, default=4)
    ap.add_argument("--iters", type=int, default=3000)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--omax", type=int, default=6)
    ap.add_argument("--max-seconds", type=float, default=None)
    args = ap.parse_args()
    net, meta = train(args.images, args.width, args.height, args.omax, iters=args.iters, max_seconds=args.max_seconds)
    print(meta)
    save(args.out, net, meta)


if __name__ == "__main__":
    main()
