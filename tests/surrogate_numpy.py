"""Float64 numpy restatement of the FED surrogate net, for checking the
CUDA training kernels (forward, backward, weight gradients) and the BF16
inference kernels.

Net: valid 3x3 convolutions 3 -> 32 -> 32 -> 32 -> 32 -> 1, ReLU after the
first four.  x: (B, C, H, W); w: (cout, cin, 3, 3); b: (cout,).
"""
import numpy as np


def conv_fwd(x, w, b, relu):
    B, C, H, W = x.shape
    co = w.shape[0]
    out = np.zeros((B, co, H - 2, W - 2))
    for ky in range(3):
        for kx in range(3):
            patch = x[:, :, ky:ky + H - 2, kx:kx + W - 2]
            out += np.einsum("bchw,oc->bohw", patch, w[:, :, ky, kx])
    out += b[None, :, None, None]
    return np.maximum(out, 0.0) if relu else out


def conv_bwd(x, w, dout, mask=None):
    """Gradients of a valid conv: (dx, dw, db).  mask multiplies dx (the
    ReLU derivative of the layer below)."""
    B, C, H, W = x.shape
    dx = np.zeros_like(x, dtype=np.float64)
    dw = np.zeros_like(w, dtype=np.float64)
    for ky in range(3):
        for kx in range(3):
            patch = x[:, :, ky:ky + H - 2, kx:kx + W - 2]
            dw[:, :, ky, kx] = np.einsum("bohw,bchw->oc", dout, patch)
            dx[:, :, ky:ky + H - 2, kx:kx + W - 2] += np.einsum("bohw,oc->bchw", dout, w[:, :, ky, kx])
    db = dout.sum(axis=(0, 2, 3))
    if mask is not None:
        dx = dx * (mask > 0)
    return dx, dw, db


def net_fwd(x, params):
    acts = [x]
    n = len(params)
    for i, (w, b) in enumerate(params):
        acts.append(conv_fwd(acts[-1], w, b, relu=i < n - 1))
    return acts


def net_bwd(acts, params, dout):
    grads = [None] * len(params)
    g = dout
    for i in range(len(params) - 1, -1, -1):
        w, _ = params[i]
        mask = acts[i] if i > 0 else None
        dx, dw, db = conv_bwd(acts[i], w, g, mask)
        grads[i] = (dw, db)
        g = dx
    return grads


def same_conv_replicate(x, w, b, relu):
    """'Same' 3x3 convolution with replicate padding (the inference form
    on a whole level: the image is extended by its border values)."""
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)), mode="edge")
    return conv_fwd(xp, w, b, relu)
