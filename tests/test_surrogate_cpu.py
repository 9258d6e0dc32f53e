"""The float64 numpy surrogate net against finite differences, and the
BF16 weight packing (CPU only)."""
import numpy as np

from akaze_gb300 import surrogate as sg

import surrogate_numpy as snp


def _params(rng, layers):
    return [(rng.normal(0, 0.3, (co, ci, 3, 3)), rng.normal(0, 0.1, co)) for ci, co in layers]


def test_numpy_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    layers = [(3, 4), (4, 4), (4, 1)]
    params = _params(rng, layers)
    x = rng.normal(0, 1, (2, 3, 9, 9))
    t = rng.normal(0, 1, (2, 1, 3, 3))

    def loss(ps):
        return 0.5 * ((snp.net_fwd(x, ps)[-1] - t) ** 2).sum()

    acts = snp.net_fwd(x, params)
    grads = snp.net_bwd(acts, params, acts[-1] - t)
    eps = 1e-6
    for li in range(len(layers)):
        w, b = params[li]
        for idx in [(0, 0, 1, 2), (0, 1, 0, 0)] if w.shape[1] > 1 else [(0, 0, 1, 2)]:
            wp = [(ww.copy(), bb.copy()) for ww, bb in params]
            wp[li][0][idx] += eps
            wm = [(ww.copy(), bb.copy()) for ww, bb in params]
            wm[li][0][idx] -= eps
            fd = (loss(wp) - loss(wm)) / (2 * eps)
            assert abs(fd - grads[li][0][idx]) <= 1e-5 * max(1.0, abs(fd)), (li, idx)
        bp = [(ww.copy(), bb.copy()) for ww, bb in params]
        bp[li][1][0] += eps
        bm = [(ww.copy(), bb.copy()) for ww, bb in params]
        bm[li][1][0] -= eps
        fd = (loss(bp) - loss(bm)) / (2 * eps)
        assert abs(fd - grads[li][1][0]) <= 1e-5 * max(1.0, abs(fd))


def test_bf16_round_trip_and_packing_layout():
    v = np.array([1.0, 1.00390625, 1.0078125, -3.5, 1e-3], np.float32)
    back = sg.from_bf16_bits(sg.to_bf16_bits(v))
    assert back[0] == 1.0 and back[3] == -3.5
    assert back[1] == 1.0  # a tie rounds to even
    rng = np.random.default_rng(1)
    params = [(rng.normal(0, 1, (co, ci, 3, 3)).astype(np.float32), rng.normal(0, 1, co).astype(np.float32))
              for ci, co in sg.LAYERS]
    blob, biases = sg.pack_inference(params)
    assert blob.size == 32 * 32 + 3 * 32 * 288 + 8 * 288
    W = sg.from_bf16_bits(blob)
    # layer 2, output 5, tap (ky=2, kx=1), input channel 7
    assert W[32 * 32 + 5 * 288 + (2 * 3 + 1) * 32 + 7] == sg.from_bf16_bits(sg.to_bf16_bits(params[1][0][5, 7, 2, 1]))
    # layer 1, output 3, tap (0, 2), channel 1 (g)
    assert W[3 * 32 + (0 * 3 + 2) * 3 + 1] == sg.from_bf16_bits(sg.to_bf16_bits(params[0][0][3, 1, 0, 2]))
    assert biases[128] == params[4][1][0] and biases[40] == params[1][1][8]
