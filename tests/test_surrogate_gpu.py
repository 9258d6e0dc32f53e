"""The surrogate's CUDA kernels against the float64 numpy net.

Training kernels (FP32): activations within 1e-4 and weight/bias gradients
within 1e-3 of the numpy values (relative to each tensor's largest
magnitude).  Inference kernel (BF16 tensor cores, FP32 accumulation): the
output residual within 2% of its range of a numpy emulation that rounds
inputs, weights and activations to BF16 the same way.
"""
import ctypes

import numpy as np
import pytest

from akaze_gb300 import surrogate as sg

import surrogate_numpy as snp

pytestmark = pytest.mark.gpu


def _close(got, want, rel):
    scale = max(float(np.abs(want).max()), 1e-12)
    return float(np.abs(np.asarray(got, np.float64) - want).max()) <= rel * scale


def test_training_kernels_match_numpy(gpu_lib):
    torch = pytest.importorskip("torch")
    net = sg.SurrogateNet(seed=3)
    rng = np.random.default_rng(4)
    x = rng.uniform(0, 1, (2, 3, 20, 22)).astype(np.float32)
    acts = net.forward(torch.from_numpy(x).cuda())
    params = [(w.astype(np.float64), b.astype(np.float64)) for w, b in net.params_numpy()]
    ref = snp.net_fwd(x.astype(np.float64), params)
    for i in range(1, len(ref)):
        assert _close(acts[i].cpu().numpy(), ref[i], 1e-4), f"activation {i}"
    dout = rng.normal(0, 1, ref[-1].shape).astype(np.float32)
    net.backward(acts, torch.from_numpy(dout).cuda())
    torch.cuda.synchronize()
    grads = snp.net_bwd(ref, params, dout.astype(np.float64))
    for i, (dw, db) in enumerate(grads):
        assert _close(net.gw[i].cpu().numpy(), dw, 1e-3), f"dw {i}"
        assert _close(net.gb[i].cpu().numpy(), db, 1e-3), f"db {i}"


@pytest.mark.parametrize("tcgen05,W,H", [(False, 100, 70), (True, 100, 70), (True, 300, 77), (True, 640, 400)])
def test_inference_kernel_matches_bf16_emulation(gpu_lib, tcgen05, W, H):
    """The persistent tcgen05 kernel gives each CTA at most one item of
    ceil(H / (CTAs per 128-pixel column block)) rows: (300, 77) has a
    partial column block and one-row items; (640, 400) has items of 5 rows
    on 152 SMs, so rows are prefetched inside the loop."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    params = [(rng.normal(0, np.sqrt(2.0 / (ci * 9)), (co, ci, 3, 3)).astype(np.float32),
               rng.normal(0, 0.05, co).astype(np.float32)) for ci, co in sg.LAYERS]
    pitch = (W + 31) // 32 * 32
    l0 = rng.uniform(0, 1, (H, W)).astype(np.float32)
    g = rng.uniform(0, 1, (H, W)).astype(np.float32)
    dtf, s_out = 0.7, sg.S_OUT
    blob, biases = sg.pack_inference(params)
    lib = gpu_lib.load()
    assert lib.akz_sg_weight_elems() == blob.size
    pl = np.zeros((H, pitch), np.float32)
    pg = np.zeros((H, pitch), np.float32)
    pl[:, :W], pg[:, :W] = l0, g
    dl, dg = torch.from_numpy(pl).cuda(), torch.from_numpy(pg).cuda()
    dout = torch.zeros((H, pitch), dtype=torch.float32, device="cuda")
    dw = torch.from_numpy(blob.view(np.int16).copy()).cuda()
    db = torch.from_numpy(biases).cuda()
    scratch = torch.empty(2 * H * W * 64, dtype=torch.uint8, device="cuda")
    lib.akz_sg_set_tcgen05(int(tcgen05))
    st = lib.akz_sg_infer_level(ctypes.c_void_p(dl.data_ptr()), ctypes.c_void_p(dg.data_ptr()), pitch, W, H,
                                ctypes.c_float(dtf), ctypes.c_float(s_out), ctypes.c_void_p(dw.data_ptr()),
                                ctypes.c_void_p(db.data_ptr()), ctypes.c_void_p(scratch.data_ptr()),
                                ctypes.c_void_p(dout.data_ptr()), None)
    assert st == 0, lib.akz_last_error()
    torch.cuda.synchronize()
    lib.akz_sg_set_tcgen05(1)  # the default
    timed_out = ctypes.c_int(-1)
    assert lib.akz_sg_tcgen05_status(ctypes.byref(timed_out)) == 0 and timed_out.value == 0
    got = (dout.cpu().numpy()[:, :W].astype(np.float64) - l0) / s_out

    def bf(a):
        return sg.from_bf16_bits(sg.to_bf16_bits(np.asarray(a, np.float32))).astype(np.float64)

    a = np.stack([bf(l0), bf(g), np.full((H, W), bf(np.float32(dtf)))])[None]
    for li, (w, b) in enumerate(params):
        out = snp.same_conv_replicate(a, bf(w), b.astype(np.float64), relu=li < len(params) - 1)
        a = bf(out) if li < len(params) - 1 else out
    want = a[0, 0]
    err = np.abs(got - want)
    assert err.max() <= 0.02 * (np.abs(want).max() + 1e-6), (err.max(), np.abs(want).max())


def test_training_lowers_the_loss(gpu_lib):
    pytest.importorskip("torch")
    net, meta = sg.train(nimages=1, width=640, height=480, omax=3, n_per_level=16, iters=120, batch=8, lr=2e-3,
                         log=lambda *_: None)
    curve = meta["loss_curve"]
    assert curve[-1][1] < curve[0][1]
    assert meta["val_mse"] < meta["val_mse_zero_residual"]


def test_surrogate_in_the_pipeline_and_exact_fallback(gpu_lib):
    pytest.importorskip("torch")
    from akaze_gb300 import synth
    W, H = 640, 480
    sizes = [(W, H)] * 2
    imgs = [synth.synth_image(800 + i, W, H) for i in range(2)]
    rng = np.random.default_rng(6)
    params = [(0.5 * rng.normal(0, np.sqrt(2.0 / (ci * 9)), (co, ci, 3, 3)).astype(np.float32), np.zeros(co, np.float32))
              for ci, co in sg.LAYERS]
    plain = gpu_lib.Batch(gpu_lib.AKAZEOptions(), sizes)
    plain.upload(imgs)
    plain.run()
    ref = [plain.results(i) for i in range(2)]
    b = gpu_lib.Batch(gpu_lib.AKAZEOptions(), sizes)
    b.upload(imgs)
    # a tolerance nothing meets: every surrogate level falls back to plain FED,
    # so the whole result equals the plain pipeline bit for bit
    b.set_surrogate(params, first_octave=1, check_tol=1e-12)
    b.run()
    errs = b.surrogate_errors()
    assert errs.size == 16 and np.all(errs[4:] > 1e-12) and np.all(errs[:4] == 0)
    for i in range(2):
        kp, d = b.results(i)
        assert kp.tobytes() == ref[i][0].tobytes() and np.array_equal(d, ref[i][1])
    # a tolerance everything meets: the net's levels stand
    b.set_surrogate(params, first_octave=1, check_tol=1e9)
    b.run()
    assert np.all(np.isfinite(b.surrogate_errors()))
    assert not np.array_equal(b.plane(0, 5, shape=(240, 320)), plain.plane(0, 5, shape=(240, 320)))
    assert np.array_equal(b.plane(0, 3, shape=(480, 640)), plain.plane(0, 3, shape=(480, 640)))
    # switched off again: plain results
    b.set_surrogate(None)
    b.run()
    kp, d = b.results(1)
    assert kp.tobytes() == ref[1][0].tobytes() and np.array_equal(d, ref[1][1])
