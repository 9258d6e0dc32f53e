"""The device's exact PM-g2 reciprocal, (float)(1 / (1 + (double)f)) as
nldiffusion_functions.cpp:81 evaluates it, against numpy's double division:
2^26 random arguments over the range the conductance sees plus arguments
placed next to rounding midpoints of the result, through the two-pixel
routine of the level kernel and the scalar one."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _arguments():
    rng = np.random.default_rng(12)
    a = np.exp(rng.uniform(np.log(1e-8), np.log(1e6), 1 << 25)).astype(np.float32)
    b = rng.uniform(0, 4, 1 << 25).astype(np.float32)
    # near midpoints: y = (k + 1/2) ulp in [2^-12, 1), f = 1/y - 1 rounded to float, and its neighbours
    e = rng.integers(-12, 0, 1 << 20)
    k = rng.integers(1 << 23, 1 << 24, 1 << 20)
    y = (k + 0.5) * np.exp2(e - 24.0)
    f = (1.0 / y - 1.0).astype(np.float32)
    near = np.concatenate([f, np.nextafter(f, np.float32(np.inf)), np.nextafter(f, np.float32(0))])
    special = np.array([0.0, 1.0, 2.0, 0.5, 1e-30, 3e38, np.inf, np.nan], np.float32)
    return np.concatenate([a, b, near[near >= 0], special])


@pytest.mark.parametrize("fn", [0, 1])
def test_pm_g2_reciprocal_is_exact(gpu_lib, fn):
    torch = pytest.importorskip("torch")
    x = _arguments()
    want = (1.0 / (1.0 + x.astype(np.float64))).astype(np.float32)
    lib = gpu_lib.load()
    dx = torch.from_numpy(x).cuda()
    dy = torch.empty_like(dx)
    assert lib.akz_selfcheck_pm_g2(ctypes.c_void_p(dx.data_ptr()), ctypes.c_void_p(dy.data_ptr()), len(x), fn, None) == 0
    got = dy.cpu().numpy()
    bad = ~((got == want) | (np.isnan(got) & np.isnan(want)))
    assert int(bad.sum()) == 0, (x[bad][:5], got[bad][:5], want[bad][:5])
