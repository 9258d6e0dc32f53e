"""The allocation-free matcher entry point against the allocating one.

akz_matcher_bfmatch_noalloc serves callers that cannot call cudaMalloc (a
plugin inside a host that owns the device memory budget, or a hot path where
an allocation would synchronise the device): they pass device buffers in and
out, and the library keeps its scratch in a fixed device array.  This file is
collected last so that a failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

from akaze_gb300 import synth

pytestmark = pytest.mark.gpu

MAX_QUERIES = 131072


def _device_rows(torch, rows61):
    rows64 = np.zeros((rows61.shape[0], 64), np.uint8)
    rows64[:, :61] = rows61
    return torch.from_numpy(rows64).cuda()


def _noalloc(lib, torch, q, t, nt):
    out = torch.zeros((q.shape[0], 2, 4), dtype=torch.int32, device="cuda")
    st = lib.akz_matcher_bfmatch_noalloc(ctypes.c_void_p(q.data_ptr()), q.shape[0], ctypes.c_void_p(t.data_ptr()),
                                         nt, ctypes.c_void_p(out.data_ptr()),
                                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, lib.akz_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _allocating(gpu_lib, torch, q, t, nt):
    m = gpu_lib.Matcher()
    out = torch.zeros((q.shape[0], 2, 4), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    m.bfmatch_device(q.data_ptr(), q.shape[0], t.data_ptr(), nt, out.data_ptr())
    torch.cuda.synchronize()
    res = out.cpu().numpy()
    m.close()
    return res


def test_noalloc_matches_allocating_entry_point(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    lib = gpu_lib.load()
    # two calls in a row on the shared scratch array, of different shapes,
    # then one with an empty train set (every match is {trainIdx 0, distance 512})
    for seed, nq, nt in ((21, 1500, 7000), (22, 700, 3000), (23, 300, 0)):
        q61, t61 = synth.matcher_rows(seed, nq, nt)
        q = _device_rows(torch, q61)
        # an empty train set still passes a valid (unread) device address
        t = _device_rows(torch, t61) if nt else torch.zeros((1, 64), dtype=torch.uint8, device="cuda")
        got = _noalloc(lib, torch, q, t, nt)
        want = _allocating(gpu_lib, torch, q, t, nt)
        assert np.array_equal(got, want), f"seed {seed}: no-alloc result differs from the allocating entry point"
        # and both equal the CPU oracle's brute-force 2-NN
        ref = oracle.bfmatch(q61, t61)
        assert got.tobytes() == ref.tobytes(), f"seed {seed}: no-alloc result differs from the oracle"
        if nt == 0:
            assert np.all(ref["distance"] == 512) and np.all(ref["trainIdx"] == 0)


def test_noalloc_rejects_more_than_the_limit(gpu_lib):
    lib = gpu_lib.load()
    st = lib.akz_matcher_bfmatch_noalloc(ctypes.c_void_p(16), MAX_QUERIES + 1, ctypes.c_void_p(16), 1,
                                         ctypes.c_void_p(16), None)
    assert st == 1  # AKZ_ERR_INVALID_ARG, checked before any device work
    assert b"131072" in lib.akz_last_error()
