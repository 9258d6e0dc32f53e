"""The tensor-core matcher (tcgen05 FP8 products, akz_match_tc.cu) against
the xor + popc matcher and the CPU oracle, bit for bit: indices and
distances, ties to the lower train index, the {trainIdx 0, distance 512}
convention, sizes that are not multiples of the 128-row tiles, train splits,
rows whose pad bits are set (all 512 bits count in both engines), and the
allocation-free entry point at a size where it takes the tensor path."""
import ctypes

import numpy as np
import pytest

from akaze_gb300 import synth

pytestmark = pytest.mark.gpu


def _match(gpu_lib, q, t, tensor):
    L = gpu_lib.load()
    assert L.akz_matcher_set_tensor_cores(1 if tensor else 0) == 0
    try:
        return gpu_lib.Matcher().bfmatch(q, t)
    finally:
        L.akz_matcher_set_tensor_cores(1)


def _status(gpu_lib):
    v = ctypes.c_int(-1)
    assert gpu_lib.load().akz_matcher_tensor_status(ctypes.byref(v)) == 0
    return v.value


@pytest.mark.parametrize("nq,nt,seed", [(3000, 5000, 1), (1024, 1024, 2), (129, 8191, 3), (4097, 300, 4),
                                        (20000, 20000, 5)])
def test_tensor_matcher_equals_popc_and_oracle(gpu_lib, oracle, nq, nt, seed):
    q, t = synth.matcher_rows(seed, nq, nt)
    rng = np.random.default_rng(seed)
    k = max(1, nt // 20)
    t[rng.integers(0, nt, k)] = t[rng.integers(0, nt, k)]  # duplicated rows: forced equal distances
    tc = _match(gpu_lib, q, t, True)
    pc = _match(gpu_lib, q, t, False)
    assert tc.tobytes() == pc.tobytes()
    assert tc.tobytes() == oracle.bfmatch(q, t).tobytes()
    assert _status(gpu_lib) == 0


def test_tensor_matcher_counts_all_512_bits(gpu_lib, oracle):
    """64-byte rows with random pad bits: both engines measure all 512."""
    rng = np.random.default_rng(9)
    q = rng.integers(0, 256, (2048, 64), dtype=np.uint8)
    t = rng.integers(0, 256, (3000, 64), dtype=np.uint8)
    t[:5] = np.bitwise_not(q[:5])  # distance 512 pairs, the popc kernel's initial record
    tc = _match(gpu_lib, q, t, True)
    assert tc.tobytes() == _match(gpu_lib, q, t, False).tobytes()
    assert tc.tobytes() == oracle.bfmatch(q, t).tobytes()
    assert _status(gpu_lib) == 0


def test_tensor_matcher_largest_sweep_size_sampled(gpu_lib, oracle):
    n = 131072
    q, t = synth.matcher_rows(77, n, n)
    got = _match(gpu_lib, q, t, True)
    idx = np.sort(np.random.default_rng(3).choice(n, 2048, replace=False))
    want = oracle.bfmatch(q[idx], t)
    want["queryIdx"] = idx[:, None]
    assert got[idx].tobytes() == want.tobytes()
    assert _status(gpu_lib) == 0


def test_tensor_matcher_train_set_beyond_21_bit_columns(gpu_lib, oracle):
    """2^21 + 5 train rows: the tensor path's packed top-two words hold a
    split's column in 21 bits, so the split count must keep every split
    shorter than 2^21 rows; the nearest neighbours are planted at both ends
    and at the split boundary region."""
    nq, nt = 64, (1 << 21) + 5
    q, t = synth.matcher_rows(31, nq, nt)
    rng = np.random.default_rng(31)
    for i, j in enumerate([0, nt - 1, (1 << 20) + 3, (1 << 21) - 1]):
        t[j] = q[i]
        t[j, rng.integers(0, 61)] ^= 1  # distance 1
    tc = _match(gpu_lib, q, t, True)
    assert tc.tobytes() == _match(gpu_lib, q, t, False).tobytes()
    assert tc.tobytes() == oracle.bfmatch(q, t).tobytes()
    assert _status(gpu_lib) == 0


def test_few_train_rows_take_the_popc_kernel(gpu_lib, oracle):
    """At least 2^20 pairs but fewer than 128 train rows: the popc kernel
    answers, with the same result as the oracle."""
    q, t = synth.matcher_rows(32, 20000, 100)
    got = _match(gpu_lib, q, t, True)
    assert got.tobytes() == oracle.bfmatch(q, t).tobytes()


def test_tensor_matcher_timeout_is_reported_and_recovers(gpu_lib, oracle):
    """Failure detection without a fault: a launch whose MMA warp issues
    nothing makes the epilogue's bounded wait run out; the kernel flags it,
    frees its tensor memory and returns, and the next calls work."""
    L = gpu_lib.load()
    t = ctypes.c_int(-1)
    assert L.akz_selfcheck_matcher_timeout(1 << 12, ctypes.byref(t)) == 0
    assert t.value == 1
    assert _status(gpu_lib) == 0  # read and cleared by the self-check
    q, tr = synth.matcher_rows(41, 2048, 3000)
    assert _match(gpu_lib, q, tr, True).tobytes() == oracle.bfmatch(q, tr).tobytes()
    assert _status(gpu_lib) == 0
