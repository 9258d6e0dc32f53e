"""The M-LDB comparison tables of the descriptor modes, on the CPU.

- The oracle's restatement of the GNU C library's rand() (which the
  reference's generateDescriptorSubsample draws from after srand(1024),
  AKAZE.cpp:535) gives libc's own sequence.
- The full 3-channel table is the reference's 486-pair order
  (InitCompareIndices, cuda_akaze.cu:2034-2111, as the oracle states it).
- The 1- and 2-channel tables keep the full table's per-grid, per-channel
  pair order with fewer channels (AKAZE.cpp:412-418).
- The random-bit subsets (AKAZE.cpp:498-603) force the 2x2 grid's 6 pairs
  first, compare equal channels of two cells of one grid, and are prefixes
  of each other for the same channel count (one draw sequence).
"""
import ctypes

import numpy as np
import pytest


def test_glibc_rand_restatement_equals_libc(oracle):
    try:
        libc = ctypes.CDLL("libc.so.6")
    except OSError:
        pytest.skip("no GNU C library")
    for seed in (1024, 1, 7, 123456789):
        libc.srand(seed)
        want = [libc.rand() for _ in range(3000)]
        assert list(oracle.glibc_rand_sequence(seed, 3000)) == want, seed


def test_full_tables(oracle):
    c1, c2 = oracle.mldb_table(3, 0)
    i1 = np.zeros(486, np.int32)
    i2 = np.zeros(486, np.int32)
    assert oracle.lib().ako_descriptor_pairs(i1.ctypes.data, i2.ctypes.data) == 486
    assert np.array_equal(c1, i1) and np.array_equal(c2, i2)
    for ch in (1, 2):
        d1, d2 = oracle.mldb_table(ch, 0)
        assert len(d1) == 162 * ch
        keep = (c1 % 3) < ch  # the 3-channel order with the other channels dropped
        assert np.array_equal(d1, c1[keep]) and np.array_equal(d2, c2[keep])


def _grid(cell):
    return np.where(cell < 4, 0, np.where(cell < 13, 1, 2))


@pytest.mark.parametrize("channels", [1, 2, 3])
def test_subset_tables(oracle, channels):
    full = 162 * channels
    c1, c2 = oracle.mldb_table(channels, full)
    assert len(c1) == full
    assert np.all(c1 % 3 == c2 % 3) and np.all(c1 % 3 < channels)  # same channel, within the count
    assert np.all(_grid(c1 // 3) == _grid(c2 // 3)) and np.all(c1 != c2)  # two cells of one grid
    # the first 6 picks are the 2x2 grid's pairs in order, each cell listed
    # in the subset's column-major order (row j % 2, column j // 2)
    first = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    col_major = {0: 0, 1: 2, 2: 1, 3: 3}
    for i, (a, b) in enumerate(first):
        for ch in range(channels):
            k = i * channels + ch
            if k < full:
                assert (c1[k], c2[k]) == (3 * col_major[a] + ch, 3 * col_major[b] + ch), (i, ch)
    for n in (1, 7, 64, 100):
        s1, s2 = oracle.mldb_table(channels, n)
        assert np.array_equal(s1, c1[:n]) and np.array_equal(s2, c2[:n])
    # a full-size subset uses every pair of every grid once per channel
    pairs = {(min(a, b), max(a, b)) for a, b in zip(c1 // 3, c2 // 3)}
    assert len(pairs) == 162
