"""CPU check of the streaming detector's ring schedule (k_detect_strip in
akaze_gb300/csrc/akz_detect.cu), restated step by step in Python.

The kernel walks each 256-row strip through three shared rings: Lsmooth
rows (32, filled by cp.async one block ahead), Lx/Ly rows (16) and
determinant rows (16).  Rows are formed in pairs (r, r + step) by the
warps of a block of BH rows, and block k + 1's Lx/Ly share a phase with
block k's maxima.  This test replays that schedule for steps 2..4 over
several image sizes and asserts, at every read, that the ring slot holds the
row being read (no row was overwritten early, none is missing); that no
cp.async in flight targets a slot read in the same phase; and that every
in-image pixel's Lx/Ly is written exactly once."""
import pytest

NS, ND, NE, CH = 32, 16, 16, 256


def geometry(st):
    a = (st + 2) & ~1
    tw = (127 - a - st) & ~1
    return a, tw


def block_rows(st):
    return 6 if st == 3 else 8


def pair_rows(base, st, bh):
    rows = []
    for w in range(0, bh, 2):  # even warps: the pair's first row; the odd warp takes the other column half
        q = w >> 1
        o = (q // st) * 2 * st + q % st
        rows += [base + o, base + o + st]
    assert sorted(rows) == list(range(base, base + bh))
    return rows


def replay_strip(st, W, H, tx0, ty0, written):
    a, tw = geometry(st)
    bh = block_rows(st)
    ch = min(CH, H - ty0)
    iters = (ch + bh - 1) // bh
    S, D, E = [None] * NS, [None] * ND, [None] * NE
    pending = []

    def issue(rows):
        pending.extend(rows)

    def land():
        for r in pending:
            S[r % NS] = r
        pending.clear()

    def comp_d(r):
        for rr in (r - st, r, r + st):
            assert S[rr % NS] == rr, ("S", st, rr)
            assert all(p % NS != rr % NS for p in pending), ("S slot in flight", st, rr)
        if ty0 <= r < ty0 + ch:
            for d in range(0, 128, 2):
                x = tx0 - a + d
                if a <= d < a + tw and x < W:
                    for xx in (x, x + 1):
                        if xx < W:
                            assert (r, xx) not in written
                            written.add((r, xx))
        D[r % ND] = r

    def comp_e(r):
        for rr in (r - st, r, r + st):
            assert D[rr % ND] == rr, ("D", st, rr)
        E[r % NE] = r

    def maxima(y):
        if y < ty0 + ch:
            for rr in (y - 1, y, y + 1):
                assert E[rr % NE] == rr, ("E", st, rr)

    # pre-roll
    issue(range(ty0 - 1 - 2 * st, ty0 + 2 * st + 1))
    land()
    issue(range(ty0 + 2 * st + 1, ty0 + 2 * st + 1 + bh))
    for r in range(ty0 - 1 - st, ty0 + st + 1):
        comp_d(r)
    for r in (ty0 - 1, ty0):
        comp_e(r)
    land()
    if iters > 1:
        issue(range(ty0 + 2 * st + bh + 1, ty0 + 2 * st + 2 * bh + 1))
    for r in pair_rows(ty0 + st + 1, st, bh):
        comp_d(r)
    for r in pair_rows(ty0 + 1, st, bh):
        comp_e(r)
    for k in range(iters):
        r = ty0 + bh * k
        land()
        if k + 2 < iters:
            issue(range(r + 2 * st + 2 * bh + 1, r + 2 * st + 3 * bh + 1))
        if k + 1 < iters:  # phase A: block k + 1's Lx, Ly and block k's maxima
            for rr in pair_rows(r + bh + st + 1, st, bh):
                comp_d(rr)
        for w in range(bh):
            maxima(r + w)
        if k + 1 < iters:  # phase B: block k + 1's determinant
            for rr in pair_rows(r + bh + 1, st, bh):
                comp_e(rr)
    land()


@pytest.mark.parametrize("st", [2, 3, 4])
@pytest.mark.parametrize("W,H", [(24, 20), (159, 81), (331, 257), (480, 270), (1000, 513)])
def test_strip_ring_schedule(st, W, H):
    a, tw = geometry(st)
    written = set()
    for ty0 in range(0, H, CH):
        for tx0 in range(0, W, tw):
            replay_strip(st, W, H, tx0, ty0, written)
    assert len(written) == W * H
