"""Literal emulation of the reference's round-based keypoint suppression.

Used by tests to check the oracle's sequential restatement.  It follows
src/lib/cuda_akaze.cu of the reference step by step:

  FindNeighbors (:1005-1070): for each sorted point, the earlier points of the
    same level and the points of the previous level within |size|/2;
  FilterExtrema_kernel (:1074-1224): rounds of three barrier-separated phases
    (pick the smallest-valued settled neighbour or add; per slot only the
    lowest challenger acts; compare responses and update memberarray);
  sortFiltered_kernel (:1227-1316): chunks of 2048 slots, sorted values,
    emitted when the point's size is positive.

The per-slot minimum of phase 1 is taken exactly (the reference writes it
with a plain read-modify-write).  Pure Python; for small point sets only.
"""
import numpy as np


def neighbours(px, py, size, level, level_off):
    n = len(px)
    out = []
    for i in range(n):
        s = np.float32(size[i])
        hs = np.float32(s * np.float32(0.5))
        lim = float(np.float32(s * s)) * 0.25
        l = level[i]
        nb = []
        j = i - 1
        while j >= level_off[l]:
            if np.float32(py[i] - py[j]) > hs:
                break
            d = np.float32(np.float32((px[i] - px[j]) ** 2) + np.float32((py[i] - py[j]) ** 2))
            if float(d) < lim:
                nb.append(j)
            j -= 1
        if l > 0:
            j = level_off[l] - 1
            while j >= level_off[l - 1]:
                if np.float32(py[j] - py[i]) > hs:
                    j -= 1
                    continue
                if np.float32(py[i] - py[j]) > hs:
                    break
                d = np.float32(np.float32((px[i] - px[j]) ** 2) + np.float32((py[i] - py[j]) ** 2))
                if float(d) < lim:
                    nb.append(j)
                j -= 1
        out.append(nb)
    return out


def filter_rounds(nb, response, max_rounds=10000):
    n = len(nb)
    mem = [-1] * n
    for _ in range(max_rounds):
        minnb = [n + 1] * n
        should_add = [True] * n
        any_unprocessed = False
        for i in range(n):
            if mem[i] != -1:
                continue
            any_unprocessed = True
            process = True
            for k in nb[i]:
                if mem[k] == -1:
                    process = False
                    should_add[i] = False
                    break
                if mem[k] >= 0:
                    should_add[i] = False
            if process and not should_add[i]:
                cands = [k for k in nb[i] if mem[k] >= 0]
                nidx = min(cands, key=lambda k: mem[k])
                minnb[nidx] = min(minnb[nidx], i)
        for i in range(n):
            if mem[i] == -1 and should_add[i]:
                mem[i] = i
        for i in range(n):
            c = minnb[i]
            if c != n + 1 and mem[c] == -1 and not should_add[c]:
                if response[c] > response[i]:
                    mem[c] = i
                    mem[i] = -2
                else:
                    mem[c] = -2
        if not any_unprocessed:
            break
    return mem


def emit(mem, size):
    n = len(mem)
    out = []
    for cs in range(0, n, 2048):
        vals = [mem[s] for s in range(cs, min(cs + 2048, n)) if mem[s] >= 0 and size[mem[s]] >= 0]
        out.extend(sorted(vals))
    return out


def suppress(ext, level_off):
    """ext: oracle extrema array (EXTREMUM_DTYPE). Returns (memberarray, emitted indices)."""
    ratio = (1 << ext["octave"].astype(np.int64))
    px = (ratio * ext["x"]).astype(np.float32)
    py = (ratio * ext["y"]).astype(np.float32)
    nb = neighbours(px, py, ext["size"], ext["level"], level_off)
    mem = filter_rounds(nb, ext["response"].astype(np.float32))
    return np.array(mem, np.int64), emit(mem, ext["size"])
