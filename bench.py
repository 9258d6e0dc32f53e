#!/usr/bin/env python3
"""Throughput of A-KAZE detect + M-LDB on 1920x1080 u8 images, on GB300.

Workload (one step): a batch of --batch seeded synthetic 1920x1080 images
(40 Gaussian blobs, 3 gratings, +-8 noise), default options (4 octaves x 4
sublevels, PM-g2, contrast percentile 0.7, threshold 0.001, full 486-bit
M-LDB), every stage of the path on the GPU: contrast factor, 16 levels with
their 166 FED steps, Hessian detector, extrema, suppression, orientation,
descriptors.  One graph replay per step.

  value   images/s with the input already in HBM (all ranks; replicas only)
  e2e     images/s through akz_batch_detect_describe_packed: pinned host u8
          in, host keypoints + 61-byte descriptors out (packed), copies inside
          the timing
  roofline  HBM roofline of the level (FED) stage, the dominant stage
  cpu_baseline  the CPU oracle on this host's cores (OpenMP), bounded sample

--impl reference times the reference's CPU path as restated by the oracle
(the reference itself needs OpenCV/Boost and an sm_30 toolchain; only its
fed.cpp compiles here) on the host cores, with the same metric and config.
Multi-GPU: replicas only, one process per GPU under torchrun, each rank its
own images, no collective on the data path; the max time over ranks counts.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

# Every group of the batch runs on three streams (compute, upload, result
# copy); with the driver's default number of hardware queues, streams share
# queues and the group streams wait behind one another's copies (end to end
# about 3% slower).  It must be set before the CUDA context exists.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "1080p images/s detect+MLDB, surrogate vs plain FED at fixed repeatability"
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of the 27 k_fed
# launches of one 1920x1080 image, from an ncu capture of an 8-image batch in
# the fused mode (399.3 MB read + 224.7 MB written, / 8) at a blocking depth
# of 8 FED steps per launch; the level stage's traffic per step is this times
# the batch.
FED_TRAFFIC_PER_1080P_IMAGE = 78.00e6
FED_TRAFFIC_DEPTH = 8
PEAKS_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--profile-e2e", action="store_true",
                    help="run two pipelined end-to-end steps of the headline batch (pinned host images in, "
                         "packed results out) and print the counts, for an ncu launch list of the per-run kernels")
    ap.add_argument("--profile-case", action="store_true",
                    help="small case for ncu: --batch images, one graph-less run of every stage, no timing line")
    ap.add_argument("--weights", default=os.path.join(ROOT, "akaze_gb300", "surrogate_weights.npz"),
                    help="surrogate4k: trained surrogate weights (python -m akaze_gb300.surrogate train)")
    ap.add_argument("--sg-tcgen05", type=int, default=1, choices=[0, 1],
                    help="surrogate4k: run the net's 32-channel layers on tcgen05 (1) or mma.sync (0)")
    ap.add_argument("--check-tol", type=float, default=2e-3,
                    help="surrogate4k: per-level tolerance of the surrogate against plain FED before it falls back")
    ap.add_argument("--groups", type=int, default=6,
                    help="1080p batch: images split into this many native batches on their own streams (BatchGroup)")
    ap.add_argument("--fed-depth", default=None, choices=["auto", "4", "5", "6", "7", "8"],
                    help="FED steps per level-kernel launch; auto times each depth per level on the batch first "
                         "(default: 8 for the 1080p batch, whose HBM traffic was captured at 8; auto for uneven64)")
    ap.add_argument("--workload", default="batch1080p",
                    choices=["batch1080p", "single640", "uneven64", "matcher", "surrogate4k"],
                    help="batch1080p: the headline line (default); single640: one 640x480 pair, GPU and CPU; "
                         "uneven64: 64 images of uneven sizes, images/s and per-image latency; "
                         "matcher: 2-NN sweep N=M 1024..131072, Gmatch/s against the popc roofline; "
                         "surrogate4k: 3840x2160, 6x4 levels, plain FED vs the learned surrogate")
    ap.add_argument("--matcher-n", type=int, nargs="*", default=None,
                    help="matcher: the N=M sizes to run (default 1024, 2048, ..., 131072)")
    ap.add_argument("--arith", default="fused", choices=["fused", "exact"],
                    help="1080p batch: arithmetic of the scale-space and detector kernels (akz_options.fast_math): "
                         "fused multiply-adds within the specification's tolerances (default), or the reference's "
                         "operation order, bit-identical to the CPU restatement; the other mode's device-resident "
                         "throughput is reported beside the headline")
    return ap.parse_args()


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return PEAKS_FALLBACK, "fallback"


def level_sizes(w, h, omax=4, nsub=4):
    out = []
    for i in range(omax):
        lw, lh = int(w / 2 ** i), int(h / 2 ** i)
        if (lw < 80 or lh < 40) and i:
            break
        out += [(lw, lh)] * nsub
    return out


def fed_algorithmic_bytes(w, h):
    """Compulsory HBM bytes of the level stage per image: for every level
    >= 1, read the predecessor level (4 B/px of its size), write the evolved
    level (4 B/px) and write its pre-diffusion smoothing Lsmooth (4 B/px),
    which the stage produces for the detector."""
    L = level_sizes(w, h)
    return sum(4 * L[i - 1][0] * L[i - 1][1] + 8 * L[i][0] * L[i][1] for i in range(1, len(L)))


def image_algorithmic_bytes(w, h, nkp):
    """Whole-pipeline compulsory bytes per image: u8 read twice (contrast and
    level 0) + per level: write Lt, read the predecessor, re-read the
    pre-diffusion smoothing for the detector, write Lx and Ly; + 5384 B per
    keypoint (441 samples x 3 planes x 4 B, a 64 B row and a 28 B record)."""
    L = level_sizes(w, h)
    b = 2 * w * h
    for i, (lw, lh) in enumerate(L):
        p = lw * lh
        b += 4 * p + (4 * L[i - 1][0] * L[i - 1][1] if i else 0) + 4 * p + 8 * p
    return b + 5384 * nkp


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_oracle_rate(w, h, seconds, seed=900, threads=None, max_runs=50):
    """Images/s of the CPU oracle on a bounded sample (all host cores unless
    threads is given)."""
    from akaze_gb300 import synth
    from oracle import oracle_ctypes as oc
    oc.build()
    cores = threads or os.cpu_count() or 1
    oc.set_threads(cores)
    img = synth.synth_image(seed, w, h)
    o = oc.Oracle(w, h)
    o.run(img)  # warm-up
    n, t0 = 0, time.perf_counter()
    while True:
        o.run(img)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds or n >= max_runs:
            break
    oc.set_threads(os.cpu_count() or 1)
    return n / el, cores, f"{n} runs of one {w}x{h} synthetic image, {cores} OpenMP threads, {el:.1f} s"


def run_reference(args):
    ws, rank, _ = dist_setup(args)
    if rank != 0:
        return 0
    from akaze_gb300 import synth  # noqa: F401
    from oracle import oracle_ctypes as oc
    oc.build()
    cores = os.cpu_count() or 1
    oc.set_threads(cores)
    w, h = args.width, args.height
    o = oc.Oracle(w, h)
    from akaze_gb300 import synth as sy
    imgs = [sy.synth_image(1000 + i, w, h) for i in range(min(4, args.steps + args.warmup))]
    for k in range(args.warmup):
        o.run(imgs[k % len(imgs)])
    t0 = time.perf_counter()
    for k in range(args.steps):
        o.run(imgs[k % len(imgs)])
    el = time.perf_counter() - t0
    v = args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "images/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"plain A-KAZE detect+MLDB, {w}x{h} u8, 4 octaves x 4 sublevels, one image per step",
                   "images_per_step": 1},
        "cpu_baseline": {"value": v, "unit": "images/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} images of {w}x{h}, one per step, {cores} OpenMP threads"},
        "e2e": {"value": v, "unit": "images/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": ("the reference's own sources need OpenCV, Boost.Python and sm_30 (no build here); this arm times "
                 "the CPU restatement of its path (oracle/), whose FED schedule is pinned to its fed.cpp"),
    }
    print(json.dumps(line))
    return 0


def _torch_stream():
    import torch
    torch.cuda.set_device(0)
    return torch, torch.cuda.Stream()


def _event_ms(torch, stream, fn, reps):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def nndr_inliers(kp1, kp2, matches, Hm, ratio=0.8, px=2.5):
    """NNDR matches and homography inliers (akaze_match.cpp:35-36, utils.cpp:154-243)."""
    from akaze_gb300 import synth
    if len(matches) == 0:
        return 0, 0
    d1, d2 = matches[:, 0]["distance"], matches[:, 1]["distance"]
    good = d1 < ratio * d2
    qi, ti = matches[good, 0]["queryIdx"], matches[good, 0]["trainIdx"]
    x, y = synth._apply(Hm, kp1["x"][qi].astype(np.float64), kp1["y"][qi].astype(np.float64))
    err = np.hypot(x - kp2["x"][ti], y - kp2["y"][ti])
    return int(good.sum()), int((err < px).sum())


def workload_single640(args):
    """One 640x480 pair through the reference's class API on the GPU, next to
    the CPU oracle on one thread and on all host cores."""
    torch, stream = _torch_stream()
    import akaze_gb300 as akz
    from akaze_gb300 import synth
    W, H = 640, 480
    img1, img2, Hm = synth.synth_pair(11, W, H)
    o = akz.AKAZEOptions()
    o.setWidth(W)
    o.setHeight(H)
    ak = akz.AKAZE(o)
    ak.set_stream(stream.cuda_stream)
    res = [ak.detect_and_compute(im) for im in (img1, img2)]
    reps = max(args.steps, 10)
    t0 = time.perf_counter()
    for _ in range(reps):
        ak.detect_and_compute(img1)
    api_ms = 1000 * (time.perf_counter() - t0) / reps
    b = akz.Batch(akz.AKAZEOptions(), [(W, H)])
    b.set_stream(stream.cuda_stream)
    b.upload([img1])
    for _ in range(max(args.warmup, 3)):
        b.run()
    dev_ms = _event_ms(torch, stream, b.run, reps)
    m = akz.Matcher()
    (k1, d1), (k2, d2) = res
    matches = m.bfmatch(d1, d2)
    t0 = time.perf_counter()
    for _ in range(reps):
        m.bfmatch(d1, d2)
    match_ms = 1000 * (time.perf_counter() - t0) / reps
    nn, inl = nndr_inliers(k1, k2, matches, Hm)
    cpu_all, cores, _ = cpu_oracle_rate(W, H, 3.0, seed=11)
    cpu_one, _, _ = cpu_oracle_rate(W, H, 3.0, seed=11, threads=1, max_runs=20)
    print(json.dumps({
        "workload": "single640", "config": "640x480 u8 pair, default options, full M-LDB, 2-NN match",
        "gpu_ms_per_image_device": dev_ms, "gpu_ms_per_image_class_api": api_ms, "match_ms_host_api": match_ms,
        "keypoints": [int(len(k1)), int(len(k2))], "nndr_matches": nn, "homography_inliers": inl,
        "cpu_ms_per_image": {"threads_%d" % cores: 1000.0 / cpu_all, "threads_1": 1000.0 / cpu_one},
        "speedup_device_vs_cpu_all_cores": (1000.0 / cpu_all) / dev_ms,
    }))
    return 0


def _pick_fed_depth(batch, args, default):
    """FED blocking depth per level: the autotuner's picks (timed on the
    uploaded batch) or the one asked for."""
    depth = args.fed_depth or default
    if depth == "auto" and hasattr(batch, "parts"):
        d, ms = batch.autotune()[0]
        return d, {str(k): round(v, 4) for k, v in ms.items()}
    if depth == "auto":
        d, ms = batch.autotune()
        return d, {str(k): round(v, 4) for k, v in ms.items()}
    batch.set_fed_depth(int(depth))
    return [int(depth)], None


def _group_event_ms(torch, stream, gstreams, fn, steps):
    """ms per call of fn, whose work runs on gstreams, timed with events on
    stream that bracket every group stream."""
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for g in gstreams:
        g.wait_event(e0)
    for _ in range(steps):
        fn()
    for g in gstreams:
        stream.wait_stream(g)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def workload_uneven64(args):
    """64 images of uneven sizes, split into stream groups of graph-replayed
    batches (images/s), and each image alone (per-image latency, p50/p99)."""
    torch, stream = _torch_stream()
    import akaze_gb300 as akz
    from akaze_gb300 import synth
    sizes = synth.uneven_sizes(2024, 64)
    imgs = [synth.synth_image(3000 + i, w, h) for i, (w, h) in enumerate(sizes)]
    opt = akz.AKAZEOptions()
    b = akz.BatchGroup(opt, sizes, groups=args.groups)
    gstreams = [torch.cuda.Stream() for _ in b.parts]
    b.set_streams([g.cuda_stream for g in gstreams])
    b.upload(imgs)
    fed_depth, depth_ms = _pick_fed_depth(b, args, "auto")
    for _ in range(max(args.warmup, 3)):
        b.run()
    step_ms = _group_event_ms(torch, stream, gstreams, b.run, args.steps)
    counts = b.counts()
    singles = []
    for (w, h), im in zip(sizes, imgs):
        s1 = akz.Batch(opt, [(w, h)])
        s1.set_stream(stream.cuda_stream)
        s1.upload([im])
        for _ in range(3):
            s1.run()
        singles.append(_event_ms(torch, stream, s1.run, 5))
        s1.close()
    lat = np.array(singles)
    mpix = sum(w * h for w, h in sizes) / 1e6
    print(json.dumps({
        "workload": "uneven64", "config": "64 synthetic images, W~U[320,1920], H~U[240,1080], multiples of 8",
        "groups": len(b.parts),
        "images_per_s": 64 * 1000.0 / step_ms, "batch_ms": step_ms, "megapixels_per_batch": mpix,
        "latency_ms_alone": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                             "min": float(lat.min()), "max": float(lat.max())},
        "latency_ms_in_batch": step_ms, "keypoints_total": int(sum(counts)),
        "fed_depth_per_level": fed_depth, "level_stage_ms_by_depth": depth_ms,
    }))
    return 0


def workload_matcher(args):
    """2-NN Hamming sweep N=M in 1024..131072 with both pair-distance engines:
    tcgen05 FP8 products (the default for >= 2^20 pairs), against twice the
    measured bf16 tensor peak (the FP8 dense rate is not measured here), and
    xor + popc, against the popc rate measured in the same run.  Each size's
    two results are compared with each other, and the top-2 of 256 sampled
    queries against numpy."""
    torch, stream = _torch_stream()
    import ctypes
    import akaze_gb300 as akz
    from akaze_gb300 import synth
    lib = akz._lib.load()
    rate = ctypes.c_double(0)
    akz._lib.check(lib.akz_measure_popc_rate(2000, ctypes.byref(rate), ctypes.c_void_p(stream.cuda_stream)))
    peak_pairs = rate.value / 16.0
    pk, pk_kind = peaks()
    fp8_peak = 2.0 * pk["bf16_tflops"] * 1e12  # FLOP/s; one pair = 2 x 512 FLOP of the K = 512 product
    m = akz.Matcher()
    m.set_stream(stream.cuda_stream)
    rows = []
    sizes = args.matcher_n or [1024 << k for k in range(8)]
    for N in sizes:
        k = max(0, int(N).bit_length() - 11)
        q61, t61 = synth.matcher_rows(5000 + k, N, N)
        q64 = np.zeros((N, 64), np.uint8)
        t64 = np.zeros((N, 64), np.uint8)
        q64[:, :61], t64[:, :61] = q61, t61
        qd, td = torch.from_numpy(q64).cuda(), torch.from_numpy(t64).cuda()
        res_by = {}
        row = {"N": N}
        for engine, on in (("tensor", 1), ("popc", 0)):
            akz._lib.check(lib.akz_matcher_set_tensor_cores(on))
            out = torch.empty((N, 2, 4), dtype=torch.int32, device="cuda")
            fn = lambda: m.bfmatch_device(qd.data_ptr(), N, td.data_ptr(), N, out.data_ptr())
            for _ in range(2):
                fn()
            reps = max(3, min(50, int(2e10 / (N * N)) * (4 if on else 1)))
            ms = _event_ms(torch, stream, fn, reps)
            res_by[engine] = out.cpu().numpy()
            pairs = N * N / (ms / 1000.0)
            row[engine] = {"ms": ms, "gmatch_per_s": pairs / 1e9}
            if on:
                row[engine]["frac_fp8_tensor_peak"] = pairs * 1024 / fp8_peak
                row[engine]["tensor_path"] = N * N >= (1 << 20) and N >= 128
            else:
                row[engine]["frac_popc_roofline"] = pairs / peak_pairs
        akz._lib.check(lib.akz_matcher_set_tensor_cores(1))
        res = res_by["tensor"]
        resf = res.view(np.float32)
        rng = np.random.default_rng(k)
        sample = rng.choice(N, min(256, N), replace=False)
        ok = True
        for i in sample:
            d = np.bitwise_count(np.bitwise_xor(t64, q64[i]).view(np.uint64)).sum(axis=1)
            order = np.lexsort((np.arange(N), d))
            want = [(int(order[0]), int(d[order[0]])), (int(order[1]), int(d[order[1]]))]
            got = [(int(res[i, j, 1]), int(resf[i, j, 3])) for j in range(2)]
            ok &= want == got
        row["engines_identical"] = bool(np.array_equal(res_by["tensor"], res_by["popc"]))
        row["sample_exact"] = bool(ok)
        rows.append(row)
    print(json.dumps({"workload": "matcher", "config": "N=M rows of 486 Bernoulli(0.5) bits in 64 B, 30% planted "
                      "copies with 5% bit flips", "popc_triples_per_s": rate.value,
                      "peak_gmatch_per_s_popc": peak_pairs / 1e9,
                      "peak_gmatch_per_s_fp8": fp8_peak / 1024 / 1e9,
                      "fp8_peak_kind": "2 x %s bf16_tflops (dense FP8 rate not measured)" % pk_kind,
                      "sweep": rows}))
    return 0


def repeatability(kp_ref, d_ref, kp, d, px=0.5):
    """Fraction of reference keypoints with a keypoint at the same level
    (class_id) within px, and the Hamming distances of those pairs'
    descriptors."""
    hits, ham = 0, []
    for c in np.unique(kp_ref["class_id"]):
        ri = np.nonzero(kp_ref["class_id"] == c)[0]
        si = np.nonzero(kp["class_id"] == c)[0]
        if len(si) == 0:
            continue
        order = si[np.argsort(kp["x"][si])]
        xs = kp["x"][order]
        for r in ri:
            lo, hi = np.searchsorted(xs, kp_ref["x"][r] - px), np.searchsorted(xs, kp_ref["x"][r] + px, side="right")
            cand = order[lo:hi]
            if len(cand) == 0:
                continue
            dd = np.hypot(kp["x"][cand] - kp_ref["x"][r], kp["y"][cand] - kp_ref["y"][r])
            j = int(np.argmin(dd))
            if dd[j] <= px:
                hits += 1
                ham.append(int(np.unpackbits(d_ref[r] ^ d[cand[j]]).sum()))
    n = len(kp_ref)
    ham = np.array(ham) if ham else np.zeros(0)
    return {"repeatability": hits / n if n else 1.0, "matched": hits, "reference": n,
            "hamming_mean": float(ham.mean()) if ham.size else 0.0,
            "hamming_le2": float((ham <= 2).mean()) if ham.size else 1.0}


def workload_surrogate4k(args):
    """3840x2160 with 6 octaves x 4 sublevels: plain FED, the learned
    surrogate for octaves >= 1 alone, and with its per-level check against
    plain FED on image 0 and fallback."""
    torch, stream = _torch_stream()
    import akaze_gb300 as akz
    from akaze_gb300 import surrogate as sg
    from akaze_gb300 import synth
    if not os.path.exists(args.weights):
        print(json.dumps({"workload": "surrogate4k", "unavailable": f"no trained weights at {args.weights}"}))
        return 0
    params = sg.load_params(args.weights)
    akz._lib.check(akz._lib.load().akz_sg_set_tcgen05(args.sg_tcgen05))
    W, H, B = 3840, 2160, min(args.batch, 8)
    imgs = [synth.synth_image(9000 + i, W, H) for i in range(B)]
    opt = akz.AKAZEOptions(omax=6)
    res = {}
    for mode, tol in (("plain", None), ("surrogate", 0.0), ("surrogate_checked", args.check_tol)):
        b = akz.Batch(opt, [(W, H)] * B)
        b.set_stream(stream.cuda_stream)
        b.upload(imgs)
        if tol is not None:
            b.set_surrogate(params, first_octave=1, check_tol=tol)
        for _ in range(max(args.warmup, 3)):
            b.run()
        ms = _event_ms(torch, stream, b.run, max(3, min(args.steps, 10)))
        out = {"ms_per_batch": ms, "images_per_s": B * 1000.0 / ms, "stage_ms": [float(x) for x in b.profile()],
               "results": [b.results(i) for i in range(B)]}
        if tol is None:
            sizes = [(int(W / 2 ** o), int(H / 2 ** o)) for o in range(6) for _ in range(4)]
            out["level_max_abs_image0"] = [float(np.abs(b.plane(0, l, shape=(h, w))).max()) for l, (w, h) in enumerate(sizes)]
        if tol:
            e = b.surrogate_errors()
            out["level_max_err_image0"] = [float(x) for x in e]
            out["levels_fallen_back"] = int(np.sum(~(e <= tol)))
        res[mode] = out
        b.close()
    line = {"workload": "surrogate4k", "config": f"{B} synthetic 3840x2160 u8, 6 octaves x 4 sublevels, surrogate on "
            "octaves >= 1 (BF16 tensor-core net, 5 layers x 32 channels)", "check_tol": args.check_tol,
            "tensor_path": "tcgen05" if args.sg_tcgen05 else "mma.sync"}
    for mode, out in res.items():
        r = {k: v for k, v in out.items() if k != "results"}
        if mode != "plain":
            for tag, lim in (("", 24), ("_octaves0to4", 20)):
                reps = []
                for i in range(B):
                    (kr, dr), (k, d) = res["plain"]["results"][i], out["results"][i]
                    mr, m = kr["class_id"] < lim, k["class_id"] < lim
                    reps.append(repeatability(kr[mr], dr[mr], k[m], d[m]))
                r["repeatability" + tag] = float(np.mean([x["repeatability"] for x in reps]))
                r["hamming_mean" + tag] = float(np.mean([x["hamming_mean"] for x in reps]))
                r["hamming_le2" + tag] = float(np.mean([x["hamming_le2"] for x in reps]))
            r["speedup_vs_plain"] = res["plain"]["ms_per_batch"] / out["ms_per_batch"]
        r["keypoints"] = [int(len(k)) for k, _ in out["results"]]
        line[mode] = r
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "batch1080p":
        return {"single640": workload_single640, "uneven64": workload_uneven64, "matcher": workload_matcher,
                "surrogate4k": workload_surrogate4k}[args.workload](args)
    ws, rank, local = dist_setup(args)
    import torch
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import akaze_gb300 as akz
    from akaze_gb300 import replicas, synth

    B, W, H = args.batch, args.width, args.height
    imgs = [synth.synth_image(s, W, H) for s in replicas.rank_seeds(rank, B)]
    opt = akz.AKAZEOptions(fast_math=1 if args.arith == "fused" else 0)
    if args.profile_e2e:
        batch = akz.BatchGroup(opt, [(W, H)] * B, groups=args.groups)
        _pick_fed_depth(batch, args, "8")
        pin = [torch.empty((H, W), dtype=torch.uint8).pin_memory() for _ in range(B)]
        for pp, im in zip(pin, imgs):
            pp.numpy()[:] = im
        cap = B * 20000
        kp_out = torch.empty(cap * 28, dtype=torch.uint8).pin_memory().numpy().view(akz.KEYPOINT_DTYPE)
        d_out = torch.empty(cap * 61, dtype=torch.uint8).pin_memory().numpy().reshape(cap, 61)
        c = batch.detect_describe_packed_steps([[pp.numpy() for pp in pin]] * 2, kp_out, d_out)
        print(json.dumps({"profile_e2e": f"{B} x {W}x{H}, {len(batch.parts)} groups, 2 steps",
                          "keypoints": int(c.sum())}))
        return 0
    if args.profile_case:
        batch = akz.Batch(opt, [(W, H)] * B)
        batch.upload(imgs)
        _pick_fed_depth(batch, args, "8")
        torch.cuda.synchronize()
        ms = batch.profile()
        print(json.dumps({"profile_case": f"{B} x {W}x{H}", "stage_ms": [float(x) for x in ms],
                          "keypoints": [int(c) for c in batch.counts()]}))
        return 0
    batch = akz.BatchGroup(opt, [(W, H)] * B, groups=args.groups)
    stream = torch.cuda.Stream()
    gstreams = [torch.cuda.Stream() for _ in batch.parts]
    batch.set_streams([g.cuda_stream for g in gstreams])
    batch.upload(imgs)
    fed_depth, depth_ms = _pick_fed_depth(batch, args, "8")
    torch.cuda.synchronize()

    # device-resident throughput: every group stream starts after e0, e1 after all of them
    for _ in range(max(args.warmup, 3)):
        batch.run()
    counts = batch.counts()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    sampler = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for g in gstreams:
        g.wait_event(e0)
    for _ in range(args.steps):
        batch.run()
    for g in gstreams:
        stream.wait_stream(g)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop() if sampler else None
    ms_max = replicas.max_over_ranks(e0.elapsed_time(e1), dist, device="cuda")
    value = replicas.job_throughput(B * args.steps, ws, ms_max / 1000.0)

    # the other arithmetic mode, same images and timing (reported beside the headline)
    other = akz.BatchGroup(akz.AKAZEOptions(fast_math=0 if args.arith == "fused" else 1), [(W, H)] * B,
                           groups=args.groups)
    other.set_streams([g.cuda_stream for g in gstreams])
    other.upload(imgs)
    other.set_fed_depth(int(fed_depth[0]) if fed_depth and fed_depth[0] else 8)
    for _ in range(max(args.warmup, 3)):
        other.run()
    torch.cuda.synchronize()
    e0.record(stream)
    for g in gstreams:
        g.wait_event(e0)
    for _ in range(args.steps):
        other.run()
    for g in gstreams:
        stream.wait_stream(g)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_other = replicas.max_over_ranks(e0.elapsed_time(e1), dist, device="cuda")
    value_other = replicas.job_throughput(B * args.steps, ws, ms_other / 1000.0)
    other.close()

    # stage profile for the roofline of the level stage: one non-graph run of
    # all B images as one batch (every k_fed launch then covers all images,
    # as the level stage of the timed step does across its concurrent groups)
    whole = akz.Batch(opt, [(W, H)] * B)
    whole.upload(imgs)
    whole.set_fed_depth(int(fed_depth[0]) if fed_depth and fed_depth[0] else 8)
    stage = [float(x) for x in whole.profile()]
    stage = [min(a, float(x)) for a, x in zip(stage, whole.profile())]
    whole.close()
    fed_ms = stage[2]
    fed_bytes = fed_algorithmic_bytes(W, H) * B
    pk, pk_kind = peaks()
    achieved = fed_bytes / (fed_ms / 1000.0) / 1e9
    n_launch = sum(b.kernel_count() for b in batch.parts)

    # end to end through the C ABI: pinned host u8 in, host results out
    pin_in = [torch.empty((H, W), dtype=torch.uint8).pin_memory() for _ in range(B)]
    for p, im in zip(pin_in, imgs):
        p.numpy()[:] = im
    cap = int(sum(counts)) + 1024
    kp_out = torch.empty(cap * 28, dtype=torch.uint8).pin_memory().numpy().view(akz.KEYPOINT_DTYPE)
    d_out = torch.empty(cap * 61, dtype=torch.uint8).pin_memory().numpy().reshape(cap, 61)
    np_in = [p.numpy() for p in pin_in]
    for _ in range(2):
        c2 = batch.detect_describe_packed(np_in, kp_out, d_out)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    e_steps = max(1, min(args.steps, 20))
    # consecutive steps pipelined per group: a group's next upload starts once its
    # results are read back, while the other groups still compute
    c2 = batch.detect_describe_packed_steps([np_in] * e_steps, kp_out, d_out)
    el = replicas.max_over_ranks(time.perf_counter() - t0, dist, device="cuda")
    e2e = replicas.job_throughput(B * e_steps, ws, el)
    h2d = B * W * H
    d2h = int(sum(c2)) * (28 + 61) + B * 32

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    cpu_v, cores, sample = cpu_oracle_rate(W, H, args.cpu_seconds)
    cpu_1, _, sample_1 = cpu_oracle_rate(W, H, min(args.cpu_seconds, 6.0), threads=1, max_runs=5)
    nkp = float(np.mean(counts))
    line = {
        "metric": METRIC, "value": value, "unit": "images/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"plain A-KAZE detect+MLDB, {W}x{H} u8, 4 octaves x 4 sublevels, default options",
                   "fed": "plain (the learned surrogate is built but 2.6x slower at 4K on this GPU: --workload surrogate4k)",
                   "images_per_step_per_gpu": B, "parallelism": f"replicas x{ws}",
                   "groups": "%d native batches of %s images, one stream and graph each"
                             % (len(batch.parts), "/".join(str(b.n) for b in batch.parts)),
                   "l2": "inputs and working set larger than L2 (~%.1f GB per step)" % (B * image_algorithmic_bytes(W, H, 0) / 1e9),
                   "keypoints_per_image": nkp,
                   "fed_depth_per_level": fed_depth, "level_stage_ms_by_depth": depth_ms,
                   "arith": ("fused: fast_math=1, FMA and the hardware reciprocal in the scale-space and detector "
                             "kernels, tested to levels 1e-4 relative, >=99% keypoints within 0.5 px, >=99% "
                             "descriptors within Hamming 2" if args.arith == "fused" else
                             "exact: fast_math=0, bit-identical to the CPU restatement of the reference")},
        "value_other_arith": {"arith": "exact" if args.arith == "fused" else "fused", "value": value_other,
                              "unit": "images/s", "ms_per_step": ms_other / args.steps},
        "roofline": {"bound": "hbm", "kernel": ("k_fed (level stage: 15 levels, 166 FED steps; its event-timed "
                                                "stage time on one %d-image batch, arith %s)" % (B, args.arith)),
                     "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"],
                     "traffic": (FED_TRAFFIC_PER_1080P_IMAGE * B
                                 if (W, H) == (1920, 1080) and set(fed_depth) == {FED_TRAFFIC_DEPTH} else None),
                     "traffic_note": "ncu DRAM bytes of the level stage, 8-image capture scaled to the batch",
                     "algorithmic_bytes_per_image": fed_algorithmic_bytes(W, H), "launch_ms": fed_ms,
                     "peak_kind": f"{pk_kind} hbm_gbs"},
        "pipeline_roofline": {"achieved": image_algorithmic_bytes(W, H, nkp) * value / 1e9,
                              "frac": image_algorithmic_bytes(W, H, nkp) * value / 1e9 / pk["hbm_gbs"],
                              "bytes_per_image": image_algorithmic_bytes(W, H, nkp)},
        "stage_ms": dict(zip(["contrast", "level0", "levels", "detector", "scan_extract", "suppression", "describe"], stage)),
        "cpu_baseline": {"value": cpu_v, "unit": "images/s", "cores": cores, "kind": "port", "sample": sample,
                         "single_thread": {"value": cpu_1, "sample": sample_1}},
        "e2e": {"value": e2e, "unit": "images/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": n_launch * args.steps,
        "clocks": clocks,
    }
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
