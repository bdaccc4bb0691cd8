"""Benchmark: Lloyd k-means iterations/s on one GB300 (headline), with the
kNN self-joins, serving and batched k-means alongside.

Workload (one "step" = one complete Lloyd k-means call): n=70,000, d=784,
k=64, each coordinate 0 with probability 0.8 else U{1..255}/255 (synthetic
stand-in for MNIST), init = 64 seeded distinct rows, 100 fixed iterations.
The input matrix (219.5 MB) is larger than the 129 MB L2, so no explicit L2
flush is needed between steps.

Beside it (same JSON line): the plain kNN self-join (n=20,000, d=16, k=10),
the tensor-core kNN self-join (n=1,000,000, d=128, k=100, integer data) with
its plain FP32 CUDA-core rate on a query subset, kNN serving (2,000,000 x 96
resident index, Poisson arrivals) and 512 batched k-means problems.  After the
timed regions every leg is checked against the oracle at its benchmarked size
(``parity``): the full Lloyd runs (fixed 100 iterations and the converging
run) against the exact-mean oracle and fuel's own f32-sum Lloyd, sampled rows
of the 10^6-point self-join and of the served requests against the oracle's
tie-inclusive lists, and the whole 20,000-point self-join; the FP64 error of
the returned distances and the near-ties / FP64 order flips are reported per
kNN leg (``fp64``).

Run: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun (N>1) each rank runs an independent replica ("replicas only";
the path is a single-device engine) and rank 0 prints one JSON line.
--quick skips the side legs and the parity checks (the headline only).

python bench.py --profile lloyd|knn_tc|knn_plain|serving|batched [--steps K] [--warmup W]
runs one workload alone (no CPU baseline, no side legs) for profiler
captures; --knn-queries sets the query count of the kNN workloads there.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "k-means Lloyd iters/s & kNN queries/s: TC+refine vs plain FP32, 1 GB300; p99"
N, D, K, ITERS = 70_000, 784, 64, 100
REF_SAMPLE_ITERS = 10    # Lloyd iterations per reference-arm step (about 1 s of CPU work)
CPU_SAMPLE_ITERS = 100   # iterations of the CPU baseline leg (one full step, about 10 s)
KNN_N, KNN_D, KNN_K = 1_000_000, 128, 100
KNN_PLAIN_QUERIES = 20_000  # plain FP32 tier on a query subset (about 0.6 s)
BATCH_PROBLEMS, BATCH_ITERS = 512, 20  # batched k-means: problems, fixed iterations
SERVE_N, SERVE_D, SERVE_RATE = 2_000_000, 96, 2000.0  # resident index rows, dims, requests/s
SERVE_SECONDS = {"fp16": 30.0, "split_bf16": 5.0}      # seconds of Poisson arrivals per tensor-core tier
SERVE_PLAIN_RATE, SERVE_PLAIN_SECONDS = 40.0, 10.0     # the plain tier at a rate it can sustain
PARITY_KNN_ROWS = 256        # sampled self-join rows checked against the oracle's tie-inclusive lists
PARITY_SERVE_ROWS = 256      # sampled served query rows checked against the oracle
CPU_KNN_TC_QUERIES = 1000    # CPU baseline sample of the 10^6-point self-join
CPU_SERVE_QUERIES = 512      # CPU baseline sample of the serving queries


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "_fallback": True}


def host_threads():
    return os.cpu_count() or 1


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_lloyd_sample(X, init, iters, threads):
    """fuel's CPU Lloyd (restated, f32 running sums, host summation order) on
    the full matrix for at most `iters` iterations; returns (seconds,
    iterations run).  fuel counts the initial assignment as iteration 1."""
    from oracle import oracle
    t0 = time.perf_counter()
    _, _, it, _ = oracle.lloyd(X, K, init, max_iter=iters, order=oracle.host_order(), threads=threads)
    return time.perf_counter() - t0, it


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    from fuel_gb300 import workloads
    from oracle import oracle
    oracle.build()
    X, init = workloads.lloyd_sparse(N, D, K)
    threads = host_threads()
    sample_iters = REF_SAMPLE_ITERS
    for _ in range(args.warmup):
        cpu_lloyd_sample(X, init, sample_iters, threads)
    runs = [cpu_lloyd_sample(X, init, sample_iters, threads) for _ in range(args.steps)]
    tot = sum(t for t, _ in runs)
    value = sum(it for _, it in runs) / tot
    times = runs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "iters/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"lloyd k={K} n={N} d={D}", "n": N, "d": D, "k": K,
                   "sample": f"{sample_iters} Lloyd iterations of the full matrix per step"},
        "cpu_baseline": {"value": value, "unit": "iters/s", "cores": threads, "kind": "port",
                         "sample": f"{sample_iters} iterations x {args.steps} steps, restated fuel CPU Lloyd "
                                   f"(f32 running sums, {oracle.host_order()} summation order)"},
        "e2e": {"value": value, "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# FP32 issue rate (the plain tiers' roofline denominator) and lane-op counts
# ---------------------------------------------------------------------------

_FP32_RATE = None


def fp32_rate(lib, _lib):
    """Measured FP32 FMA issue rate of this GPU, 10^12 lane-ops/s (fuelg_fp32_rate)."""
    global _FP32_RATE
    if _FP32_RATE is None:
        r = ctypes.c_double()
        _lib.check(lib.fuelg_fp32_rate(ctypes.byref(r)))
        _FP32_RATE = r.value
    return _FP32_RATE


def lane_ops_per_eval(d, order):
    """FP32 lane operations of one exact distance in fuel's order: 'arm' (unroll.rs
    8-lane sub, mul, add per coordinate) = 3d; 'x86' (AVX2: sub + FMA per coordinate)
    = 2d.  The lane folds and the tail are left out (a lower bound of the work)."""
    return (3 if order == "arm" else 2) * d


def plain_roofline(lib, _lib, evals, d, kernel_ms, kernel):
    peak = fp32_rate(lib, _lib)
    ops = evals * lane_ops_per_eval(d, _lib.default_order())
    ach = ops / (kernel_ms / 1e3) / 1e12
    return {"bound": "fp32", "achieved": ach, "peak": peak, "unit": "Tlane-op/s", "frac": ach / peak,
            "kernel": kernel, "lane_ops_per_eval": lane_ops_per_eval(d, _lib.default_order()),
            "peak_source": "measured (fuelg_fp32_rate: FMA chains, CUDA events, this run)"}


# ---------------------------------------------------------------------------
# parity against the oracle at the benchmarked sizes
# ---------------------------------------------------------------------------

def lloyd_parity(lib, _lib, X, init, gpu_fixed, threads):
    """Config 2 at full size.  gpu_fixed = (centres, labels, iterations, inertia)
    of a 100-fixed-iteration GPU call.  Checks: (a) that run against the
    exact-mean oracle (labels, centre bits, iteration count, inertia within
    1e-7 of its FP64 value); (b) the converging run (fuel's changed == 0 stop,
    max_iter 300) the same way; (c) fuel's own f32-sum Lloyd at this host's
    thread count (the restated reference): same iteration count / partition or not."""
    from fuel_gb300 import kmeans
    from oracle import oracle
    order = _lib.default_order()
    out = {}
    t0 = time.perf_counter()
    rc, rl, rit, rinert = oracle.lloyd_exact(X, K, init, max_iter=ITERS, order=order, threads=threads,
                                             fixed_iters=True)
    gc, gl, git, ginert = gpu_fixed
    out["fixed_100"] = {
        "labels_equal": bool(np.array_equal(gl, rl)), "centers_bit_equal": bool(np.array_equal(
            np.ascontiguousarray(gc).view(np.uint32), rc.view(np.uint32))),
        "iterations": [int(git), int(rit)], "inertia_gpu": ginert, "inertia_fp64": rinert,
        "inertia_rel_err_fp64": abs(ginert - rinert) / rinert, "oracle_s": time.perf_counter() - t0}
    t0 = time.perf_counter()
    g = kmeans(X, k=K, variant="lloyd", init=init, max_iter=300, tol=0, order=order, precision="split_bf16")
    rc2, rl2, rit2, rinert2 = oracle.lloyd_exact(X, K, init, max_iter=300, order=order, threads=threads)
    out["converging"] = {
        "labels_equal": bool(np.array_equal(g.labels, rl2)), "centers_bit_equal": bool(np.array_equal(
            g.centers.view(np.uint32), rc2.view(np.uint32))), "iterations": [g.n_iter, int(rit2)],
        "inertia_rel_err_fp64": abs(g.inertia - rinert2) / rinert2, "oracle_s": time.perf_counter() - t0}
    t0 = time.perf_counter()
    fc, fl, fit, _ = oracle.lloyd(X, K, init, max_iter=300, order=order, threads=threads)
    out["vs_fuel_f32_sums"] = {
        "threads": threads, "iterations": [g.n_iter, int(fit)], "labels_differ": int((fl != g.labels).sum()),
        "centers_max_rel_diff": float(np.max(np.abs(fc.astype(np.float64) - g.centers) /
                                            np.maximum(np.abs(g.centers.astype(np.float64)), 1e-30))),
        "note": "fuel keeps f32 running sums per rayon chunk; the engine's centres are exact means",
        "oracle_s": time.perf_counter() - t0}
    out["bit_exact"] = all(out[k_]["labels_equal"] and out[k_]["centers_bit_equal"] and
                           out[k_]["iterations"][0] == out[k_]["iterations"][1] and
                           out[k_]["inertia_rel_err_fp64"] <= 1e-7 for k_ in ("fixed_100", "converging"))
    return out


def _reference_rows(X, Q, rows_self, k, metric, threads):
    """The reference's answer for query rows Q: its tie-inclusive list
    (KNNHeap::into_vec), index rows_self[j] dropped from row j when given (the
    linear-index exclude rule, python/search.rs:485-488), truncated to k and
    padded (python/search.rs:1195-1216).  Rows run in parallel threads."""
    from oracle import oracle

    def one(j):
        ii, dd = oracle.knn_with_ties(X, Q[j], k, metric=metric)
        if rows_self is not None:
            keep = ii != rows_self[j]
            ii, dd = ii[keep], dd[keep]
        oi = np.full(k, -1, np.int64)
        od = np.full(k, np.inf, np.float32)
        oi[:min(k, len(ii))] = ii[:k]
        od[:min(k, len(dd))] = dd[:k]
        return oi, od

    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(one, range(Q.shape[0])))
    return np.stack([r[0] for r in res]), np.stack([r[1] for r in res])


def knn_rows_parity(X, Q, rows_self, k, gi, gd, metric, threads, what):
    t0 = time.perf_counter()
    ri, rd = _reference_rows(X, Q, rows_self, k, metric, threads)
    return {"rows": int(Q.shape[0]), "what": what,
            "indices_equal": bool(np.array_equal(gi, ri)),
            "distance_bits_equal": bool(np.array_equal(np.ascontiguousarray(gd, np.float32).view(np.uint32),
                                                       rd.view(np.uint32))),
            "oracle_s": time.perf_counter() - t0}


def error_report(lib, _lib, handle, queries_ptr, m, k, idx_ptr, dist_ptr):
    rep = _lib.ErrorReport()
    _lib.check(lib.fuelg_knn_error(handle, queries_ptr, m, k, idx_ptr, dist_ptr, ctypes.byref(rep)))
    return rep.as_dict()


# ---------------------------------------------------------------------------
# the headline leg and the JSON line
# ---------------------------------------------------------------------------

def run_ours(args):
    import torch
    from fuel_gb300 import _lib, build, workloads

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
        torch.cuda.set_device(local)
    build.build()
    lib = _lib.load()
    prec = _lib.PRECISION[args.precision]
    order = _lib.ORDER[_lib.default_order()]

    X, init = workloads.lloyd_sparse(N, D, K)
    Xd = torch.from_numpy(X).cuda()
    Cd = torch.from_numpy(init).cuda()
    oc = torch.empty((K, D), dtype=torch.float32, device="cuda")
    ol = torch.empty((N,), dtype=torch.int64, device="cuda")
    # pinned host copies for the end-to-end leg
    Xh = torch.empty((N, D), dtype=torch.float32, pin_memory=True)
    Xh.copy_(torch.from_numpy(X))
    Ch = torch.empty((K, D), dtype=torch.float32, pin_memory=True)
    Ch.copy_(torch.from_numpy(init))
    och = torch.empty((K, D), dtype=torch.float32, pin_memory=True)
    olh = torch.empty((N,), dtype=torch.int64, pin_memory=True)

    def step(device_resident=True, precision=None):
        st = _lib.Stats()
        it = ctypes.c_int32()
        inert = ctypes.c_double()
        src = (Xd, Cd, oc, ol) if device_resident else (Xh, Ch, och, olh)
        pr = prec if precision is None else precision
        _lib.check(lib.fuelg_kmeans_lloyd(_lib.ptr(src[0]), N, D, K, _lib.ptr(src[1]), ITERS, 0.0, pr, order,
                                          _lib.LLOYD_FIXED_ITERS, _lib.ptr(src[2]), _lib.ptr(src[3]),
                                          ctypes.byref(it), ctypes.byref(inert), ctypes.byref(st)))
        assert it.value == ITERS
        return st, inert.value

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step(True)
    barrier()
    with ClockSampler(local) as clk:
        stats = [step(True) for _ in range(args.steps)]
    barrier()
    dev_ms = sum(s.device_ms for s, _ in stats)
    rescored = sum(s.rescored for s, _ in stats)
    prec_used = stats[-1][0].precision_used
    hot_ms = sum(s.hot_kernel_ms for s, _ in stats)
    hot_n = sum(s.hot_kernel_launches for s, _ in stats)
    launches = sum(s.kernel_launches for s, _ in stats)
    inertia = stats[-1][1]

    # end-to-end through the C ABI with pinned host buffers (copies inside the timed call)
    for _ in range(max(1, args.warmup // 2)):
        step(False)
    barrier()
    e2e = [step(False) for _ in range(args.steps)]
    barrier()
    e2e_ms = sum(s.device_ms for s, _ in e2e)
    h2d = e2e[0][0].h2d_bytes
    d2h = e2e[0][0].d2h_bytes
    gpu_fixed = (och.numpy().copy(), olh.numpy().copy(), ITERS, e2e[-1][1])

    t_max = dev_ms
    e2e_max = e2e_ms
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([dev_ms, e2e_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_max, e2e_max = float(t[0]), float(t[1])
    if rank != 0:
        return

    # the plain FP32 CUDA-core tier on the same workload, for the TC-vs-plain ratio
    plain = None
    if prec != 0:
        step(True, 0)
        pst = [step(True, 0) for _ in range(2)]
        pms = sum(s.device_ms for s, _ in pst)
        # average over the launches timed one by one (passes outside the replayed graph)
        p_launch = sum(s.hot_kernel_ms for s, _ in pst) / max(1, sum(s.hot_kernel_launches for s, _ in pst))
        plain = {"iters_per_s": ITERS * len(pst) / (pms / 1e3), "hot_kernel_ms": p_launch,
                 "roofline": plain_roofline(lib, _lib, N * K, D, p_launch,
                                            "scan_topk_kernel (exact FP32 Lloyd assignment, one pass)")}
    # the same tensor-core tier on data that is not small integers times one scale
    # (the split form reads hi and lo BF16 copies: twice the screen's bytes)
    general = None
    if prec == 2 and not args.quick:
        os.environ["FUELG_TC_NO_SCALED"] = "1"
        try:
            step(True)
            gst = [step(True) for _ in range(3)]
        finally:
            del os.environ["FUELG_TC_NO_SCALED"]
        g_hot = sum(s.hot_kernel_ms for s, _ in gst) / max(1, sum(s.hot_kernel_launches for s, _ in gst))
        g_bytes = N * D * 2 * 2 + K * D * 2 + N * 4
        general = {"iters_per_s": ITERS * len(gst) / (sum(s.device_ms for s, _ in gst) / 1e3),
                   "precision_used": _lib.PRECISION_NAMES[gst[-1][0].precision_used],
                   "screen_ms": g_hot, "screen_gbs": g_bytes / (g_hot / 1e3) / 1e9,
                   "note": "split-BF16 tier with the scaled-integer copy disabled (FUELG_TC_NO_SCALED=1): "
                           "the form any float32 data takes"}

    pk = peaks()
    value = world * ITERS * args.steps / (t_max / 1e3)
    e2e_value = world * ITERS * args.steps / (e2e_max / 1e3)
    # roofline of the hot kernel.  Tensor-core tier: one read of the BF16 copies of X
    # (n*d*2 each: hi and lo for split-BF16, the one exact scaled-integer copy for
    # split_bf16_scaled), the BF16 centres (k*d*2 per copy) and one int32 label per
    # point.  Plain tier: one read of X (n*d*4) + the centres (k*d*4) + one 8-byte
    # key per point.
    if prec_used != 0:
        x_copies = 2 if prec_used == 2 else 1
        c_copies = 2 if prec_used == 3 else 1
        alg_bytes = N * D * 2 * x_copies + K * D * 2 * c_copies + N * 4
        hot_name = "lloyd_tc_kernel (tcgen05 BF16 screen of the Lloyd assignment)"
    else:
        alg_bytes = N * D * 4 + K * D * 4 + N * 8
        hot_name = "scan_topk_kernel (exact FP32 Lloyd assignment)"
    avg_launch_ms = hot_ms / max(1, hot_n)
    # DRAM bytes (read + write) per launch of the screen on this workload, from
    # ncu captures of the same kernel: split-BF16 233.8 MB + 3.2 MB; the scaled
    # integer copy (8-bit values / 255) 117.6 MB + 3.0 MB
    traffic = {2: 237.0e6, 3: 120.6e6}.get(prec_used)
    achieved = alg_bytes / (avg_launch_ms / 1e3) / 1e9
    hbm_peak = pk.get("hbm_gbs", 6800.0)
    threads = host_threads()

    side = {}
    if not args.quick:
        side["knn_plain"] = knn_plain_rate(lib, _lib, torch, args, parity=True)
        side["knn_tc"] = knn_tc_rate(lib, _lib, torch, args, parity=True)
        if not args.no_serving:
            side["knn_serving"] = serving_rates(parity=True)
        if not args.no_batched:
            side["kmeans_batched"] = batched_rate()
        side["lloyd_parity"] = lloyd_parity(lib, _lib, X, init, gpu_fixed, threads)

    # CPU baseline: restated fuel CPU Lloyd on the host cores, bounded sample
    sample_iters = CPU_SAMPLE_ITERS
    cpu_t, cpu_it = cpu_lloyd_sample(X, init, sample_iters, threads)
    cpu_value = cpu_it / cpu_t

    line = {
        "metric": METRIC, "value": value, "unit": "iters/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16+f32" if prec_used else "f32", "data": "synthetic",
        "config": {"workload": f"lloyd k={K} n={N} d={D}, {ITERS} fixed iterations per step", "n": N, "d": D,
                   "k": K, "iters_per_step": ITERS, "precision": args.precision,
                   "summation_order": _lib.default_order(),
                   "l2": "inputs (219.5 MB) larger than L2; no flush", "parallelism": "replicas"},
        "e2e": {"value": e2e_value, "unit": "iters/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic,
                     "kernel": hot_name, "alg_bytes_per_launch": alg_bytes,
                     "avg_launch_ms": avg_launch_ms, "peak_source": "measured" if "_fallback" not in pk else
                     "fallback"},
        "cpu_baseline": {"value": cpu_value, "unit": "iters/s", "cores": threads, "kind": "port",
                         "sample": f"{cpu_it} iterations of the full n={N} matrix (one call, max_iter="
                                   f"{sample_iters}), restated fuel CPU Lloyd, {cpu_t:.1f} s"},
        "clocks": clk.summary(),
        "inertia": inertia,
        "precision_used": _lib.PRECISION_NAMES[prec_used],
        "rescored_fraction": rescored / float(N * ITERS * args.steps),
        "plain_fp32": plain,
        "tc_vs_plain": (value / plain["iters_per_s"]) if plain else None,
        "general_split_bf16": general,
    }
    if side:
        line["parity"] = {
            "lloyd": side["lloyd_parity"],
            "knn_plain": side["knn_plain"].pop("parity"),
            "knn_tc_sample": side["knn_tc"].pop("parity"),
            "serving_sample": side["knn_serving"].pop("parity") if "knn_serving" in side else None,
        }
        line["parity"]["all_bit_exact"] = bool(
            line["parity"]["lloyd"]["bit_exact"] and
            all(v["indices_equal"] and v["distance_bits_equal"]
                for k_, v in line["parity"].items() if k_ not in ("lloyd",) and isinstance(v, dict)))
        for k_ in ("knn_plain", "knn_tc", "knn_serving", "kmeans_batched"):
            if k_ in side:
                line[k_] = side[k_]
    print(json.dumps(line), flush=True)


def pairwise_rate(lib, _lib, torch, args):
    """pairwise_distances on the kNN self-join points (n=20,000, d=16): condensed and
    square forms, device-resident output; roofline = bytes written / kernel time."""
    from fuel_gb300 import workloads
    X = workloads.knn_plain()
    n, d = X.shape
    Xd = torch.from_numpy(X).cuda()
    out = {}
    for form, nout in ((0, n * (n - 1) // 2), (1, n * n)):
        o = torch.empty(nout, dtype=torch.float32, device="cuda")
        sts = []
        for i in range(max(3, args.warmup) + max(1, args.steps)):
            st = _lib.Stats()
            _lib.check(lib.fuelg_pairwise(_lib.ptr(Xd), n, d, 1, _lib.ORDER[_lib.default_order()], form, _lib.ptr(o),
                                          ctypes.byref(st)))
            sts.append(st)
        sts = sts[max(3, args.warmup):]
        hot = sum(s.hot_kernel_ms for s in sts) / len(sts)
        out["condensed" if form == 0 else "square"] = {
            "kernel_ms": hot, "pairs_per_s": n * (n - 1) / 2 / (hot / 1e3),
            "written_gbs": nout * 4 / (hot / 1e3) / 1e9}
        del o
    return {"workload": f"pairwise euclidean n={n} d={d}", **out}


def knn_plain_rate(lib, _lib, torch, args, parity=False):
    """Plain exact kNN self-join n=20,000, d=16, k=10 (6-Gaussian mixture),
    linear-index exclude rule; device-resident queries and outputs (value) and
    pinned host buffers through the C ABI (e2e); the whole output checked
    against the oracle; CPU baseline = the oracle on all host cores."""
    from fuel_gb300 import workloads
    X = workloads.knn_plain()
    n, d, k = X.shape[0], X.shape[1], 10
    h = ctypes.c_void_p()
    _lib.check(lib.fuelg_index_create(_lib.ptr(X), n, d, 0, _lib.ORDER[_lib.default_order()], ctypes.byref(h)))
    try:
        Qd = torch.from_numpy(X).cuda()
        oi = torch.empty((n, k), dtype=torch.int64, device="cuda")
        od = torch.empty((n, k), dtype=torch.float32, device="cuda")
        Qh = torch.empty((n, d), dtype=torch.float32, pin_memory=True)
        Qh.copy_(torch.from_numpy(X))
        oih = torch.empty((n, k), dtype=torch.int64, pin_memory=True)
        odh = torch.empty((n, k), dtype=torch.float32, pin_memory=True)

        def call(q, i, o):
            st = _lib.Stats()
            _lib.check(lib.fuelg_knn(h, _lib.ptr(q), n, k, 1, 0, _lib.ptr(i), _lib.ptr(o), ctypes.byref(st)))
            return st

        ms, hot, e2e = [], [], []
        for it in range(args.warmup + args.steps):
            st = call(Qd, oi, od)
            if it >= args.warmup:
                ms.append(st.device_ms)
                hot.append(st.hot_kernel_ms / max(1, st.hot_kernel_launches))
        for it in range(args.warmup + args.steps):
            st = call(Qh, oih, odh)
            if it >= args.warmup:
                e2e.append(st.device_ms)
        t = sum(ms) / len(ms)
        te = sum(e2e) / len(e2e)
        hk = sum(hot) / len(hot)
        out = {"workload": "knn self-join n=20000 d=16 k=10 sqeuclidean", "queries_per_s": n / (t / 1e3),
               "ms_per_call": t, "distance_evals_per_s": n * n / (t / 1e3), "hot_kernel_ms": hk,
               "precision": "fp32",
               "e2e": {"queries_per_s": n / (te / 1e3), "ms_per_call": te, "h2d_bytes_per_call": n * d * 4,
                       "d2h_bytes_per_call": n * k * 12},
               "roofline": plain_roofline(lib, _lib, n * n, d, hk, "scan_topk_kernel (exact FP32 kNN scan)")}
        out["fp64"] = error_report(lib, _lib, h, _lib.ptr(Qd), n, k, _lib.ptr(oi), _lib.ptr(od))
        if parity:
            from oracle import oracle
            threads = host_threads()
            ci, cd = oracle.knn(X, X, k, metric="sqeuclidean", order=_lib.default_order(), exclude="linear",
                                threads=threads)
            t0 = time.perf_counter()
            oracle.knn(X, X, k, metric="sqeuclidean", order=_lib.default_order(), exclude="linear",
                       threads=threads)
            cpu_s = time.perf_counter() - t0
            gi, gd = oih.numpy(), odh.numpy()
            out["parity"] = {"rows": n, "what": "whole self-join vs the oracle (linear exclude rule)",
                             "indices_equal": bool(np.array_equal(gi, ci)),
                             "distance_bits_equal": bool(np.array_equal(gd.view(np.uint32), cd.view(np.uint32)))}
            out["cpu_baseline"] = {"value": n / cpu_s, "unit": "queries/s", "cores": threads, "kind": "port",
                                   "sample": f"the whole self-join ({n} queries), restated fuel linear scan, "
                                             f"{cpu_s:.2f} s"}
        return out
    finally:
        lib.fuelg_index_destroy(h)


def knn_tc_rate(lib, _lib, torch, args, m_tc=None, plain=True, reps=1, n_index=KNN_N, parity=False):
    """Exact kNN self-join n=1e6, d=128, k=100 (integer data), linear-index
    exclude rule: tensor-core tier over m_tc queries (default all n), plain
    FP32 tier over a query subset; device-resident queries and outputs;
    distance evaluations = m * n.  With parity: sampled rows against the
    oracle's tie-inclusive lists, the FP64 report of the whole output, the
    tie counts of every row (fuelg_knn_ties), the end-to-end call with pinned
    host buffers and the CPU baseline on a query sample."""
    from fuel_gb300 import workloads
    X = workloads.knn_geometric(n_index, KNN_D)
    n, d, k = n_index, KNN_D, KNN_K
    m_tc = n if m_tc is None else m_tc
    h = ctypes.c_void_p()
    _lib.check(lib.fuelg_index_create(_lib.ptr(X), n, d, 0, _lib.ORDER[_lib.default_order()], ctypes.byref(h)))
    try:
        Qd = torch.from_numpy(X[:m_tc]).cuda()
        oi = torch.empty((m_tc, k), dtype=torch.int64, device="cuda")
        od = torch.empty((m_tc, k), dtype=torch.float32, device="cuda")

        def call(m, prec, q=Qd, i=oi, o=od):
            st = _lib.Stats()
            _lib.check(lib.fuelg_knn(h, _lib.ptr(q), m, k, 1, prec, _lib.ptr(i), _lib.ptr(o), ctypes.byref(st)))
            return st

        call(min(m_tc, 4096), 1)
        sts = [call(m_tc, 1) for _ in range(reps)]
        t = sum(s.device_ms for s in sts) / len(sts)
        hot = sum(s.hot_kernel_ms for s in sts) / max(1, sum(s.hot_kernel_launches for s in sts))
        out = {"workload": f"knn self-join n={n} d={d} k={k} sqeuclidean, integer geometric(0.1) data",
               "queries": m_tc, "queries_per_s": m_tc / (t / 1e3), "ms_per_call": t,
               "distance_evals_per_s": m_tc * float(n) / (t / 1e3), "hot_kernel_ms": hot,
               "hot_kernel_launches": sts[-1].hot_kernel_launches, "rescored": sts[-1].rescored,
               "precision_used": _lib.PRECISION_NAMES[sts[-1].precision_used],
               "kernel_launches": sts[-1].kernel_launches}
        # tensor pipe: 2*m*n*dp flops in the screen kernel
        dp = ((d + 63) // 64) * 64
        out["screen_tflops"] = 2.0 * m_tc * n * dp / (hot * sts[-1].hot_kernel_launches / 1e3) / 1e12
        pk = peaks()
        tp = pk.get("bf16_tflops_sustained", 1700.0)  # the screen runs for tenths of a second
        out["roofline"] = {"bound": "tensor", "achieved": out["screen_tflops"], "peak": tp, "unit": "TFLOP/s",
                           "frac": out["screen_tflops"] / tp, "kernel": "knn_tc_kernel",
                           "peak_source": "measured" if "_fallback" not in pk else "fallback"}
        if parity:
            threads = host_threads()
            rng = np.random.default_rng(7)
            rows = np.sort(rng.choice(m_tc, size=min(PARITY_KNN_ROWS, m_tc), replace=False))
            gi = oi[torch.from_numpy(rows).cuda()].cpu().numpy()
            gd = od[torch.from_numpy(rows).cuda()].cpu().numpy()
            out["parity"] = knn_rows_parity(X, X[rows], rows, k, gi, gd, "sqeuclidean", threads,
                                            "sampled rows of the full self-join vs the oracle's tie-inclusive "
                                            "lists (self dropped, truncated to k)")
            out["fp64"] = error_report(lib, _lib, h, _lib.ptr(Qd), m_tc, k, _lib.ptr(oi), _lib.ptr(od))
            # ties at the k-th distance over every row (tie-inclusive lists of the whole self-join)
            res = ctypes.c_void_p()
            st = _lib.Stats()
            _lib.check(lib.fuelg_knn_ties(h, None, n, k, 1, 1, ctypes.byref(res), ctypes.byref(st)))
            try:
                from fuel_gb300.search import _take_csr
                off, _, _ = _take_csr(lib, res, n)
            finally:
                lib.fuelg_range_free(res)
            lens = np.diff(off)
            out["ties"] = {"rows_with_ties_at_k": int((lens > k).sum()), "extra_tied_entries": int(np.maximum(
                lens - k, 0).sum()), "longest_list": int(lens.max()), "call_ms": st.device_ms,
                "note": "tie-inclusive lists (KNNHeap::into_vec) of all rows, linear exclude rule"}
            # end to end: pinned host queries in, pinned host results out, one call per 10^6 rows
            Qh = torch.empty((m_tc, d), dtype=torch.float32, pin_memory=True)
            Qh.copy_(torch.from_numpy(X[:m_tc]))
            oih = torch.empty((m_tc, k), dtype=torch.int64, pin_memory=True)
            odh = torch.empty((m_tc, k), dtype=torch.float32, pin_memory=True)
            call(m_tc, 1, Qh, oih, odh)
            se = call(m_tc, 1, Qh, oih, odh)
            out["e2e"] = {"queries_per_s": m_tc / (se.device_ms / 1e3), "ms_per_call": se.device_ms,
                          "h2d_bytes_per_call": se.h2d_bytes, "d2h_bytes_per_call": se.d2h_bytes}
            from oracle import oracle
            mq = CPU_KNN_TC_QUERIES
            t0 = time.perf_counter()
            oracle.knn(X, X[:mq], k, metric="sqeuclidean", order=_lib.default_order(), threads=threads)
            cpu_s = time.perf_counter() - t0
            out["cpu_baseline"] = {"value": mq / cpu_s, "unit": "queries/s", "cores": threads, "kind": "port",
                                   "distance_evals_per_s": mq * float(n) / cpu_s,
                                   "sample": f"{mq} queries of the 10^6-point self-join, restated fuel linear "
                                             f"scan, {cpu_s:.1f} s"}
        if plain:
            mp = min(KNN_PLAIN_QUERIES, m_tc)
            call(min(mp, 2048), 0)
            st = call(mp, 0)
            pr = mp * float(n) / (st.device_ms / 1e3)
            p_hot = st.hot_kernel_ms
            out["plain_fp32"] = {"queries": mp, "ms_per_call": st.device_ms, "distance_evals_per_s": pr,
                                 "roofline": plain_roofline(lib, _lib, mp * n, d, p_hot,
                                                            "scan_topk_kernel (exact FP32 kNN scan)")}
            out["tc_vs_plain"] = out["distance_evals_per_s"] / pr
        return out
    finally:
        lib.fuelg_index_destroy(h)


def batched_rate(reps=1, count=BATCH_PROBLEMS, plain=True):
    """Batched k-means: 512 Gaussian-mixture problems (n log-uniform in
    [1e3, 2e5], d in {2, 8, 32, 64}, k log-uniform in [4, 256]), 20 fixed
    Lloyd iterations, all in one engine call, against one plain FP32
    fuelg_kmeans_lloyd call per problem; inputs in pinned host memory for
    both.  Unit: problem-iterations/s.  Roofline: one read of every problem's
    points per iteration (sum n*d*4 bytes) over the iteration loop's time."""
    import torch
    from fuel_gb300 import kmeans, kmeans_batched, workloads
    descs = workloads.batched_kmeans_problems(count=count, seed=0)
    # inputs in pinned host memory (numpy views of pinned tensors, kept alive
    # here), as for the other end-to-end legs: the copies inside each call
    # run at the host link's rate, not at that of pageable staging
    keep = []

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True)
        keep.append(t)
        v = t.numpy()
        v[...] = a
        return v

    probs = [tuple(pinned(a) for a in workloads.batched_kmeans_data(t)) for t in descs]
    kmeans_batched(probs[:8], max_iter=3, fixed_iters=True)  # warm-up
    kmeans_batched(probs, max_iter=BATCH_ITERS, fixed_iters=True)  # launch-shape tuning for this mix
    ms = []
    for _ in range(reps):
        kmeans_batched(probs, max_iter=BATCH_ITERS, fixed_iters=True)
        ms.append(kmeans_batched.last_stats["device_ms"])
    t = sum(ms) / len(ms)
    hot = kmeans_batched.last_stats["hot_kernel_ms"]
    plain_ms = 0.0
    for X, init in (probs if plain else []):
        r = kmeans(X, k=init.shape[0], variant="lloyd", init=init, max_iter=BATCH_ITERS, fixed_iters=True,
                   precision="fp32")
        plain_ms += r.stats["device_ms"]
    pi = count * BATCH_ITERS
    plain_ms = plain_ms or float("nan")
    bytes_it = float(sum(dsc[0] * dsc[1] * 4 for dsc in descs))
    flops_it = float(sum(2 * dsc[0] * dsc[2] * dsc[1] for dsc in descs))
    loop_s = hot / 1e3
    pk = peaks()
    ach = bytes_it * BATCH_ITERS / loop_s / 1e9
    return {"workload": f"batched k-means {count} problems n~logU[1e3,2e5] d in {{2,8,32,64}} "
                        f"k~logU[4,256], {BATCH_ITERS} fixed iterations",
            "points": int(sum(d[0] for d in descs)), "ms_per_call": t, "iteration_loop_ms": hot,
            "problem_iters_per_s": pi / (t / 1e3), "plain_per_problem_ms": plain_ms,
            "plain_problem_iters_per_s": pi / (plain_ms / 1e3), "batched_vs_plain": plain_ms / t,
            "kernel_launches": kmeans_batched.last_stats["kernel_launches"],
            "rescored_rows": kmeans_batched.last_stats.get("rescored"),
            "roofline": {"bound": "hbm", "achieved": ach, "peak": pk.get("hbm_gbs", 6800.0), "unit": "GB/s",
                         "frac": ach / pk.get("hbm_gbs", 6800.0), "alg_bytes_per_iteration": bytes_it,
                         "flops_per_iteration": flops_it,
                         "tflops": flops_it * BATCH_ITERS / loop_s / 1e12,
                         "note": "sum n*d*4 bytes per iteration over the iteration loop (CUDA events)"}}


def serving_run(precision, seconds, X=None, seed=1, rate=SERVE_RATE, sample=0):
    """kNN serving: resident index n=2,000,000, d=96 (unit-norm rows);
    Poisson arrivals (`rate` requests/s) of query batches of log-uniform size
    in [1, 4096] with k drawn from {1, 10, 100}, submitted in real time to the
    continuous-batching server; latency = submit to completion.  sample > 0
    keeps the results of about that many query rows (whole small requests)
    for the parity check."""
    from fuel_gb300 import SearchIndex, workloads
    from fuel_gb300.serving import Server
    X = workloads.unit_normal_rows(SERVE_N, SERVE_D, seed=0) if X is None else X
    ix = SearchIndex(X, distance="sqeuclidean", tree="linear", precision=precision)
    rng = np.random.default_rng(seed)
    pool = workloads.unit_normal_rows(1 << 16, SERVE_D, seed=2)
    reqs, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > seconds:
            break
        m = int(np.exp(rng.uniform(0.0, np.log(4096.0))))
        o = int(rng.integers(0, pool.shape[0] - m))
        reqs.append((t, pool[o:o + m], int(rng.choice([1, 10, 100]))))
    with Server(ix, precision=precision, max_batch_queries=16384, budget_bytes=8 << 30, workers=3) as sv:
        sv.submit(pool[:256], 10).result()  # warm-up (tensor-core form, streams)
        handles = []
        t0 = time.perf_counter()

        def feed():
            for ta, Q, k in reqs:
                dt = t0 + ta - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                handles.append(sv.submit(Q, k))

        th = threading.Thread(target=feed)
        th.start()
        th.join()
        for h in handles:
            h.result()
        wall = time.perf_counter() - t0
        st = sv.stats()
    lat = np.array([h.latency_ms for h in handles])
    q = sum(Q.shape[0] for _, Q, _ in reqs)
    out = {"precision": precision, "requests": len(reqs), "queries": q, "arrival_seconds": seconds,
           "arrival_rate_req_per_s": rate, "offered_queries_per_s": q / seconds, "queries_per_s": q / wall,
           "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "batches": st["batches"] - 1, "max_batch_requests": st["max_batch_requests"],
           "device_ms": st["device_ms"]}
    if sample:
        # whole requests, spread over the run, until about `sample` query rows
        picks, rows = [], 0
        for j in np.random.default_rng(3).permutation(len(reqs)):
            if rows >= sample:
                break
            if reqs[j][1].shape[0] <= 64:
                picks.append(j)
                rows += reqs[j][1].shape[0]
        out["_sample"] = [(reqs[j][1], reqs[j][2], handles[j].result()) for j in sorted(picks)]
        out["_index"] = ix
    return out


def serving_rates(parity=False):
    from fuel_gb300 import _lib, workloads
    X = workloads.unit_normal_rows(SERVE_N, SERVE_D, seed=0)
    tc16 = serving_run("fp16", SERVE_SECONDS["fp16"], X, sample=PARITY_SERVE_ROWS if parity else 0)
    tc = serving_run("split_bf16", SERVE_SECONDS["split_bf16"], X)
    plain = serving_run("fp32", SERVE_PLAIN_SECONDS, X, rate=SERVE_PLAIN_RATE)
    out = {"workload": f"knn serving n={SERVE_N} d={SERVE_D} unit-norm rows, Poisson {SERVE_RATE:.0f} req/s, "
                       "batch log-U[1,4096], k in {1,10,100}", "tc_fp16": tc16, "tc": tc, "plain_fp32": plain,
           "note": f"fp16 tier over {SERVE_SECONDS['fp16']:.0f} s of arrivals at {SERVE_RATE:.0f} req/s; "
                   f"split_bf16 over {SERVE_SECONDS['split_bf16']:.0f} s; the plain FP32 tier cannot sustain "
                   f"that load, so it runs at {SERVE_PLAIN_RATE:.0f} req/s for {SERVE_PLAIN_SECONDS:.0f} s"}
    if parity:
        lib = _lib.load()
        threads = host_threads()
        sample = tc16.pop("_sample")
        ix = tc16.pop("_index")
        Q = np.concatenate([s[0] for s in sample])
        gi, gd, checks, fp64 = [], [], [], []
        for Qr, k, (ii, dd) in sample:
            from oracle import oracle
            ci, cd = oracle.knn(X, Qr, k, metric="sqeuclidean", order=_lib.default_order(), threads=threads)
            checks.append(np.array_equal(ii, ci) and np.array_equal(dd.view(np.uint32), cd.view(np.uint32)))
            fp64.append(error_report(lib, _lib, ix._handle, _lib.ptr(Qr), Qr.shape[0], k, _lib.ptr(ii),
                                     _lib.ptr(dd)))
        out["parity"] = {"rows": int(Q.shape[0]), "requests": len(sample),
                         "what": "whole served requests (fp16 tier, mixed k) vs the oracle",
                         "indices_equal": bool(all(checks)), "distance_bits_equal": bool(all(checks))}
        tc16["fp64"] = {"max_rel_err": max(f["max_rel_err"] for f in fp64),
                        "max_abs_err": max(f["max_abs_err"] for f in fp64),
                        "pairs": sum(f["pairs"] for f in fp64), "near_ties": sum(f["near_ties"] for f in fp64),
                        "order_flips": sum(f["order_flips"] for f in fp64)}
        from oracle import oracle
        pool = workloads.unit_normal_rows(1 << 16, SERVE_D, seed=2)
        mq = CPU_SERVE_QUERIES
        t0 = time.perf_counter()
        oracle.knn(X, pool[:mq], 10, metric="sqeuclidean", order=_lib.default_order(), threads=threads)
        cpu_s = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": mq / cpu_s, "unit": "queries/s", "cores": threads, "kind": "port",
                               "sample": f"{mq} queries (k=10) against the 2,000,000-row index, restated fuel "
                                         f"linear scan, {cpu_s:.1f} s"}
        del ix
    tc16.pop("_index", None)
    return out


def run_profile(args):
    """One workload alone, for profiler captures."""
    import torch
    from fuel_gb300 import _lib, build, workloads
    build.build()
    lib = _lib.load()
    if args.profile == "lloyd":
        X, init = workloads.lloyd_sparse(N, D, K)
        Xd = torch.from_numpy(X).cuda()
        Cd = torch.from_numpy(init).cuda()
        oc = torch.empty((K, D), dtype=torch.float32, device="cuda")
        ol = torch.empty((N,), dtype=torch.int64, device="cuda")
        ms = []
        for i in range(args.warmup + args.steps):
            st = _lib.Stats()
            it = ctypes.c_int32()
            inert = ctypes.c_double()
            _lib.check(lib.fuelg_kmeans_lloyd(_lib.ptr(Xd), N, D, K, _lib.ptr(Cd), args.iters, 0.0,
                                              _lib.PRECISION[args.precision], _lib.ORDER[_lib.default_order()],
                                              _lib.LLOYD_FIXED_ITERS, _lib.ptr(oc), _lib.ptr(ol), ctypes.byref(it),
                                              ctypes.byref(inert), ctypes.byref(st)))
            if i >= args.warmup:
                ms.append(st.device_ms)
        print(json.dumps({"profile": "lloyd", "iters": args.iters, "ms_per_call": sum(ms) / max(1, len(ms))}))
    elif args.profile == "knn_tc":
        r = knn_tc_rate(lib, _lib, torch, args, m_tc=args.knn_queries, plain=False, reps=max(1, args.steps),
                        n_index=args.knn_n)
        print(json.dumps({"profile": "knn_tc", **r}))
    elif args.profile == "serving":
        print(json.dumps({"profile": "serving", **serving_rates()}))
    elif args.profile == "batched":
        print(json.dumps({"profile": "batched", **batched_rate(count=args.batched_problems, plain=False)}))
    elif args.profile == "pairwise":
        print(json.dumps({"profile": "pairwise", **pairwise_rate(lib, _lib, torch, args)}))
    else:
        args.steps = max(1, args.steps)
        print(json.dumps({"profile": "knn_plain", **knn_plain_rate(lib, _lib, torch, args)}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["fp32", "bf16", "split_bf16"], default="split_bf16")
    ap.add_argument("--profile", choices=["lloyd", "knn_tc", "knn_plain", "serving", "batched", "pairwise"],
                    default=None)
    ap.add_argument("--iters", type=int, default=ITERS, help="Lloyd iterations per call (--profile lloyd)")
    ap.add_argument("--knn-queries", type=int, default=20_000, help="query count (--profile knn_tc)")
    ap.add_argument("--knn-n", type=int, default=KNN_N, help="index rows (--profile knn_tc)")
    ap.add_argument("--quick", action="store_true", help="headline only: no side legs, no parity checks")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving leg")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched k-means leg")
    ap.add_argument("--batched-problems", type=int, default=BATCH_PROBLEMS, help="problems (--profile batched)")
    args = ap.parse_args()
    if args.profile:
        run_profile(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
