#!/usr/bin/env python
"""ε-self-join benchmark: prints one JSON line.

Workload (default): the SUSY-shaped low-dimensional join, n = 5,000,000
points, d = 18, FP64, k = 6 reference points, ε calibrated for a mean of 64
neighbours (seeded synthetic stand-in: the real SUSY file is not available).

One step = one complete self-join through the library's C ABI (index build,
neighbour enumeration, join with pair compaction; the full pair list is
written), i.e. the work the reference's nodeLauncher5 does per dataset.

  value  points joined per second with the input resident in HBM and the
         pair list written to a device buffer (CUDA events on the library's
         stream, which is torch's current stream).
  e2e    the same metric through the same call with a host input array and
         the pair list returned in host memory (host->device copy of the
         points and device->host copy of the pairs inside the timed region).

Also reported: wall time per join, distance evaluations/s (unordered
candidate pairs the join evaluated / step time), pairs/s, the plain FP64
CUDA-core join on the same index (identical pair set required), the roofline
of the dominant kernel, the whole step against its lower bound, and a CPU
baseline (the reference's brute-force algorithm, src/utils.cu:285-317, as
the oracle's C port, on a bounded row sample, extrapolated to the whole job).

The line also carries `tiny384_5m`: the 5M x 384 clustered FP32 workload
(TINY-shaped, k = 8, 16 mean neighbours) measured in the same run -- mixed
precision at full size, and mixed precision against the plain FP64 join
(and TF32) on a fixed full-density sample of home points (mistic_opts.
home_sample), with the pair sets compared bit for bit.

`--impl reference` times that CPU implementation alone (rank 0 only).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "self-join-mistic_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

from mistic import workloads as W  # noqa: E402

METRIC = "self-join wall time & distance evals/s: mixed-prec vs FP64 plain, exact pair set"
UNIT = "points/s"

#: workload name -> (constructor, description)
def _subset(make, full_n):
    """The workload at full size, or its first n points with the full
    configuration's ε (a smaller case of the same kernel, for profiling)."""
    def f(n):
        if not n or n == full_n:
            return make(full_n)
        full_eps = float.fromhex(W.EPS_HEX[f"{make.__name__}:{full_n}"])
        wl = make.__wrapped_gen__(n)
        return W.Workload(f"{make.__name__}:{n}", wl[0], wl[1], full_eps, wl[2])
    return f


W.susy18.__wrapped_gen__ = lambda n: (W.gen_susy_like(n), 6, 64.0)
W.uniform18.__wrapped_gen__ = lambda n: (W.gen_uniform(n, 18, seed=0), 6, 32.0)
W.msd90.__wrapped_gen__ = lambda n: (W.gen_msd_like(n), 8, 16.0)

WORKLOADS = {
    "susy18": (_subset(W.susy18, 5_000_000),
               "SUSY-shaped n=5e6 d=18 FP64, k=6, 64 mean neighbours"),
    "uniform18": (_subset(W.uniform18, 100_000),
                  "uniform n=1e5 d=18 FP64, k=6, 32 mean neighbours"),
    "msd90": (_subset(W.msd90, 515_345),
              "MSD-shaped n=515,345 d=90 FP64, k=8, 16 mean neighbours"),
    # ε calibrated on each generated set (drawn on the GPU at this size)
    "tiny384": (lambda n: W.tiny384(n or 5_000_000),
                "TINY-shaped n=5e6 d=384 FP32, 1000 Zipf(1.1) clusters with full-rank covariance "
                "(eigenvalues log-uniform in [1e-3,1]), L2-normalised, k=8, 16 mean neighbours"),
}

FALLBACK_PEAKS = {"hbm_gbs": 6785.9, "bf16_tflops": 1922.1, "bf16_tflops_sustained": 1711.2}

#: DRAM bytes (read + write) per evaluated cell of k_join_tc on the SUSY-shaped
#: data, from an ncu capture of the 2.5M-point case (317.9 MB over 2.3567e10
#: cells); scaled by the cells of the measured launch.
TC_DRAM_BYTES_PER_CELL_SUSY18 = 317.9e6 / 2.3567e10


def load_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        d["_source"] = "MEASURED_PEAKS.json"
        return d
    except Exception:
        d = dict(FALLBACK_PEAKS)
        d["_source"] = "MEASURED_PEAKS.json values recorded at build time"
        return d


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                c = [x.strip() for x in line.split(",")]
                if len(c) < 9:
                    continue
                try:
                    sm.append(float(c[1]))
                    smax.append(float(c[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, c[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU baseline
def cpu_sample(x: np.ndarray, eps: float, seconds: float) -> dict:
    """The reference's brute-force algorithm (oracle C port, all host
    threads) on rows [0, R) against all n rows; R grows until the sample takes
    about `seconds`.  Extrapolates to the whole n x n job."""
    from oracle import oracle as O
    threads = O.max_threads()
    n = x.shape[0]
    rows = max(threads, 16)
    t = 0.0
    while True:
        t0 = time.perf_counter()
        O.count_rows(x, eps, 0, min(rows, n), threads)
        t = time.perf_counter() - t0
        if t >= seconds / 4 or rows >= n:
            break
        rows = min(n, int(rows * max(2.0, seconds / 4 / max(t, 1e-3))))
    rows = min(n, max(rows, int(rows * seconds / max(t, 1e-6))))
    t0 = time.perf_counter()
    O.count_rows(x, eps, 0, rows, threads)
    t = time.perf_counter() - t0
    job_s = t * n / rows
    return {"rows": rows, "seconds": t, "job_seconds": job_s, "threads": threads,
            "points_per_s": n / job_s, "evals_per_s": rows * n / t}


def host_join_sample(x: np.ndarray, eps: float, k: int, seconds: float) -> dict:
    """The project's own indexed host join (oracle/hostjoin.c: the same
    reference-point bins, FP64 predicate, OpenMP on all host threads).  The
    index build and the neighbour enumeration run in full; the distance work
    runs on every S-th home bin, S chosen so that it takes about `seconds`,
    and is scaled to the whole join by candidate pairs."""
    from oracle import oracle as O
    threads = O.max_threads()
    rp = O.pca_far_points(x, k)
    probe = O.host_join(x, eps, rp, home_stride=4096, threads=threads)
    per_cand = probe["s_join"] / max(1, probe["cand_sampled"])
    full_join = per_cand * probe["cand_all"]
    stride = max(1, int(math.ceil(full_join / max(seconds, 1e-3)))) if probe["cand_sampled"] else 4096
    r = O.host_join(x, eps, rp, home_stride=stride, threads=threads)
    join_s = r["s_join"] * r["cand_all"] / max(1, r["cand_sampled"])
    job_s = r["s_index"] + join_s
    return {"value": x.shape[0] / job_s, "unit": UNIT, "cores": threads, "kind": "project host join",
            "job_seconds": job_s, "index_and_enumeration_s": r["s_index"], "join_s_extrapolated": join_s,
            "sample": f"every {stride}-th of {r['bins']} home bins joined ({r['s_join']:.1f} s, "
                      f"{r['cand_sampled']} of {r['cand_all']} candidate pairs), scaled by candidate pairs",
            "evals_per_s": r["cand_sampled"] / max(r["s_join"], 1e-9)}


# ------------------------------------------------------------------ arms
def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(ms: float, world: int, device=None) -> float:
    """Per-step time of the job: the slowest replica's (all_reduce MAX over
    the process group; NCCL on GPUs, gloo in the CPU tests)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_points_per_s(n_per_rank: int, world: int, ms: float) -> float:
    """Whole-job throughput of `world` replicas that each join n_per_rank
    points per step (weak scaling)."""
    return world * n_per_rank / (ms * 1e-3)


def config_for(args, wl, world: int) -> dict:
    """The `config` of the line: the same dict in both arms."""
    return {"workload": args.workload, "n": wl.n, "d": wl.d, "k": wl.k, "eps_hex": float(wl.eps).hex(),
            "desc": WORKLOADS[args.workload][1], "parallelism": "replicas" if world > 1 else "single",
            "l2": f"inputs larger than L2 ({wl.n * wl.d * wl.pts.itemsize / 1e6:.0f} MB points per step)",
            "pairs_to": "caller device buffer"}


def run_reference(args, wl) -> None:
    rank, world, _ = dist_env()
    if rank != 0:
        return
    x, eps = wl.pts, wl.eps
    per_step = args.ref_seconds
    for _ in range(args.warmup):
        cpu_sample(x, eps, per_step / 4)
    samples = [cpu_sample(x, eps, per_step) for _ in range(args.steps)]
    job = statistics.mean(s["job_seconds"] for s in samples)
    value = wl.n / job
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": job * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_for(args, wl, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": samples[0]["threads"], "kind": "port",
                         "sample": f"rows [0,{samples[0]['rows']}) x all {wl.n} rows per step, "
                                   "extrapolated to n rows; brute_force of src/utils.cu:285-317 "
                                   "(oracle C port, OpenMP)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_mistic(args, wl) -> None:
    import torch
    import mistic
    from mistic import _lib as L

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    h = mistic.Handle(local, stream=stream.cuda_stream)

    x = np.ascontiguousarray(wl.pts)
    n, d = x.shape
    dt = L.F64 if x.dtype == np.float64 else L.F32
    xt = torch.from_numpy(x).to(dev)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # first call sizes the caller-owned device pair buffer
    r0 = h.to_result(h.selfjoin_raw(xt.data_ptr(), n, d, dt, wl.k, wl.eps,
                                    h.opts(input_on_device=True, mode=args.mode)))
    cap = int(r0.pairs_ij * 1.02) + 1024
    pbuf = torch.empty((cap,), dtype=torch.int64, device=dev)
    o_dev = h.opts(input_on_device=True, pairs="device", pair_capacity=cap, pair_buffer=pbuf.data_ptr(),
                   mode=args.mode)

    def step(opts):
        return h.to_result(h.selfjoin_raw(xt.data_ptr(), n, d, dt, wl.k, wl.eps, opts))

    for _ in range(args.warmup):
        step(o_dev)
    barrier()
    clocks = ClockSampler()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    results = []
    e0.record(stream)
    for _ in range(args.steps):
        results.append(step(o_dev))
    e1.record(stream)
    barrier()
    clk = clocks.stop()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, world, dev)
    r = results[-1]
    assert all(q.pairs_ij == r.pairs_ij for q in results)
    join_ms = statistics.mean(q.ms["join"] for q in results)
    launches = sum(q.kernel_launches for q in results)

    # ---- e2e: host input, host pair list, through the same C ABI call
    o_host = h.opts(pairs="host", mode=args.mode)
    for _ in range(1):
        h.to_result(h.selfjoin_raw(x.ctypes.data, n, d, dt, wl.k, wl.eps, o_host))
    barrier()
    t0 = time.perf_counter()
    e2e_res = []
    for _ in range(args.steps):
        raw = h.selfjoin_raw(x.ctypes.data, n, d, dt, wl.k, wl.eps, o_host)
        e2e_res.append((raw.pairs_ij, raw.ms_h2d, raw.ms_d2h))
        h.lib.mistic_result_free(ctypes.byref(raw))
    barrier()
    e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / args.steps, world, dev)

    # ---- full-size check: neighbour counts of sampled row blocks from the
    # GPU FP64 brute force (mistic_bruteforce_rows) against the degrees of
    # the timed run's pair list
    verify = None
    if args.verify_rows < 0:  # default: 16,384 rows where the brute force takes seconds (n * d <= 2e8)
        args.verify_rows = 16384 if n * d <= 2e8 else 0
    if args.verify_rows > 0:
        pr = pbuf[:r.pairs_ij]
        deg = torch.zeros(n, dtype=torch.int64, device=dev)
        ones = torch.ones(pr.numel(), dtype=torch.int64, device=dev)
        deg.index_add_(0, (pr >> 32) & 0xFFFFFFFF, ones)  # packed (i << 32 | j) or (j << 32 | i)
        deg.index_add_(0, pr & 0xFFFFFFFF, ones)
        half = max(1, args.verify_rows // 2)
        lo0 = int(np.random.default_rng(7).integers(0, max(1, n - half)))
        ok = True
        for lo in (lo0, max(0, n - half)):
            hi = min(n, lo + half)
            bf = h.bruteforce_rows(None, wl.eps, lo, hi, on_device_ptr=xt.data_ptr(), n=n, d=d, dtype=dt)
            ok = ok and bool(np.array_equal(bf.astype(np.int64), deg[lo:hi].cpu().numpy()))
        verify = {"rows": 2 * half, "degrees_match": ok,
                  "source": "GPU FP64 brute force over two row blocks (mistic_bruteforce_rows)"}

    # ---- plain FP64 CUDA-core join on the same inputs (or on the first
    # --fp64-rows rows, where the full plain join would take hours), identical pair set
    fp64 = None
    if not args.no_fp64:
        m = n if args.fp64_rows <= 0 else min(n, args.fp64_rows)
        rm = h.to_result(h.selfjoin_raw(xt.data_ptr(), m, d, dt, wl.k, wl.eps,
                                        h.opts(input_on_device=True, mode=args.mode)))
        capm = int(rm.pairs_ij * 1.02) + 1024
        pa = torch.empty((capm,), dtype=torch.int64, device=dev)
        pb2 = torch.empty_like(pa)
        o_s = h.opts(input_on_device=True, pairs="device", pair_capacity=capm, pair_buffer=pa.data_ptr(),
                     sort_pairs=True, mode=args.mode)
        o_f = h.opts(input_on_device=True, pairs="device", pair_capacity=capm, pair_buffer=pb2.data_ptr(),
                     sort_pairs=True, mode="fp64")

        def step_m(opts):
            return h.to_result(h.selfjoin_raw(xt.data_ptr(), m, d, dt, wl.k, wl.eps, opts))

        barrier()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        rs = step_m(o_s)
        s1.record(stream)
        barrier()
        mms = s0.elapsed_time(s1) if m < n else ms
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        rf = step_m(o_f)
        f1.record(stream)
        barrier()
        fms = f0.elapsed_time(f1)
        same = (rs.pairs_ij == rf.pairs_ij and
                bool(torch.equal(pa[:rs.pairs_ij], pb2[:rf.pairs_ij])))
        fp64 = {"ms_per_step": fms, "join_ms": rf.ms["join"], "pairs_ij": rf.pairs_ij,
                "identical_pair_set": same, "mixed_speedup": fms / mms,
                "ulp_ambiguous": rf.ulp_ambiguous}
        if m < n:
            fp64.update({"rows": m, "mixed_ms_same_rows": mms,
                         "note": f"plain FP64 and mixed precision both timed on the first {m} rows of the "
                                 "workload (same k and eps); the full-size plain FP64 join is too long to time"})

    if rank != 0:
        return
    peaks = load_peaks()
    fp32_peak = measure_fp32_peak()
    simt_ms = statistics.mean(q.ms["join_simt"] for q in results)
    tc_ms = statistics.mean(q.ms["join_tc"] for q in results)
    if r.mode_used == "bf16" and tc_ms >= simt_ms:
        # dominant kernel: the tensor-core join; algorithmic work 2*d flops per
        # evaluated (home row, candidate) cell, one contraction of length d
        work = r.tc_cells * 2.0 * d
        achieved = work / (tc_ms * 1e-3) / 1e12
        wide = r.tc_kernel == "k-chunked"  # rows prepared once (long rows, or medium rows whose bound allows)
        kname = "k_join_tcw" if wide else "k_join_tc"
        kstage = 64 if r.tc_operands == "bf16" else 32
        kmma = ((d + kstage - 1) // kstage * kstage) if wide else (d + 2 + 15) // 16 * 16
        nprod = 3 if r.tc_operands == "split-bf16" else 1
        roof = {"bound": "tensor", "kernel": kname, "achieved": achieved,
                "peak": peaks.get("bf16_tflops"), "unit": "TFLOP/s",
                "frac": achieved / peaks["bf16_tflops"] if peaks.get("bf16_tflops") else None,
                "traffic": None, "work": "2*d flops per evaluated cell (one d-long contraction)",
                "peak_source": peaks["_source"] + " bf16 burst (of measured)", "kernel_ms": tc_ms,
                "cells": r.tc_cells, "fp32_simt_peak_tflops": fp32_peak,
                # tensor-pipe work actually issued: 3 split products x 2 * K per
                # 128 x 128 tile cell (padding and empty rows/columns included)
                # (K-chunked kernel: tiles count 128 x 128 MMA tiles; the short-row
                # kernel counts candidate tiles, each issued once per home chunk)
                "issued_tflops": (r.tc_tiles * 128 * 128 * nprod * 2.0 * kmma / (tc_ms * 1e-3) / 1e12)
                if wide else None}
        if args.workload == "susy18":
            roof["traffic"] = TC_DRAM_BYTES_PER_CELL_SUSY18 * r.tc_cells
            roof["traffic_source"] = ("ncu dram__bytes_read+write per cell of a 2.5M-point capture of the "
                                      "same kernel x this launch's cells")
    else:
        # dominant kernel: the FP32 filter join; 3*d flops per candidate pair
        # (d subtractions, d multiply-adds) on the CUDA-core FP32 pipe, over
        # the candidate pairs it evaluated (those the tensor cores did not)
        work = max(0, r.candidates - r.tc_cells) * 3.0 * d
        achieved = work / (simt_ms * 1e-3) / 1e12
        roof = {"bound": "fp32", "kernel": "k_join_f32r" if d <= 32 else "k_join_f32", "achieved": achieved,
                "peak": fp32_peak,
                "unit": "TFLOP/s", "frac": achieved / fp32_peak if fp32_peak else None, "traffic": None,
                "work": "3*d FP32 flops per candidate pair", "kernel_ms": simt_ms,
                "peak_source": "mistic_peaks FFMA probe, this run (CUDA-core FP32 pipe)"}
    roof["hbm_peak_gbs"] = peaks.get("hbm_gbs")
    step_roof = step_lower_bound(r, n, d, wl.k, ms, peaks)
    # the nested and baseline measurements report a failure in their own
    # field rather than take the headline line down with them
    def guarded(fn, *a):
        try:
            return fn(*a)
        except Exception as e:  # noqa: BLE001
            return {"error": f"{type(e).__name__}: {e}"[:300]}

    big384 = None if (args.no_tiny384 or args.workload == "tiny384") else \
        guarded(run_tiny384_full, h, args, dev, stream, peaks)
    cpu = guarded(cpu_sample, x, wl.eps, args.cpu_seconds) if not args.no_cpu else None
    host = guarded(host_join_sample, x, wl.eps, wl.k, args.cpu_seconds) if not args.no_cpu else None
    ref_gpu = reference_gpu(x, wl.k, wl.eps, r.pairs_ordered_incl_self, args.ref_gpu_timeout) \
        if args.ref_gpu else None
    value = job_points_per_s(n, world, ms)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_for(args, wl, world),
        "mode_used": r.mode_used, "tc_operands": r.tc_operands, "tc_kernel": r.tc_kernel,
        "tc_min_bin": r.tc_min_bin, "tuned": r.tuned,
        "pairs_ij": r.pairs_ij, "pairs_ordered_incl_self": r.pairs_ordered_incl_self,
        "candidates": r.candidates, "band_pairs": r.band_pairs, "ulp_ambiguous": r.ulp_ambiguous,
        "band_fraction": r.band_pairs / max(1, r.candidates),
        "distance_evals_per_s": r.candidates / (ms * 1e-3), "pairs_per_s": r.pairs_ij / (ms * 1e-3),
        "phase_ms": {k: round(v, 3) for k, v in r.ms.items()},
        "bins": r.n_bins, "bin_pairs": r.n_bin_pairs, "units": r.n_units, "units_tc": r.n_units_tc,
        "tc_tiles": r.tc_tiles, "tc_fill": r.tc_cells / max(1, r.tc_tiles * 128 * 128),
        "k_used": r.k_used,
        "fp64_plain": fp64,
        "verify": verify,
        "roofline": roof,
        "step_roofline": step_roof,
        "tiny384_5m": big384,
        "reference_gpu": ref_gpu,
        "e2e": {"value": job_points_per_s(n, world, e2e_ms), "unit": UNIT, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": n * d * x.itemsize, "d2h_bytes_per_step": int(r.pairs_ij) * 8,
                "h2d_ms": statistics.mean(t[1] for t in e2e_res), "d2h_ms": statistics.mean(t[2] for t in e2e_res)},
        "gpu_launches": launches,
        "clocks": clk,
        "cpu_baseline": cpu if (cpu is None or "error" in cpu) else {
            "value": cpu["points_per_s"], "unit": UNIT, "cores": cpu["threads"], "kind": "port",
            "sample": f"rows [0,{cpu['rows']}) x all {n} rows ({cpu['seconds']:.1f} s), extrapolated to "
                      f"n rows; brute_force of src/utils.cu:285-317 (oracle C port, OpenMP)",
            "evals_per_s": cpu["evals_per_s"]},
        "cpu_host_join": host,
    }
    print(json.dumps(line), flush=True)
    h.close()


def reference_gpu(x: np.ndarray, k: int, eps: float, ours_ordered: int, timeout: float) -> dict | None:
    """The reference's own GPU join (build/main of the reference, built for
    sm_103a by oracle/build_ref_gpu.sh, one binary per DIM) on the same
    points as an FP64 file: its "Total results Set Size" (ordered pairs
    including self pairs, src/launcher.cu:3513), "Kernel Time" and "Total
    Time" (index build + join, file read excluded, src/main.cu:444).  It
    always builds its own 6 index layers (numRP is not read, src/main.cu:174).
    None when no binary was built for this d."""
    d = x.shape[1]
    exe = os.path.join(ROOT, "oracle", "_ref", f"ref_main_d{d}")
    if not os.path.exists(exe):
        return None
    with tempfile.TemporaryDirectory() as td:
        fn = os.path.join(td, "points.bin")
        np.ascontiguousarray(x, dtype=np.float64).tofile(fn)
        t0 = time.perf_counter()
        try:
            pr = subprocess.run([exe, fn, str(d), str(k), repr(float(eps))], capture_output=True, text=True,
                                timeout=timeout)
        except subprocess.TimeoutExpired:
            return {"status": f"not finished within {timeout:.0f} s"}
        wall = time.perf_counter() - t0
    out = pr.stdout

    def grab(tag):
        for line in out.splitlines():
            if line.startswith(tag):
                try:
                    return float(line[len(tag):].split()[0])
                except ValueError:
                    return None
        return None

    total = grab("Total results Set Size:")
    res = {"status": "ok" if pr.returncode == 0 else f"exit {pr.returncode}",
           "ordered_pairs_incl_self": None if total is None else int(total),
           "kernel_s": grab("Kernel Time:"), "total_s": grab("Total Time:"), "process_wall_s": wall,
           "same_count": None if total is None else int(total) == int(ours_ordered),
           "binary": os.path.relpath(exe, ROOT)}
    if pr.returncode != 0:
        res["stderr_tail"] = pr.stderr[-400:]
    return res


def step_lower_bound(r, n: int, d: int, k: int, ms: float, peaks: dict) -> dict:
    """The whole step against its lower bound: T_lb = index bytes / HBM +
    max(join tensor flops / BF16, pair bytes / HBM), with 8d + s d + 3 (4k + 4)
    index bytes a point (FP64 read for the reference-point distances, one
    read in the join's dtype, key write plus one sort pass), 2 ceil16(d)
    tensor flops per candidate pair, 8 bytes per result pair."""
    hbm = peaks["hbm_gbs"] * 1e9
    bf16 = peaks["bf16_tflops"] * 1e12
    idx_bytes = n * (8 * d + 4 * d + 3 * (4 * k + 4))
    join_flops = r.candidates * 2.0 * ((d + 15) // 16 * 16)
    out_bytes = r.pairs_ij * 8.0
    t_lb = idx_bytes / hbm + max(join_flops / bf16, out_bytes / hbm)
    return {"t_lb_ms": t_lb * 1e3, "frac": t_lb * 1e3 / ms, "index_bytes": idx_bytes,
            "join_tensor_flops": join_flops, "pair_bytes": out_bytes,
            "model": "index bytes/HBM + max(2*ceil16(d) flops per candidate / BF16, 8 B per pair / HBM)"}


def run_tiny384_full(h, args, dev, stream, peaks) -> dict:
    """The 5M x 384 clustered FP32 workload in the same run: mixed precision
    at full size (args.tiny384_steps timed steps after one warm-up), then mixed
    precision, plain FP64 and TF32 on one full-density sample of home points
    (mistic_opts.home_sample, about 1.5e10 candidate pairs), pair sets
    compared on the device."""
    import torch
    from mistic import _lib as L
    t0 = time.perf_counter()
    wl = W.tiny384(args.tiny384_n or 5_000_000)
    gen_s = time.perf_counter() - t0
    x = np.ascontiguousarray(wl.pts)
    n, d = x.shape
    xt = torch.from_numpy(x).to(dev)
    del x
    torch.cuda.synchronize()

    def call(opts, m=n):
        return h.to_result(h.selfjoin_raw(xt.data_ptr(), m, d, L.F32, wl.k, wl.eps, opts))

    r0 = call(h.opts(input_on_device=True))
    cap = int(r0.pairs_ij * 1.02) + 1024
    pbuf = torch.empty((cap,), dtype=torch.int64, device=dev)
    o_dev = h.opts(input_on_device=True, pairs="device", pair_capacity=cap, pair_buffer=pbuf.data_ptr())
    call(o_dev)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    res = [call(o_dev) for _ in range(args.tiny384_steps)]
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.tiny384_steps
    r = res[-1]
    tc_ms = statistics.mean(q.ms["join_tc"] for q in res)
    kd = {"split-bf16": (d + 31) // 32 * 32, "bf16": (d + 63) // 64 * 64, "tf32": (d + 31) // 32 * 32}.get(
        r.tc_operands, d)
    products = 3 if r.tc_operands == "split-bf16" else 1
    tflops_2d = r.tc_cells * 2.0 * d / (tc_ms * 1e-3) / 1e12
    issued = r.tc_tiles * 128 * 128 * products * 2.0 * kd / (tc_ms * 1e-3) / 1e12
    tf32_scale = 2.0 if r.tc_operands == "tf32" else 1.0  # tf32 MMAs run at half the bf16 rate
    roof = {"bound": "tensor", "kernel": "k_join_tcw", "operands": r.tc_operands, "achieved": tflops_2d,
            "peak": peaks["bf16_tflops"], "unit": "TFLOP/s", "frac": tflops_2d / peaks["bf16_tflops"],
            "issued_tflops": issued, "issued_frac": issued * tf32_scale / peaks["bf16_tflops"],
            "kernel_ms": tc_ms, "cells": r.tc_cells,
            "work": "2*d flops per evaluated cell; issued = tiles x 128 x 128 x products x 2 x K"}
    # ---- the same full-density sample in every mode
    S = max(1, int(round(r.candidates / args.tiny384_sample_cands)))
    cap_s = max(1 << 20, int(r.pairs_ij / max(1, S) * 4) + 4096)
    bufs = {}
    out = {}
    for mode in ("auto", "fp64", "tf32"):
        bufs[mode] = torch.empty((cap_s,), dtype=torch.int64, device=dev)
        o = h.opts(input_on_device=True, pairs="device", pair_capacity=cap_s, pair_buffer=bufs[mode].data_ptr(),
                   sort_pairs=True, mode=mode, home_sample=S)
        torch.cuda.synchronize()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        q = call(o)
        a1.record(stream)
        torch.cuda.synchronize()
        out[mode] = (q, a0.elapsed_time(a1))
    qa, qf, qt = out["auto"][0], out["fp64"][0], out["tf32"][0]
    same = (qa.pairs_ij == qf.pairs_ij == qt.pairs_ij and
            bool(torch.equal(bufs["auto"][:qa.pairs_ij], bufs["fp64"][:qf.pairs_ij])) and
            bool(torch.equal(bufs["tf32"][:qt.pairs_ij], bufs["fp64"][:qf.pairs_ij])))
    fp64_full_ms = qf.ms["join"] * r.candidates / max(1, qf.candidates) + (r.ms["total"] - r.ms["join"])
    line = {
        "workload": "tiny384", "n": n, "d": d, "k": wl.k, "eps_hex": float(wl.eps).hex(),
        "desc": WORKLOADS["tiny384"][1], "generation_s": gen_s,
        "steps": args.tiny384_steps, "warmup": 1, "ms_per_step": ms, "value": n / (ms * 1e-3), "unit": UNIT,
        "mode_used": r.mode_used, "tc_operands": r.tc_operands, "tc_kernel": r.tc_kernel,
        "tc_min_bin": r.tc_min_bin, "tuned": r.tuned,
        "pairs_ij": r.pairs_ij, "candidates": r.candidates, "band_pairs": r.band_pairs,
        "band_fraction": r.band_pairs / max(1, r.candidates), "ulp_ambiguous": r.ulp_ambiguous,
        "distance_evals_per_s": r.candidates / (ms * 1e-3), "pairs_per_s": r.pairs_ij / (ms * 1e-3),
        "phase_ms": {k2: round(v, 3) for k2, v in r.ms.items()},
        "bins": r.n_bins, "units": r.n_units, "units_tc": r.n_units_tc, "tc_tiles": r.tc_tiles,
        "tc_min_bin": r.tc_min_bin, "tuned": r.tuned,
        "roofline": roof,
        "sample": {
            "home_sample": S, "candidates": qf.candidates, "pairs_ij": qf.pairs_ij,
            "identical_pair_set_mixed_fp64_tf32": same,
            "mixed": {"join_ms": qa.ms["join"], "step_ms": out["auto"][1], "band_pairs": qa.band_pairs,
                      "tc_operands": qa.tc_operands},
            "fp64": {"join_ms": qf.ms["join"], "step_ms": out["fp64"][1]},
            "tf32": {"join_ms": qt.ms["join"], "step_ms": out["tf32"][1], "band_pairs": qt.band_pairs,
                     "band_fraction": qt.band_pairs / max(1, qt.candidates)},
            "mixed_vs_fp64_join": qf.ms["join"] / max(1e-9, qa.ms["join"]),
            "note": "home points of about 1 in S groups of 512 sorted points per bin, each joined with all "
                    "its candidates, identical in every mode; join_ms from the library's CUDA events"},
        "fp64_full_ms_extrapolated": fp64_full_ms,
        "mixed_vs_fp64_full_step": fp64_full_ms / ms,
    }
    del xt, pbuf, bufs
    torch.cuda.empty_cache()
    return line


def run_batch(args) -> None:
    """The batch: 2,000 independent instances (n log-uniform in [1e3, 2e5], d in
    {2,8,18,32,57,90}, FP32 Gaussian mixtures) through one
    mistic_batch_selfjoin call per step.  value: inputs resident in HBM,
    counts only; e2e: host inputs and host pair lists.  The batch call is
    synchronous and spreads instances over worker streams, so a step is timed
    by the host clock between two device synchronisations."""
    import torch
    import mistic
    from mistic import _lib as L

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    count = args.n or 2000
    t_gen = time.perf_counter()
    wls = W.batch_instances_device(count=count, device=f"cuda:{local}")
    t_gen = time.perf_counter() - t_gen
    h = mistic.Handle(local)
    m = len(wls)
    xs = [np.ascontiguousarray(w.pts) for w in wls]
    xts = [torch.from_numpy(x).to(dev) for x in xs]
    torch.cuda.synchronize()
    inst_h, inst_d = (L.Instance * m)(), (L.Instance * m)()
    for i, (w, x, xt) in enumerate(zip(wls, xs, xts)):
        for arr, ptr in ((inst_h, x.ctypes.data), (inst_d, xt.data_ptr())):
            arr[i].pts, arr[i].n, arr[i].d = ptr, x.shape[0], x.shape[1]
            arr[i].dtype, arr[i].k, arr[i].eps = L.F32, w.k, float(w.eps)
    tot_n = sum(x.shape[0] for x in xs)

    def batch(inst, opts):
        res = (L.Result * m)()
        st = h.lib.mistic_batch_selfjoin(h.h, inst, m, ctypes.byref(opts), res)
        mistic._check(h.lib, h.h, st)
        out = [(int(r.pairs_ij), int(r.kernel_launches), int(r.candidates)) for r in res]
        for i in range(m):
            h.lib.mistic_result_free(ctypes.byref(res[i]))
        return out

    def timed(inst, opts, steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        outs = [batch(inst, opts) for _ in range(steps)]
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) * 1e3 / steps, outs[-1]

    o_cnt = h.opts(input_on_device=True, mode=args.mode)
    for _ in range(args.warmup):
        batch(inst_d, o_cnt)
    clocks = ClockSampler()
    clocks.start()
    ms, res = timed(inst_d, o_cnt, args.steps)
    clk = clocks.stop()
    # the same batch with one pipeline per instance: on 8 worker streams, and
    # one instance after another (one launch of each join kernel per instance)
    os.environ["MISTIC_BATCH_FUSED"] = "0"
    batch(inst_d, o_cnt)
    streams_ms, res_s = timed(inst_d, o_cnt, 1)
    os.environ["MISTIC_BATCH_STREAMS"] = "1"
    serial_ms, _ = timed(inst_d, o_cnt, 1)
    del os.environ["MISTIC_BATCH_STREAMS"]
    del os.environ["MISTIC_BATCH_FUSED"]
    counts_same = [p[0] for p in res] == [p[0] for p in res_s]
    o_host = h.opts(pairs="host", mode=args.mode)
    batch(inst_h, o_host)
    e2e_ms, _ = timed(inst_h, o_host, args.steps)

    parity = None
    if not args.no_fp64:
        f_ms, res64 = timed(inst_d, h.opts(input_on_device=True, mode="fp64"), 1)
        from oracle import oracle as O
        small = sorted(range(m), key=lambda i: xs[i].shape[0])[:20]
        ok = True
        for i in small:
            r = h.selfjoin(xs[i], wls[i].k, wls[i].eps, pairs="host", sort_pairs=True, mode=args.mode)
            ok &= bool(np.array_equal(r.pairs, O.brute_pairs(xs[i], wls[i].eps)))
        parity = {"fp64_batch_ms": f_ms, "counts_identical_to_fp64": [p[0] for p in res] == [p[0] for p in res64],
                  "oracle_pair_sets_identical": ok, "oracle_instances": len(small)}
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu:
        # brute force on a row sample of 8 instances; the n^2 d cost model
        # scales it to the whole batch
        from oracle import oracle as O
        threads = O.max_threads()
        t_s, cost_s = 0.0, 0.0
        for i in list(range(0, m, max(1, m // 8)))[:8]:
            x = xs[i]
            rows = min(x.shape[0], max(256, int(args.cpu_seconds * 2e9 / 8 / max(1, x.shape[0] * x.shape[1]))))
            t0 = time.perf_counter()
            O.count_rows(x, wls[i].eps, 0, rows, threads)
            t_s += time.perf_counter() - t0
            cost_s += rows * x.shape[0] * x.shape[1]
        job_s = t_s * sum(x.shape[0] ** 2 * x.shape[1] for x in xs) / cost_s
        cpu = {"value": tot_n / job_s, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"row samples of 8 instances ({t_s:.1f} s), scaled by sum n^2 d to all {m}; "
                         "brute_force of src/utils.cu:285-317 (oracle C port, OpenMP)"}
    pairs = sum(p[0] for p in res)
    # the whole fused step against the tensor peak: 2*d flops per candidate
    # pair, summed over the instances (their joins run on the short-row
    # tensor-core kernel and the FP32 filter, so the FP32 CUDA-core peak is
    # given beside it)
    peaks = load_peaks()
    work = sum(2.0 * x.shape[1] * p[2] for x, p in zip(xs, res))
    achieved = work / (ms * 1e-3) / 1e12
    fp32_peak = measure_fp32_peak()
    roof = {"bound": "tensor", "kernel": "fused batch join (all join kernels of the step)", "achieved": achieved,
            "peak": peaks["bf16_tflops"], "unit": "TFLOP/s", "frac": achieved / peaks["bf16_tflops"],
            "traffic": None, "work": "2*d flops per candidate pair, summed over the instances; whole step time",
            "peak_source": peaks["_source"] + " bf16 burst (of measured)",
            "fp32_simt_peak_tflops": fp32_peak,
            "frac_of_fp32_simt": achieved / fp32_peak if fp32_peak else None}
    line = {
        "metric": METRIC, "value": world * tot_n / (ms * 1e-3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "batch2000", "instances": m, "points": tot_n,
                   "desc": "2,000 instances, n log-uniform [1e3,2e5], d in {2,8,18,32,57,90}, FP32 "
                           "Gaussian mixtures, 4/16/64 mean neighbours", "mode": args.mode,
                   "parallelism": "replicas" if world > 1 else "single",
                   "streams": "index builds on worker handles; the join of all instances fused into one "
                              "persistent launch per (kernel, d) class, captured as one CUDA graph",
                   "pairs_to": "counts only",
                   "timing": "host clock around the synchronous batch call, device synchronised",
                   "l2": f"inputs {sum(x.nbytes for x in xs) / 1e9:.1f} GB in total"},
        "pairs_ij": pairs, "candidates": sum(p[2] for p in res),
        "per_instance_streams_ms_per_step": streams_ms, "per_instance_serial_ms_per_step": serial_ms,
        "fused_vs_serial": serial_ms / ms, "fused_vs_streams": streams_ms / ms,
        "counts_identical_fused_vs_per_instance": counts_same,
        "generation_s": t_gen, "parity": parity,
        "roofline": roof,
        "e2e": {"value": world * tot_n / (e2e_ms * 1e-3), "unit": UNIT, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": sum(x.nbytes for x in xs), "d2h_bytes_per_step": pairs * 8},
        "gpu_launches": sum(p[1] for p in res),
        "clocks": clk,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    h.close()


_FP32_PEAK = None


def measure_fp32_peak() -> float | None:
    """CUDA-core FP32 FFMA peak of this GPU from the mistic_peaks probe."""
    global _FP32_PEAK
    if _FP32_PEAK is not None:
        return _FP32_PEAK
    from mistic import build as B
    try:
        out = subprocess.run([B.PEAKS], capture_output=True, text=True, timeout=120).stdout
        _FP32_PEAK = float(json.loads(out.strip().splitlines()[-1])["fp32_tflops"])
    except Exception:
        _FP32_PEAK = None
    return _FP32_PEAK


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["mistic", "reference"], default="mistic")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["batch2000"], default="susy18")
    ap.add_argument("--n", "--points", dest="n", type=int, default=0,
                    help="override the point count (testing; --points under torchrun, whose parser takes --n)")
    ap.add_argument("--k", type=int, default=0, help="override the reference-point count (testing)")
    ap.add_argument("--mode", choices=["auto", "fp32", "bf16", "fp64"], default="auto",
                    help="join mode of the timed steps")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison")
    ap.add_argument("--fp64-rows", type=int, default=0,
                    help="time the plain FP64 comparison on the first N rows only (0: all rows)")
    ap.add_argument("--verify-rows", type=int, default=-1,
                    help="check the neighbour counts of this many rows against the GPU FP64 brute force "
                         "(default: 16,384 where n * d <= 2e8, else none)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-tiny384", action="store_true", help="skip the nested 5M x 384 measurement")
    ap.add_argument("--tiny384-n", type=int, default=0, help="points of the nested 5M x 384 workload (default 5,000,000)")
    ap.add_argument("--tiny384-steps", type=int, default=2, help="timed full-size steps of the nested 5M x 384 workload")
    ap.add_argument("--tiny384-sample-cands", type=float, default=1.5e10,
                    help="candidate pairs of the nested 5M x 384 workload's mixed/FP64 sample")
    ap.add_argument("--ref-seconds", type=float, default=6.0)
    ap.add_argument("--ref-gpu", action="store_true",
                    help="also run the reference's own GPU build (oracle/build_ref_gpu.sh) on the same points")
    ap.add_argument("--ref-gpu-timeout", type=float, default=900.0)
    args = ap.parse_args()
    if args.workload == "batch2000":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference arm times the single-instance "
                              "workloads; the batch reports its CPU baseline in the mistic line"}), flush=True)
        else:
            run_batch(args)
        return
    wl = WORKLOADS[args.workload][0](args.n)
    if args.k:
        wl.k = args.k
    if args.impl == "reference":
        run_reference(args, wl)
    else:
        run_mistic(args, wl)


if __name__ == "__main__":
    main()
