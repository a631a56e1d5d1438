#!/usr/bin/env python
"""Benchmark of the FPS hot path on one GB300 (one JSON line on stdout).

Workload (default "batched-256"): 256 seeded synthetic clouds, N log-uniform
in [1,024, 131,072], D=3 uniform in a box with a per-cloud per-axis scale in
[0.1, 10], K = N // 4, start_idx 0, QuickFPS (bucket_fps_kdline) with the
tree height picked per size class.  One step = all 256 clouds sampled.

  value   clouds/s with every cloud already resident in HBM (device entry
          point), L2 flushed before each step, timed with CUDA events on the
          launching stream; max over ranks.
  e2e     clouds/s through the public drop-in API from host numpy arrays
          (fpsample.bucket_fps_kdline_sampling / fps_sampling), host<->device
          copies inside the timed region; one-cloud workloads add where the
          end-to-end time goes (e2e_phases).
  roofline  the sampling kernel: algorithmic bytes per launch -- kd-line:
          sum over clouds of 2^h (8D+8) (K-1) B of bucket records plus the
          running distances recomputed (device counter) x (4D+8) B; vanilla:
          N (K-1) (4D+8) B -- over its event-timed average launch duration,
          against the measured HBM copy bandwidth (frac), and the measured L2
          and shared-memory read bandwidths (frac_l2, frac_smem); actual_* are
          the bytes the pruned sampler really touches.
  bit_exact  every sample of every cloud of the timed step against the
          reference's answer: the full-size fixtures (tests/golden/fullsize.npz)
          for the one-cloud benchmark sizes, else the oracle.
  cpu_baseline  the reference compiled from its own sources on this host (the
          oracle port where that build is absent) on a bounded sample, 1 core.

Other workloads (--workload), each one of the reference's configurations:
  gmm-1m            one 1,048,576-point Gaussian-mixture cloud, kd-line h=7,
                    K=16,384
  gmm-1m-vanilla    the same cloud, vanilla FPS
  single-4k         vanilla FPS, 4,096 uniform points, K=1,024
  large-16m         16,777,216 points, D=6, kd-line h=9, K=65,536
  large-16m-vanilla the same cloud, vanilla FPS
  served            a Poisson request stream into the request server
Where the reference cannot finish a cloud in seconds (the 1M-point vanilla
and 16.7M-point clouds), the CPU numbers come from two truncated runs
extrapolated linearly in K (said so in the line).

--impl reference runs the reference's CPU implementation of the same path on
all host cores (rank 0 only) and prints the same metric.  The reference is
single-threaded per cloud, so a one-cloud workload uses one core.  Both arms
use the floating-point mode of the host's stock reference build.
Multi-GPU (torchrun): replicas only -- every rank samples its own copy of the
batch; value = all clouds / max step time over ranks ("weak" scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# 32 hardware work queues (default 8) before anything touches CUDA: the request
# server's worker streams must not share queues (a small batch would wait
# behind a large batch's kernel in the same queue)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = "clouds/sec"
UNIT = "clouds/s"
L2_FLUSH_BYTES = 256 << 20


def h_for(n: int) -> int:
    """Tree height by size class (the reference README's guidance: h=5 for small
    clouds, 7 for medium, 9 for large)."""
    if n < 8192:
        return 5
    if n < 262144:
        return 7
    return 9


WORKLOADS = ["batched-256", "gmm-1m", "gmm-1m-vanilla", "single-4k", "large-16m",
             "large-16m-vanilla", "served"]


class Workload:
    """algo: "kdline" or "vanilla"; clouds: [(points, k, h, start)]."""

    def __init__(self, name, algo, clouds):
        self.name, self.algo, self.clouds = name, algo, clouds
        self.dim = int(clouds[0][0].shape[1])


def workload(name: str) -> Workload:
    import workloads as W

    if name == "batched-256":
        clouds = W.batched_clouds(seed=W.SEEDS["batched-256"])
        return Workload(name, "kdline", [(p, k, h_for(p.shape[0]), 0) for p, k in clouds])
    if name in ("gmm-1m", "gmm-1m-vanilla"):
        p = W.gmm_cloud(1 << 20, seed=W.SEEDS["gmm-1m"])
        return Workload(name, "vanilla" if name.endswith("vanilla") else "kdline", [(p, 16384, 7, 0)])
    if name == "single-4k":
        p = W.uniform_cloud(4096, 3, seed=W.SEEDS["single-4k"])
        return Workload(name, "vanilla", [(p, 1024, 5, 0)])
    if name in ("large-16m", "large-16m-vanilla"):
        p = W.large_cloud(1 << 24, seed=W.SEEDS["large-16m"])
        return Workload(name, "vanilla" if name.endswith("vanilla") else "kdline", [(p, 65536, 9, 0)])
    raise ValueError(name)


def truncated_k(algo: str, n: int, k: int):
    """None when the oracle finishes (n, k) in seconds; else the smaller K of
    the two truncated runs (the other is twice as many samples)."""
    if algo == "vanilla" and n * k > 5e8:
        return max(8, min(k // 4, int(2e8 // n)))
    if algo == "kdline" and n > (4 << 20):
        return min(k // 4, 128)
    return None


def max_over_ranks(x: float, world: int, device) -> float:
    """The largest x over all ranks (the step time of the slowest replica)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(units_per_rank: int, world: int, seconds: float) -> float:
    """Whole-job throughput of N replicas: every rank processes its own copy of
    the workload, the job lasts as long as the slowest rank."""
    return units_per_rank * world / seconds


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


class ClockSampler:
    def __init__(self, gpu_index: int):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={CLOCK_FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# CPU side: oracle / reference
# ---------------------------------------------------------------------------
def fp_mode() -> str:
    """The distance arithmetic both arms run: FPSAMPLE_FP_MODE, else the mode
    of the reference's stock build on this host ("fma" on aarch64, where GCC
    contracts a*b+c by default; "nofma" on x86-64).  The GPU library picks the
    same default by itself; the reference arm must not import it."""
    import platform

    m = os.environ.get("FPSAMPLE_FP_MODE", "").lower()
    if m in ("fma", "nofma"):
        return m
    return "fma" if platform.machine() in ("aarch64", "arm64") else "nofma"


def _cpu_impl():
    """('reference', module) when the reference compiled from its own sources
    (oracle/_ref, built for this host by `make -C oracle ref`) is importable
    here, else ('port', Oracle): the C restatement."""
    from oracle import oracle as O

    if O.reference_available(fp_mode()):
        return "reference", O.load_reference(fp_mode())
    return "port", O.Oracle()


def _cpu_run(impl, obj, algo, pts, k, h, start):
    if algo == "vanilla":
        if impl == "reference":
            return obj.fps_sampling(pts, k, start)
        return obj.fps(pts, k, start, fp_mode())
    if impl == "reference":
        return obj.bucket_fps_kdline_sampling(pts, k, h, start)
    return obj.kdline(pts, k, h, start, fp_mode())


def _cpu_describe(impl: str) -> str:
    from oracle import oracle as O

    if impl == "reference":
        return (f"the reference's own src/lib.cpp compiled on this host ({fp_mode()} build: "
                f"{O.reference_build_flags(fp_mode())})")
    return f"the oracle port oracle/fps_oracle.c ({fp_mode()} arithmetic)"


def _cpu_cloud_seconds(impl, obj, algo, p, k, h, s):
    """(seconds for one cloud, how it was obtained): measured, or extrapolated
    linearly in K from two truncated runs."""
    kt = truncated_k(algo, p.shape[0], k)
    if kt is None:
        t0 = time.perf_counter()
        _cpu_run(impl, obj, algo, p, k, h, s)
        return time.perf_counter() - t0, None
    t = []
    for kk in (kt, 2 * kt):
        t0 = time.perf_counter()
        _cpu_run(impl, obj, algo, p, kk, h, s)
        t.append(time.perf_counter() - t0)
    est = t[0] + (t[1] - t[0]) * (k - kt) / kt
    return est, f"K={kt} and K={2 * kt} timed ({t[0]:.2f} s, {t[1]:.2f} s), extrapolated linearly to K={k}"


_W = {}


def _worker_init(name):
    sys.path.insert(0, ROOT)
    _W["wl"] = workload(name)
    _W["impl"], _W["obj"] = _cpu_impl()


def _worker_run(i):
    wl = _W["wl"]
    p, k, h, s = wl.clouds[i % len(wl.clouds)]
    return _cpu_cloud_seconds(_W["impl"], _W["obj"], wl.algo, p, k, h, s)


def cpu_baseline(wl: Workload, budget_s: float = 12.0):
    impl, obj = _cpu_impl()
    t0 = time.perf_counter()
    done = 0
    pts_done = 0
    secs = 0.0
    how = None
    for p, k, h, s in wl.clouds:
        dt, how = _cpu_cloud_seconds(impl, obj, wl.algo, p, k, h, s)
        secs += dt
        done += 1
        pts_done += p.shape[0]
        if time.perf_counter() - t0 > budget_s:
            break
    sample = (f"first {done} of {len(wl.clouds)} clouds ({pts_done} points), one thread, "
              f"{secs:.1f} s of {wl.algo} on {_cpu_describe(impl)}")
    if how:
        sample += f"; {how}"
    return {"value": done / secs, "unit": UNIT, "cores": 1, "kind": impl, "sample": sample}


def run_reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp

    wl = workload(args.workload)
    clouds = wl.clouds
    impl, _ = _cpu_impl()
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    # the reference samples one cloud on one thread: a one-cloud workload
    # cannot use more than one core
    copies = 1
    cores = min(cores, len(clouds))
    # largest clouds first so that the pool drains evenly
    order = sorted(range(len(clouds) * copies),
                   key=lambda i: -clouds[i % len(clouds)][0].shape[0] * clouds[i % len(clouds)][1])
    big = any(truncated_k(wl.algo, p.shape[0], k) for p, k, _, _ in clouds)
    warmup = 1 if big else args.warmup
    steps = 1 if big else args.steps
    how = None
    with ctx.Pool(cores, initializer=_worker_init, initargs=(args.workload,)) as pool:
        for _ in range(warmup):
            list(pool.imap_unordered(_worker_run, order))
        times = []
        for _ in range(steps):
            t0 = time.perf_counter()
            out = list(pool.imap_unordered(_worker_run, order))
            wall = time.perf_counter() - t0
            how = next((h for _, h in out if h), None)
            # a truncated run stands for the whole cloud: the step lasts as
            # long as the busiest core's extrapolated work
            times.append(max(wall, max(sec for sec, _ in out)) if how else wall)
    step = statistics.mean(times)
    v = len(clouds) * copies / step
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generators)",
            "config": config_of(wl),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": impl,
                             "sample": f"{copies} cop{'y' if copies == 1 else 'ies'} of all "
                                       f"{len(clouds)} clouds per step, {cores} processes, "
                                       f"{wl.algo} on {_cpu_describe(impl)}"
                                       + (f"; per cloud: {how}" if how else "")},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _gen_points(job):
    """Writes request i's cloud (from its own seed) to folder/i.npy."""
    import workloads as W

    i, n, seed, folder = job
    np.save(os.path.join(folder, f"{i}.npy"), W.sphere_cloud(np.random.default_rng(seed), n))
    return i


def _scratch_dir():
    return "/dev/shm" if os.path.isdir("/dev/shm") else None


def served_requests(window_s: float):
    """The first window_s seconds of the served stream (2000 requests/s)."""
    import workloads as W

    return list(W.request_stream(rate=2000.0, duration_s=window_s, seed=W.SEEDS["served"]))


def admitted_requests(rho: float, samples_per_s: float):
    """The whole 10 s stream thinned at random (a seeded coin per request) so
    that the samples it offers per second are rho x samples_per_s: an admitted
    load the server can sustain."""
    import workloads as W

    reqs = list(W.request_stream(rate=2000.0, duration_s=10.0, seed=W.SEEDS["served"]))
    offered = sum(r.k for r in reqs) / 10.0
    keep = min(1.0, rho * samples_per_s / offered)
    coin = np.random.default_rng(W.SEEDS["served"] + 1000).random(len(reqs))
    return [r for r, c in zip(reqs, coin) if c < keep], keep


def materialize(reqs, folder):
    """Every request's points, generated in parallel from the requests' seeds
    (spawned processes, so this may run after CUDA is initialised)."""
    import multiprocessing as mp

    jobs = sorted(((i, r.n, r.seed, folder) for i, r in enumerate(reqs)), key=lambda j: -j[1])
    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        for _ in pool.imap_unordered(_gen_points, jobs):
            pass
    pts = []
    for i in range(len(reqs)):
        f = os.path.join(folder, f"{i}.npy")
        pts.append(np.load(f))
        os.unlink(f)
    return pts


def _served_worker_init():
    sys.path.insert(0, ROOT)
    _W["impl"], _W["obj"] = _cpu_impl()


def _served_worker_run(job):
    import workloads as W

    i, n, seed, k, h, s = job
    pts = W.sphere_cloud(np.random.default_rng(seed), n)
    t0 = time.perf_counter()
    _cpu_run(_W["impl"], _W["obj"], "kdline", pts, k, h, s)
    return i, time.perf_counter() - t0


def _latency_summary(reqs, lat, queue, wall):
    small = np.array([r.n <= 65536 for r in reqs])
    pct = lambda x, q: float(np.percentile(x, q)) if len(x) else None
    return {
        "requests": len(reqs), "requests_per_s": len(reqs) / wall,
        "samples_per_s": sum(r.k for r in reqs) / wall, "wall_s": wall,
        "latency_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99), "max": float(lat.max())},
        "latency_ms_n_le_65536": {"p50": pct(lat[small], 50), "p99": pct(lat[small], 99),
                                  "count": int(small.sum())},
        "queue_ms": {"p50": pct(queue, 50), "p99": pct(queue, 99)},
    }


def run_served_reference(args):
    """The served workload on the reference's CPU path: every request of the
    same replayed window is sampled once on the host cores (one process per
    core, the reference samples a cloud on one thread) and its time measured;
    the requests are then served first come, first served by that many cores
    at their arrival times, which gives requests/s and the latency
    percentiles of the GPU line."""
    rank, _, _ = dist_env()
    if rank != 0:
        return
    import heapq
    import multiprocessing as mp

    reqs = served_requests(args.served_window)
    impl, _ = _cpu_impl()
    cores = min(os.cpu_count() or 1, len(reqs))
    jobs = sorted(((i, r.n, r.seed, r.k, h_for(r.n), r.start) for i, r in enumerate(reqs)),
                  key=lambda j: -j[1] * j[3])
    with mp.get_context("spawn").Pool(cores, initializer=_served_worker_init) as pool:
        service = dict(pool.imap_unordered(_served_worker_run, jobs))
    free = [0.0] * cores  # first come, first served on `cores` servers
    lat, queue = [], []
    for i, r in enumerate(reqs):
        t = heapq.heappop(free)
        start = max(t, r.arrival_s)
        done = start + service[i]
        heapq.heappush(free, done)
        lat.append((done - r.arrival_s) * 1e3)
        queue.append((start - r.arrival_s) * 1e3)
    wall = max(free)
    summ = _latency_summary(reqs, np.array(lat), np.array(queue), wall)
    v = summ["requests_per_s"]
    line = {
        "impl": "reference", "metric": "requests/sec (served)", "value": v, "unit": "requests/s",
        "n_gpus": 0, "higher_is_better": True, "data": "synthetic (seeded generators)",
        "config": {"workload": "served", "offered_rate_per_s": 2000, "window_s": args.served_window,
                   "requests": len(reqs), "points_total": int(sum(r.n for r in reqs)),
                   "samples_total": int(sum(r.k for r in reqs)), "fp_mode": fp_mode()},
        **{k: summ[k] for k in ("latency_ms", "latency_ms_n_le_65536", "queue_ms",
                                "samples_per_s", "wall_s")},
        "cpu_baseline": {"value": v, "unit": "requests/s", "cores": cores, "kind": impl,
                         "sample": f"every request of the {args.served_window} s window timed once "
                                   f"on {cores} processes ({_cpu_describe(impl)}), served first "
                                   f"come first served by {cores} cores at the arrival times"},
        "e2e": {"value": v, "unit": "requests/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def config_of(wl: Workload):
    name, clouds = wl.name, wl.clouds
    ns = [p.shape[0] for p, _, _, _ in clouds]
    return {"workload": name, "algo": wl.algo, "n_clouds": len(clouds),
            "points_total": int(sum(ns)),
            "samples_total": int(sum(k for _, k, _, _ in clouds)), "dim": wl.dim,
            "k": "N//4" if name == "batched-256" else int(clouds[0][1]),
            "h": ("size class: 5 (<8K), 7 (<256K), 9" if name == "batched-256"
                  else (clouds[0][2] if wl.algo == "kdline" else None)),
            "start_idx": 0, "l2": "flushed before every step (256 MiB write)",
            "fp_mode": fp_mode(), "parallelism": "replicas"}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def _peaks():
    """(HBM GB/s and where it comes from, on-chip peaks {smem_gbs, l2_gbs})."""
    try:
        hbm = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
        src = "MEASURED_PEAKS.json hbm_gbs (of measured)"
    except (OSError, KeyError, ValueError):
        hbm, src = 6800.0, "fallback 6800 GB/s (of fallback)"
    try:
        onchip = json.load(open(os.path.join(ROOT, "profiles", "peaks.json")))
    except (OSError, ValueError):
        onchip = {}
    return hbm, src, onchip


def roofline(wl: Workload, st: dict, steps: int, step_ms: float):
    """The sampling kernel's roofline line and the vanilla-equivalent bytes.

    Algorithmic bytes per launch (one launch samples every cloud of a step):
      kd-line  sum over clouds of 2^h (8D + 8) (K - 1) B of bucket records
               (box and max key of every bucket, once per sample) plus the
               running distances recomputed x (4D + 8) B (coordinates, old and
               new distance), the recomputed count taken from the device
               counter, not assumed;
      vanilla  N (K - 1) (4D + 8) B per cloud: every point read and its
               running distance read and written once per sample.
    achieved = those bytes / the kernel's average event-timed launch time,
    against the measured HBM copy bandwidth; frac_l2 / frac_smem put the same
    figure against the measured on-chip read bandwidths.  The pruned sampler
    does not move all of these bytes: actual_* counts what it touches (boxes
    tested x (8D + 8) + distances recomputed x (4D + 8))."""
    d = wl.dim
    launches = max(1, st["sampler_launches"])
    launch_ms = st["sampler_ms"] / launches
    per_step = launches / max(1, steps)  # sampler launches per step
    touched = st["points_touched"] / launches
    tested = st["pieces_tested"] / launches
    if wl.algo == "kdline":
        alg = sum((2 ** h) * (8 * d + 8) * (k - 1) for _, k, h, _ in wl.clouds) / per_step \
            + touched * (4 * d + 8)
        rule = "sum 2^h (8D+8)(K-1) + recomputed distances x (4D+8)"
    else:
        alg = sum(p.shape[0] * (k - 1) * (4 * d + 8) for p, k, _, _ in wl.clouds) / per_step
        rule = "N (K-1) (4D+8)"
    actual = tested * (8 * d + 8) + touched * (4 * d + 8)
    hbm, src, onchip = _peaks()
    sec = launch_ms / 1e3
    achieved = alg / sec / 1e9 if sec > 0 else None
    act_gbs = actual / sec / 1e9 if sec > 0 else None
    samples = sum(k for _, k, _, _ in wl.clouds) / per_step
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm if achieved else None, "kernel": "sampler",
            "alg_bytes_per_launch": alg, "alg_bytes_rule": rule, "launch_ms": launch_ms,
            "peak_source": src,
            "frac_l2": achieved / onchip["l2_gbs"] if achieved and onchip.get("l2_gbs") else None,
            "frac_smem": (achieved / onchip["smem_gbs"]
                          if achieved and onchip.get("smem_gbs") else None),
            "onchip_peaks_source": "profiles/peaks.json (bench.py --probe peaks)" if onchip else None,
            "actual_bytes_per_launch": actual, "actual_gbs": act_gbs,
            "actual_frac": act_gbs / hbm if act_gbs else None,
            "boxes_tested_per_sample": tested / samples if samples else None,
            "distances_recomputed_per_sample": touched / samples if samples else None}
    veq = None
    if wl.algo == "vanilla":
        b = sum(p.shape[0] * (k - 1) * (4 * d + 8) for p, k, _, _ in wl.clouds)
        veq = {"bytes_per_step": b, "gbs_whole_step": b / (step_ms / 1e3) / 1e9}
    return roof, veq


def _check_worker(job):
    from oracle.oracle import Oracle

    i, algo, p, k, h, s, mode = job
    orc = _W.get("orc") or _W.setdefault("orc", Oracle())
    want = orc.fps(p, k, s, mode) if algo == "vanilla" else orc.kdline(p, k, h, s, mode)
    return i, want


def check_step(wl: Workload, res, koffs, mode: str):
    """(all equal, what was checked): the GPU's complete output for the step
    against the reference answers -- the committed full-size fixtures
    (tests/golden/fullsize.npz) for the one-cloud benchmark sizes, else the
    oracle on every cloud (a process pool, outside the timed region)."""
    from tests.golden import fullsize as F

    case = F.BY_WORKLOAD.get(wl.name)
    if case and F.available():
        c = F.case(case)
        if not F.input_matches(c["cloud"], wl.clouds[0][0]):
            return False, f"input differs from the fixture's {c['cloud']} cloud (sha256)"
        want = F.expected(case, mode)
        ok = bool(np.array_equal(res[: len(want)], want)) and len(res) == len(want)
        return ok, (f"all {len(want)} samples against tests/golden/fullsize.npz "
                    f"{case}__{mode} (source: {c['source']})")
    import multiprocessing as mp

    jobs = [(i, wl.algo, p, k, h, s, mode) for i, (p, k, h, s) in enumerate(wl.clouds)]
    jobs.sort(key=lambda j: -j[2].shape[0] * j[3])
    ok = True
    procs = max(1, min(len(jobs), os.cpu_count() or 1))
    with mp.get_context("spawn").Pool(procs) as pool:
        for i, want in pool.imap_unordered(_check_worker, jobs):
            ok &= bool(np.array_equal(res[koffs[i]:koffs[i + 1]], want))
    return ok, f"all {len(jobs)} clouds, every sample, against the oracle ({mode})"


def run_gpu_arm(args):
    import torch
    import torch.distributed as dist

    import fpsample as fps
    from fpsample_gb300 import capi

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()

    wl = workload(args.workload)
    clouds = wl.clouds
    D = wl.dim
    # inputs resident in HBM: one buffer, per-cloud views
    sizes = [p.shape[0] for p, _, _, _ in clouds]
    offs = np.concatenate([[0], np.cumsum(sizes)])
    host_all = np.concatenate([p for p, _, _, _ in clouds]).astype(np.float32)
    d_all = torch.from_numpy(host_all).to(dev)
    ks = [k for _, k, _, _ in clouds]
    koffs = np.concatenate([[0], np.cumsum(ks)])
    d_out = torch.empty(int(koffs[-1]), dtype=torch.int64, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    base_pts = d_all.data_ptr()
    base_out = d_out.data_ptr()
    sptr = stream.cuda_stream

    hs = [h for _, _, h, _ in clouds]
    ss = [s for _, _, _, s in clouds]

    def step_plain():
        # the plain form: one GPU call per cloud
        for i, (p, k, h, s) in enumerate(clouds):
            if wl.algo == "vanilla":
                capi.fps_device(base_pts + int(offs[i]) * 4 * D, sizes[i], D, k, [s],
                                base_out + int(koffs[i]) * 8, 0, sptr)
            else:
                capi.kdline_device(base_pts + int(offs[i]) * 4 * D, sizes[i], D, k, s, h,
                                   base_out + int(koffs[i]) * 8, 0, sptr)

    def step_device():
        if wl.algo == "vanilla":
            step_plain()  # vanilla has no batched entry point: one call per cloud
        else:
            # the batched engine: every cloud in one call
            capi.kdline_batch_device(base_pts, offs, D, ks, hs, ss, base_out, sptr)

    pcs = [p for p, _, _, _ in clouds]

    def step_e2e():
        if wl.algo == "vanilla":
            for p, k, _, s in clouds:
                fps.fps_sampling(p, k, s)
        elif len(clouds) == 1:
            fps.bucket_fps_kdline_sampling(pcs[0], ks[0], hs[0], ss[0])
        else:
            fps.bucket_fps_kdline_sampling_batch(pcs, ks, hs, ss)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    # correctness of what is timed, outside the timed region: every cloud of
    # the step, every sample, against its reference answer
    step_device()
    torch.cuda.synchronize()
    res = d_out.cpu().numpy().astype(np.uint64)
    bit_exact, checked = check_step(wl, res, koffs, fps.get_fp_mode())

    for _ in range(args.warmup):
        flush.zero_()
        step_device()
    barrier()

    capi.stats_reset()
    capi.stats_timing(True)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        barrier()
        t_wall = time.perf_counter()
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            step_device()
            ev[i][1].record(stream)
        barrier()
        t_wall = time.perf_counter() - t_wall
    capi.stats_timing(False)
    st = capi.stats()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms = max_over_ranks(statistics.mean(step_ms), world, dev)
    value = job_value(len(clouds), world, ms / 1e3)

    # e2e through the public API (host arrays, copies inside the timed region)
    e2e_steps = max(1, min(args.steps, 3))
    step_e2e()
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        step_e2e()
    barrier()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, world, dev)
    e2e_v = job_value(len(clouds), world, e2e_s)
    # where the end-to-end time goes beyond the device step: the host->device
    # copy of the same host arrays (pageable numpy memory, as the public API
    # receives them) and the indices back, each timed alone
    phases = None
    if len(clouds) == 1:
        ht = []
        for _ in range(e2e_steps):
            barrier()
            t1 = time.perf_counter()
            tmp = torch.from_numpy(pcs[0]).to(dev)
            torch.cuda.synchronize()
            ht.append(time.perf_counter() - t1)
            del tmp
        dt = []
        for _ in range(e2e_steps):
            barrier()
            t1 = time.perf_counter()
            d_out.cpu()
            dt.append(time.perf_counter() - t1)
        phases = {"e2e_ms": e2e_s * 1e3, "device_step_ms": ms,
                  "h2d_pageable_ms": min(ht) * 1e3, "h2d_bytes": int(pcs[0].nbytes),
                  "h2d_gbs": pcs[0].nbytes / min(ht) / 1e9, "d2h_ms": min(dt) * 1e3,
                  "rest_ms": e2e_s * 1e3 - ms - min(ht) * 1e3 - min(dt) * 1e3}

    # the plain one-call-per-cloud GPU form on the same data, for comparison
    barrier()
    pe0 = torch.cuda.Event(enable_timing=True)
    pe1 = torch.cuda.Event(enable_timing=True)
    flush.zero_()
    pe0.record(stream)
    step_plain()
    pe1.record(stream)
    barrier()
    plain_ms = pe0.elapsed_time(pe1)
    plain_ok = bool(np.array_equal(d_out.cpu().numpy().astype(np.uint64), res))

    if rank == 0:
        launches = int(st["kernel_launches"])
        roof, vanilla_equiv = roofline(wl, st, args.steps, ms)
        traffic = None
        tpath = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tpath):
            tj = json.load(open(tpath)).get(args.workload)
            if tj:
                traffic = tj.get("dram_bytes_per_launch")
        cpu = cpu_baseline(wl) if world == 1 or rank == 0 else None
        lat = sorted(step_ms)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generators, workloads.py)",
            "config": config_of(wl),
            "bit_exact": bit_exact, "bit_exact_checked": checked,
            "vanilla_equivalent": vanilla_equiv,
            "plain_per_cloud": {"value": len(clouds) / (plain_ms / 1e3), "unit": UNIT,
                                "ms_per_step": plain_ms, "identical_to_batched": plain_ok,
                                "batched_speedup": plain_ms / ms},
            "e2e_phases": phases,
            "e2e": {"value": e2e_v, "unit": UNIT,
                    "h2d_bytes_per_step": int(host_all.nbytes),
                    "d2h_bytes_per_step": int(koffs[-1]) * 8},
            "roofline": dict(roof, traffic=traffic),
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": launches,
            "step_ms": {"min": lat[0], "median": statistics.median(lat), "max": lat[-1]},
            "wall_s_timed_region": t_wall,
            "stats": st,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def _replay(srv, reqs, pts):
    """Submits every request at its arrival time (relative to now) and waits
    for all results: (results, wall seconds)."""
    tickets = [None] * len(reqs)
    t0 = time.perf_counter()
    for i, r in enumerate(reqs):
        dt = t0 + r.arrival_s - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        tickets[i] = srv.submit(pts[i], r.k, h_for(r.n), r.start)
    res = [srv.result(t) for t in tickets]
    return res, time.perf_counter() - t0


def run_served(args):
    """The served workload: a Poisson stream of requests (2000/s) into the
    request server, in two parts.

      offered   the first --served-window seconds of the stream, replayed at
                its arrival times: far more work than one GPU can do, so the
                server runs saturated; completed samples/s over the replay is
                the saturation throughput (requests wait in the queue, which
                their latency shows);
      admitted  the whole 10 s stream thinned at random to --served-load times
                that saturation throughput, replayed the same way: latency at
                a load the server sustains.

    Every request's points come from its own seed and are generated on the
    host cores before the replay.  Reports requests/s and samples/s, latency
    percentiles (submit to result) overall and for requests of <= 65536
    points; a sample of results is compared with one call per cloud."""
    import tempfile as tf

    from fpsample_gb300 import capi

    reqs = served_requests(args.served_window)
    with tf.TemporaryDirectory(dir=_scratch_dir()) as folder:
        pts = materialize(reqs, folder)
    with capi.Server(150 << 30, small_workers=args.small_workers,
                     large_workers=args.large_workers) as srv:
        for i in range(min(8, len(reqs))):  # warm-up (not timed)
            srv.result(srv.submit(pts[i], reqs[i].k, h_for(reqs[i].n), reqs[i].start))
        res, wall = _replay(srv, reqs, pts)
        offered = _latency_summary(reqs, np.array([r[2] for r in res]),
                                   np.array([r[1] for r in res]), wall)
        check = list(range(0, len(reqs), max(1, len(reqs) // 8)))
        same = all(np.array_equal(res[i][0], capi.bucket_fps_kdline(pts[i], reqs[i].k,
                                                                    reqs[i].start, h_for(reqs[i].n)))
                   for i in check)
        del pts, res
        adm, keep = admitted_requests(args.served_load, offered["samples_per_s"])
        with tf.TemporaryDirectory(dir=_scratch_dir()) as folder:
            apts = materialize(adm, folder)
        ares, awall = _replay(srv, adm, apts)
        admitted = _latency_summary(adm, np.array([r[2] for r in ares]),
                                    np.array([r[1] for r in ares]), awall)
        acheck = list(range(0, len(adm), max(1, len(adm) // 8)))
        same &= all(np.array_equal(ares[i][0], capi.bucket_fps_kdline(apts[i], adm[i].k,
                                                                       adm[i].start, h_for(adm[i].n)))
                    for i in acheck)
    line = {
        "metric": "requests/sec (served)", "value": offered["requests_per_s"], "unit": "requests/s",
        "n_gpus": 1, "higher_is_better": True, "data": "synthetic (seeded generators)",
        "config": {"workload": "served", "offered_rate_per_s": 2000, "window_s": args.served_window,
                   "requests": len(reqs), "points_total": int(sum(r.n for r in reqs)),
                   "samples_total": int(sum(r.k for r in reqs)),
                   "small_workers": args.small_workers, "large_workers": args.large_workers,
                   "memory_budget_gb": 150, "fp_mode": fp_mode()},
        "offered": offered,
        "saturation": {"samples_per_s": offered["samples_per_s"],
                       "requests_per_s": offered["requests_per_s"]},
        "admitted": dict(admitted, load_of_saturation=args.served_load, stream_s=10.0,
                         kept_fraction=keep),
        "latency_ms": admitted["latency_ms"],
        "latency_ms_n_le_65536": admitted["latency_ms_n_le_65536"],
        "identical_to_single_calls": same,
    }
    print(json.dumps(line), flush=True)


def run_latency_probe(args):
    """Per-sample latency of one cloud at a time (not the headline metric):
    uniform box clouds, D=3, K=N/4, timed end to end (build + sampling) through
    the batched entry point with one cloud and through the single-cloud entry
    point; plus the gmm-1m workload (kd-line h=7 and vanilla, K=16384)."""
    import torch

    from fpsample_gb300 import capi
    import workloads as W

    def best_of(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return min(ts)

    res = {}
    rng = np.random.default_rng(0)
    s = torch.cuda.current_stream().cuda_stream
    for n in (4096, 16384, 32768, 65536, 124000):
        p = (rng.random((n, 3)) * rng.uniform(0.1, 10, 3)).astype(np.float32)
        t = torch.from_numpy(p).cuda()
        k = n // 4
        h = h_for(n)
        out = torch.empty(k, dtype=torch.int64, device="cuda")
        dt = best_of(lambda: capi.kdline_batch_device(t.data_ptr(), [0, n], 3, [k], [h], [0],
                                                      out.data_ptr(), s))
        res[f"batched_one_cloud_n{n}"] = {"ms": dt * 1e3, "us_per_sample": dt * 1e6 / k}
        dt = best_of(lambda: capi.kdline_device(t.data_ptr(), n, 3, k, 0, h, out.data_ptr(), 0, s))
        res[f"single_cloud_n{n}"] = {"ms": dt * 1e3, "us_per_sample": dt * 1e6 / k}
    g = torch.from_numpy(W.gmm_cloud(1 << 20, seed=W.SEEDS["gmm-1m"])).cuda()
    out = torch.empty(16384, dtype=torch.int64, device="cuda")
    dt = best_of(lambda: capi.kdline_device(g.data_ptr(), 1 << 20, 3, 16384, 0, 7, out.data_ptr(), 0, s))
    res["gmm1m_kdline_h7"] = {"ms": dt * 1e3, "us_per_sample": dt * 1e6 / 16384}
    dt = best_of(lambda: capi.fps_device(g.data_ptr(), 1 << 20, 3, 16384, [0], out.data_ptr(), 0, s))
    res["gmm1m_vanilla"] = {"ms": dt * 1e3, "us_per_sample": dt * 1e6 / 16384}
    dt = best_of(lambda: capi.kdtree_tensor(g, 16384, 0))
    res["gmm1m_kdtree"] = {"ms": dt * 1e3, "us_per_sample": dt * 1e6 / 16384}
    print(json.dumps({"probe": "latency", "results": res}), flush=True)


SAMPLER_CASES = {
    # name: (what it runs, the kernel it is there for)
    "resident-4k": ("vanilla FPS, 4,096 x 3 uniform, K=1,024", "vanilla_resident"),
    "stream-400k-d12": ("vanilla FPS, 400,000 x 12 uniform, K=128", "vanilla_stream"),
    "onecta-8k": ("kd-line h=5, 8,192 x 3 scaled box, K=2,048",
                  "lead_sample (one CTA: leader warp and worker warps)"),
    "onecta-124k": ("kd-line h=7, 124,000 x 3 scaled box, K=31,000",
                    "lead_sample (one CTA: leader warp and worker warps)"),
    "cluster-gmm1m": ("kd-line h=7, the 1,048,576-point Gaussian mixture, K=4,096",
                      "batch_sample (cluster), split_kernel exact levels"),
    "gridsmem-200k": ("vanilla FPS with the fp32 trace, 200,000-point Gaussian mixture, K=2,000",
                      "grid_sample_smem"),
    "gridreg-8m-d6": ("vanilla FPS, 8,388,608 x 6 (the large cloud's generator), K=512",
                      "grid_sample_reg"),
    "stream-40m-d1": ("vanilla FPS, 41,943,040 x 1 uniform, K=64", "fps_sample"),
}


def run_sampler_probe(args):
    """One call per sampler kind on a small seeded case, each timed alone
    (CUDA events around the call, after one untimed call): the cases that the
    ncu summaries under profiles/ capture one kernel of (ncu -k <kernel>
    -c 1 python bench.py --probe samplers --case <name>)."""
    import torch

    import workloads as W
    from fpsample_gb300 import capi

    names = [args.case] if args.case else list(SAMPLER_CASES)
    res = {}
    for name in names:
        if name == "resident-4k":
            pts, call = W.uniform_cloud(4096, 3, seed=0), ("fps", 1024, 0)
        elif name == "stream-400k-d12":
            pts, call = W.uniform_cloud(400_000, 12, seed=5), ("fps", 128, 0)
        elif name == "onecta-8k":
            rng = np.random.default_rng(12)
            pts = (rng.random((8192, 3)) * rng.uniform(0.1, 10, 3)).astype(np.float32)
            call = ("kdline", 2048, 5)
        elif name == "onecta-124k":
            rng = np.random.default_rng(11)
            pts = (rng.random((124_000, 3)) * rng.uniform(0.1, 10, 3)).astype(np.float32)
            call = ("kdline", 31_000, 7)
        elif name == "cluster-gmm1m":
            pts, call = W.gmm_cloud(1 << 20, seed=W.SEEDS["gmm-1m"]), ("kdline", 4096, 7)
        elif name == "gridsmem-200k":
            pts, call = W.gmm_cloud(200_000, seed=7), ("fps-trace", 2000, 0)
        elif name == "gridreg-8m-d6":
            pts, call = W.large_cloud(1 << 23, seed=W.SEEDS["large-16m"]), ("fps", 512, 0)
        elif name == "stream-40m-d1":
            pts, call = W.uniform_cloud(40 << 20, 1, seed=6), ("fps", 64, 0)
        else:
            raise ValueError(name)
        t = torch.from_numpy(pts).cuda()
        kind, k, h = call
        out = torch.empty(k, dtype=torch.int64, device="cuda")
        tr = torch.empty(k, dtype=torch.float32, device="cuda")
        s = torch.cuda.current_stream().cuda_stream

        def once():
            if kind == "kdline":
                capi.kdline_device(t.data_ptr(), t.shape[0], t.shape[1], k, 0, h, out.data_ptr(), 0, s)
            else:
                capi.fps_device(t.data_ptr(), t.shape[0], t.shape[1], k, [0], out.data_ptr(),
                                tr.data_ptr() if kind == "fps-trace" else 0, s)

        once()
        torch.cuda.synchronize()
        capi.stats_reset()
        capi.stats_timing(True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        once()
        e1.record()
        torch.cuda.synchronize()
        capi.stats_timing(False)
        st = capi.stats()
        res[name] = {"what": SAMPLER_CASES[name][0], "kernel": SAMPLER_CASES[name][1],
                     "call_ms": e0.elapsed_time(e1), "sampler_ms": st["sampler_ms"],
                     "samples": st["samples"], "boxes_tested": st["pieces_tested"],
                     "distances_recomputed": st["points_touched"]}
        del t
    print(json.dumps({"probe": "samplers", "results": res}), flush=True)


def _bench_peaks_lib():
    """bench_peaks.cu compiled into _build/ (not part of the library)."""
    import ctypes
    import shutil

    out_dir = os.path.join(ROOT, "_build")
    os.makedirs(out_dir, exist_ok=True)
    so = os.path.join(out_dir, "libbenchpeaks.so")
    src = os.path.join(ROOT, "bench_peaks.cu")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
        nvcc = nvcc if os.path.exists(nvcc) else (shutil.which("nvcc") or "nvcc")
        subprocess.run([nvcc, "-gencode=arch=compute_103a,code=sm_103a", "-O3", "-shared",
                        "-Xcompiler", "-fPIC", "-o", so, src], check=True)
    lib = ctypes.CDLL(so)
    lib.bench_measure_bandwidth.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    lib.bench_measure_bandwidth.restype = ctypes.c_int
    return lib


def run_peaks_probe(args):
    """Shared-memory and L2 read bandwidth of this GPU (the roofline of vanilla
    FPS on clouds that stay on chip), best of five, beside the HBM copy
    bandwidth measured for this GPU type (MEASURED_PEAKS.json)."""
    import ctypes

    import torch

    torch.cuda.init()
    lib = _bench_peaks_lib()
    out = {"probe": "peaks", "command": "python bench.py --probe peaks",
           "device": torch.cuda.get_device_name(0)}
    for level, key in ((0, "smem_gbs"), (1, "l2_gbs")):
        best = 0.0
        for _ in range(5):
            v = ctypes.c_double(0.0)
            rc = lib.bench_measure_bandwidth(level, ctypes.byref(v))
            if rc != 0:
                raise RuntimeError(f"bench_measure_bandwidth({level}) failed: {rc}")
            best = max(best, v.value)
        out[key] = best
    try:
        out["hbm_gbs"] = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except (OSError, KeyError):
        out["hbm_gbs"] = None
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batched-256", choices=WORKLOADS)
    ap.add_argument("--served-window", type=float, default=1.0,
                    help="seconds of the served request stream to replay at the offered rate")
    ap.add_argument("--served-load", type=float, default=0.8,
                    help="admitted load, as a fraction of the measured saturation throughput")
    ap.add_argument("--small-workers", type=int, default=8)
    ap.add_argument("--large-workers", type=int, default=2)
    ap.add_argument("--probe", default=None, choices=["latency", "peaks", "samplers"],
                    help="print a diagnostic table instead of the benchmark line")
    ap.add_argument("--case", default=None, choices=sorted(SAMPLER_CASES),
                    help="with --probe samplers: run this case only")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.probe == "latency":
        run_latency_probe(args)
        return
    if args.probe == "peaks":
        run_peaks_probe(args)
        return
    if args.probe == "samplers":
        run_sampler_probe(args)
        return
    if args.workload == "served":
        run_served(args) if args.impl != "reference" else run_served_reference(args)
        return
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_gpu_arm(args)


if __name__ == "__main__":
    main()
