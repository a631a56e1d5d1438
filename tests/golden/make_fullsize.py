"""Generate tests/golden/fullsize.npz: complete answers at the benchmark sizes.

Run where the reference sources are staged (``make -C oracle stage ref``):

    python tests/golden/make_fullsize.py [--cache DIR]   # both FP modes, ~30 min

With --cache, every answer is also saved to DIR as it is computed and reused
by the next run.

Which answer comes from where:

  gmm1m_kdline_h7    1,048,576 x 3 Gaussian mixture, kd-line h=7, K=16,384:
                     the reference (bucket_fps_kdline_sampling), each build
  gmm1m_vanilla      same cloud, vanilla FPS, K=16,384: the reference
                     (fps_sampling), each build; the multithreaded oracle
                     must agree on every index
  large16m_kdline_h9 16,777,216 x 6, kd-line h=9, K=65,536: the reference,
                     each build
  large16m_vanilla   same cloud, vanilla FPS, K=65,536: the multithreaded
                     oracle (oracle_fps_mt; the reference's single thread
                     would need ~3 h per build); its first samples are checked
                     here against the reference, and tests/test_oracle.py
                     checks it against the serial oracle and the reference on
                     smaller clouds

"nofma" is the reference built without FMA contraction, "fma" the same
sources with contraction everywhere, as GCC compiles them on aarch64 (on
x86-64: -mfma --param=avoid-fma-max-bits=0, see oracle/Makefile).  Indices are stored as uint32
(every cloud has fewer than 2**32 points) beside the sha256 of the input the
seeded generator produced, so a test can tell a changed generator from a
wrong answer.
"""
from __future__ import annotations

import hashlib
import json
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

MODES = ("nofma", "fma")
CLOUDS = {
    "gmm1m": ("gmm_cloud", {"n": 1 << 20, "seed": 1}),
    "large16m": ("large_cloud", {"n": 1 << 24, "seed": 4}),
}
# name -> (cloud, op, k, h, start, source)
CASES = {
    "gmm1m_kdline_h7": ("gmm1m", "kdline", 16384, 7, 0, "reference"),
    "gmm1m_vanilla": ("gmm1m", "fps", 16384, None, 0, "reference"),
    "large16m_kdline_h9": ("large16m", "kdline", 65536, 9, 0, "reference"),
    "large16m_vanilla": ("large16m", "fps", 65536, None, 0, "oracle_fps_mt"),
}
REF_PREFIX_CHECK = 24  # reference samples checked against the oracle's 16.7M vanilla


def cloud(name: str) -> np.ndarray:
    import workloads as W

    gen, args = CLOUDS[name]
    return np.ascontiguousarray(getattr(W, gen)(**args), dtype=np.float32)


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float32).tobytes()).hexdigest()


def _reference_job(job):
    case, mode = job
    from oracle.oracle import load_reference

    cl, op, k, h, s, _ = CASES[case]
    pts = cloud(cl)
    ref = load_reference(mode)
    t0 = time.perf_counter()
    if op == "kdline":
        out = ref.bucket_fps_kdline_sampling(pts, k, h, s)
    else:
        out = ref.fps_sampling(pts, k, s)
    return case, mode, np.asarray(out, np.uint64), time.perf_counter() - t0


def _cached(cache, case, mode):
    if cache and os.path.exists(os.path.join(cache, f"{case}__{mode}.npy")):
        return np.load(os.path.join(cache, f"{case}__{mode}.npy"))
    return None


def _store(cache, case, mode, out):
    if cache:
        os.makedirs(cache, exist_ok=True)
        np.save(os.path.join(cache, f"{case}__{mode}.npy"), out)


def main() -> None:
    import argparse

    from oracle.oracle import Oracle, load_reference, reference_build_flags

    ap = argparse.ArgumentParser()
    ap.add_argument("--cache", default=None)
    cache = ap.parse_args().cache
    results, seconds = {}, {}
    for c in CASES:
        for m in MODES:
            got = _cached(cache, c, m)
            if got is not None:
                results[(c, m)], seconds[(c, m)] = got, None
    jobs = [(c, m) for c, v in CASES.items() if v[5] == "reference" for m in MODES
            if (c, m) not in results]
    # the reference is single-threaded: one process per run, the longest first
    jobs.sort(key=lambda j: -CASES[j[0]][2] * (1 << 20 if "16m" in j[0] else 1))
    t_all = time.perf_counter()
    if jobs:
        with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
            for case, mode, out, dt in pool.imap_unordered(_reference_job, jobs):
                results[(case, mode)] = out
                seconds[(case, mode)] = dt
                _store(cache, case, mode, out)
                print(f"{case} {mode}: {dt:.0f} s (reference)", flush=True)
    orc = Oracle()
    big = cloud("large16m")
    for mode in MODES:
        if ("large16m_vanilla", mode) in results:
            continue
        t0 = time.perf_counter()
        _, _, k, _, s, _ = CASES["large16m_vanilla"]
        results[("large16m_vanilla", mode)] = orc.fps_mt(big, k, s, mode)
        seconds[("large16m_vanilla", mode)] = time.perf_counter() - t0
        _store(cache, "large16m_vanilla", mode, results[("large16m_vanilla", mode)])
        print(f"large16m_vanilla {mode}: {seconds[('large16m_vanilla', mode)]:.0f} s", flush=True)

    # cross-checks: the multithreaded oracle against the reference
    gmm = cloud("gmm1m")
    orc = Oracle()
    for mode in MODES:
        mt = orc.fps_mt(gmm, 16384, 0, mode)
        if not np.array_equal(mt, results[("gmm1m_vanilla", mode)]):
            raise SystemExit(f"oracle_fps_mt differs from the reference on gmm1m ({mode})")
        ref = load_reference(mode)
        head = np.asarray(ref.fps_sampling(big, REF_PREFIX_CHECK, 0), np.uint64)
        if not np.array_equal(head, results[("large16m_vanilla", mode)][:REF_PREFIX_CHECK]):
            raise SystemExit(f"oracle_fps_mt differs from the reference on large16m ({mode})")

    arrays, manifest = {}, {"clouds": {}, "cases": {}}
    for name, (gen, args) in CLOUDS.items():
        manifest["clouds"][name] = {"generator": f"workloads.{gen}", "args": args,
                                    "sha256": sha(cloud(name) if name != "large16m" else big)}
    for case, (cl, op, k, h, s, src) in CASES.items():
        manifest["cases"][case] = {"cloud": cl, "op": op, "k": k, "h": h, "start": s,
                                   "source": src, "seconds": {}}
        for mode in MODES:
            out = results[(case, mode)]
            assert out.shape == (k,) and int(out.max()) < 2**32
            arrays[f"{case}__{mode}"] = out.astype(np.uint32)
            sec = seconds[(case, mode)]
            manifest["cases"][case]["seconds"][mode] = None if sec is None else round(sec, 1)
            if src == "reference":
                manifest["cases"][case].setdefault("reference_flags", {})[mode] = \
                    reference_build_flags(mode)
    manifest["generated_on"] = {"machine": os.uname().machine, "numpy": np.__version__,
                                "wall_s": round(time.perf_counter() - t_all)}
    np.savez_compressed(os.path.join(HERE, "fullsize.npz"), **arrays)
    with open(os.path.join(HERE, "fullsize.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    print("wrote fullsize.npz")


if __name__ == "__main__":
    main()
