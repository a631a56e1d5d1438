"""The golden cases: inputs (generator specs or stored arrays) and the calls
made on them.  Expected outputs live in golden.npz, produced by
make_golden.py from the unmodified reference."""
from __future__ import annotations

import numpy as np

import workloads as W


def _grid(n, d, levels, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(0, levels, (n, d)).astype(np.float32)


def _bench42(n, d):
    # the reference bench's own data: np.random.seed(42); np.random.rand (float64)
    rs = np.random.RandomState(42)
    return rs.rand(n, d)


def _dups(n, d, seed):
    # a few distinct points, each repeated many times
    rng = np.random.default_rng(seed)
    base = rng.random((max(2, n // 16), d)).astype(np.float32)
    return base[rng.integers(0, base.shape[0], n)]


GENERATORS = {
    "uniform": lambda a: W.uniform_cloud(a["n"], a["d"], a["seed"]),
    "gmm": lambda a: W.gmm_cloud(a["n"], seed=a["seed"]),
    "grid": lambda a: _grid(a["n"], a["d"], a["levels"], a["seed"]),
    "bench42": lambda a: _bench42(a["n"], a["d"]),
    "dups": lambda a: _dups(a["n"], a["d"], a["seed"]),
    "equal": lambda a: np.full((a["n"], a["d"]), 0.25, np.float32),
}


def make_input(case) -> np.ndarray:
    spec = case["input"]
    return np.asarray(GENERATORS[spec["gen"]](spec["args"]))


def _c(name, op, gen, args, k, start, h=None, stored=False):
    return {"name": name, "op": op, "k": k, "start": start, "h": h,
            "input": {"kind": "stored" if stored else "gen", "gen": gen, "args": args}}


CASES = []
# single-4k workload (uniform 4096 x 3, seed 0)
U4 = {"n": 4096, "d": 3, "seed": 0}
CASES.append(_c("u4k_fps", "fps", "uniform", U4, 1024, 0))
CASES.append(_c("u4k_fps_multi", "fps", "uniform", U4, 1024, [0, 23, 64, 128]))
for h in (3, 5, 7):
    CASES.append(_c(f"u4k_kdline_h{h}", "kdline", "uniform", U4, 1024, 0, h))
CASES.append(_c("u4k_kdline_h3_s4095", "kdline", "uniform", U4, 1024, 4095, 3))
# the reference's own benchmark data (seed 42, float64 input cast by the wrapper)
B = {"n": 4096, "d": 3}
CASES.append(_c("bench42_fps", "fps", "bench42", B, 1024, 0))
CASES.append(_c("bench42_fps_multi", "fps", "bench42", B, 1024, [0, 23, 64, 128]))
for h in (3, 5, 7):
    CASES.append(_c(f"bench42_kdline_h{h}", "kdline", "bench42", B, 1024, 0, h))
# 50k shape of the reference benchmark
CASES.append(_c("u50k_fps", "fps", "uniform", {"n": 50000, "d": 3, "seed": 5}, 512, 0))
CASES.append(_c("u50k_kdline_h7", "kdline", "uniform", {"n": 50000, "d": 3, "seed": 5}, 4096, 0, 7))
# dimensions 1..8, several heights and starts
for d in range(1, 9):
    a = {"n": 1500, "d": d, "seed": 10 + d}
    CASES.append(_c(f"d{d}_fps", "fps", "uniform", a, 300, 5))
    for h in (1, 2, 4, 6):
        for s in (0, 777, 1499):
            CASES.append(_c(f"d{d}_kdline_h{h}_s{s}", "kdline", "uniform", a, 300, s, h))
# heavy ties: integer grids and repeated points, up to K = N
for d in (1, 2, 3, 5):
    g = {"n": 3000, "d": d, "levels": 4, "seed": 30 + d}
    CASES.append(_c(f"grid{d}_fps", "fps", "grid", g, 300, 7, stored=True))
    for h in (1, 3, 6):
        CASES.append(_c(f"grid{d}_kdline_h{h}", "kdline", "grid", g, 300, 7, h, stored=True))
gs = {"n": 200, "d": 2, "levels": 5, "seed": 40}
CASES.append(_c("grid_small_fps_all", "fps", "grid", gs, 200, 3, stored=True))
CASES.append(_c("grid_small_kdline_all", "kdline", "grid", gs, 200, 3, 4, stored=True))
dp = {"n": 2048, "d": 3, "seed": 41}
CASES.append(_c("dups_fps", "fps", "dups", dp, 512, 0, stored=True))
CASES.append(_c("dups_kdline_h5", "kdline", "dups", dp, 512, 0, 5, stored=True))
eq = {"n": 64, "d": 3}
CASES.append(_c("equal_fps", "fps", "equal", eq, 64, 0))
CASES.append(_c("equal_kdline_h3", "kdline", "equal", eq, 64, 10, 3))
# 2**h == N, and h = 1
CASES.append(_c("pow2_kdline_h10", "kdline", "uniform", {"n": 1024, "d": 3, "seed": 50}, 1024, 0, 10))
CASES.append(_c("tiny_kdline_h1", "kdline", "uniform", {"n": 2, "d": 3, "seed": 51}, 2, 1, 1))
CASES.append(_c("one_fps", "fps", "uniform", {"n": 1, "d": 4, "seed": 52}, 1, 0))
# Gaussian mixture where the FMA and non-FMA builds diverge (at sample 3912)
CASES.append(_c("gmm128k_kdline_h7", "kdline", "gmm", {"n": 131072, "seed": 1}, 8192, 0, 7))
# bucket_fps_kdtree (unbounded-height tree, ties to the last position):
# continuous data, every dimension, integer grids and repeated points
CASES.append(_c("u4k_kdtree", "kdtree", "uniform", U4, 1024, 0))
CASES.append(_c("bench42_kdtree", "kdtree", "bench42", B, 1024, 0))
for d in range(1, 9):
    CASES.append(_c(f"d{d}_kdtree_s777", "kdtree", "uniform",
                    {"n": 1500, "d": d, "seed": 10 + d}, 300, 777))
for d in (1, 2, 3, 5):
    CASES.append(_c(f"grid{d}_kdtree", "kdtree", "grid",
                    {"n": 3000, "d": d, "levels": 4, "seed": 30 + d}, 300, 7, stored=True))
CASES.append(_c("grid_small_kdtree_all", "kdtree", "grid", gs, 200, 3, stored=True))
CASES.append(_c("dups_kdtree", "kdtree", "dups", dp, 512, 0, stored=True))
CASES.append(_c("equal_kdtree", "kdtree", "equal", eq, 64, 10))
CASES.append(_c("tiny_kdtree", "kdtree", "uniform", {"n": 2, "d": 3, "seed": 51}, 2, 1))
CASES.append(_c("one_kdtree", "kdtree", "uniform", {"n": 1, "d": 4, "seed": 52}, 1, 0))
