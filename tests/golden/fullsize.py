"""Loader for tests/golden/fullsize.npz (written by make_fullsize.py): complete
reference answers for the benchmark-size clouds, checked against the sha256
of the input each seeded generator must reproduce."""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NPZ = os.path.join(HERE, "fullsize.npz")
MANIFEST = os.path.join(HERE, "fullsize.json")


def available() -> bool:
    return os.path.exists(NPZ) and os.path.exists(MANIFEST)


def manifest() -> dict:
    with open(MANIFEST) as f:
        return json.load(f)


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float32).tobytes()).hexdigest()


def cloud(name: str) -> np.ndarray:
    """The input cloud `name` ("gmm1m", "large16m"), regenerated from its seed."""
    import workloads as W

    spec = manifest()["clouds"][name]
    gen = getattr(W, spec["generator"].split(".", 1)[1])
    return np.ascontiguousarray(gen(**spec["args"]), dtype=np.float32)


def input_matches(name: str, pts: np.ndarray) -> bool:
    return sha(pts) == manifest()["clouds"][name]["sha256"]


def expected(case: str, mode: str) -> np.ndarray:
    """The full answer of `case` for FP mode `mode`, as uint64 indices."""
    with np.load(NPZ) as z:
        return z[f"{case}__{mode}"].astype(np.uint64)


def case(name: str) -> dict:
    return manifest()["cases"][name]


# bench workload name -> fixture case
BY_WORKLOAD = {
    "gmm-1m": "gmm1m_kdline_h7",
    "gmm-1m-vanilla": "gmm1m_vanilla",
    "large-16m": "large16m_kdline_h9",
    "large-16m-vanilla": "large16m_vanilla",
}
