"""Loader for the golden cases: regenerates or reads each input, checks its
sha256 against the manifest, and returns the reference's outputs."""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np

from tests.golden.cases import make_input

HERE = os.path.dirname(os.path.abspath(__file__))


def _sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float32).tobytes()).hexdigest()


def load_cases():
    with open(os.path.join(HERE, "manifest.json")) as f:
        manifest = json.load(f)
    data = np.load(os.path.join(HERE, "golden.npz"))
    out = []
    for case in manifest:
        if case["input"]["kind"] == "stored":
            pts = data[case["name"] + "__points"]
        else:
            pts = np.ascontiguousarray(make_input(case), dtype=np.float32)
        c = dict(case)
        c["points"] = np.ascontiguousarray(pts, dtype=np.float32)
        c["input_ok"] = _sha(pts) == case["sha256"]
        c["expected"] = {m: data[f"{case['name']}__{m}"] for m in ("nofma", "fma")}
        out.append(c)
    return out
