"""Generate tests/golden/golden.npz from the UNMODIFIED reference.

Run where the reference sources are mounted (they are not on the GPU hosts):

    make -C oracle ref            # compiles the reference's own src/lib.cpp twice
    python tests/golden/make_golden.py

Every expected output comes from the reference's public Python API
(``fpsample.fps_sampling`` / ``bucket_fps_kdline_sampling`` /
``bucket_fps_kdtree_sampling``), run
through its two builds: "nofma" (default x86-64 code, no contraction) and
"fma" (same source with FMA contraction enabled).  Inputs that a seeded
generator reproduces are stored as (generator, sha256) and regenerated by the
tests; the others are stored verbatim.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tests.golden.cases import CASES, make_input  # noqa: E402
from oracle.oracle import load_reference  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float32).tobytes()).hexdigest()


def main() -> None:
    refs = {m: load_reference(m) for m in ("nofma", "fma")}
    arrays = {}
    manifest = []
    for case in CASES:
        pts = make_input(case)
        entry = dict(case)
        entry["sha256"] = sha(pts)
        if case["input"]["kind"] == "stored":
            arrays[case["name"] + "__points"] = np.ascontiguousarray(pts, dtype=np.float32)
        for mode, ref in refs.items():
            if case["op"] == "fps":
                out = ref.fps_sampling(pts, case["k"], case["start"])
            elif case["op"] == "kdtree":
                out = ref.bucket_fps_kdtree_sampling(pts, case["k"], case["start"])
            else:
                out = ref.bucket_fps_kdline_sampling(pts, case["k"], case["h"], case["start"])
            arrays[f"{case['name']}__{mode}"] = np.asarray(out, dtype=np.uint64)
        manifest.append(entry)
        print(case["name"], "ok")
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)


if __name__ == "__main__":
    main()
