"""On the host that drives the GPU: the reference compiled there from its own
sources (oracle/_ref, `make -C oracle ref` inside build()) against the golden
vectors, the full-size fixtures and the GPU.

The golden vectors and fixtures were produced on an x86-64 host by two builds
of the reference: "nofma" (the stock x86-64 build, which cannot contract) and
"fma" (the same sources with -mfma and --param=avoid-fma-max-bits=0, so that
GCC contracts every a*b+c, loop-carried ones included).  On an aarch64 host
such as Grace the reference's stock build contracts by itself.
These tests show that the host's stock build gives exactly the vectors of the
mode it is said to match -- so the GPU, tested against those vectors in both
modes, matches the reference as it is really built on this host -- and they
compare the GPU in the library's default mode with that stock build directly
on fresh random clouds.
"""
import numpy as np
import pytest

import fpsample as fps
from oracle import oracle as O
from tests.golden import fullsize as F
from tests.golden.golden import load_cases

pytestmark = pytest.mark.gpu

CASES = load_cases()


def _stock():
    mode = O.stock_mode()
    if mode is None or not O.reference_available(mode):
        pytest.skip("the reference was not compiled on this host (no staged sources)")
    return mode, O.load_reference(mode)


def _call(ref, case):
    pts = case["points"]
    if case["op"] == "fps":
        return ref.fps_sampling(pts, case["k"], case["start"])
    if case["op"] == "kdtree":
        return ref.bucket_fps_kdtree_sampling(pts, case["k"], case["start"])
    return ref.bucket_fps_kdline_sampling(pts, case["k"], case["h"], case["start"])


def test_library_default_mode_is_the_host_stock_build():
    mode, _ = _stock()
    assert fps.get_fp_mode() == mode


@pytest.mark.parametrize("build", ["stock", "other"])
def test_host_builds_reproduce_the_golden_vectors(build):
    """Every golden case, through the reference's public API, in the host's
    stock build and in the other mode's build."""
    stock, _ = _stock()
    mode = stock if build == "stock" else ({"fma": "nofma", "nofma": "fma"}[stock])
    if not O.reference_available(mode):
        pytest.skip(f"no {mode} build of the reference on this host")
    ref = O.load_reference(mode)
    bad = [c["name"] for c in CASES
           if not np.array_equal(np.asarray(_call(ref, c), np.uint64), c["expected"][mode])]
    assert not bad, f"{mode} build ({O.reference_build_flags(mode)}) differs on {bad}"


def test_host_stock_build_reproduces_the_fullsize_fixtures():
    """The 1M-point Gaussian mixture: kd-line h=7 at full K, and vanilla FPS on
    its first 11,000 samples (FPS is prefix-stable in K), stock build vs
    fixture.  Vanilla's two arithmetics first differ at sample 10,691 on this
    cloud, so the prefix shows which one the host's compiler produced for the
    loop-carried `dist += d * d` (src/lib.cpp:214-221)."""
    mode, ref = _stock()
    pts = F.cloud("gmm1m")
    assert F.input_matches("gmm1m", pts)
    np.testing.assert_array_equal(np.asarray(ref.bucket_fps_kdline_sampling(pts, 16384, 7, 0),
                                             np.uint64), F.expected("gmm1m_kdline_h7", mode))
    np.testing.assert_array_equal(np.asarray(ref.fps_sampling(pts, 11000, 0), np.uint64),
                                  F.expected("gmm1m_vanilla", mode)[:11000])


@pytest.mark.parametrize("seed", range(8))
def test_gpu_default_mode_equals_host_stock_build(seed):
    """Random clouds (continuous, tie grids, Gaussian), D = 1..8: the GPU in
    the library's default mode against the host's stock reference build."""
    mode, ref = _stock()
    rng = np.random.default_rng(7000 + seed)
    d = 1 + seed % 8
    n = int(np.exp(rng.uniform(np.log(64), np.log(60000))))
    kind = seed % 3
    if kind == 0:
        p = rng.random((n, d)) * rng.uniform(0.1, 50, d)
    elif kind == 1:
        p = rng.integers(0, 7, (n, d)).astype(np.float64)
    else:
        p = rng.standard_normal((n, d)) * 20
    p = p.astype(np.float32)
    h = int(rng.integers(1, max(1, int(np.log2(n))) + 1))
    k = int(rng.integers(1, min(n, 4000) + 1))
    s = int(rng.integers(0, n))
    np.testing.assert_array_equal(fps.bucket_fps_kdline_sampling(p, k, h, s),
                                  np.asarray(ref.bucket_fps_kdline_sampling(p, k, h, s), np.uint64))
    kv = min(k, 1500)
    np.testing.assert_array_equal(fps.fps_sampling(p, kv, s),
                                  np.asarray(ref.fps_sampling(p, kv, s), np.uint64))
