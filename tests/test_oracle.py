"""CPU: the oracle (C restatement of the reference) against the golden vectors
produced by the unmodified reference, and internal consistency checks."""
import numpy as np
import pytest

from oracle.oracle import Oracle, fp64_trace
from tests.golden.golden import load_cases

CASES = load_cases()
ORACLE = Oracle()


def test_golden_inputs_regenerate():
    bad = [c["name"] for c in CASES if not c["input_ok"]]
    assert not bad, f"regenerated inputs differ from the ones the reference saw: {bad}"


@pytest.mark.parametrize("mode", ["nofma", "fma"])
@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_matches_reference(case, mode):
    pts = case["points"]
    if case["op"] == "fps":
        got = ORACLE.fps(pts, case["k"], case["start"], mode)
    elif case["op"] == "kdtree":
        got = ORACLE.kdtree(pts, case["k"], case["start"], mode)
    else:
        got = ORACLE.kdline(pts, case["k"], case["h"], case["start"], mode)
    np.testing.assert_array_equal(got, case["expected"][mode])


def test_kdtree_cases_contain_ties_that_separate_it_from_kdline():
    # on tie-heavy grids the kd-tree (ties to the last position) and an
    # unbounded kd-line (ties to the first) disagree, so the tie rule is pinned
    c = next(c for c in CASES if c["name"] == "grid2_kdtree")
    line = ORACLE.kdline(c["points"], c["k"], 64, c["start"], "nofma")
    assert not np.array_equal(line, c["expected"]["nofma"])


def test_fma_builds_really_differ():
    # the golden set contains a case where the two reference builds disagree,
    # so the mode switch is exercised for real
    c = next(c for c in CASES if c["name"] == "gmm128k_kdline_h7")
    d = np.nonzero(c["expected"]["nofma"] != c["expected"]["fma"])[0]
    assert d.size > 0 and d[0] == 3912


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("mode", ["nofma", "fma"])
def test_kdline_equals_fps_over_permuted_order(seed, mode):
    """The bucket pruning never changes a value: kd-line output equals plain FPS
    over the build's permuted order with first-position ties."""
    rng = np.random.default_rng(seed)
    n = int(rng.integers(50, 3000))
    d = int(rng.integers(1, 9))
    pts = rng.random((n, d)).astype(np.float32)
    if seed % 2:
        pts = np.round(pts * 3) / 3  # ties
    h = int(rng.integers(1, 8))
    k = int(rng.integers(1, n + 1))
    s = int(rng.integers(0, n))
    a = ORACLE.kdline(pts, k, h, s, mode)
    b = ORACLE.kdline_direct(pts, k, h, s, mode)
    np.testing.assert_array_equal(a, b)


def test_build_permutation_is_a_permutation_and_buckets_ordered():
    rng = np.random.default_rng(3)
    pts = rng.random((5000, 3)).astype(np.float32)
    perm, bst = ORACLE.kdline_build(pts, 6)
    assert np.array_equal(np.sort(perm), np.arange(5000))
    assert bst[0] == 0 and np.all(np.diff(bst.astype(np.int64)) > 0) and len(bst) == 64


def test_fp64_trace_close_to_fp32():
    rng = np.random.default_rng(4)
    pts = rng.random((2000, 3)).astype(np.float32)
    idx, tr = ORACLE.fps(pts, 200, 0, "nofma", trace=True)
    ref = fp64_trace(pts, idx)
    np.testing.assert_allclose(tr[1:], ref[1:], rtol=1e-5)


@pytest.mark.parametrize("mode", ["nofma", "fma"])
def test_oracle_matches_the_live_reference_on_random_clouds(mode):
    """Beyond the golden vectors: random clouds (continuous, integer grids full
    of ties, Gaussian), every dimension 1..8, random heights, sample counts and
    starts, against the reference compiled from its own sources -- where that
    build exists (it does not on hosts without the reference's sources)."""
    from oracle import oracle as O

    if not O.reference_available(mode):
        pytest.skip("the reference build is not available on this host")
    ref = O.load_reference(mode)
    rng = np.random.default_rng(2024 if mode == "nofma" else 4202)
    for i in range(24):
        d = 1 + i % 8
        n = int(np.exp(rng.uniform(np.log(16), np.log(12000))))
        kind = i % 3
        if kind == 0:
            p = rng.random((n, d)) * rng.uniform(0.1, 50, d)
        elif kind == 1:
            p = rng.integers(0, 7, (n, d)).astype(np.float64)
        else:
            p = rng.standard_normal((n, d)) * 20
        p = p.astype(np.float32)
        h = int(rng.integers(1, max(1, int(np.log2(n))) + 1))
        k = int(rng.integers(1, min(n, 1500) + 1))
        s = int(rng.integers(0, n))
        np.testing.assert_array_equal(ORACLE.kdline(p, k, h, s, mode),
                                      ref.bucket_fps_kdline_sampling(p, k, h, s))
        np.testing.assert_array_equal(ORACLE.fps(p, min(k, 300), s, mode),
                                      ref.fps_sampling(p, min(k, 300), s))
        np.testing.assert_array_equal(ORACLE.fps_mt(p, min(k, 300), s, mode, threads=5),
                                      ref.fps_sampling(p, min(k, 300), s))


@pytest.mark.parametrize("mode", ["nofma", "fma"])
def test_multithreaded_vanilla_oracle_equals_serial(mode):
    """oracle_fps_mt (chunked updates, chunk maxima folded in order) gives the
    serial restatement's answer: continuous and tie-heavy clouds, NaN
    coordinates, start lists, every dimension 1..11, 1 to 16 threads."""
    rng = np.random.default_rng(77 if mode == "nofma" else 78)
    for i in range(22):
        d = 1 + i % 11
        n = int(rng.integers(1, 6000))
        p = rng.random((n, d)).astype(np.float32)
        if i % 3 == 1:
            p = np.round(p * 4).astype(np.float32)  # ties
        if i % 7 == 3 and n > 10:
            p[rng.integers(0, n, 3), 0] = np.nan
        k = int(rng.integers(1, min(n, 800) + 1))
        m = int(rng.integers(1, min(k, 4) + 1))
        starts = [int(x) for x in rng.integers(0, n, m)]
        want = ORACLE.fps(p, k, starts, mode)
        for threads in (1, 3, 16):
            np.testing.assert_array_equal(ORACLE.fps_mt(p, k, starts, mode, threads=threads), want)


@pytest.mark.parametrize("mode", ["nofma", "fma"])
def test_fullsize_fixtures_agree_with_the_oracle(mode):
    """tests/golden/fullsize.npz: the seeded generators still produce the
    fixtures' inputs, and the oracle reproduces each answer (the 1M-point
    kd-line in full, the others on prefixes -- FPS is prefix-stable in K)."""
    from tests.golden import fullsize as F

    if not F.available():
        pytest.fail("tests/golden/fullsize.npz is missing (tests/golden/make_fullsize.py)")
    gmm = F.cloud("gmm1m")
    assert F.input_matches("gmm1m", gmm)
    np.testing.assert_array_equal(ORACLE.kdline(gmm, 16384, 7, 0, mode),
                                  F.expected("gmm1m_kdline_h7", mode))
    np.testing.assert_array_equal(ORACLE.fps_mt(gmm, 16384, 0, mode),
                                  F.expected("gmm1m_vanilla", mode))
    big = F.cloud("large16m")
    assert F.input_matches("large16m", big)
    np.testing.assert_array_equal(ORACLE.kdline(big, 256, 9, 0, mode),
                                  F.expected("large16m_kdline_h9", mode)[:256])
    np.testing.assert_array_equal(ORACLE.fps_mt(big, 16, 0, mode),
                                  F.expected("large16m_vanilla", mode)[:16])
    assert len(np.unique(F.expected("large16m_vanilla", mode))) == 65536


def test_fullsize_fixtures_separate_the_fp_modes():
    """At the benchmark sizes the two arithmetics pick different points, for
    vanilla FPS as well as for the kd-line (the 1M-point vanilla cloud first
    differs at sample 10691): the fma mode is exercised for both."""
    from tests.golden import fullsize as F

    if not F.available():
        pytest.fail("tests/golden/fullsize.npz is missing (tests/golden/make_fullsize.py)")
    for case in ("gmm1m_vanilla", "gmm1m_kdline_h7", "large16m_vanilla", "large16m_kdline_h9"):
        a, b = F.expected(case, "nofma"), F.expected(case, "fma")
        assert not np.array_equal(a, b), case
    d = np.nonzero(F.expected("gmm1m_vanilla", "nofma") != F.expected("gmm1m_vanilla", "fma"))[0]
    assert d[0] == 10691
