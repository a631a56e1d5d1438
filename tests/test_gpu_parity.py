"""GPU parity: every result must equal the reference's, bit for bit.

Sources of truth, in order:
  1. golden vectors produced by the unmodified reference (tests/golden/);
  2. complete answers at the benchmark sizes (tests/golden/fullsize.npz: the
     reference itself, or for the 16.7M-point vanilla case the multithreaded
     oracle, see tests/golden/make_fullsize.py);
  3. the oracle (oracle/fps_oracle.c, itself pinned to 1.) on seeded inputs;
  plus size-independent FPS properties (non-increasing max-min trace, fp64
  trace).
Indices are compared exactly; the fp32 trace against an fp64 recomputation
within rtol 1e-5.
"""
import numpy as np
import pytest

import fpsample as fps
from fpsample_gb300 import capi
import workloads as W
from oracle.oracle import Oracle, fp64_trace
from tests.golden import fullsize as F
from tests.golden.golden import load_cases

pytestmark = pytest.mark.gpu

CASES = load_cases()
ORACLE = Oracle()
MODES = ["nofma", "fma"]


@pytest.fixture(params=MODES)
def mode(request):
    before = fps.get_fp_mode()
    fps.set_fp_mode(request.param)
    yield request.param
    fps.set_fp_mode(before)


def _api(case):
    pts = case["points"]
    if case["op"] == "fps":
        st = case["start"]
        return fps.fps_sampling(pts, case["k"], st)
    if case["op"] == "kdtree":
        return fps.bucket_fps_kdtree_sampling(pts, case["k"], case["start"])
    return fps.bucket_fps_kdline_sampling(pts, case["k"], case["h"], case["start"])


def _cabi(case):
    pts = case["points"]
    if case["op"] == "fps":
        return capi.fps(pts, case["k"], case["start"])
    if case["op"] == "kdtree":
        return capi.bucket_fps_kdtree(pts, case["k"], case["start"])
    return capi.bucket_fps_kdline(pts, case["k"], case["start"], case["h"])


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_golden_python_api(case, mode):
    got = _api(case)
    assert got.dtype == np.uint64
    np.testing.assert_array_equal(got, case["expected"][mode])


ABI_CASES = CASES[::3] + [c for c in CASES if c["op"] == "kdtree"][1::3]


@pytest.mark.parametrize("case", ABI_CASES, ids=[c["name"] for c in ABI_CASES])
def test_golden_c_abi(case, mode):
    np.testing.assert_array_equal(_cabi(case), case["expected"][mode])


def _random_case(seed):
    rng = np.random.default_rng(1000 + seed)
    n = int(rng.integers(2, 20000))
    d = int(rng.integers(1, 9))
    kind = seed % 3
    if kind == 0:
        pts = rng.random((n, d)).astype(np.float32)
    elif kind == 1:
        pts = rng.integers(0, 5, (n, d)).astype(np.float32)
    else:
        pts = (rng.standard_normal((n, d)) * rng.uniform(0.01, 100)).astype(np.float32)
    k = int(rng.integers(1, min(n, 3000) + 1))
    s = int(rng.integers(0, n))
    h = int(rng.integers(1, max(2, int(np.log2(n)) + 1)))
    return pts, k, s, h


@pytest.mark.parametrize("seed", range(24))
def test_random_vs_oracle(seed, mode):
    pts, k, s, h = _random_case(seed)
    np.testing.assert_array_equal(fps.fps_sampling(pts, k, s), ORACLE.fps(pts, k, s, mode))
    np.testing.assert_array_equal(fps.bucket_fps_kdline_sampling(pts, k, h, s),
                                  ORACLE.kdline(pts, k, h, s, mode))


@pytest.mark.parametrize("seed", range(12))
def test_kdtree_random_vs_oracle(seed, mode):
    pts, k, s, _ = _random_case(seed)
    if pts.shape[1] > 8:
        pts = pts[:, :8]
    np.testing.assert_array_equal(fps.bucket_fps_kdtree_sampling(pts, k, s),
                                  ORACLE.kdtree(pts, k, s, mode))


def test_kdtree_large_cloud_and_trace(mode):
    """300K points: the kd-tree build reaches ~20 exact levels; plain calls run
    on a cluster, traced calls on the grid sampler."""
    torch = pytest.importorskip("torch")
    pts = W.gmm_cloud(300_000, seed=12)
    want = ORACLE.kdtree(pts, 2000, 17, mode)
    np.testing.assert_array_equal(fps.bucket_fps_kdtree_sampling(pts, 2000, 17), want)
    out, tr = capi.kdtree_tensor(torch.from_numpy(pts).cuda(), 2000, 17, trace=True)
    np.testing.assert_array_equal(out.cpu().numpy().astype(np.uint64), want)
    assert np.all(np.diff(tr.cpu().numpy()[1:]) <= 0)


@pytest.mark.parametrize("seed", range(6))
def test_multi_start_vs_oracle(seed, mode):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(100, 30000))
    pts = rng.random((n, 3)).astype(np.float32)
    m = int(rng.integers(1, 8))
    starts = [int(x) for x in rng.integers(0, n, m)]
    if seed == 0:
        starts = [5, 5, 5]  # duplicated starts are allowed
    k = int(rng.integers(m, min(n, 2000) + 1))
    np.testing.assert_array_equal(fps.fps_sampling(pts, k, starts), ORACLE.fps(pts, k, starts, mode))


@pytest.mark.parametrize("h", [0, 1, 3, 7, 11, 40])
def test_build_permutation_vs_oracle(h):
    rng = np.random.default_rng(h)
    for pts in (rng.random((3000, 3)).astype(np.float32),
                rng.integers(0, 3, (2000, 2)).astype(np.float32),
                np.full((300, 4), 1.5, np.float32)):
        perm, bst = capi.kdline_build(pts, h)
        operm, obst = ORACLE.kdline_build(pts, h)
        np.testing.assert_array_equal(perm, operm)
        np.testing.assert_array_equal(bst, obst)


@pytest.mark.parametrize("n,h", [(100, 40), (37, 64), (5, 3), (1, 5), (1000, 0)])
def test_c_abi_heights_beyond_the_python_check(n, h, mode):
    # the C ABI accepts any height (the Python wrapper asserts 2**h <= n)
    pts = np.random.default_rng(n).random((n, 3)).astype(np.float32)
    k = min(n, 50)
    np.testing.assert_array_equal(capi.bucket_fps_kdline(pts, k, n // 2, h),
                                  ORACLE.kdline(pts, k, h, n // 2, mode))


def test_more_samples_than_points_c_abi(mode):
    pts = np.random.default_rng(9).random((40, 3)).astype(np.float32)
    np.testing.assert_array_equal(capi.bucket_fps_kdline(pts, 100, 3, 2), ORACLE.kdline(pts, 100, 2, 3, mode))
    np.testing.assert_array_equal(capi.fps(pts, 100, 3), ORACLE.fps(pts, 100, 3, mode))


@pytest.mark.parametrize("n", [9000, 60_000, 240_000, 400_000])
def test_single_call_both_sides_of_the_one_cta_limit(n, mode):
    # single calls whose pieces fit one CTA run on one CTA, larger clouds on
    # the multi-CTA sampler; kd-line and single-start vanilla on both sides
    rng = np.random.default_rng(n)
    pts = rng.random((n, 3), dtype=np.float32)
    k = 1500
    np.testing.assert_array_equal(fps.bucket_fps_kdline_sampling(pts, k, 7, n // 3),
                                  ORACLE.kdline(pts, k, 7, n // 3, mode))
    np.testing.assert_array_equal(fps.fps_sampling(pts, k, n // 5), ORACLE.fps(pts, k, n // 5, mode))


def test_high_dimension_vanilla(mode):
    rng = np.random.default_rng(5)
    for d in (9, 16, 33):
        pts = rng.random((3000, d)).astype(np.float32)
        np.testing.assert_array_equal(fps.fps_sampling(pts, 300, 1), ORACLE.fps(pts, 300, 1, mode))


def test_nan_coordinates_vanilla_exact():
    pts = np.random.default_rng(6).random((500, 3)).astype(np.float32)
    pts[[3, 77, 400], 1] = np.nan
    np.testing.assert_array_equal(fps.fps_sampling(pts, 100, 0),
                                  ORACLE.fps(pts, 100, 0, fps.get_fp_mode()))


def test_kdline_nan_in_split_dimension_is_reported():
    pts = np.random.default_rng(6).random((500, 3)).astype(np.float32)
    pts[3, :] = np.nan
    with pytest.raises(RuntimeError, match="error code 6"):
        fps.bucket_fps_kdline_sampling(pts, 10, 3, 0)


def test_device_tensor_entry_points():
    torch = pytest.importorskip("torch")
    pts = W.gmm_cloud(200_000, seed=7)
    t = torch.from_numpy(pts).cuda()
    m = fps.get_fp_mode()
    out, tr = capi.kdline_tensor(t, 2000, 7, 0, trace=True)
    np.testing.assert_array_equal(out.cpu().numpy().astype(np.uint64),
                                  ORACLE.kdline(pts, 2000, 7, 0, m))
    out2, tr2 = capi.fps_tensor(t, 2000, [0, 9], trace=True)
    np.testing.assert_array_equal(out2.cpu().numpy().astype(np.uint64),
                                  ORACLE.fps(pts, 2000, [0, 9], m))
    ref = fp64_trace(pts, out2.cpu().numpy())
    np.testing.assert_allclose(tr2.cpu().numpy()[2:], ref[2:], rtol=1e-5)
    t1 = tr.cpu().numpy()
    assert np.all(np.diff(t1[1:]) <= 0)  # FPS max-min trace never increases


def _fixture_cloud(name):
    if not F.available():
        pytest.fail("tests/golden/fullsize.npz is missing (tests/golden/make_fullsize.py)")
    pts = F.cloud(name)
    assert F.input_matches(name, pts), f"the {name} generator no longer reproduces the fixture's input"
    return pts


@pytest.fixture(scope="module")
def gmm1m():
    return _fixture_cloud("gmm1m")


@pytest.fixture(scope="module")
def large16m():
    return _fixture_cloud("large16m")


def test_gmm_1m_kdline_h7_full(gmm1m, mode):
    """gmm-1m workload at full size: N=1,048,576, h=7, K=16,384, every sample
    against the reference's own answer."""
    got = fps.bucket_fps_kdline_sampling(gmm1m, 16384, 7, 0)
    np.testing.assert_array_equal(got, F.expected("gmm1m_kdline_h7", mode))


def test_gmm_1m_vanilla_full(gmm1m, mode):
    """Vanilla FPS on the same cloud, K=16,384: the plain call (thread-block
    cluster) and the traced call (grid sampler) both equal the reference's
    answer sample for sample; the fp32 trace never increases and follows the
    fp64 recomputation on its first samples."""
    torch = pytest.importorskip("torch")
    want = F.expected("gmm1m_vanilla", mode)
    np.testing.assert_array_equal(fps.fps_sampling(gmm1m, 16384, 0), want)
    out, tr = capi.fps_tensor(torch.from_numpy(gmm1m).cuda(), 16384, 0, trace=True)
    np.testing.assert_array_equal(out.cpu().numpy().astype(np.uint64), want)
    t = tr.cpu().numpy()
    assert np.all(np.diff(t[1:]) <= 0)
    ref = fp64_trace(gmm1m, want[:400])
    np.testing.assert_allclose(t[1:400], ref[1:400], rtol=1e-5)


def test_large_16m_d6_kdline_h9_full(large16m, mode):
    """large-16m workload at full size (N=16,777,216, D=6), kd-line h=9,
    K=65,536: every sample against the reference's answer, through the Python
    API and the traced device entry point (non-increasing trace)."""
    torch = pytest.importorskip("torch")
    want = F.expected("large16m_kdline_h9", mode)
    np.testing.assert_array_equal(fps.bucket_fps_kdline_sampling(large16m, 65536, 9, 0), want)
    out, tr = capi.kdline_tensor(torch.from_numpy(large16m).cuda(), 65536, 9, 0, trace=True)
    np.testing.assert_array_equal(out.cpu().numpy().astype(np.uint64), want)
    assert np.all(np.diff(tr.cpu().numpy()[1:]) <= 0)


def test_large_16m_d6_vanilla_full(large16m, mode):
    """Vanilla FPS on the 16.7M-point 6-D cloud, K=65,536: every sample
    against the multithreaded oracle's complete answer (whose first samples
    the reference confirmed)."""
    want = F.expected("large16m_vanilla", mode)
    np.testing.assert_array_equal(fps.fps_sampling(large16m, 65536, 0), want)


def test_beyond_register_capacity_uses_streaming_sampler():
    """33.5M points in one dimension: more pieces than the whole grid holds in
    registers, so the streaming sampler (piece records in HBM) runs."""
    rng = np.random.default_rng(33)
    pts = rng.random((1 << 25, 1), dtype=np.float32)
    m = fps.get_fp_mode()
    v = fps.fps_sampling(pts, 64, 7)
    np.testing.assert_array_equal(v, ORACLE.fps_mt(pts, 64, 7, m))
    assert len(np.unique(v)) == 64
    idx, xyz = fps.fps_sampling_points(pts, 64, 7)
    np.testing.assert_array_equal(idx, v)
    np.testing.assert_array_equal(xyz, pts[v.astype(np.int64)])
    kd = fps.bucket_fps_kdline_sampling(pts, 64, 1, 7)
    np.testing.assert_array_equal(kd, ORACLE.kdline(pts, 64, 1, 7, m))


@pytest.mark.parametrize("n,d", [(3000, 3), (20000, 3), (300_000, 3), (5000, 12),
                                 (2_500_000, 2)])
def test_sampled_points_are_the_gather(n, d, mode):
    """The *_points calls return the same indices as the plain calls and
    pc[indices] bit for bit, on every sampler: resident and streaming vanilla,
    one CTA, a cluster, forced starts on the grid, the register grid."""
    rng = np.random.default_rng(n + d)
    pts = (rng.standard_normal((n, d)) * 7).astype(np.float32)
    k = 700
    idx, xyz = fps.fps_sampling_points(pts, k, 11)
    np.testing.assert_array_equal(idx, fps.fps_sampling(pts, k, 11))
    np.testing.assert_array_equal(xyz, pts[idx.astype(np.int64)])
    idx, xyz = fps.fps_sampling_points(pts, k, [11, 5, 999])
    np.testing.assert_array_equal(idx, fps.fps_sampling(pts, k, [11, 5, 999]))
    np.testing.assert_array_equal(xyz, pts[idx.astype(np.int64)])
    if d <= 8:
        idx, xyz = fps.bucket_fps_kdline_sampling_points(pts, k, 7, 3)
        np.testing.assert_array_equal(idx, fps.bucket_fps_kdline_sampling(pts, k, 7, 3))
        np.testing.assert_array_equal(xyz, pts[idx.astype(np.int64)])
        idx, xyz = fps.bucket_fps_kdtree_sampling_points(pts, k, 3)
        np.testing.assert_array_equal(idx, fps.bucket_fps_kdtree_sampling(pts, k, 3))
        np.testing.assert_array_equal(xyz, pts[idx.astype(np.int64)])


def test_batch_points_are_the_gather():
    torch = pytest.importorskip("torch")
    clouds, ks, hs, ss = _batch_clouds(77, 12, 300, 30000)
    clouds.append(W.gmm_cloud(400_000, seed=9))  # more pieces than one CTA: a cluster
    ks.append(1500)
    hs.append(7)
    ss.append(5)
    sizes = [p.shape[0] for p in clouds]
    off = np.concatenate([[0], np.cumsum(sizes)])
    t = torch.from_numpy(np.concatenate(clouds)).cuda()
    out = torch.empty(sum(ks), dtype=torch.int64, device="cuda")
    xyz = torch.empty((sum(ks), 3), dtype=torch.float32, device="cuda")
    capi.kdline_batch_points_device(t.data_ptr(), off, 3, ks, hs, ss, out.data_ptr(),
                                    xyz.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got, pts_got = out.cpu().numpy(), xyz.cpu().numpy()
    want = capi.kdline_batch(clouds, ks, hs, ss)
    kb = np.concatenate([[0], np.cumsum(ks)])
    for c, p in enumerate(clouds):
        np.testing.assert_array_equal(got[kb[c]:kb[c + 1]].astype(np.uint64), want[c])
        np.testing.assert_array_equal(pts_got[kb[c]:kb[c + 1]], p[want[c].astype(np.int64)])


def _batch_clouds(seed, count, lo, hi, d=3):
    rng = np.random.default_rng(seed)
    clouds, ks, hs, ss = [], [], [], []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        kind = i % 3
        if kind == 0:
            p = rng.random((n, d)) * rng.uniform(0.1, 10, d)
        elif kind == 1:
            p = rng.integers(0, 6, (n, d))  # ties
        else:
            p = rng.standard_normal((n, d)) * 50
        clouds.append(p.astype(np.float32))
        ks.append(int(rng.integers(1, n + 1)))
        hs.append(int(rng.integers(1, max(1, int(np.log2(n))) + 1)))  # 2**h <= n
        ss.append(int(rng.integers(0, n)))
    return clouds, ks, hs, ss


@pytest.mark.parametrize("seed,d", [(0, 3), (1, 1), (2, 5), (3, 8)])
def test_batch_equals_oracle_per_cloud(seed, d, mode):
    clouds, ks, hs, ss = _batch_clouds(seed, 24, 2, 20000, d)
    got = fps.bucket_fps_kdline_sampling_batch(clouds, ks, hs, ss)
    for p, k, h, s, g in zip(clouds, ks, hs, ss, got):
        np.testing.assert_array_equal(g, ORACLE.kdline(p, k, h, s, mode))


@pytest.mark.parametrize("kind", ["kdline", "vanilla"])
def test_one_cta_sampler_epochs_with_ties(kind, mode):
    """Clouds of D <= 3 that one CTA samples with a hot table and many epochs,
    on a coarse lattice (many equal distances, some repeated points: ties
    decided by position, also between a hot piece and the workers' bound);
    every sample against the oracle."""
    rng = np.random.default_rng(21)
    cases = []
    for n, d in ((9000, 3), (40000, 3), (30000, 2), (20000, 1)):
        p = (np.round(rng.random((n, d)) * 40) / 4).astype(np.float32)  # 0.25 lattice
        cases.append((p, n // 4, 7, int(rng.integers(0, n))))
    if kind == "kdline":
        for d in (3, 2, 1):
            sub = [c for c in cases if c[0].shape[1] == d]
            got = fps.bucket_fps_kdline_sampling_batch([c[0] for c in sub], [c[1] for c in sub],
                                                        [c[2] for c in sub], [c[3] for c in sub])
            for (p, k, h, s), g in zip(sub, got):
                np.testing.assert_array_equal(g, ORACLE.kdline(p, k, h, s, mode))
    else:
        for p, k, _, s in cases:
            np.testing.assert_array_equal(fps.fps_sampling(p, k, s), ORACLE.fps(p, k, [s], mode))


_BATCH_CHILD = r"""
import sys
import numpy as np
import fpsample as fps
data = np.load(sys.argv[1], allow_pickle=True)
fps.set_fp_mode(str(data["mode"]))
got = fps.bucket_fps_kdline_sampling_batch(list(data["clouds"]), list(data["ks"]), list(data["hs"]),
                                           list(data["ss"]))
np.save(sys.argv[2], np.array(got, dtype=object), allow_pickle=True)
"""


def test_lockstep_one_cta_sampler_d3(mode, tmp_path):
    """The lockstep one-CTA sampler (batch_sample), which D <= 3 clouds take
    only with FPSGPU_ONECTA_SAMPLER=lockstep (read once per process, hence a
    child process), against the oracle."""
    import os
    import subprocess
    import sys

    clouds, ks, hs, ss = _batch_clouds(31, 12, 500, 60000, 3)
    inp, out = tmp_path / "in.npz", tmp_path / "out.npy"
    np.savez(inp, clouds=np.array(clouds, dtype=object), ks=ks, hs=hs, ss=ss, mode=mode)
    env = dict(os.environ, FPSGPU_ONECTA_SAMPLER="lockstep")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.run([sys.executable, "-c", _BATCH_CHILD, str(inp), str(out)], env=env, cwd=root,
                   check=True, timeout=600)
    got = np.load(out, allow_pickle=True)
    for p, k, h, s, g in zip(clouds, ks, hs, ss, got):
        np.testing.assert_array_equal(g, ORACLE.kdline(p, k, h, s, mode))


@pytest.mark.parametrize("hot", ["5", "7"])
def test_both_hot_table_widths_on_every_cloud_size(mode, hot, tmp_path):
    """The leader/worker sampler's two tables (55 and 77 hot pieces; a launch
    takes the wide one when it holds a cloud of 512 pieces or more) forced with
    FPSGPU_LEAD_HOT for clouds of every size, ties and a two-point cloud
    included, against the oracle (a child process: the setting is read
    once per process)."""
    import os
    import subprocess
    import sys

    clouds, ks, hs, ss = _batch_clouds(37, 14, 300, 120000, 3)
    clouds.append(np.array([[0, 0, 0], [1, 2, 3]], np.float32))  # the smallest cloud h = 1 allows
    ks.append(2)
    hs.append(1)
    ss.append(1)
    inp, out = tmp_path / "in.npz", tmp_path / "out.npy"
    np.savez(inp, clouds=np.array(clouds, dtype=object), ks=ks, hs=hs, ss=ss, mode=mode)
    env = dict(os.environ, FPSGPU_LEAD_HOT=hot)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.run([sys.executable, "-c", _BATCH_CHILD, str(inp), str(out)], env=env, cwd=root,
                   check=True, timeout=600)
    got = np.load(out, allow_pickle=True)
    for p, k, h, s, g in zip(clouds, ks, hs, ss, got):
        np.testing.assert_array_equal(g, ORACLE.kdline(p, k, h, s, mode))


def test_batch_with_clouds_too_big_for_shared_memory(mode):
    # one cloud with more piece records than fit in shared memory takes the
    # multi-CTA path inside the same batched call
    clouds, ks, hs, ss = _batch_clouds(7, 6, 500, 5000)
    big = W.gmm_cloud(400_000, seed=8)
    clouds.insert(2, big)
    ks.insert(2, 3000)
    hs.insert(2, 7)
    ss.insert(2, 11)
    got = capi.kdline_batch(clouds, ks, hs, ss)
    for p, k, h, s, g in zip(clouds, ks, hs, ss, got):
        np.testing.assert_array_equal(g, ORACLE.kdline(p, k, h, s, mode))


def test_batch_identical_to_one_call_per_cloud():
    clouds, ks, hs, ss = _batch_clouds(11, 40, 1000, 60000)
    got = fps.bucket_fps_kdline_sampling_batch(clouds, ks, hs, ss)
    for p, k, h, s, g in zip(clouds, ks, hs, ss, got):
        np.testing.assert_array_equal(g, fps.bucket_fps_kdline_sampling(p, k, h, s))


def test_batch_list_form_equals_contiguous_form():
    """One host buffer per cloud (fpsgpu_kdline_batch_list, the Python batch API's
    path) gives the same indices as the concatenated buffer (fpsgpu_kdline_batch),
    including clouds that are strided or float64 on the Python side."""
    clouds, ks, hs, ss = _batch_clouds(12, 30, 200, 40000)
    clouds[3] = np.asfortranarray(clouds[3])
    clouds[5] = clouds[5].astype(np.float64)
    want = capi.kdline_batch(clouds, ks, hs, ss)
    got_c = capi.kdline_batch_list(clouds, ks, hs, ss)
    got_py = fps.bucket_fps_kdline_sampling_batch(clouds, ks, hs, ss)
    for w, a, b in zip(want, got_c, got_py):
        np.testing.assert_array_equal(a, w)
        np.testing.assert_array_equal(b, w)


def _kdline_job(job):
    from oracle.oracle import Oracle

    p, k, h, s, m = job
    return Oracle().kdline(p, k, h, s, m)


def test_batched_workload_all_clouds_vs_oracle(mode):
    """The bench's 256-cloud workload: every sample of every cloud against the
    oracle (computed by a process pool)."""
    import multiprocessing as mp
    import os

    clouds = W.batched_clouds(seed=W.SEEDS["batched-256"])
    hs = [5 if p.shape[0] < 8192 else 7 for p, _ in clouds]
    got = fps.bucket_fps_kdline_sampling_batch([p for p, _ in clouds], [k for _, k in clouds], hs, 0)
    jobs = [(p, k, h, 0, mode) for (p, k), h in zip(clouds, hs)]
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        want = pool.map(_kdline_job, jobs)
    for i in range(len(clouds)):
        np.testing.assert_array_equal(got[i], want[i], err_msg=f"cloud {i}")


def test_cloud_beyond_shared_memory(mode):
    """1.2M points in 8 dimensions: plain calls run on a thread-block cluster;
    calls with a trace take the multi-CTA samplers, and these points do not fit
    the grid's shared memory, so the global-memory sampler runs.  All must give
    the oracle's answer."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    pts = rng.random((1_200_000, 8), dtype=np.float32)
    ref_kd = ORACLE.kdline(pts, 1500, 6, 5, mode)
    ref_v = ORACLE.fps(pts, 300, 5, mode)
    np.testing.assert_array_equal(fps.bucket_fps_kdline_sampling(pts, 1500, 6, 5), ref_kd)
    np.testing.assert_array_equal(fps.fps_sampling(pts, 300, 5), ref_v)
    t = torch.from_numpy(pts).cuda()
    out, _ = capi.kdline_tensor(t, 1500, 6, 5, trace=True)
    np.testing.assert_array_equal(out.cpu().numpy().astype(np.uint64), ref_kd)
    out, _ = capi.fps_tensor(t, 300, 5, trace=True)
    np.testing.assert_array_equal(out.cpu().numpy().astype(np.uint64), ref_v)


@pytest.mark.parametrize("d", [2, 3, 6])
def test_batch_with_several_cluster_clouds(d, mode):
    # clouds with more pieces than one CTA holds each get a thread-block
    # cluster; several of them share the cluster queue with small clouds
    clouds, ks, hs, ss = _batch_clouds(30 + d, 5, 300, 3000, d)
    rng = np.random.default_rng(d)
    for n in (300_000, 520_000, 760_000):
        clouds.append((rng.random((n, d)) * rng.uniform(1, 50, d)).astype(np.float32))
        ks.append(1200)
        hs.append(7)
        ss.append(int(rng.integers(0, n)))
    got = capi.kdline_batch(clouds, ks, hs, ss)
    for p, k, h, s, g in zip(clouds, ks, hs, ss, got):
        np.testing.assert_array_equal(g, ORACLE.kdline(p, k, h, s, mode))
