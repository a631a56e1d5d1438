"""GPU: the request server (continuous batching) returns, for every request,
exactly what one bucket_fps_kdline call on that cloud alone returns -- whether
requests arrive together, from several threads, or under a memory budget that
forces them to wait for each other."""
import threading

import numpy as np
import pytest

import fpsample as fps
from fpsample_gb300 import capi
import workloads as W
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _requests(seed, count, lo, hi):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        pts = W.sphere_cloud(rng, n)
        k = int(rng.integers(max(1, n // 16), n // 4 + 1))
        h = 5 if n < 8192 else (7 if n < 262144 else 9)
        out.append((pts, k, h, int(rng.integers(0, n))))
    return out


def test_server_mixed_sizes_equal_single_calls():
    reqs = _requests(0, 24, 600, 400_000)  # includes the large-request class
    with capi.Server(8 << 30, small_workers=4, large_workers=2) as srv:
        tickets = [srv.submit(p, k, h, s) for p, k, h, s in reqs]
        results = [srv.result(t) for t in tickets]
    for (p, k, h, s), (idx, q_ms, tot_ms) in zip(reqs, results):
        np.testing.assert_array_equal(idx, fps.bucket_fps_kdline_sampling(p, k, h, s))
        assert 0 <= q_ms <= tot_ms


def test_server_against_oracle_and_from_two_threads():
    reqs = _requests(1, 16, 500, 40_000)
    orc = Oracle()
    results = {}
    with capi.Server(4 << 30, small_workers=3, large_workers=1) as srv:
        def client(part):
            for i in part:
                p, k, h, s = reqs[i]
                results[i] = srv.result(srv.submit(p, k, h, s))[0]
        ts = [threading.Thread(target=client, args=(range(j, len(reqs), 2),)) for j in (0, 1)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
    for i, (p, k, h, s) in enumerate(reqs):
        np.testing.assert_array_equal(results[i], orc.kdline(p, k, h, s, fps.get_fp_mode()))


def test_server_tight_memory_budget():
    # a budget smaller than one request: requests run one at a time, in order
    reqs = _requests(2, 6, 20_000, 60_000)
    with capi.Server(1 << 20, small_workers=2, large_workers=1) as srv:
        tickets = [srv.submit(p, k, h, s) for p, k, h, s in reqs]
        results = [srv.result(t)[0] for t in tickets]
    for (p, k, h, s), idx in zip(reqs, results):
        np.testing.assert_array_equal(idx, capi.bucket_fps_kdline(p, k, s, h))


def test_server_refuses_a_second_waiter_on_one_ticket():
    # one waiter per ticket: of two threads waiting on the same ticket, the
    # one that claims it gets the result and the other an argument error,
    # instead of touching a request the first waiter frees
    import ctypes

    rng = np.random.default_rng(5)
    pts = np.ascontiguousarray(W.sphere_cloud(rng, 300_000), np.float32)
    out = np.empty(60_000, np.uint64)
    with capi.Server(8 << 30, small_workers=1, large_workers=1) as srv:
        t = ctypes.c_uint64(0)
        rc = capi.lib().fpsgpu_server_submit(srv._h, pts.ctypes.data_as(capi._f32p), pts.shape[0],
                                             3, out.size, 0, 9, out.ctypes.data_as(capi._szp),
                                             ctypes.byref(t))
        assert rc == 0
        rcs = []
        lock = threading.Lock()

        def waiter():
            rc = capi.lib().fpsgpu_server_wait(srv._h, t.value, None, None)
            with lock:
                rcs.append(rc)

        ths = [threading.Thread(target=waiter) for _ in range(2)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
    # FPSGPU_ERR_ARG (3): ticket already waited on, or already gone
    assert sorted(rcs) == [0, 3]
    np.testing.assert_array_equal(out, capi.bucket_fps_kdline(pts, out.size, 0, 9))
