"""GPU: failure handling without a GPU fault.

* The multi-CTA samplers' grid exchange waits on other CTAs with a bounded
  poll count; fpsgpu_selftest_exchange_timeout runs that exchange with a
  partner that never arrives (one CTA launched for a grid of two, a limit of
  4096 polls).  The call must return FPSGPU_ERR_DEVICE, and the GPU must stay
  usable: a normal call right after it is still bit-exact.
* The one-CTA leader/worker sampler's worker warps wait for the leader's next
  sample with a bounded poll count; fpsgpu_selftest_lead_timeout runs it with
  the leader muted (a limit of 4096 polls) and must return FPSGPU_ERR_DEVICE,
  the next call still exact.
* Host-side fault injection: fpsgpu_debug_fail_allocations refuses the N-th
  scratch allocation.  For every N up to the first one the call survives, the
  call must raise the reference's RuntimeError, and the next call must succeed
  with the same indices as before.  In the request server, a refused batch
  fails its requests and the workers keep serving.
"""
import numpy as np
import pytest

import fpsample as fps
from fpsample_gb300 import capi
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

FPSGPU_ERR_DEVICE = 5


def test_bounded_exchange_wait_reports_an_error_and_the_gpu_stays_usable():
    lib = capi.lib()
    assert lib.fpsgpu_selftest_exchange_timeout() == FPSGPU_ERR_DEVICE
    assert "gave up" in lib.fpsgpu_last_error().decode()
    pts = np.random.default_rng(71).random((3000, 3)).astype(np.float32)
    got = fps.bucket_fps_kdline_sampling(pts, 300, 5, 0)
    np.testing.assert_array_equal(got, Oracle().kdline(pts, 300, 5, 0, fps.get_fp_mode()))


def test_bounded_worker_wait_of_the_one_cta_sampler_reports_an_error():
    """The leader/worker sampler's worker warps wait for the leader's next
    sample with a bounded poll count; with the leader muted they must give
    up, the call must return FPSGPU_ERR_DEVICE, and the next call must still
    be exact."""
    lib = capi.lib()
    assert lib.fpsgpu_selftest_lead_timeout() == FPSGPU_ERR_DEVICE
    assert "gave up" in lib.fpsgpu_last_error().decode()
    rng = np.random.default_rng(73)
    clouds = [rng.random((n, 3)).astype(np.float32) for n in (20000, 3000)]
    got = fps.bucket_fps_kdline_sampling_batch(clouds, [5000, 700], 5, 0)
    oracle = Oracle()
    for p, k, g in zip(clouds, (5000, 700), got):
        np.testing.assert_array_equal(g, oracle.kdline(p, k, 5, 0, fps.get_fp_mode()))


@pytest.mark.parametrize("algo", ["kdline", "vanilla", "batch"])
def test_refused_allocations_fail_cleanly_and_the_next_call_recovers(algo):
    lib = capi.lib()
    rng = np.random.default_rng(72)
    pts = rng.random((20000, 3)).astype(np.float32)
    clouds = [rng.random((n, 3)).astype(np.float32) for n in (900, 5000, 30000)]

    def call():
        if algo == "kdline":
            return fps.bucket_fps_kdline_sampling(pts, 500, 7, 3)
        if algo == "vanilla":
            return fps.fps_sampling(pts, 500, 3)
        return np.concatenate(fps.bucket_fps_kdline_sampling_batch(clouds, [100, 700, 2000], 5, 0))

    want = call()
    refused = 0
    for after in range(200):
        lib.fpsgpu_debug_fail_allocations(after)
        try:
            got = call()
        except RuntimeError as e:
            # the reference's message (kd-line: "... failed with error code 4");
            # the library's own message says why
            assert "error code 4" in str(e)
            assert "injected" in lib.fpsgpu_last_error().decode()
            refused += 1
            got = None
        finally:
            lib.fpsgpu_debug_fail_allocations(-1)
        np.testing.assert_array_equal(call(), want)
        if got is not None:  # every allocation of the call fit in the budget
            np.testing.assert_array_equal(got, want)
            break
    else:
        pytest.fail("the call never completed within 200 allocations")
    assert refused >= 3


def test_request_server_fails_requests_cleanly_and_keeps_serving():
    """A batch whose scratch allocation is refused fails its requests with
    FPSGPU_ERR_CUDA; the server's workers carry on and later requests are
    exact."""
    import workloads as W

    lib = capi.lib()
    rng = np.random.default_rng(73)
    reqs = []
    for n in (5000, 12000, 30000):
        p = W.sphere_cloud(rng, n)
        reqs.append((p, n // 8, 7 if n >= 8192 else 5, int(rng.integers(0, n))))
    want = [fps.bucket_fps_kdline_sampling(p, k, h, s) for p, k, h, s in reqs]
    with capi.Server(1 << 30, small_workers=1, large_workers=1) as srv:
        lib.fpsgpu_debug_fail_allocations(0)
        try:
            p, k, h, s = reqs[0]
            t = srv.submit(p, k, h, s)
            with pytest.raises(capi.FpsGpuError) as e:
                srv.result(t)
            assert e.value.code == 4
        finally:
            lib.fpsgpu_debug_fail_allocations(-1)
        tickets = [srv.submit(p, k, h, s) for p, k, h, s in reqs]
        for t, w in zip(tickets, want):
            np.testing.assert_array_equal(srv.result(t)[0], w)
