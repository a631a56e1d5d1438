"""GPU: fpsgpu_fps_device_noalloc, the vanilla FPS entry point that allocates
no GPU memory, for callers that cannot call cudaMalloc (memory owned by another
allocator or pool, loops with a no-allocation rule).  Its scratch is a fixed
array inside the library that every call reuses, so each case below calls it
twice in a row and both results must equal, index for index (the tolerance is
zero: indices are integers):
  * the oracle's answer (the C restatement of the reference's vanilla FPS,
    src/lib.cpp:111-246), in both floating-point modes;
  * the allocating entry point fpsgpu_fps_device on the same input.
For clouds of at most 8192 points both entry points run the same resident
kernel, so the oracle is the independent check there; beyond that the
allocating entry point takes the pruned engine.
This file is collected last on purpose and must also pass on its own."""
import numpy as np
import pytest

from fpsample_gb300 import capi
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

ORACLE = Oracle()


@pytest.fixture(params=["nofma", "fma"])
def mode(request):
    before = capi.get_fp_mode()
    capi.set_fp_mode(request.param)
    yield request.param
    capi.set_fp_mode(before)


def _noalloc(torch, t, k, starts):
    out = torch.full((k,), -1, dtype=torch.int64, device=t.device)
    capi.fps_device_noalloc(t.data_ptr(), t.shape[0], t.shape[1], k, starts, out.data_ptr(),
                            0, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return out.cpu().numpy().astype(np.uint64)


@pytest.mark.parametrize("n,d,k,starts", [
    (4096, 3, 1024, [0]),          # one CTA, cloud in shared memory
    (50000, 3, 2000, [5, 77, 5]),  # several CTAs exchanging through the fixed slots
    (65536, 6, 700, [1]),          # the size limit, 16 CTAs
    (300, 8, 300, [299]),
    (2000, 2, 2000, [3]),          # integer grid: ties everywhere, K = N
])
def test_noalloc_equals_oracle_and_allocating_entry_point_twice(n, d, k, starts, mode):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n + d)
    pts = rng.random((n, d), dtype=np.float32)
    if d == 2:
        pts = np.round(pts * 6).astype(np.float32)
    t = torch.from_numpy(pts).cuda()
    want = ORACLE.fps(pts, k, starts, mode)
    allocating = capi.fps_tensor(t, k, starts).cpu().numpy().astype(np.uint64)
    first = _noalloc(torch, t, k, starts)
    second = _noalloc(torch, t, k, starts)
    np.testing.assert_array_equal(first, want)
    np.testing.assert_array_equal(second, want)
    np.testing.assert_array_equal(allocating, want)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    t = torch.zeros((65537, 3), dtype=torch.float32, device="cuda")
    with pytest.raises(capi.FpsGpuError, match="at most 65536 points") as e:
        _noalloc(torch, t, 10, [0])
    assert e.value.code == 3
    t = torch.zeros((100, 3), dtype=torch.float32, device="cuda")
    with pytest.raises(capi.FpsGpuError, match="at most 512 start indices"):
        _noalloc(torch, t, 600, list(range(100)) * 6)
