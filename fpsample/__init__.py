"""fpsample, GB300 build: farthest point sampling on NVIDIA GB300 behind the
reference package's own module path.

``import fpsample`` and keep calling ``fps_sampling``,
``bucket_fps_kdline_sampling`` and ``bucket_fps_kdtree_sampling`` with the same
numpy arrays, ``n_samples``, ``h`` and ``start_idx``: the returned uint64 index
arrays are identical to the reference CPU library's.  The extension module is
``fpsample._fpsample`` with the reference's five function names.  The argument
checks below are the reference's own (reference ``src/fpsample/__init__.py:19-65``,
``:145-171`` and ``:174-206``), including their ``AssertionError`` messages and
the random start drawn from numpy's global ``np.random`` state when
``start_idx`` is None.

All sampling runs in the CUDA library ``fpsample_gb300/libfpsgpu.so`` through
the compiled extension ``_fpsample``; there is no CPU fallback.  Importing this
package fails with an ImportError if the extension has not been built (run
``python -c "import __graft_entry__ as g; g.build()"`` or
``python fpsample_gb300/_build.py``).

Floating point: distances follow the reference's fp32 operation order.  A
reference built by a compiler that contracts ``a*b+c`` into FMAs (GCC on
aarch64, the default there) picks different points at scale than one that
does not (x86-64 default); ``set_fp_mode("fma" | "nofma")`` selects which one
to match.  The default is the reference's stock build on this host's CPU
architecture ("fma" on aarch64, "nofma" elsewhere), or the environment
variable FPSAMPLE_FP_MODE.
"""
from __future__ import annotations

import os
from typing import List, Optional, Union

import numpy as np

# More hardware work queues than the default 8, so that kernels on different
# streams (request-server workers, the batched engine's side stream) never wait
# for each other by sharing a queue.  Read when the process first uses CUDA, so
# it only takes effect if this package is imported before that.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

try:
    from ._fpsample import (
        __doc__ as _ext_doc,
        __version__,
        _bucket_fps_kdline_sampling,
        _bucket_fps_kdline_sampling_batch,
        _bucket_fps_kdline_sampling_batch_list,
        _bucket_fps_kdtree_sampling,
        _fps_npdu_kdtree_sampling,
        _fps_npdu_sampling,
        _fps_sampling,
        _get_fp_mode,
        _kdline_build,
        _sample_points,
        _set_fp_mode,
        ALGO_FPS,
        ALGO_KDLINE,
        ALGO_KDTREE,
    )
except ImportError as e:  # loud: no CPU fallback exists
    raise ImportError(
        "fpsample's CUDA extension is not built or cannot be loaded "
        "(build it with `python fpsample_gb300/_build.py`): " + str(e)
    ) from e


def get_start_idx(n_pts: int, start_idx: Optional[Union[int, List[int]]]) -> Union[int, np.ndarray]:
    """None -> a random start from np.random; int -> itself; list -> uint64 array
    (reference src/fpsample/__init__.py:19-32)."""
    if start_idx is None:
        return np.random.randint(low=0, high=n_pts)
    if isinstance(start_idx, int):
        return start_idx
    if isinstance(start_idx, list):
        return np.array(start_idx, dtype=np.uint64)
    raise ValueError("start_idx should be None, int or list")


def fps_sampling(
    pc: np.ndarray, n_samples: int, start_idx: Optional[Union[int, List[int]]] = None
) -> np.ndarray:
    """
    Vanilla FPS sampling on the GPU.

    Args:
        pc (np.ndarray): The input point cloud of shape (n_pts, D).
        n_samples (int): Number of samples.
        start_idx (int or list[int], default=None): The starting index of sampling. If set to None, it will be randomly picked.
            If multiple start indices are given, they are used as a start set for the FPS and will all be present in the final samples.
    Returns:
        np.ndarray: The selected indices of shape (n_samples,), uint64.
    """
    assert n_samples >= 1, "n_samples should be >= 1"
    assert pc.ndim == 2
    n_pts, _ = pc.shape
    assert n_pts >= n_samples, "n_pts should be >= n_samples"
    if isinstance(start_idx, int):
        assert 0 <= start_idx < n_pts, "start_idx should be None or 0 <= start_idx < n_pts"
    if isinstance(start_idx, list):
        assert len(start_idx) <= n_samples, "len(start_idx) should be <= n_samples"
        for idx in start_idx:
            assert 0 <= idx < n_pts, "start_idx should be None or 0 <= start_idx < n_pts"
    pc = np.ascontiguousarray(pc, dtype=np.float32)
    start_idx = get_start_idx(n_pts, start_idx)
    return _fps_sampling(pc, n_samples, start_idx)


def bucket_fps_kdline_sampling(
    pc: np.ndarray, n_samples: int, h: int, start_idx: Optional[Union[int, List[int]]] = None
) -> np.ndarray:
    """
    Bucket-based FPS sampling with a kd-line tree of height ``h`` ("QuickFPS") on the GPU.

    Args:
        pc (np.ndarray): The input point cloud of shape (n_pts, D), D <= 8.
        n_samples (int): Number of samples.
        h (int): Height of the kd tree; the tree has up to ``2**h`` buckets.
            h=3 or 5 suits small clouds, h=7 medium ones, h=9 very large ones.
        start_idx (int, default=None): The starting index of sampling. If set to None, it will be randomly picked.
            As in the reference, it names a position of the tree build's permuted order.

    Returns:
        np.ndarray: The selected indices of shape (n_samples,), uint64.
    """
    assert n_samples >= 1, "n_samples should be >= 1"
    assert pc.ndim == 2
    n_pts, _ = pc.shape
    assert n_pts >= n_samples, "n_pts should be >= n_samples"
    assert h >= 1, "h should be >= 1"
    assert 2**h <= n_pts, "2**h should be <= n_pts"
    assert start_idx is None or 0 <= start_idx < n_pts, "start_idx should be None or 0 <= start_idx < n_pts"
    if isinstance(start_idx, list):
        assert len(start_idx) <= n_samples, "len(start_idx) should be <= n_samples"
    pc = np.ascontiguousarray(pc, dtype=np.float32)
    start_idx = get_start_idx(n_pts, start_idx)
    return _bucket_fps_kdline_sampling(pc, n_samples, h, start_idx)


def bucket_fps_kdline_sampling_batch(pcs, n_samples, h, start_idx=0):
    """
    Many clouds in one GPU call (no counterpart in the reference): the result
    for every cloud is identical to ``bucket_fps_kdline_sampling`` on it alone.

    Args:
        pcs (list[np.ndarray]): point clouds of shape (n_i, D), same D <= 8.
        n_samples (int or list[int]): samples per cloud.
        h (int or list[int]): tree height per cloud.
        start_idx (int or list[int], default=0): start per cloud (no random start).

    Returns:
        list[np.ndarray]: uint64 indices per cloud.
    """
    m = len(pcs)
    ks = [n_samples] * m if isinstance(n_samples, int) else list(n_samples)
    hs = [h] * m if isinstance(h, int) else list(h)
    ss = [start_idx] * m if isinstance(start_idx, int) else list(start_idx)
    assert len(ks) == m and len(hs) == m and len(ss) == m, "one value per cloud"
    if m == 0:
        return []
    dims = {np.asarray(p).shape[1] for p in pcs}
    assert len(dims) == 1, "all clouds must have the same dimension"
    for p, k, hh, s in zip(pcs, ks, hs, ss):
        n_pts = np.asarray(p).shape[0]
        assert np.asarray(p).ndim == 2
        assert 1 <= k <= n_pts, "n_pts should be >= n_samples >= 1"
        assert hh >= 1, "h should be >= 1"
        assert 2**hh <= n_pts, "2**h should be <= n_pts"
        assert 0 <= s < n_pts, "0 <= start_idx < n_pts"
    # one buffer per cloud goes to the library as is: no host-side concatenation
    clouds = [np.ascontiguousarray(p, dtype=np.float32) for p in pcs]
    out = _bucket_fps_kdline_sampling_batch_list(clouds, np.array(ks, np.uint64),
                                                 np.array(hs, np.uint64), np.array(ss, np.uint64))
    bounds = np.concatenate([[0], np.cumsum(ks)])
    return [out[bounds[i]:bounds[i + 1]] for i in range(m)]


def fps_npdu_sampling(pc, n_samples, w=None, start_idx=None):
    """Not part of the GB300 build (heuristic NPDU variant); raises NotImplementedError."""
    return _fps_npdu_sampling(pc, n_samples, w, start_idx)


def fps_npdu_kdtree_sampling(pc, n_samples, w=None, start_idx=None):
    """Not part of the GB300 build (heuristic NPDU + kd-tree variant); raises NotImplementedError."""
    return _fps_npdu_kdtree_sampling(pc, n_samples, w, start_idx)


def bucket_fps_kdtree_sampling(
    pc: np.ndarray, n_samples: int, start_idx: Optional[Union[int, List[int]]] = None
) -> np.ndarray:
    """
    Bucket-based FPS sampling using KDTree. Also called "QuickFPS" in the paper.

    Args:
        pc (np.ndarray): The input point cloud of shape (n_pts, D).
        n_samples (int): Number of samples.
        start_idx (int or list[int], default=None): The starting index of sampling. If set to None, it will be randomly picked.
            If multiple start indices are given, they are used as a start set for the FPS and will all be present in the final samples.
    Returns:
        np.ndarray: The selected indices of shape (n_samples,).

    Same checks and results as the reference (src/fpsample/__init__.py:145-171),
    computed on the GPU: the kd-line engine with no height limit and ties to
    the last position of the tree's order (KDNode.h:41-46).
    """
    assert n_samples >= 1, "n_samples should be >= 1"
    assert pc.ndim == 2
    n_pts, _ = pc.shape
    assert n_pts >= n_samples, "n_pts should be >= n_samples"
    assert (
        start_idx is None or 0 <= start_idx < n_pts
    ), "start_idx should be None or 0 <= start_idx < n_pts"
    if isinstance(start_idx, list):
        assert len(start_idx) <= n_samples, "len(start_idx) should be <= n_samples"
    pc = np.ascontiguousarray(pc, dtype=np.float32)
    # Random pick a start if not given
    start_idx = get_start_idx(n_pts, start_idx)
    return _bucket_fps_kdtree_sampling(pc, n_samples, start_idx)


def _starts_array(start_idx) -> np.ndarray:
    return np.atleast_1d(np.asarray(start_idx, dtype=np.uint64))


def fps_sampling_points(pc: np.ndarray, n_samples: int,
                        start_idx: Optional[Union[int, List[int]]] = None):
    """fps_sampling plus the gather the caller would do next: returns
    (indices, pc[indices]) with the points as float32 [n_samples, D], written by
    the sampler as it picks them (no second pass over the cloud).  Same
    checks and indices as fps_sampling."""
    assert n_samples >= 1, "n_samples should be >= 1"
    assert pc.ndim == 2
    n_pts, _ = pc.shape
    assert n_pts >= n_samples, "n_pts should be >= n_samples"
    if isinstance(start_idx, int):
        assert 0 <= start_idx < n_pts, "start_idx should be None or 0 <= start_idx < n_pts"
    if isinstance(start_idx, list):
        assert len(start_idx) <= n_samples, "len(start_idx) should be <= n_samples"
        for idx in start_idx:
            assert 0 <= idx < n_pts, "start_idx should be None or 0 <= start_idx < n_pts"
    pc = np.ascontiguousarray(pc, dtype=np.float32)
    start_idx = get_start_idx(n_pts, start_idx)
    return _sample_points(ALGO_FPS, pc, n_samples, _starts_array(start_idx), 0)


def bucket_fps_kdline_sampling_points(pc: np.ndarray, n_samples: int, h: int,
                                      start_idx: Optional[int] = None):
    """bucket_fps_kdline_sampling plus the fused gather: (indices, points)."""
    assert n_samples >= 1, "n_samples should be >= 1"
    assert pc.ndim == 2
    n_pts, _ = pc.shape
    assert n_pts >= n_samples, "n_pts should be >= n_samples"
    assert h >= 1, "h should be >= 1"
    assert 2**h <= n_pts, "2**h should be <= n_pts"
    assert (
        start_idx is None or 0 <= start_idx < n_pts
    ), "start_idx should be None or 0 <= start_idx < n_pts"
    pc = np.ascontiguousarray(pc, dtype=np.float32)
    start_idx = get_start_idx(n_pts, start_idx)
    return _sample_points(ALGO_KDLINE, pc, n_samples, _starts_array(start_idx), h)


def bucket_fps_kdtree_sampling_points(pc: np.ndarray, n_samples: int,
                                      start_idx: Optional[int] = None):
    """bucket_fps_kdtree_sampling plus the fused gather: (indices, points)."""
    assert n_samples >= 1, "n_samples should be >= 1"
    assert pc.ndim == 2
    n_pts, _ = pc.shape
    assert n_pts >= n_samples, "n_pts should be >= n_samples"
    assert (
        start_idx is None or 0 <= start_idx < n_pts
    ), "start_idx should be None or 0 <= start_idx < n_pts"
    pc = np.ascontiguousarray(pc, dtype=np.float32)
    start_idx = get_start_idx(n_pts, start_idx)
    return _sample_points(ALGO_KDTREE, pc, n_samples, _starts_array(start_idx), 0)


def set_fp_mode(mode: str) -> None:
    """Select the distance arithmetic to match: "nofma" (reference built without
    FMA contraction, the x86-64 default) or "fma" (contracting build)."""
    _set_fp_mode(mode)


def get_fp_mode() -> str:
    return _get_fp_mode()


def kdline_build(pc: np.ndarray, h: int):
    """The kd-line tree build alone: (perm, bucket_starts), both uint64.
    perm[p] is the original index of the point at position p of the permuted
    order; bucket_starts lists the first position of every bucket."""
    pc = np.ascontiguousarray(pc, dtype=np.float32)
    return _kdline_build(pc, h)


__doc__ = (__doc__ or "") + (_ext_doc or "")

__all__ = [
    "__doc__",
    "__version__",
    "fps_sampling",
    "fps_npdu_sampling",
    "fps_npdu_kdtree_sampling",
    "bucket_fps_kdtree_sampling",
    "fps_sampling_points",
    "bucket_fps_kdline_sampling_points",
    "bucket_fps_kdtree_sampling_points",
    "bucket_fps_kdline_sampling",
    "bucket_fps_kdline_sampling_batch",
    "set_fp_mode",
    "get_fp_mode",
    "kdline_build",
]
