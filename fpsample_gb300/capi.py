"""ctypes view of libfpsgpu's C ABI (include/fpsgpu.h).

For callers that hold device buffers (for example torch CUDA tensors) or want
to call the C entry points directly from Python.  Everything here runs on the
GPU; failures raise ``FpsGpuError`` with the library's code and message.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfpsgpu.so")

_sz = ctypes.c_size_t
_vp = ctypes.c_void_p
_u64p = ctypes.POINTER(ctypes.c_uint64)
_f32p = ctypes.POINTER(ctypes.c_float)
_szp = ctypes.POINTER(ctypes.c_size_t)

# name -> (restype, argtypes)
SIGNATURES = {
    "bucket_fps_kdline": (ctypes.c_int, [_f32p, _sz, _sz, _sz, _sz, _sz, _szp]),
    "bucket_fps_kdtree": (ctypes.c_int, [_f32p, _sz, _sz, _sz, _sz, _szp]),
    "fpsgpu_kdtree_device": (ctypes.c_int, [_vp, _sz, _sz, _sz, _sz, _vp, _vp, _vp]),
    "fpsgpu_fps": (ctypes.c_int, [_f32p, _sz, _sz, _sz, _szp, _sz, _szp]),
    "fpsgpu_kdline_device": (ctypes.c_int, [_vp, _sz, _sz, _sz, _sz, _sz, _vp, _vp, _vp]),
    "fpsgpu_fps_device": (ctypes.c_int, [_vp, _sz, _sz, _sz, _szp, _sz, _vp, _vp, _vp]),
    "fpsgpu_fps_device_noalloc": (ctypes.c_int, [_vp, _sz, _sz, _sz, _szp, _sz, _vp, _vp, _vp]),
    "fpsgpu_kdline_build": (ctypes.c_int, [_f32p, _sz, _sz, _sz, _u64p, _u64p, _szp]),
    "fpsgpu_kdline_batch": (ctypes.c_int, [_f32p, _szp, _sz, _sz, _szp, _szp, _szp, _szp]),
    "fpsgpu_kdline_batch_list": (ctypes.c_int, [ctypes.POINTER(_f32p), _szp, _sz, _sz, _szp, _szp,
                                                _szp, _szp]),
    "fpsgpu_kdline_batch_device": (ctypes.c_int, [_vp, _szp, _sz, _sz, _szp, _szp, _szp, _vp, _vp]),
    "fpsgpu_server_create": (ctypes.c_int, [_sz, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_vp)]),
    "fpsgpu_server_submit": (ctypes.c_int, [_vp, _f32p, _sz, _sz, _sz, _sz, _sz, _szp, _u64p]),
    "fpsgpu_server_wait": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_double)]),
    "fpsgpu_server_destroy": (ctypes.c_int, [_vp]),
    "fpsgpu_set_fp_mode": (ctypes.c_int, [ctypes.c_int]),
    "fpsgpu_get_fp_mode": (ctypes.c_int, []),
    "fpsgpu_stats_reset": (None, []),
    "fpsgpu_stats_get": (None, [ctypes.c_void_p]),
    "fpsgpu_stats_timing": (None, [ctypes.c_int]),
    "fpsgpu_last_error": (ctypes.c_char_p, []),
    "fpsgpu_selftest_exchange_timeout": (ctypes.c_int, []),
    "fpsgpu_selftest_lead_timeout": (ctypes.c_int, []),
    "fpsgpu_debug_fail_allocations": (None, [ctypes.c_longlong]),
    "fpsgpu_sample_points": (ctypes.c_int, [ctypes.c_int, _f32p, _sz, _sz, _sz, _szp, _sz, _sz,
                                            _szp, _f32p]),
    "fpsgpu_sample_points_device": (ctypes.c_int, [ctypes.c_int, _vp, _sz, _sz, _sz, _szp, _sz,
                                                   _sz, _vp, _vp, _vp]),
    "fpsgpu_kdline_batch_points_device": (ctypes.c_int, [_vp, _szp, _sz, _sz, _szp, _szp, _szp,
                                                         _vp, _vp, _vp]),
    "fpsgpu_version": (ctypes.c_char_p, []),
}

FP_MODES = {"nofma": 0, "fma": 1}


class Stats(ctypes.Structure):
    """fpsgpu_stats (include/fpsgpu.h)."""

    _fields_ = [("kernel_launches", ctypes.c_uint64), ("sampler_launches", ctypes.c_uint64),
                ("sampler_ms", ctypes.c_double), ("samples", ctypes.c_uint64),
                ("pieces_tested", ctypes.c_uint64), ("points_touched", ctypes.c_uint64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


def stats_reset() -> None:
    lib().fpsgpu_stats_reset()


def stats_timing(enable: bool) -> None:
    lib().fpsgpu_stats_timing(1 if enable else 0)


def stats() -> dict:
    s = Stats()
    lib().fpsgpu_stats_get(ctypes.byref(s))
    return s.as_dict()


class FpsGpuError(RuntimeError):
    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn} failed with error code {code}: {msg}")
        self.code = code


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is not built (python fpsample_gb300/_build.py)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(fn: str, rc: int) -> None:
    if rc != 0:
        raise FpsGpuError(fn, rc, lib().fpsgpu_last_error().decode())


def _rows(pc) -> np.ndarray:
    a = np.ascontiguousarray(pc, dtype=np.float32)
    if a.ndim != 2:
        raise ValueError("points must be 2D")
    return a


def set_fp_mode(mode: str) -> None:
    _check("fpsgpu_set_fp_mode", lib().fpsgpu_set_fp_mode(FP_MODES[mode]))


def get_fp_mode() -> str:
    return {v: k for k, v in FP_MODES.items()}[lib().fpsgpu_get_fp_mode()]


def bucket_fps_kdline(pc, n_samples: int, start_idx: int, height: int) -> np.ndarray:
    """The reference-compatible C entry point, host buffers."""
    a = _rows(pc)
    out = np.zeros(n_samples, np.uint64)
    rc = lib().bucket_fps_kdline(a.ctypes.data_as(_f32p), a.shape[0], a.shape[1], n_samples,
                                 start_idx, height, out.ctypes.data_as(_szp))
    _check("bucket_fps_kdline", rc)
    return out


def bucket_fps_kdtree(pc, n_samples: int, start_idx: int) -> np.ndarray:
    """The reference-compatible kd-tree C entry point, host buffers."""
    a = _rows(pc)
    out = np.zeros(n_samples, np.uint64)
    rc = lib().bucket_fps_kdtree(a.ctypes.data_as(_f32p), a.shape[0], a.shape[1], n_samples,
                                 start_idx, out.ctypes.data_as(_szp))
    _check("bucket_fps_kdtree", rc)
    return out


def kdtree_tensor(points, n_samples: int, start_idx: int = 0, trace: bool = False):
    """bucket_fps_kdtree on a torch CUDA tensor [N, D] float32; int64 CUDA tensor out."""
    import torch

    pts = points.contiguous()
    if pts.dtype != torch.float32 or not pts.is_cuda or pts.dim() != 2:
        raise ValueError("points must be a 2D float32 CUDA tensor")
    out = torch.empty(n_samples, dtype=torch.int64, device=pts.device)
    tr = torch.empty(n_samples, dtype=torch.float32, device=pts.device) if trace else None
    with torch.cuda.device(pts.device):
        stream = torch.cuda.current_stream().cuda_stream
        _check("fpsgpu_kdtree_device",
               lib().fpsgpu_kdtree_device(pts.data_ptr(), pts.shape[0], pts.shape[1], n_samples,
                                          start_idx, out.data_ptr(), tr.data_ptr() if trace else 0,
                                          stream))
    return (out, tr) if trace else out


def fps(pc, n_samples: int, starts) -> np.ndarray:
    a = _rows(pc)
    st = np.atleast_1d(np.asarray(starts, dtype=np.uint64))
    out = np.zeros(n_samples, np.uint64)
    rc = lib().fpsgpu_fps(a.ctypes.data_as(_f32p), a.shape[0], a.shape[1], n_samples,
                          st.ctypes.data_as(_szp), st.size, out.ctypes.data_as(_szp))
    _check("fpsgpu_fps", rc)
    return out


def kdline_build(pc, height: int):
    a = _rows(pc)
    n = a.shape[0]
    perm = np.zeros(n, np.uint64)
    bst = np.zeros(n, np.uint64)
    nb = _sz(0)
    rc = lib().fpsgpu_kdline_build(a.ctypes.data_as(_f32p), n, a.shape[1], height,
                                   perm.ctypes.data_as(_u64p), bst.ctypes.data_as(_u64p),
                                   ctypes.byref(nb))
    _check("fpsgpu_kdline_build", rc)
    return perm, bst[: nb.value].copy()


def kdline_device(points_ptr: int, n: int, dim: int, n_samples: int, start_idx: int, height: int,
                  out_ptr: int, trace_ptr: int = 0, stream: int = 0) -> None:
    """Device pointers (e.g. tensor.data_ptr()); out: n_samples uint64 (int64 tensor)."""
    rc = lib().fpsgpu_kdline_device(points_ptr, n, dim, n_samples, start_idx, height, out_ptr,
                                    trace_ptr or None, stream or None)
    _check("fpsgpu_kdline_device", rc)


def fps_device(points_ptr: int, n: int, dim: int, n_samples: int, starts, out_ptr: int,
               trace_ptr: int = 0, stream: int = 0) -> None:
    st = np.atleast_1d(np.asarray(starts, dtype=np.uint64))
    rc = lib().fpsgpu_fps_device(points_ptr, n, dim, n_samples, st.ctypes.data_as(_szp), st.size,
                                 out_ptr, trace_ptr or None, stream or None)
    _check("fpsgpu_fps_device", rc)


def kdline_tensor(points, n_samples: int, height: int, start_idx: int = 0, trace: bool = False):
    """torch CUDA tensor [N, D] float32 in, int64 CUDA tensor [K] out (same values
    as the uint64 indices), on the tensor's device and torch's current stream."""
    import torch

    pts = points.contiguous()
    if pts.dtype != torch.float32 or not pts.is_cuda or pts.dim() != 2:
        raise ValueError("points must be a 2D float32 CUDA tensor")
    out = torch.empty(n_samples, dtype=torch.int64, device=pts.device)
    tr = torch.empty(n_samples, dtype=torch.float32, device=pts.device) if trace else None
    with torch.cuda.device(pts.device):
        stream = torch.cuda.current_stream().cuda_stream
        kdline_device(pts.data_ptr(), pts.shape[0], pts.shape[1], n_samples, start_idx, height,
                      out.data_ptr(), tr.data_ptr() if trace else 0, stream)
    return (out, tr) if trace else out


def fps_tensor(points, n_samples: int, starts=0, trace: bool = False):
    """torch CUDA tensor [N, D] float32 in, int64 CUDA tensor [K] out."""
    import torch

    pts = points.contiguous()
    if pts.dtype != torch.float32 or not pts.is_cuda or pts.dim() != 2:
        raise ValueError("points must be a 2D float32 CUDA tensor")
    out = torch.empty(n_samples, dtype=torch.int64, device=pts.device)
    tr = torch.empty(n_samples, dtype=torch.float32, device=pts.device) if trace else None
    with torch.cuda.device(pts.device):
        stream = torch.cuda.current_stream().cuda_stream
        fps_device(pts.data_ptr(), pts.shape[0], pts.shape[1], n_samples, starts, out.data_ptr(),
                   tr.data_ptr() if trace else 0, stream)
    return (out, tr) if trace else out


def kdline_batch(pcs, n_samples, heights, starts):
    """Host-buffer batched QuickFPS through the C ABI; list of uint64 arrays."""
    sizes = [np.asarray(p).shape[0] for p in pcs]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    pts = np.ascontiguousarray(np.concatenate([np.asarray(p, np.float32) for p in pcs]))
    ks = np.asarray(n_samples, np.uint64)
    out = np.zeros(int(ks.sum()), np.uint64)
    hs = np.asarray(heights, np.uint64)
    ss = np.asarray(starts, np.uint64)
    rc = lib().fpsgpu_kdline_batch(pts.ctypes.data_as(_f32p), off.ctypes.data_as(_szp), len(pcs),
                                   pts.shape[1], ks.ctypes.data_as(_szp), ss.ctypes.data_as(_szp),
                                   hs.ctypes.data_as(_szp), out.ctypes.data_as(_szp))
    _check("fpsgpu_kdline_batch", rc)
    b = np.concatenate([[0], np.cumsum(ks)]).astype(np.int64)
    return [out[b[i]:b[i + 1]] for i in range(len(pcs))]


def kdline_batch_list(pcs, n_samples, heights, starts):
    """Host-buffer batched QuickFPS with one buffer per cloud (no concatenation)
    through the C ABI; list of uint64 arrays."""
    clouds = [np.ascontiguousarray(p, np.float32) for p in pcs]
    ptrs = (_f32p * max(1, len(clouds)))(*[c.ctypes.data_as(_f32p) for c in clouds])
    npts = np.asarray([c.shape[0] for c in clouds], np.uint64)
    dim = clouds[0].shape[1] if clouds else 3
    ks = np.asarray(n_samples, np.uint64)
    out = np.zeros(max(1, int(ks.sum())), np.uint64)
    hs = np.asarray(heights, np.uint64)
    ss = np.asarray(starts, np.uint64)
    rc = lib().fpsgpu_kdline_batch_list(ptrs, npts.ctypes.data_as(_szp), len(clouds), dim,
                                        ks.ctypes.data_as(_szp), ss.ctypes.data_as(_szp),
                                        hs.ctypes.data_as(_szp), out.ctypes.data_as(_szp))
    _check("fpsgpu_kdline_batch_list", rc)
    b = np.concatenate([[0], np.cumsum(ks)]).astype(np.int64)
    return [out[b[i]:b[i + 1]] for i in range(len(clouds))]


def kdline_batch_device(points_ptr: int, offsets, dim: int, n_samples, heights, starts,
                        out_ptr: int, stream: int = 0) -> None:
    """Device buffers (points [sum n, dim] float32, out [sum k] uint64); host per-cloud arrays."""
    off = np.ascontiguousarray(offsets, np.uint64)
    ks = np.ascontiguousarray(n_samples, np.uint64)
    hs = np.ascontiguousarray(heights, np.uint64)
    ss = np.ascontiguousarray(starts, np.uint64)
    rc = lib().fpsgpu_kdline_batch_device(points_ptr, off.ctypes.data_as(_szp), len(ks), dim,
                                          ks.ctypes.data_as(_szp), ss.ctypes.data_as(_szp),
                                          hs.ctypes.data_as(_szp), out_ptr, stream or None)
    _check("fpsgpu_kdline_batch_device", rc)


def fps_device_noalloc(points_ptr: int, n: int, dim: int, n_samples: int, starts, out_ptr: int,
                       trace_ptr: int = 0, stream: int = 0) -> None:
    """fpsgpu_fps_device_noalloc: vanilla FPS whose scratch is a fixed array in
    the library (no GPU allocation; at most 65536 points, 512 starts)."""
    st = np.atleast_1d(np.asarray(starts, dtype=np.uint64))
    rc = lib().fpsgpu_fps_device_noalloc(points_ptr, n, dim, n_samples, st.ctypes.data_as(_szp),
                                         st.size, out_ptr, trace_ptr or None, stream or None)
    _check("fpsgpu_fps_device_noalloc", rc)


class Server:
    """QuickFPS request server with continuous batching (fpsgpu_server_*).

    submit() returns a ticket immediately; result(ticket) blocks and returns
    (indices, queue_ms, total_ms).  Indices equal bucket_fps_kdline_sampling's.
    """

    def __init__(self, max_device_bytes: int = 150 << 30, small_workers: int = 8,
                 large_workers: int = 2):
        h = _vp()
        _check("fpsgpu_server_create",
               lib().fpsgpu_server_create(max_device_bytes, small_workers, large_workers,
                                          ctypes.byref(h)))
        self._h = h
        self._live = {}

    def submit(self, pc, n_samples: int, height: int, start_idx: int = 0) -> int:
        a = _rows(pc)
        out = np.empty(n_samples, np.uint64)
        t = ctypes.c_uint64(0)
        _check("fpsgpu_server_submit",
               lib().fpsgpu_server_submit(self._h, a.ctypes.data_as(_f32p), a.shape[0], a.shape[1],
                                          n_samples, start_idx, height, out.ctypes.data_as(_szp),
                                          ctypes.byref(t)))
        self._live[t.value] = (a, out)  # keep the buffers alive until the result is taken
        return t.value

    def result(self, ticket: int):
        q = ctypes.c_double(0)
        tot = ctypes.c_double(0)
        rc = lib().fpsgpu_server_wait(self._h, ticket, ctypes.byref(q), ctypes.byref(tot))
        _, out = self._live.pop(ticket)
        _check("fpsgpu_server_wait", rc)
        return out, q.value, tot.value

    def close(self) -> None:
        if self._h:
            lib().fpsgpu_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


ALGO_FPS, ALGO_KDLINE, ALGO_KDTREE = 0, 1, 2


def sample_points(algo: int, pc, n_samples: int, starts, height: int = 0):
    """fpsgpu_sample_points, host buffers: (uint64 indices, float32 [K, D] points)."""
    a = _rows(pc)
    st = np.atleast_1d(np.asarray(starts, dtype=np.uint64))
    out = np.zeros(n_samples, np.uint64)
    xyz = np.zeros((n_samples, a.shape[1]), np.float32)
    _check("fpsgpu_sample_points",
           lib().fpsgpu_sample_points(algo, a.ctypes.data_as(_f32p), a.shape[0], a.shape[1],
                                      n_samples, st.ctypes.data_as(_szp), st.size, height,
                                      out.ctypes.data_as(_szp), xyz.ctypes.data_as(_f32p)))
    return out, xyz


def kdline_batch_points_device(points_ptr: int, offsets, dim: int, n_samples, heights, starts,
                               out_ptr: int, out_points_ptr: int, stream=0) -> None:
    off = np.asarray(offsets, dtype=np.uint64)
    ks = np.asarray(n_samples, dtype=np.uint64)
    hs = np.asarray(heights, dtype=np.uint64)
    ss = np.asarray(starts, dtype=np.uint64)
    _check("fpsgpu_kdline_batch_points_device",
           lib().fpsgpu_kdline_batch_points_device(
               points_ptr, off.ctypes.data_as(_szp), len(ks), dim, ks.ctypes.data_as(_szp),
               ss.ctypes.data_as(_szp), hs.ctypes.data_as(_szp), out_ptr, out_points_ptr, stream))
