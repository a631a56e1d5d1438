"""Python handle on the oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arm, always as the reference answer that
GPU results are compared with, or as the timed CPU baseline.  The product
package (fpsample_gb300) never imports it.

Two things live here:

* ``Oracle``: ctypes bindings to ``liboracle.so``, the C restatement of the
  reference's algorithm in ``fps_oracle.c`` (which cites the reference's
  file:line for every step).
* ``load_reference(mode)``: the unmodified reference package, assembled from
  its own ``src/fpsample/__init__.py`` and the extension that ``make -C oracle
  ref`` compiled from its own ``src/lib.cpp``.  Both come from the copy of the
  reference's sources that ``make -C oracle stage`` places in the git-ignored
  ``baseline/_ref/``; where that copy is absent, so is the reference.  Used to
  generate and check golden vectors and, on the host that runs the GPU, as the
  timed reference CPU path.
"""
from __future__ import annotations

import ctypes
import importlib.util
import os
import platform
import subprocess
import sys
import sysconfig

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
ROOT = os.path.dirname(HERE)
REF_SRC = os.path.join(ROOT, "baseline", "_ref", "src", "fpsample")
# builds of the reference for this host's CPU architecture (oracle/Makefile ref)
REF_OUT = os.path.join(HERE, "_ref", platform.machine())
REF_FLAGS = os.path.join(REF_OUT, "flags.txt")

FP_MODES = {"nofma": 0, "fma": 1}

_u64p = ctypes.POINTER(ctypes.c_uint64)
_f32p = ctypes.POINTER(ctypes.c_float)
_sz = ctypes.c_size_t


def build(quiet: bool = True) -> str:
    """Compile liboracle.so with the committed Makefile."""
    out = subprocess.run(["make", "-C", HERE, "all"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)
    return LIB_PATH


def _ptr(a, t):
    return a.ctypes.data_as(t)


class Oracle:
    """ctypes view of liboracle.so."""

    def __init__(self, path: str = LIB_PATH):
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        lib.oracle_fps.argtypes = [_f32p, _sz, _sz, _sz, _u64p, _sz, ctypes.c_int, _u64p, _f32p]
        lib.oracle_fps_mt.argtypes = [_f32p, _sz, _sz, _sz, _u64p, _sz, ctypes.c_int, _sz, _u64p,
                                      _f32p]
        lib.oracle_kdline.argtypes = [_f32p, _sz, _sz, _sz, _sz, _sz, ctypes.c_int, _u64p, _f32p, _u64p]
        lib.oracle_kdline_direct.argtypes = [_f32p, _sz, _sz, _sz, _sz, _sz, ctypes.c_int, _u64p]
        lib.oracle_kdtree.argtypes = [_f32p, _sz, _sz, _sz, _sz, ctypes.c_int, _u64p]
        lib.oracle_kdline_build.argtypes = [_f32p, _sz, _sz, _sz, _u64p, _u64p, ctypes.POINTER(_sz)]
        for f in ("oracle_fps", "oracle_fps_mt", "oracle_kdline", "oracle_kdline_direct", "oracle_kdline_build",
                  "oracle_kdtree"):
            getattr(lib, f).restype = ctypes.c_int
        self.lib = lib

    @staticmethod
    def _pts(pc):
        pc = np.ascontiguousarray(pc, dtype=np.float32)
        assert pc.ndim == 2
        return pc

    def fps(self, pc, k, starts, fp_mode="nofma", trace=False):
        """Vanilla FPS (reference src/lib.cpp:111-246).  starts: int or list."""
        pc = self._pts(pc)
        st = np.atleast_1d(np.asarray(starts, dtype=np.uint64))
        out = np.zeros(k, np.uint64)
        tr = np.zeros(k, np.float32) if trace else None
        rc = self.lib.oracle_fps(_ptr(pc, _f32p), pc.shape[0], pc.shape[1], k, _ptr(st, _u64p),
                                 st.size, FP_MODES[fp_mode], _ptr(out, _u64p),
                                 _ptr(tr, _f32p) if trace else None)
        if rc:
            raise RuntimeError(f"oracle_fps failed with code {rc}")
        return (out, tr) if trace else out

    def fps_mt(self, pc, k, starts, fp_mode="nofma", threads=None, trace=False):
        """Vanilla FPS on several host threads: the same answer as fps() (the
        per-point updates are independent and the argmax folds exactly)."""
        pc = self._pts(pc)
        st = np.atleast_1d(np.asarray(starts, dtype=np.uint64))
        out = np.zeros(k, np.uint64)
        tr = np.zeros(k, np.float32) if trace else None
        nt = threads or os.cpu_count() or 1
        rc = self.lib.oracle_fps_mt(_ptr(pc, _f32p), pc.shape[0], pc.shape[1], k, _ptr(st, _u64p),
                                    st.size, FP_MODES[fp_mode], nt, _ptr(out, _u64p),
                                    _ptr(tr, _f32p) if trace else None)
        if rc:
            raise RuntimeError(f"oracle_fps_mt failed with code {rc}")
        return (out, tr) if trace else out

    def kdline(self, pc, k, h, start, fp_mode="nofma", trace=False, perm=False):
        """bucket_fps_kdline (reference src/wrapper.hpp:118-132 and src/_ext)."""
        pc = self._pts(pc)
        out = np.zeros(k, np.uint64)
        tr = np.zeros(k, np.float32) if trace else None
        pm = np.zeros(pc.shape[0], np.uint64) if perm else None
        rc = self.lib.oracle_kdline(_ptr(pc, _f32p), pc.shape[0], pc.shape[1], k, start, h,
                                    FP_MODES[fp_mode], _ptr(out, _u64p),
                                    _ptr(tr, _f32p) if trace else None,
                                    _ptr(pm, _u64p) if perm else None)
        if rc:
            raise RuntimeError(f"oracle_kdline failed with code {rc}")
        res = [out]
        if trace:
            res.append(tr)
        if perm:
            res.append(pm)
        return res[0] if len(res) == 1 else tuple(res)

    def kdline_direct(self, pc, k, h, start, fp_mode="nofma"):
        pc = self._pts(pc)
        out = np.zeros(k, np.uint64)
        rc = self.lib.oracle_kdline_direct(_ptr(pc, _f32p), pc.shape[0], pc.shape[1], k, start, h,
                                           FP_MODES[fp_mode], _ptr(out, _u64p))
        if rc:
            raise RuntimeError(f"oracle_kdline_direct failed with code {rc}")
        return out

    def kdtree(self, pc, k, start, fp_mode="nofma"):
        """bucket_fps_kdtree: unbounded-height build, ties to the last position."""
        pc = self._pts(pc)
        out = np.zeros(k, np.uint64)
        rc = self.lib.oracle_kdtree(_ptr(pc, _f32p), pc.shape[0], pc.shape[1], k, start,
                                    FP_MODES[fp_mode], _ptr(out, _u64p))
        if rc:
            raise RuntimeError(f"oracle_kdtree failed with code {rc}")
        return out

    def kdline_build(self, pc, h):
        """(perm, bucket_starts) of the kd-line tree (KDTreeBase.h:84-207)."""
        pc = self._pts(pc)
        n = pc.shape[0]
        perm = np.zeros(n, np.uint64)
        bst = np.zeros(n, np.uint64)
        nb = _sz(0)
        rc = self.lib.oracle_kdline_build(_ptr(pc, _f32p), n, pc.shape[1], h, _ptr(perm, _u64p),
                                          _ptr(bst, _u64p), ctypes.byref(nb))
        if rc:
            raise RuntimeError(f"oracle_kdline_build failed with code {rc}")
        return perm, bst[: nb.value].copy()


def fp64_trace(pc, idx):
    """For each output i >= 1, the float64 squared distance from point idx[i]
    to its nearest earlier sample idx[0..i-1] (the max-min trace of FPS)."""
    p = np.asarray(pc, dtype=np.float64)[np.asarray(idx, dtype=np.int64)]
    k = p.shape[0]
    out = np.full(k, np.inf)
    best = np.full(k, np.inf)
    for i in range(1, k):
        d = ((p[i:] - p[i - 1]) ** 2).sum(axis=1)
        best[i:] = np.minimum(best[i:], d)
        out[i] = best[i]
    return out


def stock_mode():
    """The FP mode of this host's stock build of the reference (default flags:
    "fma" where GCC contracts by default, i.e. aarch64; "nofma" on x86-64), or
    None when the reference was not compiled here."""
    try:
        for line in open(REF_FLAGS):
            if line.startswith("stock="):
                return line.strip().split("=", 1)[1]
    except OSError:
        pass
    return None


def reference_build_flags(mode: str) -> str | None:
    """The compiler flags `make ref` used for that build on this host."""
    try:
        for line in open(REF_FLAGS):
            if line.startswith(mode + "="):
                return line.strip().split("=", 1)[1]
    except OSError:
        pass
    return None


def reference_available(mode: str = "nofma") -> bool:
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    return os.path.isdir(REF_SRC) and os.path.exists(os.path.join(REF_OUT, mode, "_fpsample" + ext))


def load_reference(mode: str = "nofma"):
    """The reference's own Python package, unmodified, with the extension that
    oracle/Makefile compiled from its own sources (mode "nofma" or "fma")."""
    if not reference_available(mode):
        raise RuntimeError(f"reference build '{mode}' not available (run make -C oracle ref)")
    name = f"_fpsample_reference_{mode}"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(
        name, os.path.join(REF_SRC, "__init__.py"),
        submodule_search_locations=[os.path.join(REF_OUT, mode), REF_SRC])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod
