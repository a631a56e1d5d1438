"""CPU: the C-ABI library loads, exports every function include/fpsgpu.h
declares, and validates arguments (codes 1/2/3 as the reference's C ABI)
before touching the GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from fpsample_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_reference_entry_point():
    assert "bucket_fps_kdline" in declared_functions()


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(capi.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    unbound = [n for n in declared_functions() if n not in capi.SIGNATURES]
    assert not unbound, f"declared but without a ctypes signature in capi: {unbound}"


def test_version_and_fp_mode_roundtrip():
    assert capi.lib().fpsgpu_version().decode().startswith("1.0.2")
    before = capi.get_fp_mode()
    try:
        capi.set_fp_mode("fma")
        assert capi.get_fp_mode() == "fma"
        capi.set_fp_mode("nofma")
        assert capi.get_fp_mode() == "nofma"
        assert capi.lib().fpsgpu_set_fp_mode(7) == 3
    finally:
        capi.set_fp_mode(before)


def test_default_fp_mode_follows_the_host_architecture():
    # the reference's stock build contracts a*b+c on aarch64 (GCC's default
    # there) and cannot on x86-64; the library starts in the matching mode
    # unless FPSAMPLE_FP_MODE says otherwise
    import os
    import platform
    import subprocess
    import sys

    code = "from fpsample_gb300 import capi; print(capi.get_fp_mode())"
    env = {k: v for k, v in os.environ.items() if k != "FPSAMPLE_FP_MODE"}
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                         cwd=os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    want = "fma" if platform.machine() in ("aarch64", "arm64") else "nofma"
    assert out.stdout.strip() == want, out.stderr
    for forced in ("fma", "nofma"):
        out = subprocess.run([sys.executable, "-c", code], env=dict(env, FPSAMPLE_FP_MODE=forced),
                             capture_output=True, text=True,
                             cwd=os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
        assert out.stdout.strip() == forced, out.stderr


def _kdline_rc(n, dim, start, k=4, h=3):
    pts = np.zeros((max(n, 1), max(dim, 1)), np.float32)
    out = np.zeros(max(k, 1), np.uint64)
    return capi.lib().bucket_fps_kdline(pts.ctypes.data_as(capi._f32p), n, dim, k, start, h,
                                        out.ctypes.data_as(capi._szp))


def test_reference_error_codes_without_gpu():
    # wrapper.hpp:121-127: 1 for dim outside [1, 8], 2 for start_idx >= n_points
    assert _kdline_rc(10, 0, 0) == 1
    assert _kdline_rc(10, 9, 0) == 1
    assert _kdline_rc(10, 3, 10) == 2
    assert _kdline_rc(0, 3, 0) == 2
    # zero samples: nothing to do, succeeds without a device
    assert _kdline_rc(10, 3, 0, k=0) == 0


def test_vanilla_argument_checks_without_gpu():
    L = capi.lib()
    pts = np.zeros((10, 3), np.float32)
    out = np.zeros(4, np.uint64)
    st = np.array([11], np.uint64)
    rc = L.fpsgpu_fps(pts.ctypes.data_as(capi._f32p), 10, 3, 4, st.ctypes.data_as(capi._szp), 1,
                      out.ctypes.data_as(capi._szp))
    assert rc == 2
    st = np.array([1, 2, 3, 4, 5], np.uint64)
    rc = L.fpsgpu_fps(pts.ctypes.data_as(capi._f32p), 10, 3, 4, st.ctypes.data_as(capi._szp), 5,
                      out.ctypes.data_as(capi._szp))
    assert rc == 3
    rc = L.fpsgpu_fps(pts.ctypes.data_as(capi._f32p), 10, 0, 4, st.ctypes.data_as(capi._szp), 1,
                      out.ctypes.data_as(capi._szp))
    assert rc == 1
    assert "dim" in L.fpsgpu_last_error().decode()


def test_batch_list_argument_checks_without_gpu():
    """fpsgpu_kdline_batch_list rejects a bad dimension and a cloud with points
    but no buffer before it touches the GPU; an empty batch succeeds."""
    L = capi.lib()
    a = np.zeros((10, 3), np.float32)
    ptrs = (capi._f32p * 2)(a.ctypes.data_as(capi._f32p), capi._f32p())
    npts = np.array([10, 10], np.uint64)
    ks = np.array([2, 2], np.uint64)
    hs = np.array([1, 1], np.uint64)
    ss = np.array([0, 0], np.uint64)
    out = np.zeros(4, np.uint64)
    args = (npts.ctypes.data_as(capi._szp),)
    rest = (ks.ctypes.data_as(capi._szp), ss.ctypes.data_as(capi._szp),
            hs.ctypes.data_as(capi._szp), out.ctypes.data_as(capi._szp))
    assert L.fpsgpu_kdline_batch_list(ptrs, *args, 2, 9, *rest) == 1
    assert L.fpsgpu_kdline_batch_list(ptrs, *args, 2, 3, *rest) == 3
    assert "null buffer" in L.fpsgpu_last_error().decode()
    assert L.fpsgpu_kdline_batch_list(ptrs, *args, 0, 3, *rest) == 0
