"""In-tree build of the native parts of fpsample_gb300.

Outputs (git-ignored):
  fpsample_gb300/libfpsgpu.so   CUDA kernels + the C ABI of include/fpsgpu.h,
                                sm_103a only
  fpsample/_fpsample<ext>       pybind11 extension (C++) calling the C ABI,
                                importable as fpsample._fpsample like the
                                reference's

Each .cu translation unit is compiled by its own nvcc process in parallel;
nothing is rebuilt when its output is newer than every source it depends on.
"""
from __future__ import annotations

import concurrent.futures as cf
import importlib.util
import os
import shutil
import subprocess
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(HERE, "_objs")
LIB = os.path.join(HERE, "libfpsgpu.so")
EXT = os.path.join(ROOT, "fpsample", "_fpsample" + sysconfig.get_config_var("EXT_SUFFIX"))

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CU_UNITS = ["api", "vanilla_nofma", "vanilla_fma", "engine_nofma", "engine_fma", "noalloc", "server"]


def _nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(cuda, "bin", "nvcc")
    return p if os.path.exists(p) else (shutil.which("nvcc") or "nvcc")


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs + [os.path.join(INCLUDE, "fpsgpu.h")]


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _pybind11_include() -> str:
    spec = importlib.util.find_spec("torch")
    if spec and spec.submodule_search_locations:
        inc = os.path.join(spec.submodule_search_locations[0], "include")
        if os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
            return inc
    spec = importlib.util.find_spec("pybind11")
    if spec and spec.submodule_search_locations:
        inc = os.path.join(spec.submodule_search_locations[0], "include")
        if os.path.exists(inc):
            return inc
    raise RuntimeError("pybind11 headers not found (expected under torch/include)")


def build(verbose: bool = False) -> None:
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    flags = [ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
             "-I" + INCLUDE, "--expt-relaxed-constexpr"]

    def compile_unit(u: str) -> str:
        src = os.path.join(CSRC, u + ".cu")
        obj = os.path.join(OBJ, u + ".o")
        if _stale(obj, [src] + headers):
            if verbose:
                print("nvcc", u)
            _run([nvcc, *flags, "-c", src, "-o", obj])
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(CU_UNITS)) as ex:
        objs = list(ex.map(compile_unit, CU_UNITS))
    if _stale(LIB, objs):
        _run([nvcc, ARCH, "-shared", "-cudart=static", "-o", LIB, *objs])

    src = os.path.join(CSRC, "pymodule.cpp")
    if _stale(EXT, [src, LIB, os.path.join(INCLUDE, "fpsgpu.h")]):
        cxx = os.environ.get("CXX", "g++")
        pyinc = sysconfig.get_paths()["include"]
        _run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden",
              "-I" + pyinc, "-I" + _pybind11_include(), "-I" + INCLUDE, src,
              "-o", EXT, "-L" + HERE, "-lfpsgpu", "-Wl,-rpath,$ORIGIN/../fpsample_gb300"])


if __name__ == "__main__":
    build(verbose=True)
