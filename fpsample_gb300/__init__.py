"""fpsample_gb300: the native side of the GB300 build of fpsample.

  csrc/          CUDA kernels, the C ABI of include/fpsgpu.h, the request
                 server and the pybind11 extension's source
  _build.py      in-tree build: libfpsgpu.so here, fpsample/_fpsample<ext>
  capi.py        ctypes view of the C ABI (device buffers, batches, server)

The drop-in Python API is the ``fpsample`` package (the reference's module
path); its functions are re-exported here as well.
"""
from fpsample import *  # noqa: F401,F403
from fpsample import __all__, __doc__ as _api_doc, __version__  # noqa: F401
