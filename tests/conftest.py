import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")
    # The native library, the extension and the oracle are built in-tree; build
    # whatever is missing so that a fresh checkout can run the suite directly.
    import importlib.util

    spec = importlib.util.spec_from_file_location(
        "fpsample_gb300_build", os.path.join(ROOT, "fpsample_gb300", "_build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"], check=True)
