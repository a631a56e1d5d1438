"""CPU: the drop-in Python API validates arguments exactly like the reference
(src/fpsample/__init__.py and src/lib.cpp) before any GPU work, and without a
GPU every sampling call fails loudly instead of falling back to the CPU."""
import numpy as np
import pytest

import fpsample as fps
from fpsample import _fpsample

PC = np.random.default_rng(0).random((64, 3))


@pytest.mark.parametrize(
    "call,exc",
    [
        (lambda: fps.fps_sampling(PC, 0, 0), AssertionError),
        (lambda: fps.fps_sampling(PC[0], 4, 0), AssertionError),
        (lambda: fps.fps_sampling(PC, 65, 0), AssertionError),
        (lambda: fps.fps_sampling(PC, 4, 64), AssertionError),
        (lambda: fps.fps_sampling(PC, 4, -1), AssertionError),
        (lambda: fps.fps_sampling(PC, 2, [0, 1, 2]), AssertionError),
        (lambda: fps.fps_sampling(PC, 4, [0, 64]), AssertionError),
        (lambda: fps.fps_sampling(PC, 4, np.int64(3)), ValueError),
        (lambda: fps.fps_sampling(PC, 4, (1, 2)), ValueError),
        (lambda: fps.bucket_fps_kdline_sampling(PC, 0, 3, 0), AssertionError),
        (lambda: fps.bucket_fps_kdline_sampling(PC, 4, 0, 0), AssertionError),
        (lambda: fps.bucket_fps_kdline_sampling(PC, 4, 7, 0), AssertionError),
        (lambda: fps.bucket_fps_kdline_sampling(PC, 4, 3, 64), AssertionError),
        (lambda: fps.bucket_fps_kdline_sampling(PC, 4, 3, [0, 1]), TypeError),
        (lambda: fps.bucket_fps_kdline_sampling(PC, 65, 3, 0), AssertionError),
    ],
)
def test_python_wrapper_errors(call, exc):
    with pytest.raises(exc):
        call()


def test_extension_errors_match_reference():
    pc = np.zeros((10, 3), np.float32)
    with pytest.raises(TypeError, match="start_idx must be int or 1D numpy array of size_t"):
        _fpsample._fps_sampling(pc, 3, 1.5)
    with pytest.raises(TypeError):
        _fpsample._fps_sampling(pc, 3, np.array([1], np.int64))
    with pytest.raises(ValueError, match="points must be a 2D array"):
        _fpsample._fps_sampling(np.zeros(10, np.float32), 3, 0)
    with pytest.raises(ValueError, match="at least one column"):
        _fpsample._fps_sampling(np.zeros((10, 0), np.float32), 3, 0)
    with pytest.raises(ValueError, match="n_samples must be less than the number of points"):
        _fpsample._fps_sampling(pc, 11, 0)
    with pytest.raises(ValueError, match="start_idx must be less than the number of points"):
        _fpsample._fps_sampling(pc, 3, 10)
    with pytest.raises(ValueError, match="The number of start indices"):
        _fpsample._fps_sampling(pc, 1, np.array([1, 2], np.uint64))
    with pytest.raises(ValueError, match="All indices in start_idx"):
        _fpsample._fps_sampling(pc, 3, np.array([1, 10], np.uint64))
    with pytest.raises(NotImplementedError, match="Array of start indices not implemented yet"):
        _fpsample._bucket_fps_kdline_sampling(pc, 3, 2, np.array([1], np.uint64))
    with pytest.raises(ValueError, match="points must be a 2D float32 array"):
        _fpsample._bucket_fps_kdline_sampling(np.zeros(10, np.float32), 3, 2, 0)
    with pytest.raises(ValueError, match="start_idx out of range"):
        _fpsample._bucket_fps_kdline_sampling(pc, 3, 2, 10)
    with pytest.raises(ValueError, match=r"n_samples must be in \[1, num_points\]"):
        _fpsample._bucket_fps_kdline_sampling(pc, 0, 2, 0)
    with pytest.raises(ValueError, match="height must be >= 1"):
        _fpsample._bucket_fps_kdline_sampling(pc, 3, 0, 0)
    # C-ABI error codes surface as RuntimeError with the reference's message
    with pytest.raises(RuntimeError, match="bucket_fps_kdline failed with error code 1"):
        _fpsample._bucket_fps_kdline_sampling(np.zeros((10, 9), np.float32), 3, 2, 0)


def test_out_of_scope_variants_raise():
    for f in (lambda: fps.fps_npdu_sampling(PC, 4), lambda: fps.fps_npdu_kdtree_sampling(PC, 4)):
        with pytest.raises(NotImplementedError):
            f()


def test_kdtree_argument_checks_match_reference():
    # reference src/fpsample/__init__.py:159-171 and src/lib.cpp:467-520
    with pytest.raises(AssertionError, match="n_samples should be >= 1"):
        fps.bucket_fps_kdtree_sampling(PC, 0)
    with pytest.raises(AssertionError, match="n_pts should be >= n_samples"):
        fps.bucket_fps_kdtree_sampling(PC, PC.shape[0] + 1)
    with pytest.raises(AssertionError, match="start_idx should be None"):
        fps.bucket_fps_kdtree_sampling(PC, 3, PC.shape[0])
    pc = np.zeros((5, 3), np.float32)
    with pytest.raises(NotImplementedError, match="Array of start indices"):
        _fpsample._bucket_fps_kdtree_sampling(pc, 3, np.array([0, 1], np.uint64))
    with pytest.raises(ValueError, match="start_idx out of range"):
        _fpsample._bucket_fps_kdtree_sampling(pc, 3, 10)
    with pytest.raises(ValueError, match=r"n_samples must be in \[1, num_points\]"):
        _fpsample._bucket_fps_kdtree_sampling(pc, 0, 0)
    with pytest.raises(TypeError):
        _fpsample._bucket_fps_kdtree_sampling(pc, 3, "0")


def test_exports_and_version():
    for name in ("fps_sampling", "bucket_fps_kdline_sampling", "fps_npdu_sampling",
                 "fps_npdu_kdtree_sampling", "bucket_fps_kdtree_sampling", "__version__"):
        assert hasattr(fps, name)
    assert fps.__version__.startswith("1.0.2")


def test_random_start_uses_numpy_global_state():
    np.random.seed(123)
    a = fps.get_start_idx(1000, None)
    np.random.seed(123)
    assert a == np.random.randint(low=0, high=1000)
    assert isinstance(fps.get_start_idx(10, [1, 2]), np.ndarray)
    assert fps.get_start_idx(10, [1, 2]).dtype == np.uint64


def test_import_raises_the_hardware_work_queues_unless_set():
    """Importing the package sets CUDA_DEVICE_MAX_CONNECTIONS=32 (the request
    server's worker streams must not share hardware queues) but keeps a value
    the caller chose."""
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = "import os, fpsample_gb300; print(os.environ['CUDA_DEVICE_MAX_CONNECTIONS'])"
    for preset, want in ((None, "32"), ("16", "16")):
        env = {k: v for k, v in os.environ.items() if k != "CUDA_DEVICE_MAX_CONNECTIONS"}
        if preset is not None:
            env["CUDA_DEVICE_MAX_CONNECTIONS"] = preset
        out = subprocess.run([sys.executable, "-c", code], cwd=root, env=env, capture_output=True,
                             text=True, check=True).stdout.strip()
        assert out == want


@pytest.mark.parametrize(
    "call",
    [
        lambda: fps.bucket_fps_kdline_sampling_batch([PC, PC[:, :2]], 4, 3),   # mixed dimensions
        lambda: fps.bucket_fps_kdline_sampling_batch([PC, PC], [4, 65], 3),    # K > n
        lambda: fps.bucket_fps_kdline_sampling_batch([PC, PC], 4, [3, 7]),     # 2**h > n
        lambda: fps.bucket_fps_kdline_sampling_batch([PC, PC], 4, 3, [0, 64]),  # start out of range
        lambda: fps.bucket_fps_kdline_sampling_batch([PC, PC], [4], 3),        # one K per cloud
        lambda: fps.bucket_fps_kdline_sampling_batch([PC, PC], 4, [0, 3]),     # h >= 1
    ],
)
def test_batch_wrapper_checks(call):
    with pytest.raises(AssertionError):
        call()


def test_batch_list_extension_checks_and_no_cpu_fallback():
    a = np.zeros((10, 3), np.float32)
    u = lambda *v: np.array(v, np.uint64)
    assert fps.bucket_fps_kdline_sampling_batch([], 4, 3) == []
    with pytest.raises(ValueError, match="one entry per cloud"):
        _fpsample._bucket_fps_kdline_sampling_batch_list([a, a], u(2), u(1, 1), u(0, 0))
    with pytest.raises(ValueError, match="empty cloud"):
        _fpsample._bucket_fps_kdline_sampling_batch_list([a, a[:0]], u(2, 1), u(1, 1), u(0, 0))
    with pytest.raises(ValueError, match="same dimension"):
        _fpsample._bucket_fps_kdline_sampling_batch_list([a, a[:, :2]], u(2, 2), u(1, 1), u(0, 0))
    with pytest.raises(ValueError, match="start_idx"):
        _fpsample._bucket_fps_kdline_sampling_batch_list([a], u(2), u(1), u(10))
    # a valid batch: sampled on the GPU, or a loud failure where there is none
    try:
        out = _fpsample._bucket_fps_kdline_sampling_batch_list([a], u(2), u(1), u(0))
    except RuntimeError as e:
        assert "fpsgpu_kdline_batch_list failed with error code 4" in str(e)
    else:
        assert out.shape == (2,)


def test_importable_under_the_reference_module_path():
    """`import fpsample` and `fpsample._fpsample` resolve to this build, with
    every public and extension name the reference defines
    (src/fpsample/__init__.py:209-217, src/lib.cpp:598-653)."""
    import os

    import fpsample

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    assert os.path.dirname(fpsample.__file__) == os.path.join(root, "fpsample")
    assert _fpsample.__name__ == "fpsample._fpsample"
    assert os.path.dirname(_fpsample.__file__) == os.path.join(root, "fpsample")
    for name in ("fps_sampling", "fps_npdu_sampling", "fps_npdu_kdtree_sampling",
                 "bucket_fps_kdtree_sampling", "bucket_fps_kdline_sampling", "__version__",
                 "__doc__"):
        assert hasattr(fpsample, name), name
    for name in ("_fps_sampling", "_fps_npdu_sampling", "_fps_npdu_kdtree_sampling",
                 "_bucket_fps_kdtree_sampling", "_bucket_fps_kdline_sampling", "__version__"):
        assert hasattr(_fpsample, name), name
    from fpsample import fps_sampling  # noqa: F401  (the form callers write)
