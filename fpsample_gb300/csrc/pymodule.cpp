// fpsample._fpsample: the Python extension module of the GPU build.
//
// It mirrors the reference's pybind11 module `fpsample._fpsample`
// (src/lib.cpp:581-660): same function names, argument order, argument
// conversion (float32, C order, forcecast), validation messages and exception
// types, uint64 outputs.  Every sampling call goes through the C ABI of
// libfpsgpu (include/fpsgpu.h) on the GPU with the GIL released; there is no
// CPU path.  The heuristic variants that are not part of the GPU build raise
// NotImplementedError.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>

#include <cstdint>
#include <optional>
#include <string>
#include <vector>

#include "../../include/fpsgpu.h"

namespace py = pybind11;

using FloatRows = py::array_t<float, py::array::c_style | py::array::forcecast>;
using Indices = py::array_t<size_t>;

namespace {

// Either one start index or an array of them (reference src/lib.cpp:16-24).
struct Start {
    bool single = true;
    size_t idx = 0;
    Indices arr;
};

Start parse_start(const py::object& obj) {
    Start s;
    if (py::isinstance<py::int_>(obj)) {
        s.idx = obj.cast<size_t>();
    } else if (py::isinstance<Indices>(obj)) {
        s.single = false;
        s.arr = obj.cast<Indices>();
    } else {
        throw py::type_error("start_idx must be int or 1D numpy array of size_t");
    }
    return s;
}

// Argument checks of the reference's vanilla path (src/lib.cpp:52-109).
void check_inputs(const FloatRows& points, size_t n_samples, const Start& start) {
    if (points.ndim() != 2)
        throw py::value_error("points must be a 2D array, but got shape " +
                              std::to_string(points.ndim()));
    const ssize_t P = points.shape(0), C = points.shape(1);
    if (C == 0) throw py::value_error("points must have at least one column");
    if (n_samples > static_cast<size_t>(P))
        throw py::value_error("n_samples must be less than the number of points: n_samples=" +
                              std::to_string(n_samples) + ", P=" + std::to_string(P));
    if (start.single) {
        if (start.idx >= static_cast<size_t>(P))
            throw py::value_error("start_idx must be less than the number of points: start_idx=" +
                                  std::to_string(start.idx) + ", P=" + std::to_string(P));
    } else {
        auto a = start.arr.unchecked<1>();
        if (static_cast<size_t>(a.shape(0)) > n_samples)
            throw py::value_error(
                "The number of start indices must be less than or equal to n_samples: " +
                std::to_string(a.shape(0)) + ", n_samples=" + std::to_string(n_samples));
        for (ssize_t i = 0; i < a.shape(0); ++i)
            if (a(i) >= static_cast<size_t>(P))
                throw py::value_error(
                    "All indices in start_idx must be less than the number of points: " +
                    std::to_string(a(i)) + ", P=" + std::to_string(P));
    }
}

[[noreturn]] void raise_gpu_failure(const char* what, int rc) {
    throw std::runtime_error(std::string(what) + " failed with error code " + std::to_string(rc) +
                             ": " + fpsgpu_last_error());
}

// _fps_sampling (reference src/lib.cpp:249-270 -> :188-246 / :111-186)
Indices fps_sampling(FloatRows points, size_t n_samples, py::object start_obj) {
    Start start = parse_start(start_obj);
    check_inputs(points, n_samples, start);
    const ssize_t P = points.shape(0), C = points.shape(1);
    std::vector<size_t> starts;
    if (start.single) {
        if (P <= 0 || C <= 0) throw py::value_error("points must be a 2D array with at least one column");
        starts.push_back(start.idx);
    } else {
        if (P <= 0 || C <= 0) throw std::runtime_error("points must be a 2D array");
        auto a = start.arr.unchecked<1>();
        for (ssize_t i = 0; i < a.shape(0); ++i) starts.push_back(a(i));
        if (starts.empty() && n_samples > 0)
            throw py::value_error("start_idx must hold at least one index");
    }
    Indices out(n_samples);
    if (n_samples == 0) return out;
    size_t* out_ptr = static_cast<size_t*>(out.mutable_data());
    const float* data = points.data();
    int rc;
    {
        py::gil_scoped_release nogil;
        rc = fpsgpu_fps(data, (size_t)P, (size_t)C, n_samples, starts.data(), starts.size(), out_ptr);
    }
    if (rc != 0) raise_gpu_failure("fps_sampling", rc);
    return out;
}

// _bucket_fps_kdline_sampling (reference src/lib.cpp:522-579)
Indices bucket_fps_kdline_sampling(FloatRows points, size_t n_samples, size_t height,
                                   py::object start_obj) {
    Start start = parse_start(start_obj);
    if (!start.single) {
        PyErr_SetString(PyExc_NotImplementedError, "Array of start indices not implemented yet");
        throw py::error_already_set();
    }
    if (points.ndim() != 2) throw py::value_error("points must be a 2D float32 array");
    const ssize_t P = points.shape(0), C = points.shape(1);
    if (start.idx >= static_cast<size_t>(P)) throw py::value_error("start_idx out of range");
    if (n_samples == 0 || n_samples > static_cast<size_t>(P))
        throw py::value_error("n_samples must be in [1, num_points]");
    if (height == 0) throw py::value_error("height must be >= 1");
    Indices out(n_samples);
    size_t* out_ptr = static_cast<size_t*>(out.mutable_data());
    const float* data = points.data();
    int rc;
    {
        py::gil_scoped_release nogil;
        rc = bucket_fps_kdline(data, (size_t)P, (size_t)C, n_samples, start.idx, height, out_ptr);
    }
    if (rc != 0)
        throw std::runtime_error("bucket_fps_kdline failed with error code " + std::to_string(rc));
    return out;
}

// _bucket_fps_kdtree_sampling (reference src/lib.cpp:467-520)
Indices bucket_fps_kdtree_sampling(FloatRows points, size_t n_samples, py::object start_obj) {
    Start start = parse_start(start_obj);
    if (!start.single) {
        PyErr_SetString(PyExc_NotImplementedError, "Array of start indices not implemented yet");
        throw py::error_already_set();
    }
    if (points.ndim() != 2) throw py::value_error("points must be a 2D float32 array");
    const ssize_t P = points.shape(0), C = points.shape(1);
    if (start.idx >= static_cast<size_t>(P)) throw py::value_error("start_idx out of range");
    if (n_samples == 0 || n_samples > static_cast<size_t>(P))
        throw py::value_error("n_samples must be in [1, num_points]");
    Indices out(n_samples);
    size_t* out_ptr = static_cast<size_t*>(out.mutable_data());
    const float* data = points.data();
    int rc;
    {
        py::gil_scoped_release nogil;
        rc = bucket_fps_kdtree(data, (size_t)P, (size_t)C, n_samples, start.idx, out_ptr);
    }
    if (rc != 0)
        throw std::runtime_error("bucket_fps_kdtree failed with error code " + std::to_string(rc));
    return out;
}

// Indices and the sampled points in one call (the gather fused into the
// sampler): algo is FPSGPU_ALGO_FPS / _KDLINE / _KDTREE; starts holds one or
// more start indices (one for the kd variants).  Returns (uint64 [K],
// float32 [K, C]).  Argument checks are the ones of the matching function.
py::tuple sample_points(int algo, FloatRows points, size_t n_samples, Indices starts,
                        size_t height) {
    if (points.ndim() != 2) throw py::value_error("points must be a 2D float32 array");
    const ssize_t P = points.shape(0), C = points.shape(1);
    const ssize_t m = starts.size();
    if (m == 0) throw py::value_error("need at least one start index");
    for (ssize_t i = 0; i < m; ++i)
        if (starts.data()[i] >= static_cast<size_t>(P)) throw py::value_error("start_idx out of range");
    if (n_samples == 0 || n_samples > static_cast<size_t>(P))
        throw py::value_error("n_samples must be in [1, num_points]");
    if (algo != FPSGPU_ALGO_FPS && m != 1) {
        PyErr_SetString(PyExc_NotImplementedError, "Array of start indices not implemented yet");
        throw py::error_already_set();
    }
    if (algo == FPSGPU_ALGO_KDLINE && height == 0) throw py::value_error("height must be >= 1");
    Indices out(n_samples);
    py::array_t<float> xyz({static_cast<ssize_t>(n_samples), C});
    size_t* out_ptr = static_cast<size_t*>(out.mutable_data());
    float* xyz_ptr = xyz.mutable_data();
    const float* data = points.data();
    const size_t* st = starts.data();
    int rc;
    {
        py::gil_scoped_release nogil;
        rc = fpsgpu_sample_points(algo, data, (size_t)P, (size_t)C, n_samples, st, (size_t)m, height,
                                  out_ptr, xyz_ptr);
    }
    if (rc != 0) raise_gpu_failure("fpsgpu_sample_points", rc);
    return py::make_tuple(out, xyz);
}

// Batched QuickFPS: clouds stored back to back in `points` (rows
// [offsets[c], offsets[c+1]) form cloud c).  Returns one uint64 array with the
// clouds' local indices back to back (cloud c at sum(n_samples[:c])).
Indices bucket_fps_kdline_sampling_batch(FloatRows points, Indices offsets, Indices n_samples,
                                         Indices heights, Indices starts) {
    if (points.ndim() != 2) throw py::value_error("points must be a 2D float32 array");
    const ssize_t C = n_samples.size();
    if (offsets.size() != C + 1 || heights.size() != C || starts.size() != C)
        throw py::value_error("offsets must have n_clouds + 1 entries; n_samples, heights and "
                              "starts n_clouds");
    const size_t* off = offsets.data();
    if (C > 0 && (off[0] != 0 || off[C] != (size_t)points.shape(0)))
        throw py::value_error("offsets must start at 0 and end at the number of points");
    size_t total = 0;
    for (ssize_t c = 0; c < C; ++c) {
        const size_t nc = off[c + 1] - off[c];
        const size_t k = n_samples.data()[c];
        if (off[c + 1] < off[c] || nc == 0) throw py::value_error("empty cloud in the batch");
        if (starts.data()[c] >= nc) throw py::value_error("start_idx out of range");
        if (k == 0 || k > nc) throw py::value_error("n_samples must be in [1, num_points]");
        if (heights.data()[c] == 0) throw py::value_error("height must be >= 1");
        total += k;
    }
    Indices out(total);
    if (C == 0) return out;
    int rc;
    const float* data = points.data();
    size_t* out_ptr = static_cast<size_t*>(out.mutable_data());
    {
        py::gil_scoped_release nogil;
        rc = fpsgpu_kdline_batch(data, off, (size_t)C, (size_t)points.shape(1), n_samples.data(),
                                 starts.data(), heights.data(), out_ptr);
    }
    if (rc != 0) raise_gpu_failure("fpsgpu_kdline_batch", rc);
    return out;
}

// Batched QuickFPS over a list of clouds, each its own (n_i, D) float32 array:
// no concatenation on the host.  Same checks and result layout as
// bucket_fps_kdline_sampling_batch.
Indices bucket_fps_kdline_sampling_batch_list(py::list pcs, Indices n_samples, Indices heights,
                                              Indices starts) {
    const ssize_t C = (ssize_t)pcs.size();
    if (n_samples.size() != C || heights.size() != C || starts.size() != C)
        throw py::value_error("n_samples, heights and starts need one entry per cloud");
    std::vector<FloatRows> arrs;
    arrs.reserve(C);
    std::vector<const float*> ptrs(C);
    std::vector<size_t> npts(C);
    size_t total = 0, dim = 0;
    for (ssize_t c = 0; c < C; ++c) {
        arrs.push_back(FloatRows::ensure(pcs[c]));
        const FloatRows& a = arrs.back();
        if (!a || a.ndim() != 2) throw py::value_error("every cloud must be a 2D float32 array");
        if (c == 0) dim = (size_t)a.shape(1);
        if ((size_t)a.shape(1) != dim) throw py::value_error("all clouds must have the same dimension");
        const size_t nc = (size_t)a.shape(0);
        const size_t k = n_samples.data()[c];
        if (nc == 0) throw py::value_error("empty cloud in the batch");
        if (starts.data()[c] >= nc) throw py::value_error("start_idx out of range");
        if (k == 0 || k > nc) throw py::value_error("n_samples must be in [1, num_points]");
        if (heights.data()[c] == 0) throw py::value_error("height must be >= 1");
        ptrs[c] = a.data();
        npts[c] = nc;
        total += k;
    }
    Indices out(total);
    if (C == 0) return out;
    int rc;
    size_t* out_ptr = static_cast<size_t*>(out.mutable_data());
    {
        py::gil_scoped_release nogil;
        rc = fpsgpu_kdline_batch_list(ptrs.data(), npts.data(), (size_t)C, dim, n_samples.data(),
                                      starts.data(), heights.data(), out_ptr);
    }
    if (rc != 0) raise_gpu_failure("fpsgpu_kdline_batch_list", rc);
    return out;
}

[[noreturn]] void not_in_gpu_build(const char* name) {
    PyErr_SetString(PyExc_NotImplementedError,
                    (std::string(name) +
                     " is not part of the GB300 build; it provides fps_sampling, "
                     "bucket_fps_kdline_sampling and bucket_fps_kdtree_sampling")
                        .c_str());
    throw py::error_already_set();
}

// extras beyond the reference: build permutation and fp mode
py::tuple kdline_build(FloatRows points, size_t height) {
    if (points.ndim() != 2) throw py::value_error("points must be a 2D float32 array");
    const ssize_t P = points.shape(0), C = points.shape(1);
    if (P == 0) throw py::value_error("points must not be empty");
    py::array_t<uint64_t> perm(P);
    std::vector<uint64_t> starts((size_t)P);
    size_t nb = 0;
    int rc;
    const float* data = points.data();
    uint64_t* perm_ptr = static_cast<uint64_t*>(perm.mutable_data());
    {
        py::gil_scoped_release nogil;
        rc = fpsgpu_kdline_build(data, (size_t)P, (size_t)C, height, perm_ptr, starts.data(), &nb);
    }
    if (rc != 0) raise_gpu_failure("kdline_build", rc);
    py::array_t<uint64_t> bst(nb);
    std::copy(starts.begin(), starts.begin() + nb, static_cast<uint64_t*>(bst.mutable_data()));
    return py::make_tuple(perm, bst);
}

std::string get_fp_mode() { return fpsgpu_get_fp_mode() == FPSGPU_FP_FMA ? "fma" : "nofma"; }

void set_fp_mode(const std::string& m) {
    int mode;
    if (m == "fma") mode = FPSGPU_FP_FMA;
    else if (m == "nofma") mode = FPSGPU_FP_NOFMA;
    else throw py::value_error("fp mode must be 'fma' or 'nofma'");
    fpsgpu_set_fp_mode(mode);
}

}  // namespace

PYBIND11_MODULE(_fpsample, m) {
    m.doc() = R"pbdoc(
        Farthest point sampling (FPS) on NVIDIA GB300
        -----------------------

        .. currentmodule:: fpsample

        .. autosummary::
           :toctree: _generate

           _fps_sampling
           _fps_npdu_sampling
           _fps_npdu_kdtree_sampling
           _bucket_fps_kdtree_sampling
           _bucket_fps_kdline_sampling
    )pbdoc";

    m.def("_fps_sampling", &fps_sampling, R"pbdoc(
            Farthest Point Sampling (FPS) on the GPU
            Args:
                points (np.ndarray[float32, 2D]): N x C point array.
                n_samples (int): number of samples to pick.
                start_idx (int or np.ndarray[uint64, 1D]): initial index or indices to start FPS.
            Returns:
                np.ndarray[uint64]: sampled point indices.
    )pbdoc");

    m.def("_bucket_fps_kdline_sampling", &bucket_fps_kdline_sampling, R"pbdoc(
            Bucket FPS sampling with a kd-line bucket tree (QuickFPS) on the GPU
            Args:
                points (np.ndarray[float32, 2D]): N x C point array, C <= 8.
                n_samples (int): number of samples to pick.
                height (int): height of the kd-line tree.
                start_idx (int): first index (a position of the tree's permuted order).
            Returns:
                np.ndarray[uint64]: sampled point indices.
    )pbdoc");

    m.def("_fps_npdu_sampling", [](py::args, py::kwargs) { not_in_gpu_build("_fps_npdu_sampling"); });
    m.def("_fps_npdu_kdtree_sampling",
          [](py::args, py::kwargs) { not_in_gpu_build("_fps_npdu_kdtree_sampling"); });
    m.def("_bucket_fps_kdtree_sampling", &bucket_fps_kdtree_sampling, R"pbdoc(
            Bucket FPS sampling with a full kd-tree (QuickFPS) on the GPU
            Args:
                points (np.ndarray[float32, 2D]): N x C point array, C <= 8.
                n_samples (int): number of samples to pick.
                start_idx (int): first index (a position of the tree's permuted order).
            Returns:
                np.ndarray[uint64]: sampled point indices.
    )pbdoc");

    m.def("_sample_points", &sample_points,
          "(algo, points, n_samples, starts uint64[], height) -> (indices, sampled points)");
    m.attr("ALGO_FPS") = FPSGPU_ALGO_FPS;
    m.attr("ALGO_KDLINE") = FPSGPU_ALGO_KDLINE;
    m.attr("ALGO_KDTREE") = FPSGPU_ALGO_KDTREE;
    m.def("_bucket_fps_kdline_sampling_batch", &bucket_fps_kdline_sampling_batch,
          "many clouds in one GPU call: (points, offsets, n_samples, heights, starts) -> indices");
    m.def("_bucket_fps_kdline_sampling_batch_list", &bucket_fps_kdline_sampling_batch_list,
          "many clouds in one GPU call, one array per cloud: (clouds, n_samples, heights, starts) "
          "-> indices");
    m.def("_kdline_build", &kdline_build,
          "kd-line tree build alone: (perm uint64[N], bucket_starts uint64[B])");
    m.def("_get_fp_mode", &get_fp_mode, "current floating-point mode: 'nofma' or 'fma'");
    m.def("_set_fp_mode", &set_fp_mode, "select 'nofma' or 'fma' for later calls");
    m.def("_library_version", []() { return std::string(fpsgpu_version()); });

    m.attr("__version__") = fpsgpu_version();
}
