// fpsgpu_fps_device_noalloc: vanilla FPS for callers that cannot allocate GPU
// memory.
//
// Who needs it: code that runs where cudaMalloc / cudaMallocAsync are not
// allowed or not wanted -- inside a memory pool owned by someone else (a
// framework's caching allocator, a fixed arena sized at start-up), in a
// real-time loop with a hard no-allocation rule, or in a process whose device
// memory is fully reserved by another component.  This entry point runs the
// same kernel as fpsgpu_fps_device for small clouds, but its scratch (the
// start list, the cross-CTA exchange slots and the error word) lives in one
// file-scope __device__ array below, so a call allocates nothing: the caller
// passes the points and the output buffer, and the library only copies into and
// clears that fixed array.
//
// Limits: at most kNoAllocMaxPoints points, kNoAllocMaxStarts start indices,
// dim in [1, 8].  The array is 4.4 KB and every GPU that loads the library
// holds it until the process exits.
//
// Concurrency: every call, from any thread or stream, uses the same array and
// it keeps the last call's contents.  Calls whose GPU work overlaps -- two
// streams, or two host threads -- race on it and may return wrong indices.
// Serialise them (one stream, or host-side locking).
//
// Set-up: the first call on each device looks up the array's device address
// with cudaGetSymbolAddress while that device is current.  Make that first call
// before any stream capture on the device.
#include <mutex>
#include <vector>

#include "vanilla.cuh"

namespace fpsgpu {
namespace {

constexpr uint64_t kNoAllocMaxPoints = 65536;  // 16 CTAs x 1024 threads x 4 points
constexpr uint32_t kNoAllocMaxStarts = 512;
constexpr int kNoAllocMaxCtas = 16;
// word layout: [0, 512) start indices | [512, 560) exchange slots | [560] error word
constexpr size_t kWordsStarts = kNoAllocMaxStarts;
constexpr size_t kWordsSlots = 3 * kNoAllocMaxCtas;
constexpr size_t kScratchWords = kWordsStarts + kWordsSlots + 1;

static __device__ __align__(256) uint64_t g_noalloc_scratch[kScratchWords];

std::mutex g_mu;
std::vector<uint64_t*> g_ptr;  // device address of g_noalloc_scratch, per device

// Looks up (once per device) the device address of the scratch array; the host
// symbol itself is only a stand-in and must never be passed to a kernel.
int scratch_address(uint64_t** out) {
    int dev = 0;
    FPSGPU_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_mu);
    if ((int)g_ptr.size() <= dev) g_ptr.resize(dev + 1, nullptr);
    if (g_ptr[dev] == nullptr) {
        void* p = nullptr;
        FPSGPU_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_ptr[dev] = static_cast<uint64_t*>(p);
    }
    *out = g_ptr[dev];
    return FPSGPU_OK;
}

template <int D, bool FMA>
int run_noalloc(const float* d_points, uint64_t n, uint64_t k, uint32_t n_start, uint64_t* d_out,
                float* d_trace, cudaStream_t stream, uint64_t* scratch) {
    constexpr int ppt_max = D <= 4 ? 8 : 4;
    int ppt;
    if (n <= (uint64_t)kVanillaThreads) ppt = 1;
    else if (n <= 2ull * kVanillaThreads) ppt = 2;
    else if (n <= 4ull * kVanillaThreads) ppt = 4;
    else ppt = ppt_max;
    const int G = (int)((n + (uint64_t)kVanillaThreads * ppt - 1) / ((uint64_t)kVanillaThreads * ppt));
    if (G > kNoAllocMaxCtas)
        return set_error(FPSGPU_ERR_ARG, "no-allocation FPS: %llu points need %d CTAs (max %d)",
                         (unsigned long long)n, G, kNoAllocMaxCtas);
    uint64_t* slots = scratch + kWordsStarts;
    int* err = reinterpret_cast<int*>(scratch + kWordsStarts + kWordsSlots);
    // the slots and the error word must start at zero on every call
    FPSGPU_CUDA_TRY(cudaMemsetAsync(slots, 0, (kWordsSlots + 1) * sizeof(uint64_t), stream));
    VanillaArgs a{};
    a.pts = d_points;
    a.n = n;
    a.dim = D;
    a.k = k;
    a.starts = scratch;
    a.n_starts = n_start;
    a.out = d_out;
    a.trace = d_trace;
    a.slots = slots;
    a.err = err;
    a.smem_cloud = (G == 1 && n * D * sizeof(float) <= 96 * 1024) ? 1 : 0;
    VanillaCall c{};
    c.n = n;
    c.stream = stream;
    int rc;
    switch (ppt) {
        case 1: rc = launch_resident<D, FMA, 1>(c, a, G); break;
        case 2: rc = launch_resident<D, FMA, 2>(c, a, G); break;
        case 4: rc = launch_resident<D, FMA, 4>(c, a, G); break;
        default: rc = launch_resident<D, FMA, ppt_max>(c, a, G); break;
    }
    if (rc) return rc;
    int h_err = 0;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    FPSGPU_CUDA_TRY(cudaStreamSynchronize(stream));
    if (h_err)
        return set_error(FPSGPU_ERR_DEVICE, "FPS kernel gave up (device error word 0x%x)", h_err);
    return FPSGPU_OK;
}

template <bool FMA>
int dispatch_noalloc(int dim, const float* p, uint64_t n, uint64_t k, uint32_t ns, uint64_t* o,
                     float* t, cudaStream_t s, uint64_t* sc) {
    switch (dim) {
        case 1: return run_noalloc<1, FMA>(p, n, k, ns, o, t, s, sc);
        case 2: return run_noalloc<2, FMA>(p, n, k, ns, o, t, s, sc);
        case 3: return run_noalloc<3, FMA>(p, n, k, ns, o, t, s, sc);
        case 4: return run_noalloc<4, FMA>(p, n, k, ns, o, t, s, sc);
        case 5: return run_noalloc<5, FMA>(p, n, k, ns, o, t, s, sc);
        case 6: return run_noalloc<6, FMA>(p, n, k, ns, o, t, s, sc);
        case 7: return run_noalloc<7, FMA>(p, n, k, ns, o, t, s, sc);
        case 8: return run_noalloc<8, FMA>(p, n, k, ns, o, t, s, sc);
        default: return set_error(FPSGPU_ERR_DIM, "dim must be in [1, 8], got %d", dim);
    }
}

}  // namespace
}  // namespace fpsgpu

using namespace fpsgpu;

extern "C" int fpsgpu_fps_device_noalloc(const float* d_points, size_t n_points, size_t dim,
                                         size_t n_samples, const size_t* h_start, size_t n_start,
                                         uint64_t* d_out, float* d_trace, void* stream) {
    clear_error();
    if (dim == 0 || dim > 8) return set_error(FPSGPU_ERR_DIM, "dim must be in [1, 8], got %zu", dim);
    if (n_points == 0) return set_error(FPSGPU_ERR_ARG, "n_points must be >= 1");
    if (n_points > kNoAllocMaxPoints)
        return set_error(FPSGPU_ERR_ARG,
                         "no-allocation FPS handles at most %llu points, got %zu",
                         (unsigned long long)kNoAllocMaxPoints, n_points);
    if (n_start == 0 || h_start == nullptr)
        return set_error(FPSGPU_ERR_ARG, "need at least one start index");
    if (n_start > kNoAllocMaxStarts)
        return set_error(FPSGPU_ERR_ARG, "no-allocation FPS handles at most %u start indices, got %zu",
                         kNoAllocMaxStarts, n_start);
    if (n_samples > 0 && n_start > n_samples)
        return set_error(FPSGPU_ERR_ARG, "more start indices (%zu) than samples (%zu)", n_start,
                         n_samples);
    for (size_t i = 0; i < n_start; ++i)
        if (h_start[i] >= n_points)
            return set_error(FPSGPU_ERR_START, "start index %zu out of range (n_points=%zu)",
                             h_start[i], n_points);
    if (n_samples == 0) return FPSGPU_OK;
    uint64_t* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);  // NULL: the legacy default stream
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(scratch, h_start, n_start * sizeof(uint64_t),
                                    cudaMemcpyHostToDevice, s));
    return fpsgpu_get_fp_mode() == FPSGPU_FP_FMA
               ? dispatch_noalloc<true>((int)dim, d_points, n_points, n_samples, (uint32_t)n_start,
                                        d_out, d_trace, s, scratch)
               : dispatch_noalloc<false>((int)dim, d_points, n_points, n_samples,
                                         (uint32_t)n_start, d_out, d_trace, s, scratch);
}
