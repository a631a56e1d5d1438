// Host-side internals shared by the translation units of libfpsgpu.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <vector>

#include "../../include/fpsgpu.h"

namespace fpsgpu {

// Records a message for fpsgpu_last_error() on this thread and returns code.
int set_error(int code, const char* fmt, ...);
void clear_error();

// On failure the error is also taken off the runtime's last-error slot, so a
// later, unrelated cudaGetLastError() does not report it again.
#define FPSGPU_CUDA_TRY(expr)                                                              \
    do {                                                                                   \
        cudaError_t e_ = (expr);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            (void)cudaGetLastError();                                                      \
            return ::fpsgpu::set_error(FPSGPU_ERR_CUDA, "%s failed: %s (%s:%d)", #expr,    \
                                       cudaGetErrorString(e_), __FILE__, __LINE__);        \
        }                                                                                  \
    } while (0)

// Properties of the current device plus the library's own stream on it.
struct DevCtx {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
};
int current_ctx(DevCtx* ctx);

// Stream-ordered scratch: every allocation is released with cudaFreeAsync on
// the same stream when the object goes out of scope.
// The memory pool that stream-ordered scratch of the calling thread comes from:
// the one set for the thread, else the library's pool of the current device
// (it keeps up to 8 GB mapped between calls), else, if that pool cannot be
// made, the device's default pool.  Server workers each use their own pool:
// a shared pool may make one stream wait for another stream's work in order
// to reuse memory freed there, which would chain independent batches together.
void set_thread_pool(cudaMemPool_t pool);
cudaMemPool_t thread_pool();

// Fault injection on the host (fpsgpu_debug_fail_allocations): the number of
// stream-ordered scratch allocations that may still succeed, or -1 (off).
bool scratch_alloc_refused();

class Scratch {
   public:
    explicit Scratch(cudaStream_t s) : s_(s) {}
    ~Scratch() {
        for (void* p : ptrs_) cudaFreeAsync(p, s_);
    }
    Scratch(const Scratch&) = delete;
    Scratch& operator=(const Scratch&) = delete;
    template <class T>
    int alloc(T** out, size_t count) {
        *out = nullptr;
        void* p = nullptr;
        size_t bytes = count ? count * sizeof(T) : sizeof(T);
        if (scratch_alloc_refused())
            return set_error(FPSGPU_ERR_CUDA, "cudaMallocAsync(%zu bytes) refused (injected fault)", bytes);
        cudaMemPool_t pool = thread_pool();
        cudaError_t e = pool ? cudaMallocFromPoolAsync(&p, bytes, pool, s_)
                             : cudaMallocAsync(&p, bytes, s_);
        if (e != cudaSuccess)
            return set_error(FPSGPU_ERR_CUDA, "cudaMallocAsync(%zu bytes) failed: %s", bytes,
                             cudaGetErrorString(e));
        ptrs_.push_back(p);
        *out = static_cast<T*>(p);
        return FPSGPU_OK;
    }

   private:
    cudaStream_t s_;
    std::vector<void*> ptrs_;
};

// A second stream that forks from and joins back into a caller's stream, for
// two launches that should run side by side.  If it is dropped without a join
// (an error path), it waits for its own work so that stream-ordered frees on
// the caller's stream cannot overtake it.
struct SideStream {
    cudaStream_t s = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    bool joined = false;
    SideStream() = default;
    SideStream(const SideStream&) = delete;
    SideStream& operator=(const SideStream&) = delete;
    int fork(cudaStream_t from) {
        FPSGPU_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        FPSGPU_CUDA_TRY(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
        FPSGPU_CUDA_TRY(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
        FPSGPU_CUDA_TRY(cudaEventRecord(ev_fork, from));
        FPSGPU_CUDA_TRY(cudaStreamWaitEvent(s, ev_fork, 0));
        return FPSGPU_OK;
    }
    int join(cudaStream_t into) {
        FPSGPU_CUDA_TRY(cudaEventRecord(ev_join, s));
        FPSGPU_CUDA_TRY(cudaStreamWaitEvent(into, ev_join, 0));
        joined = true;
        return FPSGPU_OK;
    }
    ~SideStream() {
        if (s && !joined) cudaStreamSynchronize(s);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (s) cudaStreamDestroy(s);
    }
};

// One vanilla FPS call on device buffers.
struct VanillaCall {
    const float* d_points;  // row-major [n][dim]
    uint64_t n;
    int dim;
    uint64_t k;
    const uint64_t* h_starts;
    uint32_t n_starts;
    uint64_t* d_out;
    float* d_trace;
    cudaStream_t stream;
    int sms;
    float* d_out_pts = nullptr;  // null, or [k][dim]: the sampled points (fused gather)
};
int run_vanilla_nofma(const VanillaCall& c);
int run_vanilla_fma(const VanillaCall& c);

// The pruned engine (engine.cuh): kd-line QuickFPS and vanilla FPS.
struct EngineCall;
struct BatchCall;
int run_engine_nofma(int dim, const EngineCall& c);
int run_engine_fma(int dim, const EngineCall& c);
int run_batch_nofma(int dim, const BatchCall& c);
int run_batch_fma(int dim, const BatchCall& c);

// fpsgpu_kdline_batch_device with the multi-CTA samplers (clouds too large for
// one CTA) limited to max_grid CTAs (0: all SMs), so that several batches can
// share the GPU.
int kdline_batch_device_capped(const float* d_points, const size_t* h_offsets, size_t n_clouds,
                               size_t dim, const size_t* h_n_samples, const size_t* h_start_idx,
                               const size_t* h_height, uint64_t* d_out, void* stream,
                               int max_grid, float* d_out_pts = nullptr, int min_cluster = 0);

// measurement counters (fpsgpu_stats_*)
void stats_count_launch(uint64_t n = 1);
bool stats_timing_enabled();
// Records the sampler's events/counters: call begin() right before the sampler
// launch and end() right after it (same stream); end() adds the device time
// after the caller's stream synchronisation via finish().
struct SamplerTimer {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    bool on = false;
    void begin(cudaStream_t s);
    void end(cudaStream_t s);
    void finish(uint64_t samples, const uint64_t* h_counters /* tested, touched */);
    ~SamplerTimer();
};

// cooperative launch helper: refuses grids that cannot be co-resident
int launch_persistent(const void* func, int grid, int block, void** args, size_t smem,
                      cudaStream_t stream, bool cooperative);
// one-time kernel attributes (see api.cu)
int allow_max_smem(const void* func);
int allow_cluster16(const void* func);

// thread-block cluster launches (batched engine's cluster sampler)
int cluster_size_for_batch();
// One-CTA batched clouds of D <= 3 take the leader/worker sampler unless
// FPSGPU_ONECTA_SAMPLER=lockstep selects the lockstep one (batch_sample).
bool lead_sampler_enabled();
// Hot pieces per worker warp of the leader/worker sampler: FPSGPU_LEAD_HOT
// (5 or 7) fixes the table for every launch; 0 (unset): the size rule.
int lead_hot_per_warp();
bool cluster_size_fixed();
uint32_t cluster_min_pieces();
int cluster_capacity(const void* func, int cl, int block, size_t smem, int* out);
int launch_clustered(const void* func, int items, int cl, int block, void** args, size_t smem,
                     cudaStream_t stream, int max_ctas = 0);

}  // namespace fpsgpu
