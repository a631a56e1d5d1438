// Bandwidth microbenchmarks for the roofline of the on-chip levels: aggregate
// shared-memory read bandwidth and L2 read bandwidth of this GPU.  The vanilla
// FPS configurations whose cloud stays on chip are bounded by these, not by
// HBM; the measured HBM copy bandwidth of this GPU type covers the rest.  Diagnostics
// only: nothing on the sampling path calls them.
#include <cuda_runtime.h>

#include "fpsgpu_internal.h"

namespace fpsgpu {
namespace {

constexpr int kBwThreads = 1024;
constexpr int kSmemFloat4 = 3072;  // 48 KB of float4 per CTA

// Every thread reads float4 words of its CTA's shared buffer; consecutive
// threads read consecutive words (no bank conflicts) and the word changes every
// iteration, so the loads cannot be hoisted.
__global__ void __launch_bounds__(kBwThreads) smem_read(int iters, float* sink) {
    __shared__ float4 buf[kSmemFloat4];
    for (int i = threadIdx.x; i < kSmemFloat4; i += blockDim.x)
        buf[i] = make_float4((float)i, 1.0f, 2.0f, 3.0f);
    __syncthreads();
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    int idx = threadIdx.x;
    for (int it = 0; it < iters; ++it) {
        const float4 v = buf[idx];
        acc.x += v.x;
        acc.y += v.y;
        acc.z += v.z;
        acc.w += v.w;
        idx += kBwThreads;
        if (idx >= kSmemFloat4) idx -= kSmemFloat4;
    }
    if (acc.x + acc.y + acc.z + acc.w == -1.0f) sink[blockIdx.x] = acc.x;  // never true
}

// Grid-stride float4 reads of a buffer that fits in L2, bypassing L1.
__global__ void __launch_bounds__(kBwThreads) l2_read(const float4* __restrict__ p, size_t n4,
                                                      int passes, float* sink) {
    float acc = 0.0f;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (int r = 0; r < passes; ++r) {
        for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
            const float4 v = __ldcg(p + i);
            acc += v.x + v.y + v.z + v.w;
        }
    }
    if (acc == -1.0f) sink[blockIdx.x] = acc;  // never true
}

int measure(int level, double* gbs) {
    int dev = 0, sms = 0;
    FPSGPU_CUDA_TRY(cudaGetDevice(&dev));
    FPSGPU_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    float* sink = nullptr;
    FPSGPU_CUDA_TRY(cudaMalloc(&sink, (size_t)sms * 8 * sizeof(float)));
    cudaEvent_t e0, e1;
    FPSGPU_CUDA_TRY(cudaEventCreate(&e0));
    FPSGPU_CUDA_TRY(cudaEventCreate(&e1));
    double bytes = 0.0;
    float ms = 0.0f;
    int rc = FPSGPU_OK;
    if (level == 0) {
        int per_sm = 0;
        FPSGPU_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, smem_read, kBwThreads, 0));
        const int grid = sms * (per_sm > 0 ? per_sm : 1);
        const int iters = 1 << 14;
        smem_read<<<grid, kBwThreads>>>(iters, sink);  // warm-up
        FPSGPU_CUDA_TRY(cudaEventRecord(e0));
        smem_read<<<grid, kBwThreads>>>(iters, sink);
        FPSGPU_CUDA_TRY(cudaEventRecord(e1));
        bytes = (double)grid * kBwThreads * iters * sizeof(float4);
    } else if (level == 1) {
        const size_t n4 = (32ull << 20) / sizeof(float4);  // 32 MB: resident in L2
        float4* buf = nullptr;
        FPSGPU_CUDA_TRY(cudaMalloc(&buf, n4 * sizeof(float4)));
        FPSGPU_CUDA_TRY(cudaMemset(buf, 0, n4 * sizeof(float4)));
        const int grid = sms * 2, passes = 64;
        l2_read<<<grid, kBwThreads>>>(buf, n4, 2, sink);  // warm-up, loads the buffer into L2
        FPSGPU_CUDA_TRY(cudaEventRecord(e0));
        l2_read<<<grid, kBwThreads>>>(buf, n4, passes, sink);
        FPSGPU_CUDA_TRY(cudaEventRecord(e1));
        bytes = (double)n4 * sizeof(float4) * passes;
        FPSGPU_CUDA_TRY(cudaEventSynchronize(e1));
        cudaFree(buf);
    } else {
        rc = set_error(FPSGPU_ERR_ARG, "unknown bandwidth level %d (0 shared memory, 1 L2)", level);
    }
    if (!rc) {
        FPSGPU_CUDA_TRY(cudaGetLastError());
        FPSGPU_CUDA_TRY(cudaEventSynchronize(e1));
        FPSGPU_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        *gbs = ms > 0.0f ? bytes / (ms * 1e-3) / 1e9 : 0.0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    return rc;
}

}  // namespace
}  // namespace fpsgpu

extern "C" int fpsgpu_measure_bandwidth(int level, double* gbs) {
    fpsgpu::clear_error();
    if (!gbs) return fpsgpu::set_error(FPSGPU_ERR_ARG, "null output");
    return fpsgpu::measure(level, gbs);
}
