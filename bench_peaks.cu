// Bandwidth microbenchmarks for bench.py's roofline of the on-chip levels:
// aggregate shared-memory read bandwidth and L2 read bandwidth of this GPU.
// The vanilla FPS configurations whose cloud stays on chip are bounded by
// these, not by HBM; the measured HBM copy bandwidth of this GPU type covers
// the rest.  Not part of the library: `bench.py --probe peaks` compiles this
// file into a small shared object of its own and prints profiles/peaks.json.
#include <cuda_runtime.h>

#define TRY(expr)                               \
    do {                                        \
        cudaError_t e_ = (expr);                \
        if (e_ != cudaSuccess) return (int)e_;  \
    } while (0)

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
    TRY(cudaGetDevice(&dev));
    TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    float* sink = nullptr;
    TRY(cudaMalloc(&sink, (size_t)sms * 8 * sizeof(float)));
    cudaEvent_t e0, e1;
    TRY(cudaEventCreate(&e0));
    TRY(cudaEventCreate(&e1));
    double bytes = 0.0;
    float ms = 0.0f;
    int rc = 0;
    if (level == 0) {
        int per_sm = 0;
        TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, smem_read, kBwThreads, 0));
        const int grid = sms * (per_sm > 0 ? per_sm : 1);
        const int iters = 1 << 14;
        smem_read<<<grid, kBwThreads>>>(iters, sink);  // warm-up
        TRY(cudaEventRecord(e0));
        smem_read<<<grid, kBwThreads>>>(iters, sink);
        TRY(cudaEventRecord(e1));
        bytes = (double)grid * kBwThreads * iters * sizeof(float4);
    } else if (level == 1) {
        const size_t n4 = (32ull << 20) / sizeof(float4);  // 32 MB: resident in L2
        float4* buf = nullptr;
        TRY(cudaMalloc(&buf, n4 * sizeof(float4)));
        TRY(cudaMemset(buf, 0, n4 * sizeof(float4)));
        const int grid = sms * 2, passes = 64;
        l2_read<<<grid, kBwThreads>>>(buf, n4, 2, sink);  // warm-up, loads the buffer into L2
        TRY(cudaEventRecord(e0));
        l2_read<<<grid, kBwThreads>>>(buf, n4, passes, sink);
        TRY(cudaEventRecord(e1));
        bytes = (double)n4 * sizeof(float4) * passes;
        TRY(cudaEventSynchronize(e1));
        cudaFree(buf);
    } else {
        rc = -1;  // unknown level (0 shared memory, 1 L2)
    }
    if (!rc) {
        TRY(cudaGetLastError());
        TRY(cudaEventSynchronize(e1));
        TRY(cudaEventElapsedTime(&ms, e0, e1));
        *gbs = ms > 0.0f ? bytes / (ms * 1e-3) / 1e9 : 0.0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    return rc;
}

}  // namespace

// Read bandwidth in GB/s of level 0 (shared memory, all SMs) or 1 (L2, a 32 MB
// buffer); 0 on success, else a cudaError_t value (-1: unknown level).
extern "C" int bench_measure_bandwidth(int level, double* gbs) {
    if (!gbs) return -1;
    return measure(level, gbs);
}
