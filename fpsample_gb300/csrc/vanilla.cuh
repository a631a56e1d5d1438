// Vanilla FPS kernels (reference: src/lib.cpp:111-246).
//
// Two persistent kernels, both one CTA of 1024 threads per SM:
//
// vanilla_resident<D,FMA,PPT>: the whole cloud lives on-chip.  Every thread
//   owns PPT points (coordinates and running min-distance in registers) for all
//   K iterations; the cloud is read from HBM once.  One iteration = update the
//   owned min-distances with the previous sample, warp argmax (redux.sync),
//   CTA argmax through shared memory, and (for G > 1 CTAs) the cross-CTA
//   all-gather exchange.  The winner's coordinates are then fetched once per
//   CTA (from a shared-memory copy of the cloud when G == 1, else from L2).
//
// vanilla_stream<D,FMA>: clouds beyond the register file (or D > 8).  The
//   cloud is transposed once to SoA in HBM and every iteration streams each
//   CTA's contiguous slice (coordinates + min-distance), writing a distance
//   back only when it drops.  D == 0 selects the runtime-dimension path.
//
// Tie rule: highest index (lib.cpp:226 scans with >=), via key_high_wins.
// The running min-distance starts at +inf and is lowered with a strict <
// (lib.cpp:206, 220), which also leaves it unchanged for NaN distances.
#pragma once

#include "fpsgpu_device.cuh"
#include "fpsgpu_internal.h"

namespace fpsgpu {

struct VanillaArgs {
    const float* pts;  // row-major [n][D]   (resident kernel)
    const float* X;    // SoA [dim][n]       (stream kernel)
    float* dis;        // [n]                (stream kernel)
    uint64_t n;
    int dim;
    uint64_t k;
    const uint64_t* starts;  // device
    uint32_t n_starts;
    uint64_t* out;
    float* trace;
    float* out_pts;  // null, or [k][dim]: coordinates of every sample (fused gather)
    uint64_t* slots;
    int* err;
    int smem_cloud;  // resident kernel, G == 1: cloud copied to shared memory
};

constexpr int kVanillaThreads = 1024;

template <int D, bool FMA, int PPT>
__global__ void __launch_bounds__(kVanillaThreads, 1) vanilla_resident(VanillaArgs a) {
    extern __shared__ float s_cloud[];
    __shared__ uint64_t s_wkey[32];
    __shared__ float s_ref[kMaxDim];
    __shared__ int s_abort;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nwarps = blockDim.x >> 5;
    const uint32_t T = blockDim.x;
    const int G = gridDim.x;
    const uint64_t base = (uint64_t)blockIdx.x * PPT * T;

    float x[PPT][D];
    float dis[PPT];
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        const uint64_t p = base + (uint64_t)j * T + tid;
        if (p < a.n) {
#pragma unroll
            for (int d = 0; d < D; ++d) x[j][d] = a.pts[p * D + d];
        } else {
#pragma unroll
            for (int d = 0; d < D; ++d) x[j][d] = 0.0f;
        }
        dis[j] = INFINITY;
    }
    const float* src = a.pts;
    if (a.smem_cloud) {
        for (uint64_t i = tid; i < a.n * D; i += T) s_cloud[i] = a.pts[i];
        src = s_cloud;
    }
    uint64_t pos = a.starts[0];
    if (tid == 0) s_abort = 0;
    if (blockIdx.x == 0 && tid == 0) {
        a.out[0] = pos;
        if (a.trace) a.trace[0] = INFINITY;
    }
    if (tid < D) {
        s_ref[tid] = a.pts[pos * D + tid];
        if (blockIdx.x == 0 && a.out_pts) a.out_pts[tid] = s_ref[tid];
    }
    __syncthreads();

    uint32_t xround = 0;
    for (uint64_t t = 1; t < a.k; ++t) {
        float r[D];
#pragma unroll
        for (int d = 0; d < D; ++d) r[d] = s_ref[d];
        const bool forced = t < a.n_starts;
        uint64_t best = 0;
#pragma unroll
        for (int j = 0; j < PPT; ++j) {
            const uint64_t p = base + (uint64_t)j * T + tid;
            if (p < a.n) {
                float dd = sqdist<D, FMA>(x[j], r);
                if (dd < dis[j]) dis[j] = dd;
                uint64_t kk = key_high_wins(dis[j], (uint32_t)p);
                best = kk > best ? kk : best;
            }
        }
        if (!forced) {
            uint64_t wk = warp_max_key(best);
            if (lane == 0) s_wkey[warp] = wk;
        }
        __syncthreads();
        if (warp == 0) {
            uint64_t g = 0;
            bool ok = true;
            if (forced) {
                pos = a.starts[t];
            } else {
                g = warp_max_key(lane < nwarps ? s_wkey[lane] : 0ull);
                if (G > 1) g = exchange_max(a.slots, G, xround++, g, a.err);
                ok = g != 0;
                pos = key_pos<false>(g);
            }
            if (!ok) {
                if (lane == 0) s_abort = 1;
            } else {
                if (lane < D) {
                    const float v = src[pos * D + lane];
                    s_ref[lane] = v;
                    if (blockIdx.x == 0 && a.out_pts) a.out_pts[t * D + lane] = v;
                }
                if (blockIdx.x == 0 && lane == 0) {
                    a.out[t] = pos;
                    if (a.trace) a.trace[t] = forced ? INFINITY : key_dist(g);
                }
            }
        }
        __syncthreads();
        if (s_abort) break;
    }
}

template <int D, bool FMA>
__global__ void __launch_bounds__(kVanillaThreads, 1) vanilla_stream(VanillaArgs a) {
    extern __shared__ float s_dyn[];  // runtime-D reference coordinates
    __shared__ uint64_t s_wkey[32];
    __shared__ int s_abort;
    constexpr int DS = D > 0 ? D : 1;
    __shared__ float s_ref_static[DS];
    float* s_ref = D > 0 ? s_ref_static : s_dyn;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nwarps = blockDim.x >> 5;
    const uint32_t T = blockDim.x;
    const int G = gridDim.x;
    const int dim = D > 0 ? D : a.dim;
    const uint64_t n = a.n;
    const uint64_t per = (n + G - 1) / G;
    const uint64_t lo = (uint64_t)blockIdx.x * per;
    const uint64_t hi = lo + per < n ? lo + per : n;
    const float* __restrict__ X = a.X;
    float* __restrict__ dis = a.dis;

    for (uint64_t p = lo + tid; p < hi; p += T) dis[p] = INFINITY;
    uint64_t pos = a.starts[0];
    if (tid == 0) s_abort = 0;
    if (blockIdx.x == 0 && tid == 0) {
        a.out[0] = pos;
        if (a.trace) a.trace[0] = INFINITY;
    }
    for (int d = tid; d < dim; d += T) {
        s_ref[d] = X[(uint64_t)d * n + pos];
        if (blockIdx.x == 0 && a.out_pts) a.out_pts[d] = s_ref[d];
    }
    __syncthreads();

    uint32_t xround = 0;
    for (uint64_t t = 1; t < a.k; ++t) {
        const bool forced = t < a.n_starts;
        uint64_t best = 0;
        if (D > 0) {
            float r[DS];
#pragma unroll
            for (int d = 0; d < DS; ++d) r[d] = s_ref[d];
#pragma unroll 4
            for (uint64_t p = lo + tid; p < hi; p += T) {
                float x[DS];
#pragma unroll
                for (int d = 0; d < DS; ++d) x[d] = X[(uint64_t)d * n + p];
                float dv = dis[p];
                float dd = sqdist<DS, FMA>(x, r);
                if (dd < dv) {
                    dv = dd;
                    dis[p] = dd;
                }
                uint64_t kk = key_high_wins(dv, (uint32_t)p);
                best = kk > best ? kk : best;
            }
        } else {
            for (uint64_t p = lo + tid; p < hi; p += T) {
                float dv = dis[p];
                float dd = sqdist_rt<FMA>(X, n, p, s_ref, dim);
                if (dd < dv) {
                    dv = dd;
                    dis[p] = dd;
                }
                uint64_t kk = key_high_wins(dv, (uint32_t)p);
                best = kk > best ? kk : best;
            }
        }
        if (!forced) {
            uint64_t wk = warp_max_key(best);
            if (lane == 0) s_wkey[warp] = wk;
        }
        __syncthreads();
        if (warp == 0) {
            uint64_t g = 0;
            bool ok = true;
            if (forced) {
                pos = a.starts[t];
            } else {
                g = warp_max_key(lane < nwarps ? s_wkey[lane] : 0ull);
                if (G > 1) g = exchange_max(a.slots, G, xround++, g, a.err);
                ok = g != 0;
                pos = key_pos<false>(g);
            }
            if (!ok) {
                if (lane == 0) s_abort = 1;
            } else {
                for (int d = lane; d < dim; d += 32) {
                    const float v = X[(uint64_t)d * n + pos];
                    s_ref[d] = v;
                    if (blockIdx.x == 0 && a.out_pts) a.out_pts[t * (uint64_t)dim + d] = v;
                }
                if (blockIdx.x == 0 && lane == 0) {
                    a.out[t] = pos;
                    if (a.trace) a.trace[t] = forced ? INFINITY : key_dist(g);
                }
            }
        }
        __syncthreads();
        if (s_abort) break;
    }
}

// row-major [n][dim] -> SoA [dim][n]
__global__ void transpose_to_soa(const float* __restrict__ pts, float* __restrict__ X, uint64_t n,
                                 int dim);

// ---------------------------------------------------------------------------
// host launcher
// ---------------------------------------------------------------------------

template <int D, bool FMA, int PPT>
int launch_resident(const VanillaCall& c, VanillaArgs a, int G) {
    auto kern = vanilla_resident<D, FMA, PPT>;
    size_t smem = a.smem_cloud ? (size_t)c.n * D * sizeof(float) : 0;
    // static + dynamic shared memory above 48 KB needs the opt-in attribute
    if (smem > 0)
        if (int arc = allow_max_smem((const void*)kern)) return arc;
    void* args[] = {&a};
    return launch_persistent((const void*)kern, G, kVanillaThreads, args, smem, c.stream, G > 1);
}

template <int D, bool FMA>
int run_vanilla_d(const VanillaCall& c) {
    Scratch sc(c.stream);
    VanillaArgs a{};
    a.pts = c.d_points;
    a.n = c.n;
    a.dim = c.dim;
    a.k = c.k;
    a.n_starts = c.n_starts;
    a.out = c.d_out;
    a.trace = c.d_trace;
    a.out_pts = c.d_out_pts;
    int rc;
    uint64_t* d_starts;
    if ((rc = sc.alloc(&d_starts, c.n_starts))) return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_starts, c.h_starts, c.n_starts * sizeof(uint64_t),
                                    cudaMemcpyHostToDevice, c.stream));
    a.starts = d_starts;
    int* d_err;
    if ((rc = sc.alloc(&d_err, 1))) return rc;
    FPSGPU_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), c.stream));
    a.err = d_err;

    constexpr int DR = D > 0 ? D : 1;  // resident kernels exist for D in [1, 8] only
    constexpr int ppt_max = (D > 0 && D <= 4) ? 8 : 4;
    const uint64_t per_cta = (uint64_t)kVanillaThreads * ppt_max;
    const int max_g = c.sms;  // one 1024-thread CTA per SM
    int G = 1, ppt = ppt_max;
    bool resident = D > 0;
    if (resident) {
        if (c.n <= (uint64_t)kVanillaThreads) ppt = 1;
        else if (c.n <= 2ull * kVanillaThreads) ppt = 2;
        else if (c.n <= 4ull * kVanillaThreads) ppt = 4;
        else ppt = ppt_max;
        uint64_t g = (c.n + (uint64_t)kVanillaThreads * ppt - 1) / ((uint64_t)kVanillaThreads * ppt);
        if (g > (uint64_t)max_g) resident = false;
        G = (int)g;
        (void)per_cta;
    }
    SamplerTimer timer;
    if (resident) {
        uint64_t* slots = nullptr;
        if (G > 1) {
            if ((rc = sc.alloc(&slots, 3ull * G))) return rc;
            FPSGPU_CUDA_TRY(cudaMemsetAsync(slots, 0, 3ull * G * sizeof(uint64_t), c.stream));
        }
        a.slots = slots;
        a.smem_cloud = (G == 1 && c.n * D * sizeof(float) <= 96 * 1024) ? 1 : 0;
        timer.begin(c.stream);
        switch (ppt) {
            case 1: rc = launch_resident<DR, FMA, 1>(c, a, G); break;
            case 2: rc = launch_resident<DR, FMA, 2>(c, a, G); break;
            case 4: rc = launch_resident<DR, FMA, 4>(c, a, G); break;
            default: rc = launch_resident<DR, FMA, ppt_max>(c, a, G); break;
        }
        if (rc) return rc;
        timer.end(c.stream);
    } else {
        G = max_g;
        float *X, *dis;
        if ((rc = sc.alloc(&X, c.n * (uint64_t)c.dim))) return rc;
        if ((rc = sc.alloc(&dis, c.n))) return rc;
        uint64_t* slots;
        if ((rc = sc.alloc(&slots, 3ull * G))) return rc;
        FPSGPU_CUDA_TRY(cudaMemsetAsync(slots, 0, 3ull * G * sizeof(uint64_t), c.stream));
        {
            uint64_t blocks = (c.n + 255) / 256;
            if (blocks > 65535ull * 64) blocks = 65535ull * 64;
            stats_count_launch();
            transpose_to_soa<<<(unsigned)blocks, 256, 0, c.stream>>>(c.d_points, X, c.n, c.dim);
            FPSGPU_CUDA_TRY(cudaGetLastError());
        }
        a.X = X;
        a.dis = dis;
        a.slots = slots;
        auto kern = vanilla_stream<D, FMA>;
        size_t smem = D > 0 ? 0 : (size_t)c.dim * sizeof(float);
        if (smem > 0)
            if (int arc = allow_max_smem((const void*)kern)) return arc;
        void* args[] = {&a};
        timer.begin(c.stream);
        if ((rc = launch_persistent((const void*)kern, G, kVanillaThreads, args, smem, c.stream,
                                    true)))
            return rc;
        timer.end(c.stream);
    }
    int h_err = 0;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    FPSGPU_CUDA_TRY(cudaStreamSynchronize(c.stream));
    {
        // brute force: every running distance is recomputed on every iteration
        const uint64_t cnt[2] = {0, c.k > 0 ? c.n * (c.k - 1) : 0};
        timer.finish(c.k, cnt);
    }
    if (h_err)
        return set_error(FPSGPU_ERR_DEVICE, "vanilla FPS kernel gave up (device error word 0x%x)",
                         h_err);
    return FPSGPU_OK;
}

template <bool FMA>
int run_vanilla_dispatch(const VanillaCall& c) {
    switch (c.dim) {
        case 1: return run_vanilla_d<1, FMA>(c);
        case 2: return run_vanilla_d<2, FMA>(c);
        case 3: return run_vanilla_d<3, FMA>(c);
        case 4: return run_vanilla_d<4, FMA>(c);
        case 5: return run_vanilla_d<5, FMA>(c);
        case 6: return run_vanilla_d<6, FMA>(c);
        case 7: return run_vanilla_d<7, FMA>(c);
        case 8: return run_vanilla_d<8, FMA>(c);
        default: return run_vanilla_d<0, FMA>(c);
    }
}

}  // namespace fpsgpu
