// Pruned FPS engine: one GPU design behind both kd-line QuickFPS
// (reference src/wrapper.hpp:45-60, src/_ext/*.h) and vanilla FPS
// (reference src/lib.cpp:111-246).
//
// Contract.  Both reference algorithms output plain farthest point sampling in
// fp32 with a fixed tie rule:
//   * kd-line: FPS over the tree build's permuted order, started at permuted
//     position start_idx, running distance capped at FLT_MAX, ties to the
//     LOWEST permuted position (the reference's bucket pruning never changes a
//     value, so its output is exactly this);
//   * vanilla: FPS over the original order, running distance starting at +inf,
//     ties to the HIGHEST original index, optional forced start list.
// Every point therefore carries a "tag" -- its permuted position (kd-line) or
// its original index (vanilla) -- and only the tag decides ties.  Where a
// point is stored on the GPU is free, so the engine reorders points into small
// spatially tight pieces purely for pruning.
//
// Build.
//   1. exact phase (kd-line only): the reference's kd-line tree, level by
//      level, one CTA per node, bit-exact (split_kernel<EXACT=true>):
//        - exact bounding box (order-free min/max, NaN ignored,
//          KDTreeBase.h:181-207), split dimension = first strictly widest
//          fp32 span (KDTreeBase.h:160-179);
//        - split value = SEQUENTIAL fp32 sum over the node in its current order
//          / (float)count (KDTreeBase.h:151-158): warps 1..31 stream the column
//          through a double-buffered shared-memory ring, thread 0 sums;
//        - the two-pointer partition (KDTreeBase.h:123-149) in parallel: with
//          L = #(x < split), the k-th element >= split in [s, s+L) trades
//          places with the k-th element < split counted from the right end of
//          [s+L, e); ranks from warp-segment ballot scans; split point L clamped
//          to [1, count-1]; leaf at depth == height or one point
//          (KDLineTree.h:37-39).
//      Then a snapshot: Xref = coordinates by permuted position, idsnap =
//      original index by permuted position, tag = permuted position.
//   2. refinement phase: every exact leaf (vanilla: the whole cloud) is split
//      further, with any cheap rule (parallel mean of the widest dimension,
//      halving by count when that does not separate), carrying the tag, until
//      every piece holds at most kPiece points.  Pieces tile the storage order.
//   3. exact bounding box of every piece.
//
// Sampling.  Every sampler keeps each piece's max key (running distance, tag)
// and box; for a new reference point r, a piece whose box_bound(r) >= its max
// cannot change (see box_bound) and is skipped; other pieces recompute their
// points.  Samplers differ in who holds the pieces and how the argmax is
// combined:
//   * batch_sample<CL=false>: one CTA per cloud from a persistent queue,
//     piece records in registers, one __syncthreads per sample;
//   * batch_sample<CL=true>: one thread-block cluster per cloud, the CTAs'
//     maxima exchanged through distributed shared memory (st.async + mbarrier);
//   * grid_sample_reg / grid_sample_smem / fps_sample: one cloud on a
//     persistent cooperative grid, the grid-wide argmax through
//     exchange_leader (which also delivers the winner's coordinates; fps_sample
//     reads them from Xref by tag).
#pragma once

#include <algorithm>
#include <cmath>

#include "fpsgpu_device.cuh"
#include "fpsgpu_internal.h"

namespace fpsgpu {

constexpr int kBuildThreads = 1024;
constexpr int kRefineThreads = 256;
constexpr int kSumChunk = 4096;   // floats per ring slot of the serial mean
constexpr int kSampleThreads = 1024;
constexpr uint32_t kPiece = 128;  // max points per piece
constexpr int kCompactChunk = 8192;

// node: {first, end, depth, height}
struct BuildArgs {
    float* X;            // SoA [D][n], storage order
    uint32_t* tag;       // [n]: original index in the exact phase, tie tag afterwards
    uint32_t* sel;       // [n] scratch: partner positions
    uint8_t* flag;       // [n] 1 at the first position of every piece
    uint4* cur;          // nodes of this level
    uint4* next;         // nodes of the next level
    uint32_t* cnt_cur;   // node count of this level
    uint32_t* cnt_next;
    uint4* refine;       // exact-phase leaves that still need refining
    uint32_t* refine_cnt;
    uint64_t n;
    int* err;
    // sampling builds: a node of at most kPiece points starts one piece and its
    // subtree (still split exactly) starts no more; build-only calls keep the
    // reference's buckets (every exact leaf starts one)
    int coarse;
    // bucket_fps_kdtree: the snapshot gives every point the REVERSED position
    // of its cloud as tag, so that "lowest tag wins" means "last position wins"
    int reverse;
    const uint64_t* cloud_off;  // [n_clouds + 1] (reverse only)
    uint32_t n_clouds;
};

// Node depth word: bit 31 marks a node inside an existing piece (coarse mode).
constexpr uint32_t kCovered = 0x80000000u;

// Block-wide exclusive rank of `f` among the block's threads (thread order),
// and the block total.  `s_w` is a 2 x 32 array that alternates between calls
// through `parity`, so one __syncthreads per call suffices.
__device__ __forceinline__ uint32_t block_rank(bool f, uint32_t* s_w, int parity, uint32_t& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const uint32_t m = __ballot_sync(kFull, f);
    const uint32_t below = __popc(m & ((1u << lane) - 1u));
    uint32_t* w = s_w + parity * 32;
    if (lane == 0) w[warp] = __popc(m);
    __syncthreads();
    const uint32_t c = lane < nwarps ? w[lane] : 0u;
    uint32_t v = c;  // inclusive scan over the warp counts
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t u = __shfl_up_sync(kFull, v, o);
        if (lane >= o) v += u;
    }
    total = __shfl_sync(kFull, v, 31);
    return __shfl_sync(kFull, v - c, warp) + below;
}

// Serial fp32 sum of m floats from shared memory, continuing `acc`.
__device__ __forceinline__ float serial_sum(float acc, const float* buf, uint32_t m) {
    uint32_t i = 0;
    for (; i + 16 <= m; i += 16) {
        float4 v0 = *reinterpret_cast<const float4*>(buf + i);
        float4 v1 = *reinterpret_cast<const float4*>(buf + i + 4);
        float4 v2 = *reinterpret_cast<const float4*>(buf + i + 8);
        float4 v3 = *reinterpret_cast<const float4*>(buf + i + 12);
        acc = __fadd_rn(acc, v0.x); acc = __fadd_rn(acc, v0.y);
        acc = __fadd_rn(acc, v0.z); acc = __fadd_rn(acc, v0.w);
        acc = __fadd_rn(acc, v1.x); acc = __fadd_rn(acc, v1.y);
        acc = __fadd_rn(acc, v1.z); acc = __fadd_rn(acc, v1.w);
        acc = __fadd_rn(acc, v2.x); acc = __fadd_rn(acc, v2.y);
        acc = __fadd_rn(acc, v2.z); acc = __fadd_rn(acc, v2.w);
        acc = __fadd_rn(acc, v3.x); acc = __fadd_rn(acc, v3.y);
        acc = __fadd_rn(acc, v3.z); acc = __fadd_rn(acc, v3.w);
    }
    for (; i < m; ++i) acc = __fadd_rn(acc, buf[i]);
    return acc;
}

// row-major points -> SoA, tag = original index; one root per cloud:
// roots[c] = {first, end, 0, height}.  The flag array is zeroed beforehand.
template <int D>
__global__ void build_prepare(const float* __restrict__ pts, BuildArgs a, const uint4* roots,
                              uint32_t n_clouds, int exact) {
    const uint64_t n = a.n;
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t p = tid; p < n; p += stride) {
#pragma unroll
        for (int d = 0; d < D; ++d) a.X[(uint64_t)d * n + p] = pts[p * D + d];
        a.tag[p] = (uint32_t)p;
    }
    for (uint64_t c = tid; c < n_clouds; c += stride) {
        const uint4 root = roots[c];
        const uint32_t len = root.y - root.x;
        if (len == 0) continue;
        a.flag[root.x] = 1;  // every cloud starts a piece
        if (exact && root.w > 0 && len > 1) {
            uint4 r = root;
            if (a.coarse && len <= kPiece) r.z |= kCovered;  // the whole cloud is one piece
            a.cur[atomicAdd(a.cnt_cur, 1u)] = r;
        } else if (len > kPiece) {
            a.refine[atomicAdd(a.refine_cnt, 1u)] = root;
        }
    }
}

// Exclusive offsets of this warp's two counts among the block's warps (warp
// order) and the block totals; one __syncthreads.  s_w holds 2 x 32 words and
// must not be reused before the next __syncthreads.
__device__ __forceinline__ void warp_offsets2(uint32_t c0, uint32_t c1, uint32_t* s_w, uint32_t& o0,
                                              uint32_t& o1, uint32_t& t0, uint32_t& t1) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    if (lane == 0) {
        s_w[warp] = c0;
        s_w[32 + warp] = c1;
    }
    __syncthreads();
    uint32_t a = lane < nwarps ? s_w[lane] : 0u, b = lane < nwarps ? s_w[32 + lane] : 0u;
    uint32_t va = a, vb = b;  // inclusive scans over the warp counts
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t ua = __shfl_up_sync(kFull, va, o), ub = __shfl_up_sync(kFull, vb, o);
        if (lane >= o) {
            va += ua;
            vb += ub;
        }
    }
    t0 = __shfl_sync(kFull, va, 31);
    t1 = __shfl_sync(kFull, vb, 31);
    o0 = __shfl_sync(kFull, va - a, warp);
    o1 = __shfl_sync(kFull, vb - b, warp);
}

// Warp w's share [lo, hi) of an index range [0, len) cut into nwarps
// contiguous, 32-aligned segments (coalesced within the warp).
__device__ __forceinline__ void warp_segment(uint32_t len, uint32_t& lo, uint32_t& hi) {
    const uint32_t nwarps = blockDim.x >> 5, warp = threadIdx.x >> 5;
    const uint32_t seg = ((len + nwarps - 1) / nwarps + 31u) & ~31u;
    lo = min(len, warp * seg);
    hi = min(len, lo + seg);
}

// Splits the nodes of one level, one CTA of T threads per node.
// EXACT: the reference's kd-line rule (bit-exact permutation).
// !EXACT: refinement (any rule; mean of the widest dimension, or halving).
// Every pass over the node streams it with U independent loads per thread in
// flight; the partition ranks come from warp-contiguous segments (two passes:
// counts, one block-wide scan of the warp counts, then ranks by ballot), so a
// node costs a handful of __syncthreads whatever its size.
template <int D, bool EXACT, int T>
__global__ void __launch_bounds__(T) split_kernel(BuildArgs a, int force_leaf) {
    constexpr int RING = EXACT ? kSumChunk : 4;
    constexpr int U = D <= 4 ? 4 : 2;  // loads in flight per thread and pass
    __shared__ __align__(16) float s_ring[2][RING];
    __shared__ float s_lo[32][D], s_hi[32][D];
    __shared__ uint32_t s_w[2 * 32];
    __shared__ uint32_t s_w2[2 * 32];
    __shared__ float s_fw[32];
    __shared__ float s_split;
    __shared__ int s_dim;
    __shared__ int s_degenerate;

    const uint32_t cnt = *a.cnt_cur;
    if (blockIdx.x >= cnt) return;
    const uint4 nd = a.cur[blockIdx.x];
    const uint32_t s = nd.x, e = nd.y, cntn = e - s;
    const uint64_t n = a.n;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = T / 32;

    if (!EXACT && force_leaf) {  // last refinement level: everything left is a piece
        if (tid == 0) a.flag[s] = 1;
        return;
    }

    // 1. bounding box and split dimension (min/max: order-free, NaN ignored)
    {
        float lo[D], hi[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            lo[d] = FLT_MAX;
            hi[d] = -FLT_MAX;
        }
        for (uint32_t b = s + tid; b < e; b += T * U) {
            float v[U][D];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t p = b + u * T;
#pragma unroll
                for (int d = 0; d < D; ++d) v[u][d] = p < e ? a.X[(uint64_t)d * n + p] : NAN;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    lo[d] = fminf(lo[d], v[u][d]);
                    hi[d] = fmaxf(hi[d], v[u][d]);
                }
            }
        }
#pragma unroll
        for (int d = 0; d < D; ++d) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                lo[d] = fminf(lo[d], __shfl_xor_sync(kFull, lo[d], o));
                hi[d] = fmaxf(hi[d], __shfl_xor_sync(kFull, hi[d], o));
            }
            if (lane == 0) {
                s_lo[warp][d] = lo[d];
                s_hi[warp][d] = hi[d];
            }
        }
        __syncthreads();
        if (tid == 0) {
            float span_best = 0.0f;
            int sd = 0;
            for (int d = 0; d < D; ++d) {
                float l = FLT_MAX, h = -FLT_MAX;
                for (int w = 0; w < nwarps; ++w) {
                    l = fminf(l, s_lo[w][d]);
                    h = fmaxf(h, s_hi[w][d]);
                }
                float span = __fsub_rn(h, l);
                if (span > span_best) {
                    span_best = span;
                    sd = d;
                }
            }
            s_dim = sd;
            s_degenerate = !(span_best > 0.0f);
        }
        __syncthreads();
    }
    const int sd = s_dim;
    const float* col = a.X + (uint64_t)sd * n;

    // 2. split value
    if (EXACT) {
        // sequential fp32 sum in current order, / (float)count.
        // Warps 1..nwarps-1 fill ring slot c+1 while thread 0 sums slot c.
        const uint32_t nchunks = (cntn + kSumChunk - 1) / kSumChunk;
        const uint32_t loaders = T - 32;
        if (warp > 0) {
            uint32_t m = cntn < (uint32_t)kSumChunk ? cntn : (uint32_t)kSumChunk;
            for (uint32_t i = tid - 32; i < m; i += loaders) s_ring[0][i] = col[s + i];
        }
        __syncthreads();
        float acc = 0.0f;
        for (uint32_t c = 0; c < nchunks; ++c) {
            if (warp > 0 && c + 1 < nchunks) {
                const uint32_t base = (c + 1) * kSumChunk;
                const uint32_t m = cntn - base < (uint32_t)kSumChunk ? cntn - base : (uint32_t)kSumChunk;
                float* dst = s_ring[(c + 1) & 1];
                for (uint32_t i = tid - 32; i < m; i += loaders) dst[i] = col[s + base + i];
            }
            if (tid == 0) {
                const uint32_t base = c * kSumChunk;
                const uint32_t m = cntn - base < (uint32_t)kSumChunk ? cntn - base : (uint32_t)kSumChunk;
                acc = serial_sum(acc, s_ring[c & 1], m);
            }
            __syncthreads();
        }
        if (tid == 0) s_split = __fdiv_rn(acc, __uint2float_rn(cntn));
        __syncthreads();
    } else {
        float part[U];
#pragma unroll
        for (int u = 0; u < U; ++u) part[u] = 0.0f;
        for (uint32_t b = s + tid; b < e; b += T * U) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t p = b + u * T;
                part[u] += p < e ? col[p] : 0.0f;
            }
        }
        float tot_t = 0.0f;
#pragma unroll
        for (int u = 0; u < U; ++u) tot_t += part[u];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) tot_t += __shfl_xor_sync(kFull, tot_t, o);
        if (lane == 0) s_fw[warp] = tot_t;
        __syncthreads();
        if (tid == 0) {
            float tot = 0.0f;
            for (int w = 0; w < nwarps; ++w) tot += s_fw[w];
            s_split = tot / (float)cntn;
        }
        __syncthreads();
    }
    const float split = s_split;

    // 3. L = #(x < split).  In the exact phase a NaN among the values or as the
    //    split value makes the reference's two scans disagree, which the rank
    //    formulation does not model: report it and stop splitting this node.
    uint32_t L = 0;
    bool bad_node = false;
    {
        uint32_t mine = 0;
        bool bad = EXACT && isnan(split);
        for (uint32_t b = s + tid; b < e; b += T * U) {
            float v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t p = b + u * T;
                v[u] = p < e ? col[p] : split;  // split: neither < split nor NaN
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                mine += v[u] < split ? 1u : 0u;
                if (EXACT) bad |= isnan(v[u]);
            }
        }
        mine = __reduce_add_sync(kFull, mine);
        const bool wbad = __any_sync(kFull, bad);
        if (lane == 0) {
            s_w[warp] = mine;
            s_w[32 + warp] = wbad ? 1u : 0u;
        }
        __syncthreads();
        for (int w = 0; w < nwarps; ++w) {
            L += s_w[w];
            bad_node |= s_w[32 + w] != 0;
        }
        __syncthreads();
    }
    if (bad_node) {
        if (tid == 0) {
            atomicOr(a.err, kErrNonFiniteSplit);
            a.flag[s] = 1;
        }
        return;
    }
    // refinement: a split that does not separate halves the node by count
    const bool halve = !EXACT && (L == 0 || L == cntn || s_degenerate);

    // 4. partition: the k-th element >= split in [s, s+L) trades places with the
    //    k-th element < split counted from the right end of [s+L, e).  Right
    //    side index i <-> position e-1-i, left side index i <-> position s+i;
    //    each warp ranks a contiguous segment of each side.
    if (!halve) {
        const uint32_t rlen = cntn - L;
        const uint32_t lt = (1u << lane) - 1u;
        uint32_t r0, r1, l0, l1;
        warp_segment(rlen, r0, r1);
        warp_segment(L, l0, l1);
        uint32_t cr = 0, cl = 0;
        for (uint32_t b = r0 + lane; b < r1; b += 32 * U) {
            float v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t i = b + 32 * u;
                v[u] = i < r1 ? col[e - 1 - i] : split;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) cr += v[u] < split ? 1u : 0u;
        }
        for (uint32_t b = l0 + lane; b < l1; b += 32 * U) {
            float v[U];
            bool in[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t i = b + 32 * u;
                in[u] = i < l1;
                v[u] = in[u] ? col[s + i] : split;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) cl += in[u] && !(v[u] < split) ? 1u : 0u;
        }
        cr = __reduce_add_sync(kFull, cr);
        cl = __reduce_add_sync(kFull, cl);
        uint32_t orr, ol, tr, tl;
        warp_offsets2(cr, cl, s_w2, orr, ol, tr, tl);
        // right side: the rank-k element < split goes to sel[s + k]
        {
            uint32_t run = orr;
            for (uint32_t b = r0; b < r1; b += 32 * U) {
                bool f[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const uint32_t i = b + 32 * u + lane;
                    f[u] = i < r1 && col[e - 1 - i] < split;
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const uint32_t m = __ballot_sync(kFull, f[u]);
                    if (f[u]) a.sel[s + run + __popc(m & lt)] = e - 1 - (b + 32 * u + lane);
                    run += __popc(m);
                }
            }
        }
        __syncthreads();
        // left side: the rank-k element >= split swaps with sel[s + k]
        {
            uint32_t run = ol;
            for (uint32_t b = l0; b < l1; b += 32 * U) {
                bool f[U];
                uint32_t rk[U], q[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const uint32_t i = b + 32 * u + lane;
                    f[u] = i < l1 && !(col[s + i] < split);
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const uint32_t m = __ballot_sync(kFull, f[u]);
                    rk[u] = run + __popc(m & lt);
                    run += __popc(m);
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    q[u] = f[u] ? a.sel[s + rk[u]] : 0u;
                    if (f[u] && !(q[u] >= s + L && q[u] < e)) {  // unreachable: both sides count the same predicate
                        atomicOr(a.err, kErrBadIndex);
                        f[u] = false;
                    }
                }
                // pairs are disjoint: every load before any store
                float xp[U][D], xq[U][D];
                uint32_t tp[U], tq[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    if (f[u]) {
                        const uint32_t p = s + b + 32 * u + lane;
#pragma unroll
                        for (int d = 0; d < D; ++d) {
                            xp[u][d] = a.X[(uint64_t)d * n + p];
                            xq[u][d] = a.X[(uint64_t)d * n + q[u]];
                        }
                        tp[u] = a.tag[p];
                        tq[u] = a.tag[q[u]];
                    }
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    if (f[u]) {
                        const uint32_t p = s + b + 32 * u + lane;
#pragma unroll
                        for (int d = 0; d < D; ++d) {
                            a.X[(uint64_t)d * n + p] = xq[u][d];
                            a.X[(uint64_t)d * n + q[u]] = xp[u][d];
                        }
                        a.tag[p] = tq[u];
                        a.tag[q[u]] = tp[u];
                    }
                }
            }
        }
    }

    // 5. children
    if (tid == 0) {
        uint32_t lim;
        if (halve) {
            lim = cntn / 2;
        } else {
            lim = L;  // KDTreeBase.h:142-147 clamp
            if (L == 0) lim = 1;
            if (L == cntn) lim = cntn - 1;
        }
        const uint32_t cs[2] = {s, s + lim}, ce[2] = {s + lim, e};
        const uint32_t depth = (nd.z & ~kCovered) + 1;
        const bool covered = EXACT && (nd.z & kCovered) != 0;
        for (int ch = 0; ch < 2; ++ch) {
            const uint32_t len = ce[ch] - cs[ch];
            bool leaf;
            if (EXACT) leaf = depth >= nd.w || len == 1;  // KDLineTree.h:37-39
            else leaf = len <= kPiece;
            uint32_t z = depth;
            if (EXACT && a.coarse) {
                if (covered) {
                    z |= kCovered;
                } else if (len <= kPiece) {  // the first node this small starts a piece
                    a.flag[cs[ch]] = 1;
                    z |= kCovered;
                }
            }
            const uint4 child = make_uint4(cs[ch], ce[ch], z, nd.w);
            if (!leaf) {
                a.next[atomicAdd(a.cnt_next, 1u)] = child;
            } else if (EXACT && len > kPiece) {
                a.refine[atomicAdd(a.refine_cnt, 1u)] = child;
            } else if (!(EXACT && a.coarse)) {
                a.flag[cs[ch]] = 1;
            }
        }
    }
}

// After the exact phase: tag = permuted position (reversed within its cloud
// for bucket_fps_kdtree), Xref/idsnap indexed by tag.
template <int D>
__global__ void build_snapshot(BuildArgs a, float* __restrict__ Xref, uint32_t* __restrict__ idsnap) {
    const uint64_t n = a.n;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n;
         p += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t t = p;
        if (a.reverse) {  // cloud of p: last c with cloud_off[c] <= p
            uint32_t lo = 0, hi = a.n_clouds;
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) / 2;
                if (a.cloud_off[mid] <= p) lo = mid;
                else hi = mid;
            }
            t = a.cloud_off[lo] + a.cloud_off[lo + 1] - 1 - p;
        }
#pragma unroll
        for (int d = 0; d < D; ++d) Xref[(uint64_t)d * n + t] = a.X[(uint64_t)d * n + p];
        if (idsnap) {
            idsnap[t] = a.tag[p];
            a.tag[p] = (uint32_t)t;
        }
    }
}

// refine list -> first refinement level list
__global__ void build_seed_refine(BuildArgs a);

// ---- compaction of piece flags into an ordered start list -----------------
__device__ __forceinline__ bool run_start(const uint8_t* flag, uint64_t p) {
    return p == 0 || flag[p] != 0;
}
__global__ void compact_count(const uint8_t* flag, uint64_t n, uint32_t* bcount);
__global__ void compact_scan(uint32_t* bcount, uint32_t nblocks, uint32_t* total);
__global__ void compact_write(const uint8_t* flag, uint64_t n, const uint32_t* boff,
                              const uint32_t* total, uint32_t* starts);
int compact_flags(const uint8_t* flag, uint64_t n, uint32_t* starts, uint32_t* d_count,
                  Scratch& sc, cudaStream_t stream);

template <int D>
__global__ void piece_bbox(const float* __restrict__ X, uint64_t n, const uint32_t* pstart,
                           const uint32_t* npieces, float* lo_out, float* hi_out) {
    const uint32_t np = *npieces;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < np; q += warps) {
        const uint32_t ps = pstart[q], pe = pstart[q + 1];
        float lo[D], hi[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            lo[d] = FLT_MAX;
            hi[d] = -FLT_MAX;
        }
        for (uint32_t p = ps + lane; p < pe; p += 32) {
#pragma unroll
            for (int d = 0; d < D; ++d) {
                float v = X[(uint64_t)d * n + p];
                lo[d] = fminf(lo[d], v);
                hi[d] = fmaxf(hi[d], v);
            }
        }
#pragma unroll
        for (int d = 0; d < D; ++d) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                lo[d] = fminf(lo[d], __shfl_xor_sync(kFull, lo[d], o));
                hi[d] = fmaxf(hi[d], __shfl_xor_sync(kFull, hi[d], o));
            }
        }
        if (lane == 0) {
#pragma unroll
            for (int d = 0; d < D; ++d) {
                lo_out[(uint64_t)q * D + d] = lo[d];
                hi_out[(uint64_t)q * D + d] = hi[d];
            }
        }
    }
}

// ---- sampling ----------------------------------------------------------------
struct SampleArgs {
    const float* X;          // SoA [D][n], storage order
    const uint32_t* tag;     // [n] tie tag of every stored point
    float* dis;              // [n] running distance
    uint64_t n;
    const uint32_t* pstart;  // [np + 1]
    const uint32_t* npieces; // device count, or null: np_fixed
    uint32_t np_fixed;
    uint64_t id_offset;      // subtracted from every output index
    const float* plo;        // [np][D]
    const float* phi;
    uint64_t* pkey;          // [np]
    const float* Xref;       // SoA [D][n]: coordinates by tag
    const uint32_t* idmap;   // kd-line: original index by tag; vanilla: null (id = tag)
    uint64_t k;
    const uint64_t* forced;  // tags of the first n_forced samples (>= 1)
    uint32_t n_forced;
    uint64_t* out;
    float* trace;
    float* out_pts;          // null, or [k][D]: coordinates of every sample (fused gather)
    uint64_t* slots;
    int* err;
    unsigned long long* counters;  // [2]: boxes tested, distances recomputed
};

template <bool KD>
__device__ __forceinline__ uint64_t make_key(float dist, uint32_t tag) {
    return KD ? key_low_wins(dist, tag) : key_high_wins(dist, tag);
}

// Applies reference point r to the warp's pieces [q0, q1).  INIT sets every
// running distance to min(start, d) with start = FLT_MAX (kd-line,
// KDNode.h:84-103) or +inf (vanilla, lib.cpp:206); otherwise only pieces whose
// box is nearer than their max are recomputed, with the reference's
// "lower only if strictly smaller" rule.  Returns the warp's best key.
template <int D, bool FMA, bool KD, bool INIT>
__device__ __forceinline__ uint64_t apply_ref(const SampleArgs& a, uint32_t q0, uint32_t q1,
                                              const float* r, unsigned long long& touched) {
    const int lane = threadIdx.x & 31;
    const uint64_t n = a.n;
    const float init = KD ? FLT_MAX : INFINITY;
    uint64_t wbest = 0;
    for (uint32_t qb = q0; qb < q1; qb += 32) {
        const uint32_t q = qb + lane;
        const bool have = q < q1;
        uint64_t key = 0;
        bool dirty = have;
        if (!INIT && have) {
            key = a.pkey[q];
            float lo[D], hi[D];
#pragma unroll
            for (int d = 0; d < D; ++d) {
                lo[d] = __ldg(a.plo + (uint64_t)q * D + d);
                hi[d] = __ldg(a.phi + (uint64_t)q * D + d);
            }
            dirty = box_bound<D, FMA>(lo, hi, r) < key_dist(key);
        }
        uint32_t m = __ballot_sync(kFull, dirty);
        while (m) {
            const int l = __ffs(m) - 1;
            m &= m - 1;
            const uint32_t qq = qb + l;
            const uint32_t ps = __ldg(a.pstart + qq), pe = __ldg(a.pstart + qq + 1);
            touched += pe - ps;
            uint64_t pk = 0;
#pragma unroll 2
            for (uint32_t p = ps + lane; p < pe; p += 32) {
                float x[D];
#pragma unroll
                for (int d = 0; d < D; ++d) x[d] = __ldg(a.X + (uint64_t)d * n + p);
                float dv = INIT ? init : a.dis[p];
                const float dd = sqdist<D, FMA>(x, r);
                if (dd < dv) {
                    dv = dd;
                    if (!INIT) a.dis[p] = dv;
                }
                if (INIT) a.dis[p] = dv;
                const uint64_t kk = make_key<KD>(dv, __ldg(a.tag + p));
                pk = kk > pk ? kk : pk;
            }
            pk = warp_max_key(pk);
            if (lane == l) {
                key = pk;
                a.pkey[qq] = pk;
            }
        }
        if (have) wbest = key > wbest ? key : wbest;
    }
    return warp_max_key(wbest);
}

template <int D, bool FMA, bool KD>
__global__ void __launch_bounds__(kSampleThreads, 1) fps_sample(SampleArgs a) {
    __shared__ uint64_t s_wkey[32];
    __shared__ float s_ref[kMaxDim];
    __shared__ int s_abort;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const int G = gridDim.x;
    const uint64_t n = a.n;
    const uint32_t np = a.npieces ? *a.npieces : a.np_fixed;
    const uint32_t total_warps = (uint32_t)G * nwarps;
    const uint32_t pw = (np + total_warps - 1) / total_warps;
    const uint32_t gw = blockIdx.x * nwarps + warp;
    const uint32_t q0 = gw * pw < np ? gw * pw : np;
    const uint32_t q1 = q0 + pw < np ? q0 + pw : np;

    const uint32_t tag0 = (uint32_t)a.forced[0];
    if (tid < D) {
        s_ref[tid] = a.Xref[(uint64_t)tid * n + tag0];
        if (blockIdx.x == 0 && a.out_pts && a.k > 0) a.out_pts[tid] = s_ref[tid];
    }
    if (tid == 0) s_abort = 0;
    if (blockIdx.x == 0 && tid == 0 && a.k > 0) {
        a.out[0] = KD ? tag0 : tag0 - a.id_offset;
        if (a.trace) a.trace[0] = KD ? FLT_MAX : INFINITY;
    }
    __syncthreads();

    uint32_t xround = 0;
    unsigned long long tested = 0, touched = 0;
    for (uint64_t t = 0; t + 1 < a.k; ++t) {
        float r[D];
#pragma unroll
        for (int d = 0; d < D; ++d) r[d] = s_ref[d];
        if (t > 0) tested += q1 - q0;
        const uint64_t wbest = t == 0 ? apply_ref<D, FMA, KD, true>(a, q0, q1, r, touched)
                                      : apply_ref<D, FMA, KD, false>(a, q0, q1, r, touched);
        const bool forced = t + 1 < a.n_forced;
        if (!forced && lane == 0) s_wkey[warp] = wbest;
        __syncthreads();
        if (warp == 0) {
            uint64_t g = 0;
            uint32_t tg;
            bool ok = true;
            if (forced) {
                tg = (uint32_t)a.forced[t + 1];
            } else {
                g = warp_max_key(lane < nwarps ? s_wkey[lane] : 0ull);
                if (G > 1) {
                    float none[1];
                    g = exchange_leader<0>(a.slots, a.slots + (uint64_t)G * leader_words<0>(), G,
                                           xround++, g, none, none, a.err);
                }
                ok = g != 0;
                tg = key_pos<KD>(g);
            }
            if (ok && tg >= n) {
                ok = false;
                if (lane == 0) atomicOr(a.err, kErrBadIndex);
            }
            if (!ok) {
                if (lane == 0) s_abort = 1;
            } else {
                if (lane < D) {
                    const float v = a.Xref[(uint64_t)lane * n + tg];
                    s_ref[lane] = v;
                    if (blockIdx.x == 0 && a.out_pts) a.out_pts[(t + 1) * D + lane] = v;
                }
                if (blockIdx.x == 0 && lane == 0) {
                    a.out[t + 1] = KD ? tg : tg - a.id_offset;
                    if (a.trace) a.trace[t + 1] = forced ? INFINITY : key_dist(g);
                }
            }
        }
        __syncthreads();
        if (s_abort) break;
    }
    if (a.counters && lane == 0) {
        atomicAdd(a.counters, tested);
        atomicAdd(a.counters + 1, touched);
    }
}

// Recomputes one dirty piece [ps, pe) against reference point r: running
// distances lowered with the reference's strict "<" rule (or initialised to
// min(init, d) on the first pass) and the piece's new max key (returned to the
// whole warp; batch_key when BK, else make_key).  The one lane holding the max point (keys are unique) writes its
// coordinates to c_base[d * c_stride]; no shuffles.  xb/disb/tagb may point to
// shared or global memory; xs is the coordinate stride.  Pieces of at most
// kPiece points take an unrolled path that issues every load of the piece
// before the first use, so a piece in global memory costs one round trip.
// Keys of the batched sampler: valid bit | distance bits | 21-bit cloud-local
// position (complemented for kd-line, where the lowest position wins ties) |
// 11-bit piece index.  Positions are unique, so the order is the one of
// make_key; the piece index rides along to locate the winner's coordinates.
constexpr uint32_t kBatchPosBits = 21, kBatchPieceBits = 11;
template <bool KD>
__device__ __forceinline__ uint64_t batch_key(float dist, uint32_t local, uint32_t q) {
    const uint32_t m = (1u << kBatchPosBits) - 1;
    const uint32_t f = KD ? m - local : local;
    return kKeyValid | ((uint64_t)__float_as_uint(dist) << 32) | (f << kBatchPieceBits) | q;
}
template <bool KD>
__device__ __forceinline__ uint32_t batch_key_pos(uint64_t key) {
    const uint32_t m = (1u << kBatchPosBits) - 1;
    const uint32_t f = ((uint32_t)key >> kBatchPieceBits) & m;
    return KD ? m - f : f;
}

template <int D, bool FMA, bool KD, bool BK = true>
__device__ __forceinline__ uint64_t recompute_piece(const float* xb, uint64_t xs, float* disb,
                                                    const uint32_t* tagb, uint32_t ps, uint32_t pe,
                                                    const float* r, bool first, float* c_base,
                                                    uint32_t c_stride, uint32_t tag_base, uint32_t q) {
    const int lane = threadIdx.x & 31;
    const float init = KD ? FLT_MAX : INFINITY;
    uint64_t pk = 0;
    float pc[D];
#pragma unroll
    for (int d = 0; d < D; ++d) pc[d] = 0.0f;
    if (pe - ps <= kPiece) {
        constexpr int PPL = kPiece / 32;
        float x[PPL][D], dv[PPL];
        uint32_t tg[PPL];
#pragma unroll
        for (int j = 0; j < PPL; ++j) {
            const uint32_t p = ps + lane + 32 * j;
            if (p < pe) {
#pragma unroll
                for (int d = 0; d < D; ++d) x[j][d] = xb[(uint64_t)d * xs + p];
                dv[j] = first ? init : disb[p];
                tg[j] = tagb[p];
            }
        }
#pragma unroll
        for (int j = 0; j < PPL; ++j) {
            const uint32_t p = ps + lane + 32 * j;
            if (p < pe) {
                const float dd = sqdist<D, FMA>(x[j], r);
                float v = dv[j];
                if (dd < v) v = dd;
                if (first || dd < dv[j]) disb[p] = v;
                const uint64_t kk = BK ? batch_key<KD>(v, tg[j] - tag_base, q) : make_key<KD>(v, tg[j]);
                if (kk > pk) {
                    pk = kk;
#pragma unroll
                    for (int d = 0; d < D; ++d) pc[d] = x[j][d];
                }
            }
        }
    } else {
        for (uint32_t p = ps + lane; p < pe; p += 32) {
            float x[D];
#pragma unroll
            for (int d = 0; d < D; ++d) x[d] = xb[(uint64_t)d * xs + p];
            const float old = first ? init : disb[p];
            const float dd = sqdist<D, FMA>(x, r);
            float v = old;
            if (dd < v) v = dd;
            if (first || dd < old) disb[p] = v;
            const uint64_t kk = BK ? batch_key<KD>(v, tagb[p] - tag_base, q) : make_key<KD>(v, tagb[p]);
            if (kk > pk) {
                pk = kk;
#pragma unroll
                for (int d = 0; d < D; ++d) pc[d] = x[d];
            }
        }
    }
    const uint64_t wk = warp_max_key(pk);
    if (pk == wk && wk != 0) {
#pragma unroll
        for (int d = 0; d < D; ++d) c_base[(size_t)d * c_stride] = pc[d];
    }
    return wk;
}

// ---- batched sampling: one CTA per cloud -------------------------------------
//
// A persistent grid pulls clouds from a queue (largest first).  Every thread
// owns up to batch_slots(D) pieces of the current cloud and keeps their boxes and
// max keys in registers; piece q belongs to warp q % nwarps, so pieces that
// are neighbours in storage order (and tend to turn dirty together) land in
// different warps.  Clouds of at most `mcap` points keep their points
// (coordinates, running distance, tag) in shared memory, larger ones read them
// from L2/HBM.  One sample:
//   1. every thread tests all its pieces against the reference point r
//      (registers only; an empty slot holds an inverted box that is never
//      dirty), then the warp recomputes its dirty pieces one after the other
//      (recompute_piece: one round trip each; the lane holding a piece's max
//      point writes its coordinates to shared memory);
//   2. lane and warp maxima are recomputed only where a key changed; each
//      warp folds its max into one shared 64-bit atomicMax word (three of
//      them rotate, so clearing the previous one never races); one
//      __syncthreads;
//   3. the max key carries the winner's piece index (batch_key), so every warp
//      reads the next r from that piece's max coordinates: two shared loads.
// kd-line outputs hold tags while sampling and are mapped to original indices
// by the CTA after the cloud's last sample.
//
// CL = true: one thread-block cluster of C CTAs per cloud, for clouds with more
// pieces than one CTA holds.  Piece q belongs to CTA q % C (neighbouring
// pieces, which turn dirty together, land in different CTAs) and to its slot
// q / C there; points stay in L2/HBM.  Step 3 becomes a cluster exchange:
// warp 0 of every CTA sends its CTA's max key and the coordinates behind it
// into every CTA's shared memory with st.async, whose bytes complete the
// receiver's mbarrier (two of them, one per record buffer); every thread waits
// on its own CTA's mbarrier and reduces the C records locally.  No cluster
// barrier and no fence per sample: the same exchange through
// barrier.cluster.arrive.release / wait.acquire took about 15% longer per
// 1M-point cloud.  Cluster rank 0 takes the items from the queue and writes
// the outputs.
// threads per cloud and pieces per thread: 2048 pieces per cloud either way;
// 512 threads x 4 slots for D >= 3 keeps the registers from spilling
constexpr int batch_threads(int D) { return D <= 2 ? 1024 : 512; }
constexpr int batch_slots(int D) { return 2048 / batch_threads(D); }
// batch_key packs a piece index below 2048 and a position below 2^21
static_assert(2048 <= (1u << kBatchPieceBits), "piece index must fit batch_key");
static_assert(2048ull * kPiece <= (1ull << kBatchPosBits), "cloud positions must fit batch_key");

// batch clouds use cloud-local positions in 21 key bits
constexpr uint64_t kBatchMaxCloudPoints = 1ull << kBatchPosBits;
// largest cluster the cluster sampler launches (16 needs the non-portable size)
constexpr int kMaxCluster = 16;

struct BatchArgs {
    const float* X;             // SoA [D][n], storage order (all clouds)
    const uint32_t* tag;
    float* dis;
    uint64_t n;
    const uint32_t* pstart;     // global piece starts
    const float* plo;           // [np][D]
    const float* phi;
    const uint32_t* cloud_piece;  // [C + 1]
    const uint64_t* cloud_off;    // [C + 1]
    const uint64_t* cloud_k;      // [C]
    const uint64_t* cloud_tag0;   // [C] tag of the first sample
    const uint64_t* out_off;      // [C]
    const uint32_t* order;        // [n_items] clouds in processing order
    uint32_t n_items;
    const float* Xref;
    const uint32_t* idmap;      // kd-line: original index by tag; vanilla: null
    uint64_t* out;
    unsigned int* queue;
    unsigned long long* counters;
    uint32_t cap;               // pieces per cloud at most (batch_slots(D) x threads)
    uint32_t mcap;              // points that fit in shared memory
    int* err;
    float* out_pts;             // null, or [sum k][D]: coordinates of every sample (fused gather)
};

inline size_t batch_smem_bytes(int D, uint32_t cap, uint32_t mcap) {
    return (size_t)cap * 8 + (size_t)cap * D * 4 + (size_t)mcap * (4 * D + 8) + 16;
}

template <int D, bool FMA, bool KD, bool CL>
__global__ void __launch_bounds__(batch_threads(D), 1) batch_sample(BatchArgs a) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    __shared__ unsigned long long s_best[3];  // rotating per-sample max key
    __shared__ uint32_t s_item;
    // cluster exchange records, double-buffered by sample parity
    __shared__ uint64_t s_xkey[2][CL ? kMaxCluster : 1];
    __shared__ float s_xc[2][CL ? kMaxCluster : 1][D];
    __shared__ __align__(8) uint64_t s_mbar[2];  // one per record buffer
    const uint32_t cap = a.cap, mcap = a.mcap;
    float* s_x = reinterpret_cast<float*>(s_dyn);                 // [D][mcap]
    float* s_dis = s_x + (size_t)D * mcap;                        // [mcap]
    uint32_t* s_tag = reinterpret_cast<uint32_t*>(s_dis + mcap);  // [mcap]
    uint32_t* s_ps = s_tag + mcap;                                // [cap] my pieces' starts
    uint32_t* s_pe = s_ps + cap;                                  // [cap] and ends
    float* s_mc = reinterpret_cast<float*>(s_pe + cap);           // [D][cap] max coordinates
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const uint32_t T = blockDim.x;
    const uint32_t C = CL ? cluster_size() : 1u, rank = CL ? cluster_rank() : 0u;
    const uint64_t n = a.n;
    unsigned long long tested = 0, touched = 0;
    uint32_t phase = 0;  // parity of each record buffer's next phase (bit px)
    if (CL) {
        if (tid == 0) {
            mbar_init(&s_mbar[0], 1);
            mbar_init(&s_mbar[1], 1);
            mbar_init_fence();
        }
        cluster_sync_all();
    }
    bool gave_up = false;

    for (;;) {
        if (CL) {
            // rank 0 takes the item; the others read it from rank 0's shared
            // memory; the second barrier keeps rank 0 from overwriting it early
            if (rank == 0 && tid == 0) s_item = atomicAdd(a.queue, 1u);
            cluster_sync_all();
            if (rank != 0 && tid == 0) s_item = dsmem_ld_u32(dsmem_addr(&s_item, 0));
            cluster_sync_all();
        } else {
            if (tid == 0) s_item = atomicAdd(a.queue, 1u);
            __syncthreads();
        }
        const uint32_t item = s_item;
        if (item >= a.n_items) break;
        const uint32_t c = a.order[item];
        const uint32_t P0 = a.cloud_piece[c];
        const uint32_t np = a.cloud_piece[c + 1] - P0;
        const uint64_t K = a.cloud_k[c];
        const uint64_t coff = a.cloud_off[c];
        const uint32_t nc = (uint32_t)(a.cloud_off[c + 1] - coff);
        const uint64_t ooff = a.out_off[c];
        const bool resident = nc <= mcap;

        // my pieces: slot j holds local piece j * T + lane * nwarps + warp,
        // which is the cloud's piece local * C + rank
        const uint32_t nmine = np > rank ? (np - rank + C - 1) / C : 0u;
        const uint32_t ns = (nmine + T - 1) / T;  // slots in use by some thread
        float lo[batch_slots(D)][D], hi[batch_slots(D)][D];
        uint64_t key[batch_slots(D)];
        uint32_t myq[batch_slots(D)];
#pragma unroll
        for (int j = 0; j < batch_slots(D); ++j) {
            myq[j] = (uint32_t)j * T + (uint32_t)lane * nwarps + warp;
            key[j] = 0;
            const bool have = myq[j] < nmine;
            const uint64_t q = (uint64_t)P0 + (uint64_t)myq[j] * C + rank;
            // an empty slot gets an inverted box: never nearer than its key 0
#pragma unroll
            for (int d = 0; d < D; ++d) {
                lo[j][d] = have ? a.plo[q * D + d] : INFINITY;
                hi[j][d] = have ? a.phi[q * D + d] : -INFINITY;
            }
        }
        for (uint32_t i = tid; i < nmine; i += T) {
            const uint64_t q = (uint64_t)P0 + (uint64_t)i * C + rank;
            s_ps[i] = a.pstart[q] - (uint32_t)coff;
            s_pe[i] = a.pstart[q + 1] - (uint32_t)coff;
        }
        if (resident) {
            for (uint32_t i = tid; i < nc; i += T) {
#pragma unroll
                for (int d = 0; d < D; ++d) s_x[(size_t)d * mcap + i] = a.X[(uint64_t)d * n + coff + i];
                s_tag[i] = a.tag[coff + i];
            }
        }
        const float* xb = resident ? s_x : a.X + coff;
        const uint64_t xs = resident ? mcap : n;
        float* disb = resident ? s_dis : a.dis + coff;
        const uint32_t* tagb = resident ? s_tag : a.tag + coff;
        const uint32_t tag0 = (uint32_t)a.cloud_tag0[c];
        float r[D];
#pragma unroll
        for (int d = 0; d < D; ++d) r[d] = a.Xref[(uint64_t)d * n + tag0];
        // outputs hold tags while sampling (kd-line tags are mapped at the end)
        if (rank == 0 && tid == 0 && K > 0) a.out[ooff] = KD ? tag0 : tag0 - coff;
        if (rank == 0 && a.out_pts && K > 0) {
#pragma unroll
            for (int d = 0; d < D; ++d)
                if (tid == d) a.out_pts[ooff * D + d] = r[d];
        }
        if (tid < 3) s_best[tid] = 0ull;
        __syncthreads();

        {
            // every held piece is tested once per sample after the second
            uint32_t mine = 0;
#pragma unroll
            for (int j = 0; j < batch_slots(D); ++j) mine += myq[j] < nmine ? 1u : 0u;
            if (K > 2) tested += (unsigned long long)mine * (K - 2);
        }
        int px = 0;   // cluster record buffer of this sample
        int par = 0;  // s_best slot of this sample, rotating over three
        uint64_t lbest = 0, wbest = 0;  // my best key; the warp's (warp-uniform)
        for (uint64_t t = 0; t + 1 < K; ++t) {
            const bool first = t == 0;
            uint32_t dm = 0;  // my dirty slots, one bit each
#pragma unroll
            for (int j = 0; j < batch_slots(D); ++j) {
                if ((uint32_t)j < ns) {  // CTA-uniform: slots no thread uses are not tested
                    const bool dj = first ? myq[j] < nmine
                                          : box_bound<D, FMA>(lo[j], hi[j], r) < key_dist(key[j]);
                    dm |= (uint32_t)dj << j;
                }
            }
            // keys change only in dirty slots: the lane and warp maxima are
            // recomputed only where something was dirty
            if (__any_sync(kFull, dm != 0)) {
#pragma unroll
                for (int j = 0; j < batch_slots(D); ++j) {
                    if ((uint32_t)j >= ns) break;
                    uint32_t m = __ballot_sync(kFull, (dm >> j) & 1u);
                    while (m) {
                        const int l = __ffs(m) - 1;
                        m &= m - 1;
                        const uint32_t q = __shfl_sync(kFull, myq[j], l);
                        const uint32_t ps = s_ps[q], pe = s_pe[q];
                        if (lane == 0) touched += pe - ps;
                        const uint64_t wk =
                            recompute_piece<D, FMA, KD>(xb, xs, disb, tagb, ps, pe, r, first,
                                                        s_mc + q, cap, (uint32_t)coff, q);
                        if (lane == l) key[j] = wk;
                    }
                }
                if (dm) {
                    lbest = 0;
#pragma unroll
                    for (int j = 0; j < batch_slots(D); ++j) lbest = key[j] > lbest ? key[j] : lbest;
                }
                wbest = warp_max_key(lbest);
            }
            // the warp's best goes into the CTA max; the key names the piece
            // whose max coordinates become the next reference point
            if (lane == 0 && wbest) atomicMax(&s_best[par], (unsigned long long)wbest);
            __syncthreads();
            uint64_t g;
            if (CL) {
                if (warp == 0) {
                    // my CTA's record into every CTA of the cluster (a CTA
                    // without pieces sends key 0, which never wins); each
                    // store counts its bytes on the receiver's mbarrier
                    const uint64_t gl = s_best[par];
                    if (lane == 0) mbar_arrive_expect_tx(&s_mbar[px], C * (8u + 4u * D));
                    if ((uint32_t)lane < C) {
                        const uint32_t qw = (uint32_t)gl & ((1u << kBatchPieceBits) - 1);
                        const uint32_t rb = dsmem_addr(&s_mbar[px], lane);
                        st_async_u64(dsmem_addr(&s_xkey[px][rank], lane), gl, rb);
#pragma unroll
                        for (int d = 0; d < D; ++d)
                            st_async_f32(dsmem_addr(&s_xc[px][rank][d], lane),
                                         gl ? s_mc[(size_t)d * cap + qw] : 0.0f, rb);
                    }
                }
                {
                    long long spins = 0;
                    while (!mbar_try_wait_cluster(&s_mbar[px], (phase >> px) & 1u)) {
                        if (++spins > kSpinLimit) {
                            gave_up = true;
                            break;
                        }
                    }
                    phase ^= 1u << px;
                }
                const uint64_t kx = (uint32_t)lane < C ? s_xkey[px][lane] : 0ull;
                g = warp_max_key(kx);
                const int w = __ffs(__ballot_sync(kFull, (uint32_t)lane < C && kx == g)) - 1;
#pragma unroll
                for (int d = 0; d < D; ++d) r[d] = s_xc[px][w][d];
                px ^= 1;
            } else {
                g = s_best[par];
                const uint32_t qw = (uint32_t)g & ((1u << kBatchPieceBits) - 1);
#pragma unroll
                for (int d = 0; d < D; ++d) r[d] = s_mc[(size_t)d * cap + qw];
            }
            if (tid == 0) {
                if (rank == 0) {
                    const uint32_t loc = batch_key_pos<KD>(g);
                    a.out[ooff + t + 1] = KD ? loc + (uint32_t)coff : loc;
                }
                s_best[par == 0 ? 2 : par - 1] = 0ull;  // last sample's slot: everyone has read it
            }
            if (rank == 0 && a.out_pts) {  // the winner's coordinates are the new r
#pragma unroll
                for (int d = 0; d < D; ++d)
                    if (tid == 32 + d) a.out_pts[(ooff + t + 1) * D + d] = r[d];
            }
            par = par == 2 ? 0 : par + 1;
        }
        __syncthreads();  // thread 0's output writes are visible to the CTA
        if (KD && rank == 0) {
            for (uint64_t i = tid; i < K; i += T) a.out[ooff + i] = a.idmap[a.out[ooff + i]] - coff;
        }
    }
    if (CL && gave_up && lane == 0 && a.err) atomicOr(a.err, kErrExchangeTimeout);
    if (a.counters) {
        // warp sums, one atomic per warp
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            tested += __shfl_xor_sync(kFull, tested, o);
            touched += __shfl_xor_sync(kFull, touched, o);
        }
        if (lane == 0) {
            atomicAdd(a.counters, tested);
            atomicAdd(a.counters + 1, touched);
        }
    }
}

#include "lead_sample.cuh"

// ---- one cloud on the whole grid, piece records in registers ----------------
//
// For clouds whose points fit neither one SM nor a cluster (e.g. 16.7M points):
// a persistent cooperative grid of G CTAs.  Piece q of the range belongs to CTA
// q mod G (neighbouring pieces, which turn dirty together, land in different
// CTAs), and there to slot j of thread lane, warp exactly as in batch_sample;
// boxes and keys live in registers, points and running distances in HBM/L2.
// Per sample: tests, recompute of the dirty pieces (recompute_piece, plain
// 32-bit-tag keys: positions may exceed batch_key's 21 bits), each warp offers
// its max key and piece, one __syncthreads, warp 0 takes the CTA's max and that
// piece's max coordinates into exchange_leader (the grid-wide argmax with the
// winner's coordinates), one __syncthreads.  Forced samples and the trace work
// as in fps_sample.  At most G x kRegThreads x kRegSlots pieces.
constexpr int kRegThreads = 512;
constexpr int kRegSlots = 4;
constexpr uint32_t kRegCap = (uint32_t)kRegThreads * kRegSlots;

inline size_t grid_reg_smem_bytes(int D) { return (size_t)kRegCap * (8 + 4 * D); }

template <int D, bool FMA, bool KD>
__global__ void __launch_bounds__(kRegThreads, 1) grid_sample_reg(SampleArgs a) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    constexpr uint32_t cap = kRegCap;
    uint32_t* s_ps = reinterpret_cast<uint32_t*>(s_dyn);  // [cap] my pieces' starts
    uint32_t* s_pe = s_ps + cap;                           // [cap] and ends
    float* s_mc = reinterpret_cast<float*>(s_pe + cap);    // [D][cap] max coordinates
    __shared__ uint64_t s_wkey[32];
    __shared__ uint32_t s_wq[32];
    __shared__ float s_ref[kMaxDim];
    __shared__ int s_abort;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const uint32_t T = blockDim.x, G = gridDim.x, rank = blockIdx.x;
    const uint64_t n = a.n;
    const uint32_t np = a.npieces ? *a.npieces : a.np_fixed;
    const uint32_t nmine = np > rank ? (np - rank + G - 1) / G : 0u;

    float lo[kRegSlots][D], hi[kRegSlots][D];
    uint64_t key[kRegSlots];
    uint32_t myq[kRegSlots];
#pragma unroll
    for (int j = 0; j < kRegSlots; ++j) {
        myq[j] = (uint32_t)j * T + (uint32_t)lane * nwarps + warp;
        key[j] = 0;
        const bool have = myq[j] < nmine;
        const uint64_t q = (uint64_t)myq[j] * G + rank;
        // an empty slot gets an inverted box: never nearer than its key 0
#pragma unroll
        for (int d = 0; d < D; ++d) {
            lo[j][d] = have ? a.plo[q * D + d] : INFINITY;
            hi[j][d] = have ? a.phi[q * D + d] : -INFINITY;
        }
    }
    for (uint32_t i = tid; i < nmine; i += T) {
        const uint64_t q = (uint64_t)i * G + rank;
        s_ps[i] = a.pstart[q];
        s_pe[i] = a.pstart[q + 1];
    }
    const uint32_t tag0 = (uint32_t)a.forced[0];
    if (tid < D) {
        s_ref[tid] = a.Xref[(uint64_t)tid * n + tag0];
        if (blockIdx.x == 0 && a.out_pts && a.k > 0) a.out_pts[tid] = s_ref[tid];
    }
    if (tid == 0) s_abort = 0;
    // outputs hold tags while sampling; kd-line tags are mapped afterwards
    if (rank == 0 && tid == 0 && a.k > 0) {
        a.out[0] = KD ? tag0 : tag0 - a.id_offset;
        if (a.trace) a.trace[0] = KD ? FLT_MAX : INFINITY;
    }
    __syncthreads();

    unsigned long long tested = 0, touched = 0;
    {
        uint32_t mine = 0;
#pragma unroll
        for (int j = 0; j < kRegSlots; ++j) mine += myq[j] < nmine ? 1u : 0u;
        if (a.k > 2) tested += (unsigned long long)mine * (a.k - 2);
    }
    uint32_t xround = 0;
    uint64_t lbest = 0, wbest = 0;  // my best key; the warp's (warp-uniform)
    uint32_t lbq = 0, wq = 0;       // and their pieces
    for (uint64_t t = 0; t + 1 < a.k; ++t) {
        float r[D];
#pragma unroll
        for (int d = 0; d < D; ++d) r[d] = s_ref[d];
        const bool first = t == 0;
        uint32_t dm = 0;
#pragma unroll
        for (int j = 0; j < kRegSlots; ++j) {
            const bool dj = first ? myq[j] < nmine
                                  : box_bound<D, FMA>(lo[j], hi[j], r) < key_dist(key[j]);
            dm |= (uint32_t)dj << j;
        }
        if (__any_sync(kFull, dm != 0)) {
#pragma unroll
            for (int j = 0; j < kRegSlots; ++j) {
                uint32_t m = __ballot_sync(kFull, (dm >> j) & 1u);
                while (m) {
                    const int l = __ffs(m) - 1;
                    m &= m - 1;
                    const uint32_t q = __shfl_sync(kFull, myq[j], l);
                    const uint32_t ps = s_ps[q], pe = s_pe[q];
                    if (lane == 0) touched += pe - ps;
                    const uint64_t wk = recompute_piece<D, FMA, KD, false>(
                        a.X, n, a.dis, a.tag, ps, pe, r, first, s_mc + q, cap, 0u, q);
                    if (lane == l) key[j] = wk;
                }
            }
            if (dm) {
                lbest = 0;
#pragma unroll
                for (int j = 0; j < kRegSlots; ++j) {
                    if (key[j] > lbest) {
                        lbest = key[j];
                        lbq = myq[j];
                    }
                }
            }
            wbest = warp_max_key(lbest);
            const int ow = __ffs(__ballot_sync(kFull, wbest != 0 && lbest == wbest)) - 1;
            wq = __shfl_sync(kFull, lbq, ow < 0 ? 0 : ow);
        }
        const bool forced = t + 1 < a.n_forced;
        if (lane == 0) {
            s_wkey[warp] = wbest;
            s_wq[warp] = wq;
        }
        __syncthreads();
        if (warp == 0) {
            uint64_t g = 0;
            uint32_t tg;
            bool ok = true;
            float wc[D];
            if (forced) {
                tg = (uint32_t)a.forced[t + 1];
#pragma unroll
                for (int d = 0; d < D; ++d) wc[d] = a.Xref[(uint64_t)d * n + tg];
            } else {
                const uint64_t kw = lane < nwarps ? s_wkey[lane] : 0ull;
                g = warp_max_key(kw);
                const int w = __ffs(__ballot_sync(kFull, lane < nwarps && kw == g)) - 1;
                const uint32_t qw = s_wq[w];
                float mc[D];
#pragma unroll
                for (int d = 0; d < D; ++d) mc[d] = g != 0 ? s_mc[(size_t)d * cap + qw] : 0.0f;
                if (G > 1) {
                    g = exchange_leader<D>(a.slots, a.slots + (uint64_t)G * leader_words<D>(), G,
                                           xround++, g, mc, wc, a.err);
                } else {
#pragma unroll
                    for (int d = 0; d < D; ++d) wc[d] = mc[d];
                }
                ok = g != 0;
                tg = key_pos<KD>(g);
            }
            if (ok && tg >= n) {
                ok = false;
                if (lane == 0) atomicOr(a.err, kErrBadIndex);
            }
            if (!ok) {
                if (lane == 0) s_abort = 1;
            } else {
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    if (lane == d) {  // static indices keep wc in registers
                        s_ref[d] = wc[d];
                        if (blockIdx.x == 0 && a.out_pts) a.out_pts[(t + 1) * D + d] = wc[d];
                    }
                }
                if (rank == 0 && lane == 0) {
                    a.out[t + 1] = KD ? tg : tg - a.id_offset;
                    if (a.trace) a.trace[t + 1] = forced ? INFINITY : key_dist(g);
                }
            }
        }
        __syncthreads();
        if (s_abort) break;
    }
    if (a.counters && lane == 0) {
        atomicAdd(a.counters, tested);
        atomicAdd(a.counters + 1, touched);
    }
}

// first piece of every cloud: lower bound of cloud_off[c] in pstart[0, np]
__global__ void cloud_piece_ranges(const uint32_t* pstart, const uint32_t* npieces,
                                   const uint64_t* cloud_off, uint32_t n_clouds, uint32_t* out);

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// A set of clouds stored back to back: cloud c holds positions
// [off[c], off[c+1]) of the row-major point buffer.
struct CloudSet {
    const float* d_points;
    std::vector<uint64_t> off;     // C + 1
    std::vector<uint64_t> height;  // kd-line tree height per cloud
    bool kd = true;
    bool tie_last = false;         // bucket_fps_kdtree: reversed tags (ties to the last position)
};

// Device arrays produced by build_clouds.
struct Built {
    float* X = nullptr;
    uint32_t* tag = nullptr;
    float* Xref = nullptr;
    uint32_t* idsnap = nullptr;
    uint8_t* flag = nullptr;
    uint4* refine = nullptr;
    uint32_t* refine_cnt = nullptr;
    uint32_t* pstart = nullptr;
    uint32_t* d_np = nullptr;
    float* plo = nullptr;
    float* phi = nullptr;
    uint64_t np_cap = 0;
    int* err = nullptr;
};

// Exact kd-line levels (kd), snapshot, refinement, pieces and their boxes for
// every cloud of the set.  build_only stops after the snapshot.
template <int D>
int build_clouds(const CloudSet& cs, cudaStream_t stream, Scratch& sc, Built& out,
                 bool build_only) {
    const size_t C = cs.off.size() - 1;
    const uint64_t n = cs.off[C];
    int rc;
    BuildArgs b{};
    b.n = n;
    b.coarse = build_only ? 0 : 1;
    b.reverse = cs.tie_last ? 1 : 0;
    b.n_clouds = (uint32_t)C;
    if (cs.tie_last) {
        uint64_t* d_off;
        if ((rc = sc.alloc(&d_off, C + 1))) return rc;
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_off, cs.off.data(), (C + 1) * sizeof(uint64_t),
                                        cudaMemcpyHostToDevice, stream));
        b.cloud_off = d_off;
    }
    if ((rc = sc.alloc(&b.X, n * D))) return rc;
    if ((rc = sc.alloc(&b.tag, n))) return rc;
    if ((rc = sc.alloc(&b.sel, n))) return rc;
    if ((rc = sc.alloc(&b.flag, n))) return rc;
    if ((rc = sc.alloc(&b.err, 1))) return rc;
    const uint64_t node_cap = n / 2 + C + 1;
    uint4 *list_a, *list_b;
    if ((rc = sc.alloc(&list_a, node_cap))) return rc;
    if ((rc = sc.alloc(&list_b, node_cap))) return rc;
    const uint64_t rcap = n / (kPiece + 1) + 2;
    if ((rc = sc.alloc(&b.refine, rcap))) return rc;

    // per-cloud exact depth and host-side bounds on node counts
    uint64_t levels = 0, max_n = 1;
    std::vector<uint64_t> lv(C);
    std::vector<uint4> h_roots(C);
    for (size_t c = 0; c < C; ++c) {
        const uint64_t nc = cs.off[c + 1] - cs.off[c];
        lv[c] = cs.kd && nc > 0 ? std::min<uint64_t>(cs.height[c], nc - 1) : 0;
        levels = std::max(levels, lv[c]);
        max_n = std::max(max_n, nc);
        h_roots[c] = make_uint4((uint32_t)cs.off[c], (uint32_t)cs.off[c + 1], 0u,
                                (uint32_t)std::min<uint64_t>(cs.height[c], 0xffffffffull));
    }
    const int refine_levels = 10 + (int)std::ceil(std::log2((double)max_n / kPiece + 1.0));
    const uint64_t ncounters = 1 + (levels + 1) + (refine_levels + 1);
    uint32_t* counters;
    if ((rc = sc.alloc(&counters, ncounters))) return rc;
    uint4* d_roots;
    if ((rc = sc.alloc(&d_roots, C))) return rc;
    FPSGPU_CUDA_TRY(cudaMemsetAsync(counters, 0, ncounters * sizeof(uint32_t), stream));
    FPSGPU_CUDA_TRY(cudaMemsetAsync(b.err, 0, sizeof(int), stream));
    FPSGPU_CUDA_TRY(cudaMemsetAsync(b.flag, 0, n, stream));
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_roots, h_roots.data(), C * sizeof(uint4),
                                    cudaMemcpyHostToDevice, stream));
    b.refine_cnt = counters;
    uint32_t* level_cnt = counters + 1;

    const unsigned elem_blocks = (unsigned)std::min<uint64_t>((n + 255) / 256 + 1, 8192);
    b.cur = list_a;
    b.next = list_b;
    b.cnt_cur = level_cnt;
    stats_count_launch();
    build_prepare<D><<<elem_blocks, 256, 0, stream>>>(cs.d_points, b, d_roots, (uint32_t)C,
                                                      cs.kd ? 1 : 0);
    FPSGPU_CUDA_TRY(cudaGetLastError());

    // exact phase: one launch per level; grid = bound on that level's nodes
    for (uint64_t j = 0; j < levels; ++j) {
        uint64_t bound = 0;
        for (size_t c = 0; c < C; ++c) {
            if (j >= lv[c]) continue;
            const uint64_t nc = cs.off[c + 1] - cs.off[c];
            bound += std::min<uint64_t>(j < 40 ? (1ull << j) : nc, nc / 2 + 1);
        }
        bound = std::min<uint64_t>(bound, node_cap);
        if (bound > 65536) {  // read the exact count instead of launching empty CTAs
            uint32_t h_cnt = 0;
            FPSGPU_CUDA_TRY(cudaMemcpyAsync(&h_cnt, level_cnt + j, sizeof(uint32_t),
                                            cudaMemcpyDeviceToHost, stream));
            FPSGPU_CUDA_TRY(cudaStreamSynchronize(stream));
            bound = h_cnt;
        }
        if (bound == 0) break;
        b.cnt_cur = level_cnt + j;
        b.cnt_next = level_cnt + j + 1;
        stats_count_launch();
        split_kernel<D, true, kBuildThreads><<<(unsigned)bound, kBuildThreads, 0, stream>>>(b, 0);
        FPSGPU_CUDA_TRY(cudaGetLastError());
        std::swap(b.cur, b.next);
    }

    if ((rc = sc.alloc(&out.Xref, n * D))) return rc;
    if (cs.kd && (rc = sc.alloc(&out.idsnap, n))) return rc;
    stats_count_launch();
    build_snapshot<D><<<elem_blocks, 256, 0, stream>>>(b, out.Xref, out.idsnap);
    FPSGPU_CUDA_TRY(cudaGetLastError());
    out.X = b.X;
    out.tag = b.tag;
    out.flag = b.flag;
    out.refine = b.refine;
    out.refine_cnt = b.refine_cnt;
    out.err = b.err;
    if (build_only) return FPSGPU_OK;

    // refinement phase
    int sms = 0;
    {
        int dev = 0;
        FPSGPU_CUDA_TRY(cudaGetDevice(&dev));
        FPSGPU_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    }
    uint32_t* rcnt = level_cnt + levels + 1;
    b.cnt_cur = rcnt;
    stats_count_launch();
    build_seed_refine<<<64, 256, 0, stream>>>(b);
    FPSGPU_CUDA_TRY(cudaGetLastError());
    uint64_t rbound = 0, nb_bound = 0;
    for (size_t c = 0; c < C; ++c) {
        const uint64_t nc = cs.off[c + 1] - cs.off[c];
        const uint64_t leaves = lv[c] < 40 ? std::min<uint64_t>(1ull << lv[c], nc) : nc;
        nb_bound += leaves;
        rbound += std::min<uint64_t>(leaves, nc / (kPiece + 1) + 1);
    }
    rbound = std::min<uint64_t>(rbound, rcap);
    for (int j = 0; j < refine_levels && rbound > 0; ++j) {
        b.cnt_cur = rcnt + j;
        b.cnt_next = rcnt + j + 1;
        const int last = j + 1 == refine_levels;
        stats_count_launch();
        // few nodes (the top levels of a large vanilla cloud): wide CTAs, so
        // that a node of millions of points streams through one SM fast
        if (rbound <= (uint64_t)2 * std::max(1, sms))
            split_kernel<D, false, kBuildThreads><<<(unsigned)rbound, kBuildThreads, 0, stream>>>(b, last);
        else
            split_kernel<D, false, kRefineThreads><<<(unsigned)rbound, kRefineThreads, 0, stream>>>(b, last);
        FPSGPU_CUDA_TRY(cudaGetLastError());
        std::swap(b.cur, b.next);
        rbound = std::min<uint64_t>(2 * rbound, rcap);
    }

    // pieces: exact leaves of <= kPiece points, two children per refined node
    // on every refinement level, everything left on the last one
    const uint64_t per_level = n / (kPiece + 1) + 1;
    out.np_cap = std::min<uint64_t>(n, nb_bound + (2ull * refine_levels + 1) * per_level + C + 1);
    if ((rc = sc.alloc(&out.pstart, out.np_cap + 1))) return rc;
    if ((rc = sc.alloc(&out.d_np, 1))) return rc;
    if ((rc = compact_flags(b.flag, n, out.pstart, out.d_np, sc, stream))) return rc;
    if ((rc = sc.alloc(&out.plo, out.np_cap * D))) return rc;
    if ((rc = sc.alloc(&out.phi, out.np_cap * D))) return rc;
    {
        const unsigned blocks = (unsigned)std::min<uint64_t>((out.np_cap * 32 + 255) / 256, 4096);
        stats_count_launch();
        piece_bbox<D><<<blocks, 256, 0, stream>>>(b.X, n, out.pstart, out.d_np, out.plo, out.phi);
        FPSGPU_CUDA_TRY(cudaGetLastError());
    }
    return FPSGPU_OK;
}

inline int check_device_error(const int* d_err, cudaStream_t stream) {
    int h_err = 0;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    FPSGPU_CUDA_TRY(cudaStreamSynchronize(stream));
    if (h_err & kErrNonFiniteSplit)
        return set_error(FPSGPU_ERR_NONFINITE,
                         "kd-line build met a NaN coordinate in a split dimension");
    if (h_err)
        return set_error(FPSGPU_ERR_DEVICE, "FPS sampler gave up (device error word 0x%x)", h_err);
    return FPSGPU_OK;
}

// ---- grid sampling with shared-memory residency ------------------------------
//
// For one large cloud: every CTA of a cooperative grid owns a contiguous run of
// pieces and keeps their points (coordinates, running distance, tag) and piece
// records (max key, box, coordinates of the max) in shared memory for the
// whole run.  One iteration = shared-memory work, one __syncthreads, and one
// exchange_leader round (the grid-wide argmax, which also delivers the winner's
// coordinates: the next reference point).
constexpr int kSmemThreads = 512;

struct GridSmemArgs {
    const float* X;
    const uint32_t* tag;
    uint64_t n;
    const uint32_t* pstart;     // global piece starts
    const float* plo;
    const float* phi;
    const uint32_t* cta_piece;  // [G + 1] global piece index where each CTA starts
    uint32_t maxq, maxm;        // shared-memory layout: pieces / points per CTA
    const float* Xref;
    const uint32_t* idmap;
    uint64_t k;
    const uint64_t* forced;
    uint32_t n_forced;
    uint64_t id_offset;
    uint64_t* out;
    float* trace;
    float* out_pts;  // null, or [k][D] (fused gather)
    uint64_t* slots;
    int* err;
    unsigned long long* counters;
};

inline size_t grid_smem_bytes(int D, uint32_t maxq, uint32_t maxm) {
    return (size_t)maxq * (8 + 12 * D) + (size_t)maxm * (4 * D + 8) + (size_t)(maxq + 1) * 4 + 16;
}

template <int D, bool FMA, bool KD>
__global__ void __launch_bounds__(kSmemThreads, 1) grid_sample_smem(GridSmemArgs a) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    const uint32_t MQ = a.maxq, MM = a.maxm;
    uint64_t* s_key = reinterpret_cast<uint64_t*>(s_dyn);
    float* s_lo = reinterpret_cast<float*>(s_key + MQ);
    float* s_hi = s_lo + (size_t)D * MQ;
    float* s_mc = s_hi + (size_t)D * MQ;
    float* s_x = s_mc + (size_t)D * MQ;
    float* s_dis = s_x + (size_t)D * MM;
    uint32_t* s_tag = reinterpret_cast<uint32_t*>(s_dis + MM);
    uint32_t* s_ps = s_tag + MM;
    __shared__ uint64_t s_wkey[32];
    __shared__ uint32_t s_wq[32];
    __shared__ float s_ref[kMaxDim];
    __shared__ int s_abort;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const int G = gridDim.x;
    const uint64_t n = a.n;
    const uint32_t P0 = a.cta_piece[blockIdx.x];
    const uint32_t nq = a.cta_piece[blockIdx.x + 1] - P0;
    const uint32_t S0 = a.pstart[P0];
    const uint32_t m = a.pstart[P0 + nq] - S0;
    const float init = KD ? FLT_MAX : INFINITY;

    for (uint32_t i = tid; i < m; i += blockDim.x) {
#pragma unroll
        for (int d = 0; d < D; ++d) s_x[(size_t)d * MM + i] = a.X[(uint64_t)d * n + S0 + i];
        s_tag[i] = a.tag[S0 + i];
    }
    for (uint32_t q = tid; q <= nq; q += blockDim.x) {
        s_ps[q] = a.pstart[P0 + q] - S0;
        if (q < nq) {
#pragma unroll
            for (int d = 0; d < D; ++d) {
                s_lo[(size_t)d * MQ + q] = a.plo[(uint64_t)(P0 + q) * D + d];
                s_hi[(size_t)d * MQ + q] = a.phi[(uint64_t)(P0 + q) * D + d];
            }
        }
    }
    const uint32_t tag0 = (uint32_t)a.forced[0];
    if (tid < D) {
        s_ref[tid] = a.Xref[(uint64_t)tid * n + tag0];
        if (blockIdx.x == 0 && a.out_pts && a.k > 0) a.out_pts[tid] = s_ref[tid];
    }
    if (tid == 0) s_abort = 0;
    // outputs hold tags while sampling; kd-line tags are mapped afterwards
    if (blockIdx.x == 0 && tid == 0 && a.k > 0) {
        a.out[0] = KD ? tag0 : tag0 - a.id_offset;
        if (a.trace) a.trace[0] = init;
    }
    __syncthreads();
    const uint32_t stride = 32u * nwarps;  // piece q belongs to warp q % nwarps

    uint32_t xround = 0;
    unsigned long long tested = 0, touched = 0;
    for (uint64_t t = 0; t + 1 < a.k; ++t) {
        float r[D];
#pragma unroll
        for (int d = 0; d < D; ++d) r[d] = s_ref[d];
        uint64_t best = 0;
        uint32_t bestq = 0;
        for (uint32_t qb = 0; qb < nq; qb += stride) {
            const uint32_t q = qb + lane * nwarps + warp;
            const bool have = q < nq;
            const uint32_t hb = __ballot_sync(kFull, have);
            if (t > 0 && lane == 0) tested += __popc(hb);
            uint64_t key = have && t > 0 ? s_key[q] : 0ull;
            bool dirty = have;
            if (have && t > 0) {
                float lo[D], hi[D];
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    lo[d] = s_lo[(size_t)d * MQ + q];
                    hi[d] = s_hi[(size_t)d * MQ + q];
                }
                dirty = box_bound<D, FMA>(lo, hi, r) < key_dist(key);
            }
            uint32_t msk = __ballot_sync(kFull, dirty);
            while (msk) {
                const int l = __ffs(msk) - 1;
                msk &= msk - 1;
                const uint32_t qq = qb + l * nwarps + warp;
                const uint32_t ps = s_ps[qq], pe = s_ps[qq + 1];
                touched += pe - ps;
                uint64_t pk = 0;
                float pc[D];
#pragma unroll
                for (int d = 0; d < D; ++d) pc[d] = 0.0f;
                for (uint32_t i = ps + lane; i < pe; i += 32) {
                    float x[D];
#pragma unroll
                    for (int d = 0; d < D; ++d) x[d] = s_x[(size_t)d * MM + i];
                    float dv = t == 0 ? init : s_dis[i];
                    const float dd = sqdist<D, FMA>(x, r);
                    if (dd < dv) dv = dd;
                    s_dis[i] = dv;
                    const uint64_t kk = make_key<KD>(dv, s_tag[i]);
                    if (kk > pk) {
                        pk = kk;
#pragma unroll
                        for (int d = 0; d < D; ++d) pc[d] = x[d];
                    }
                }
                const uint64_t wk = warp_max_key(pk);
                const int owner = __ffs(__ballot_sync(kFull, pk == wk)) - 1;
#pragma unroll
                for (int d = 0; d < D; ++d) pc[d] = __shfl_sync(kFull, pc[d], owner);
                if (lane == l) {
                    key = wk;
                    s_key[qq] = wk;
#pragma unroll
                    for (int d = 0; d < D; ++d) s_mc[(size_t)d * MQ + qq] = pc[d];
                }
            }
            if (have && key > best) {
                best = key;
                bestq = q;
            }
        }
        const uint64_t wb = warp_max_key(best);
        const int wl = __ffs(__ballot_sync(kFull, best == wb)) - 1;
        bestq = __shfl_sync(kFull, bestq, wl);
        const bool forced = t + 1 < a.n_forced;
        if (lane == 0) {
            s_wkey[warp] = wb;
            s_wq[warp] = bestq;
        }
        __syncthreads();
        if (warp == 0) {
            uint64_t g = 0;
            uint32_t tg = 0;
            bool ok = true;
            float wc[D];
            if (forced) {
                tg = (uint32_t)a.forced[t + 1];
#pragma unroll
                for (int d = 0; d < D; ++d) wc[d] = a.Xref[(uint64_t)d * n + tg];
            } else {
                const uint64_t kw = lane < nwarps ? s_wkey[lane] : 0ull;
                g = warp_max_key(kw);
                const int w = __ffs(__ballot_sync(kFull, lane < nwarps && kw == g)) - 1;
                const uint32_t qwin = s_wq[w];
                float mc[D];
#pragma unroll
                for (int d = 0; d < D; ++d) mc[d] = nq > 0 ? s_mc[(size_t)d * MQ + qwin] : 0.0f;
                if (G > 1) {
                    g = exchange_leader<D>(a.slots, a.slots + (uint64_t)G * leader_words<D>(), G,
                                           xround++, g, mc, wc, a.err);
                } else {
#pragma unroll
                    for (int d = 0; d < D; ++d) wc[d] = mc[d];
                }
                ok = g != 0;
                tg = key_pos<KD>(g);
                if (ok && tg >= n) {
                    ok = false;
                    if (lane == 0) atomicOr(a.err, kErrBadIndex);
                }
            }
            if (!ok) {
                if (lane == 0) s_abort = 1;
            } else {
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    if (lane == d) {  // static indices keep wc in registers
                        s_ref[d] = wc[d];
                        if (blockIdx.x == 0 && a.out_pts) a.out_pts[(t + 1) * D + d] = wc[d];
                    }
                }
                if (blockIdx.x == 0 && lane == 0) {
                    a.out[t + 1] = KD ? tg : tg - a.id_offset;
                    if (a.trace) a.trace[t + 1] = forced ? INFINITY : key_dist(g);
                }
            }
        }
        __syncthreads();
        if (s_abort) break;
    }
    if (a.counters && lane == 0) {
        atomicAdd(a.counters, tested);
        atomicAdd(a.counters + 1, touched);
    }
}

// out[i] = idmap[out[i]] - id_offset: kd-line tags to original indices
__global__ void map_tags(uint64_t* out, uint64_t k, const uint32_t* idmap, uint64_t id_offset);

constexpr int kNoFit = -1;

// The shared-memory-resident grid sampler, if the range fits on chip;
// returns kNoFit (nothing launched) otherwise.
template <int D, bool FMA>
int sample_grid_smem(const Built& bt, uint64_t n, bool kd, uint32_t piece0, uint32_t np,
                     uint64_t k, const uint64_t* h_forced, uint32_t n_forced, uint64_t id_offset,
                     uint64_t* d_out, float* d_trace, float* d_out_pts, cudaStream_t stream, int sms,
                     Scratch& sc) {
    int rc;
    if (np == ~0u) {
        uint32_t h_np = 0;
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(&h_np, bt.d_np, 4, cudaMemcpyDeviceToHost, stream));
        FPSGPU_CUDA_TRY(cudaStreamSynchronize(stream));
        np = h_np;
    }
    if (np == 0) return kNoFit;
    std::vector<uint32_t> ps(np + 1);
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(ps.data(), bt.pstart + piece0, (np + 1) * 4,
                                    cudaMemcpyDeviceToHost, stream));
    FPSGPU_CUDA_TRY(cudaStreamSynchronize(stream));
    const uint64_t pts = ps[np] - ps[0];
    int dev = 0, smem_max = 0;
    FPSGPU_CUDA_TRY(cudaGetDevice(&dev));
    FPSGPU_CUDA_TRY(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa{};
    FPSGPU_CUDA_TRY(cudaFuncGetAttributes(&fa, (const void*)grid_sample_smem<D, FMA, true>));
    const size_t budget = (size_t)smem_max - fa.sharedSizeBytes - 256;
    uint64_t G = std::min<uint64_t>({(uint64_t)sms, (uint64_t)kMaxGridCoords,
                                     std::max<uint64_t>(1, pts / 2048)});
    // cut the piece range at the pieces nearest to equal point shares
    std::vector<uint32_t> cut(G + 1);
    cut[0] = 0;
    cut[G] = np;
    for (uint64_t c = 1; c < G; ++c) {
        const uint64_t target = ps[0] + pts * c / G;
        cut[c] = (uint32_t)(std::lower_bound(ps.begin(), ps.end() - 1, (uint32_t)target) - ps.begin());
        cut[c] = std::max(cut[c], cut[c - 1]);
    }
    uint32_t maxq = 1, maxm = 1;
    for (uint64_t c = 0; c < G; ++c) {
        maxq = std::max(maxq, cut[c + 1] - cut[c]);
        maxm = std::max(maxm, ps[cut[c + 1]] - ps[cut[c]]);
    }
    const size_t smem = grid_smem_bytes(D, maxq, maxm);
    if (smem > budget) return kNoFit;
    for (auto& x : cut) x += piece0;

    uint32_t* d_cut;
    uint64_t* slots;
    uint64_t* d_forced;
    unsigned long long* cnt;
    const uint64_t nslots = (G + 1) * leader_words<D>();
    if ((rc = sc.alloc(&d_cut, G + 1))) return rc;
    if ((rc = sc.alloc(&slots, nslots))) return rc;
    if ((rc = sc.alloc(&d_forced, n_forced))) return rc;
    if ((rc = sc.alloc(&cnt, 2))) return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_cut, cut.data(), (G + 1) * 4, cudaMemcpyHostToDevice, stream));
    FPSGPU_CUDA_TRY(cudaMemsetAsync(slots, 0, nslots * sizeof(uint64_t), stream));
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_forced, h_forced, n_forced * sizeof(uint64_t),
                                    cudaMemcpyHostToDevice, stream));
    FPSGPU_CUDA_TRY(cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned long long), stream));
    GridSmemArgs a{};
    a.X = bt.X;
    a.tag = bt.tag;
    a.n = n;
    a.pstart = bt.pstart;
    a.plo = bt.plo;
    a.phi = bt.phi;
    a.cta_piece = d_cut;
    a.maxq = maxq;
    a.maxm = maxm;
    a.Xref = bt.Xref;
    a.idmap = bt.idsnap;
    a.k = k;
    a.forced = d_forced;
    a.n_forced = n_forced;
    a.id_offset = id_offset;
    a.out = d_out;
    a.trace = d_trace;
    a.out_pts = d_out_pts;
    a.slots = slots;
    a.err = bt.err;
    a.counters = cnt;
    const void* kern = kd ? (const void*)grid_sample_smem<D, FMA, true>
                          : (const void*)grid_sample_smem<D, FMA, false>;
    if (int arc = allow_max_smem((const void*)kern)) return arc;
    void* args[] = {&a};
    SamplerTimer timer;
    timer.begin(stream);
    if ((rc = launch_persistent(kern, (int)G, kSmemThreads, args, smem, stream, G > 1))) return rc;
    timer.end(stream);
    if (kd) {
        stats_count_launch();
        map_tags<<<(unsigned)std::min<uint64_t>((k + 255) / 256, 4096), 256, 0, stream>>>(
            d_out, k, bt.idsnap, id_offset);
        FPSGPU_CUDA_TRY(cudaGetLastError());
    }
    unsigned long long h_cnt[2] = {0, 0};
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(h_cnt, cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, stream));
    if ((rc = check_device_error(bt.err, stream))) return rc;
    const uint64_t cn[2] = {h_cnt[0], h_cnt[1]};
    timer.finish(k, cn);
    return FPSGPU_OK;
}

// Multi-CTA sampler over pieces [piece0, piece0 + np) (np == ~0u: the device
// count of the whole build).
template <int D, bool FMA>
int sample_grid(const Built& bt, uint64_t n, bool kd, uint32_t piece0, uint32_t np,
                uint64_t points_in_range, uint64_t k, const uint64_t* h_forced, uint32_t n_forced,
                uint64_t id_offset, uint64_t* d_out, float* d_trace, float* d_out_pts,
                cudaStream_t stream, int sms, Scratch& sc) {
    int rc = sample_grid_smem<D, FMA>(bt, n, kd, piece0, np, k, h_forced, n_forced, id_offset,
                                      d_out, d_trace, d_out_pts, stream, sms, sc);
    if (rc != kNoFit) return rc;
    uint32_t h_np = np;
    if (np == ~0u) {
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(&h_np, bt.d_np, 4, cudaMemcpyDeviceToHost, stream));
        FPSGPU_CUDA_TRY(cudaStreamSynchronize(stream));
    }
    // registers hold the piece records when the grid has room for them
    const uint64_t g_reg = std::min<uint64_t>((uint64_t)sms, (uint64_t)kMaxGridCoords);
    const bool reg = h_np <= g_reg * kRegCap;
    float* dis;
    uint64_t* pkey = nullptr;
    const uint64_t nkeys = np == ~0u ? bt.np_cap : np;
    if ((rc = sc.alloc(&dis, n))) return rc;
    if (!reg && (rc = sc.alloc(&pkey, nkeys))) return rc;
    // grid: about two pieces per warp (pieces hold ~kPiece/2..kPiece points)
    uint64_t G = (points_in_range / (kPiece / 2) + 63) / 64;
    G = std::max<uint64_t>(1, std::min<uint64_t>({G, (uint64_t)sms, (uint64_t)kMaxGridCoords}));
    if (reg) G = std::max<uint64_t>(1, std::min<uint64_t>(g_reg, (h_np + 127) / 128));
    uint64_t* slots;
    const uint64_t nslots = (G + 1) * (reg ? leader_words<D>() : leader_words<0>());
    if ((rc = sc.alloc(&slots, nslots))) return rc;
    FPSGPU_CUDA_TRY(cudaMemsetAsync(slots, 0, nslots * sizeof(uint64_t), stream));
    uint64_t* d_forced;
    if ((rc = sc.alloc(&d_forced, n_forced))) return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_forced, h_forced, n_forced * sizeof(uint64_t),
                                    cudaMemcpyHostToDevice, stream));
    unsigned long long* cnt;
    if ((rc = sc.alloc(&cnt, 2))) return rc;
    FPSGPU_CUDA_TRY(cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned long long), stream));

    SampleArgs s{};
    s.X = bt.X;
    s.tag = bt.tag;
    s.dis = dis;
    s.n = n;
    s.pstart = bt.pstart + piece0;
    s.npieces = np == ~0u ? bt.d_np : nullptr;
    s.np_fixed = np == ~0u ? 0 : np;
    s.id_offset = id_offset;
    s.plo = bt.plo + (uint64_t)piece0 * D;
    s.phi = bt.phi + (uint64_t)piece0 * D;
    s.pkey = pkey;
    s.Xref = bt.Xref;
    s.idmap = bt.idsnap;
    s.k = k;
    s.forced = d_forced;
    s.n_forced = n_forced;
    s.out = d_out;
    s.trace = d_trace;
    s.out_pts = d_out_pts;
    s.slots = slots;
    s.err = bt.err;
    s.counters = cnt;
    void* args[] = {&s};
    SamplerTimer timer;
    timer.begin(stream);
    if (reg) {
        const void* kern = kd ? (const void*)grid_sample_reg<D, FMA, true>
                              : (const void*)grid_sample_reg<D, FMA, false>;
        const size_t smem = grid_reg_smem_bytes(D);
        if (int arc = allow_max_smem((const void*)kern)) return arc;
        if ((rc = launch_persistent(kern, (int)G, kRegThreads, args, smem, stream, G > 1))) return rc;
    } else {
        const void* kern = kd ? (const void*)fps_sample<D, FMA, true> : (const void*)fps_sample<D, FMA, false>;
        if ((rc = launch_persistent(kern, (int)G, kSampleThreads, args, 0, stream, G > 1))) return rc;
    }
    timer.end(stream);
    if (kd) {
        stats_count_launch();
        map_tags<<<(unsigned)std::min<uint64_t>((k + 255) / 256, 4096), 256, 0, stream>>>(
            d_out, k, bt.idsnap, id_offset);
        FPSGPU_CUDA_TRY(cudaGetLastError());
    }
    unsigned long long h_cnt[2] = {0, 0};
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(h_cnt, cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, stream));
    if ((rc = check_device_error(bt.err, stream))) return rc;
    const uint64_t cn[2] = {h_cnt[0], h_cnt[1]};
    timer.finish(k, cn);
    return FPSGPU_OK;
}

struct EngineCall {
    const float* d_points;  // row-major [n][D]
    uint64_t n;
    uint64_t k;
    bool kd;                // kd-line (true) or vanilla
    uint64_t height;        // kd-line
    const uint64_t* h_forced;  // kd-line: {start_idx}; vanilla: start list
    uint32_t n_forced;
    uint64_t* d_out;
    float* d_trace;
    cudaStream_t stream;
    int sms;
    bool tie_last = false;  // bucket_fps_kdtree
    float* d_out_pts = nullptr;  // null, or [k][D]: the sampled points (fused gather)
    // build-only mode (kd-line): host outputs
    uint64_t* h_perm;
    uint64_t* h_bucket_start;
    size_t* h_n_buckets;
};

template <int D, bool FMA>
int run_engine(const EngineCall& c) {
    Scratch sc(c.stream);
    CloudSet cs;
    cs.d_points = c.d_points;
    cs.off = {0, c.n};
    cs.height = {c.height};
    cs.kd = c.kd;
    cs.tie_last = c.tie_last;
    Built bt;
    int rc;
    if ((rc = build_clouds<D>(cs, c.stream, sc, bt, c.h_perm != nullptr))) return rc;
    const uint64_t n = c.n;

    if (c.h_perm) {  // build-only: reference permutation and buckets
        std::vector<uint32_t> h_id(n);
        uint32_t h_nref = 0;
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(h_id.data(), bt.idsnap, n * sizeof(uint32_t),
                                        cudaMemcpyDeviceToHost, c.stream));
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(&h_nref, bt.refine_cnt, sizeof(uint32_t),
                                        cudaMemcpyDeviceToHost, c.stream));
        if ((rc = check_device_error(bt.err, c.stream))) return rc;
        // buckets = exact leaves: the ones queued for refinement plus the small
        // ones already flagged as pieces
        std::vector<uint4> h_ref(h_nref);
        std::vector<uint8_t> h_flag(n);
        if (h_nref)
            FPSGPU_CUDA_TRY(cudaMemcpy(h_ref.data(), bt.refine, h_nref * sizeof(uint4),
                                       cudaMemcpyDeviceToHost));
        FPSGPU_CUDA_TRY(cudaMemcpy(h_flag.data(), bt.flag, n, cudaMemcpyDeviceToHost));
        for (const uint4& r : h_ref) h_flag[r.x] = 1;
        h_flag[0] = 1;
        size_t nb = 0;
        for (uint64_t p = 0; p < n; ++p)
            if (h_flag[p]) c.h_bucket_start[nb++] = p;
        for (uint64_t i = 0; i < n; ++i) c.h_perm[i] = h_id[i];
        *c.h_n_buckets = nb;
        return FPSGPU_OK;
    }
    // kd-tree: the start's tag is its reversed position
    const uint64_t f0 = c.tie_last ? n - 1 - c.h_forced[0] : c.h_forced[0];
    return sample_grid<D, FMA>(bt, n, c.kd, 0, ~0u, n, c.k, c.tie_last ? &f0 : c.h_forced,
                               c.n_forced, 0, c.d_out, c.d_trace, c.d_out_pts, c.stream, c.sms, sc);
}

// Many clouds in one go: build all of them together, then one CTA per cloud
// (clouds whose piece records do not fit in shared memory use sample_grid).
struct BatchCall {
    const float* d_points;            // all clouds, row-major, back to back
    std::vector<uint64_t> off;        // C + 1
    std::vector<uint64_t> k;          // C
    std::vector<uint64_t> start;      // C (local start index / position)
    std::vector<uint64_t> height;     // C
    bool kd;
    uint64_t* d_out;                  // sum(k), cloud c at out_off[c]
    cudaStream_t stream;
    int sms;
    bool tie_last = false;            // bucket_fps_kdtree
    float* d_out_pts = nullptr;       // null, or [sum k][D], cloud c at row out_off[c]
    // smallest cluster for clouds that need one (0: the latency default,
    // cluster_size_for_batch(), or 16 when every cloud of the call fits the
    // GPU at once with that size; 1: just as many CTAs as the pieces need,
    // which leaves more SMs to other work, e.g. in the server)
    int min_cluster = 0;
    // self-test of lead_sample's bounded wait (fpsgpu_selftest_lead_timeout):
    // the leader publishes nothing, the workers give up after 4096 polls
    bool lead_selftest = false;
};

// The one-CTA clouds of a batched call (D <= 3) on lead_sample: float4 point
// records and low key words for the whole call, then one persistent launch
// over the clouds in `small` (beside the clusters, which hold `cl` CTAs each,
// when both kinds run).
template <int D, bool FMA>
int launch_lead_sampler(const BatchCall& bc, const Built& bt, const std::vector<uint32_t>& small,
                        const std::vector<uint32_t>& clustered, const uint32_t* d_order, unsigned int* d_queue,
                        const uint64_t* d_coff, const uint32_t* d_cpiece, const uint64_t* d_k,
                        const uint64_t* d_tag0, const uint64_t* d_ooff, unsigned long long* cnt, bool both,
                        int cl, int maxc, int smem_optin, uint32_t max_pieces, Scratch& sc) {
    const size_t C = bc.off.size() - 1;
    const uint64_t n = bc.off[C];
    int rc;
    float4* P4;
    uint32_t* LW;
    if ((rc = sc.alloc(&P4, n))) return rc;
    if ((rc = sc.alloc(&LW, n))) return rc;
    {
        const int blocks = std::max(1, std::min(bc.sms * 8, (int)((n / 64 + 7) / 8)));
        stats_count_launch();
        if (bc.kd)
            lead_prepare<D, true><<<blocks, 256, 0, bc.stream>>>(bt.X, bt.tag, n, bt.pstart, d_cpiece, d_coff,
                                                                (uint32_t)C, P4, LW);
        else
            lead_prepare<D, false><<<blocks, 256, 0, bc.stream>>>(bt.X, bt.tag, n, bt.pstart, d_cpiece, d_coff,
                                                                 (uint32_t)C, P4, LW);
        FPSGPU_CUDA_TRY(cudaGetLastError());
    }
    // the 77-entry table when the launch holds a cloud of kLeadHotWideMin
    // pieces or more (D = 3 only; FPSGPU_LEAD_HOT=5|7 forces one)
    const int hpw_forced = lead_hot_per_warp();
    const bool wide = D == 3 && (hpw_forced ? hpw_forced == kLeadHotPerWarp : max_pieces >= kLeadHotWideMin);
    const void* kern = nullptr;
    if constexpr (D == 3) {
        if (wide)
            kern = bc.kd ? (const void*)lead_sample<D, FMA, true, kLeadHotPerWarp>
                         : (const void*)lead_sample<D, FMA, false, kLeadHotPerWarp>;
    }
    if (!kern)
        kern = bc.kd ? (const void*)lead_sample<D, FMA, true, kLeadHotSmall>
                     : (const void*)lead_sample<D, FMA, false, kLeadHotSmall>;
    size_t static_smem = 0;
    {
        cudaFuncAttributes fa{};
        FPSGPU_CUDA_TRY(cudaFuncGetAttributes(&fa, kern));
        static_smem = fa.sharedSizeBytes;
    }
    const size_t smem = lead_smem_bytes((uint32_t)kLeadWorkers * (wide ? kLeadHotPerWarp : kLeadHotSmall));
    if (static_smem + smem + 256 > (size_t)smem_optin)
        return set_error(FPSGPU_ERR_CUDA, "lead_sample needs %zu bytes of shared memory, the device offers %d",
                         static_smem + smem, smem_optin);
    LeadArgs la{};
    la.P4 = P4;
    la.LW = LW;
    la.pstart = bt.pstart;
    la.plo = bt.plo;
    la.phi = bt.phi;
    la.cloud_piece = d_cpiece;
    la.cloud_off = d_coff;
    la.cloud_k = d_k;
    la.cloud_tag0 = d_tag0;
    la.out_off = d_ooff;
    la.order = d_order;
    la.n_items = (uint32_t)small.size();
    la.n = n;
    la.Xref = bt.Xref;
    la.idmap = bc.kd ? bt.idsnap : nullptr;
    la.out = bc.d_out;
    la.queue = d_queue;
    la.counters = cnt;
    la.err = bt.err;
    la.out_pts = bc.d_out_pts;
    la.spin_limit = bc.lead_selftest ? 4096 : kSpinLimit;
    la.mute = bc.lead_selftest ? 1 : 0;
    if (int arc = allow_max_smem(kern)) return arc;
    int per_sm = 0;
    FPSGPU_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kLeadThreads, smem));
    int slots = std::max(1, per_sm) * bc.sms;
    if (both) slots = std::max(1, slots - cl * std::min<int>((int)clustered.size(), maxc));
    const int G = (int)std::min<uint64_t>(small.size(), (uint64_t)slots);
    void* args[] = {&la};
    return launch_persistent(kern, G, kLeadThreads, args, smem, bc.stream, false);
}

template <int D, bool FMA>
int run_batch(const BatchCall& bc) {
    Scratch sc(bc.stream);
    const size_t C = bc.off.size() - 1;
    const uint64_t n = bc.off[C];
    int rc;
    CloudSet cs;
    cs.d_points = bc.d_points;
    cs.off = bc.off;
    cs.height = bc.height;
    cs.kd = bc.kd;
    cs.tie_last = bc.tie_last;
    Built bt;
    if ((rc = build_clouds<D>(cs, bc.stream, sc, bt, false))) return rc;

    uint64_t* d_coff;
    uint32_t* d_cpiece;
    if ((rc = sc.alloc(&d_coff, C + 1))) return rc;
    if ((rc = sc.alloc(&d_cpiece, C + 1))) return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_coff, bc.off.data(), (C + 1) * sizeof(uint64_t),
                                    cudaMemcpyHostToDevice, bc.stream));
    stats_count_launch();
    cloud_piece_ranges<<<(unsigned)((C + 1 + 255) / 256), 256, 0, bc.stream>>>(
        bt.pstart, bt.d_np, d_coff, (uint32_t)C, d_cpiece);
    FPSGPU_CUDA_TRY(cudaGetLastError());
    std::vector<uint32_t> h_cpiece(C + 1);
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(h_cpiece.data(), d_cpiece, (C + 1) * sizeof(uint32_t),
                                    cudaMemcpyDeviceToHost, bc.stream));
    if ((rc = check_device_error(bt.err, bc.stream))) return rc;

    int dev = 0, smem_optin = 0;
    FPSGPU_CUDA_TRY(cudaGetDevice(&dev));
    FPSGPU_CUDA_TRY(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    size_t static_smem = 0;
    {
        cudaFuncAttributes fa{};
        FPSGPU_CUDA_TRY(cudaFuncGetAttributes(&fa, (const void*)batch_sample<D, FMA, true, false>));
        static_smem = fa.sharedSizeBytes;
    }
    const size_t avail = (size_t)smem_optin - static_smem - 256;
    const uint32_t cap_max = (uint32_t)batch_slots(D) * batch_threads(D);
    // one-CTA clouds of D <= 3 take the leader/worker sampler (lead_sample)
    const bool use_lead = D <= 3 && lead_sampler_enabled();
    const uint32_t one_cap = use_lead ? kLeadCap : cap_max;
    if (bc.lead_selftest && !use_lead)
        return set_error(FPSGPU_ERR_ARG, "the leader/worker sampler is off (FPSGPU_ONECTA_SAMPLER)");
    const int want_cluster = bc.min_cluster > 0 ? bc.min_cluster : cluster_size_for_batch();
    const uint32_t promote = cluster_min_pieces();
    std::vector<uint64_t> out_off(C), tag0(C);
    std::vector<uint32_t> small, clustered, big;
    uint64_t acc = 0;
    uint32_t cap = 1, need_cl = 1;
    for (size_t c = 0; c < C; ++c) {
        out_off[c] = acc;
        acc += bc.k[c];
        // kd-line: the start is a position of the cloud's permuted order, i.e.
        // a tag (reversed within the cloud for the kd-tree); vanilla: the
        // start is an original index, also a tag
        tag0[c] = bc.off[c] + (bc.tie_last ? bc.off[c + 1] - bc.off[c] - 1 - bc.start[c] : bc.start[c]);
        const uint32_t np = h_cpiece[c + 1] - h_cpiece[c];
        const uint64_t nc = bc.off[c + 1] - bc.off[c];
        if (bc.k[c] == 0) continue;
        const bool to_cluster = cluster_size_for_batch() > 1 && np <= (uint64_t)kMaxCluster * cap_max &&
                                nc <= kBatchMaxCloudPoints;
        if (np <= one_cap && !(to_cluster && promote > 0 && np >= promote)) {
            small.push_back((uint32_t)c);
            cap = std::max(cap, np);
        } else if (to_cluster) {
            clustered.push_back((uint32_t)c);
            need_cl = std::max<uint32_t>(need_cl, (np + cap_max - 1) / cap_max);
        } else {
            big.push_back((uint32_t)c);
        }
    }
    // largest first
    auto by_work = [&](uint32_t x, uint32_t y) {
        return bc.k[x] * (bc.off[x + 1] - bc.off[x]) > bc.k[y] * (bc.off[y + 1] - bc.off[y]);
    };
    std::sort(small.begin(), small.end(), by_work);
    std::sort(clustered.begin(), clustered.end(), by_work);
    int cl = want_cluster;
    while ((uint32_t)cl < need_cl) cl *= 2;
    const void* cl_kern = bc.kd ? (const void*)batch_sample<D, FMA, true, true>
                                : (const void*)batch_sample<D, FMA, false, true>;
    const size_t cl_smem = batch_smem_bytes(D, cap_max, 0);
    int maxc = 0;
    if (!clustered.empty() && bc.min_cluster == 0 && !cluster_size_fixed() && cl < kMaxCluster &&
        small.size() + clustered.size() * kMaxCluster <= (size_t)bc.sms) {
        int m16 = 0;
        if ((rc = cluster_capacity(cl_kern, kMaxCluster, batch_threads(D), cl_smem, &m16))) return rc;
        if ((size_t)m16 >= clustered.size()) cl = kMaxCluster;
    }
    if (!clustered.empty()) {
        if ((rc = cluster_capacity(cl_kern, cl, batch_threads(D), cl_smem, &maxc))) return rc;
        if (maxc < 1) {  // no such cluster on this device: the other samplers take them
            for (uint32_t c : clustered) {
                const uint32_t np = h_cpiece[c + 1] - h_cpiece[c];
                if (np <= one_cap) {
                    small.push_back(c);
                    cap = std::max(cap, np);
                } else {
                    big.push_back(c);
                }
            }
            clustered.clear();
            std::sort(small.begin(), small.end(), by_work);
        }
    }

    if (!small.empty() || !clustered.empty()) {
        uint64_t *d_k, *d_tag0, *d_ooff;
        uint32_t* d_order;
        unsigned int* d_queue;
        unsigned long long* cnt;
        float* dis;
        if ((rc = sc.alloc(&d_k, C))) return rc;
        if ((rc = sc.alloc(&d_tag0, C))) return rc;
        if ((rc = sc.alloc(&d_ooff, C))) return rc;
        if ((rc = sc.alloc(&d_order, small.size() + clustered.size()))) return rc;
        if ((rc = sc.alloc(&d_queue, 2))) return rc;
        if ((rc = sc.alloc(&cnt, 2))) return rc;
        if ((rc = sc.alloc(&dis, n))) return rc;
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_k, bc.k.data(), C * 8, cudaMemcpyHostToDevice, bc.stream));
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_tag0, tag0.data(), C * 8, cudaMemcpyHostToDevice, bc.stream));
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_ooff, out_off.data(), C * 8, cudaMemcpyHostToDevice, bc.stream));
        std::vector<uint32_t> order(small);
        order.insert(order.end(), clustered.begin(), clustered.end());
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_order, order.data(), order.size() * 4,
                                        cudaMemcpyHostToDevice, bc.stream));
        FPSGPU_CUDA_TRY(cudaMemsetAsync(d_queue, 0, 2 * sizeof(unsigned int), bc.stream));
        FPSGPU_CUDA_TRY(cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned long long), bc.stream));
        BatchArgs a{};
        a.X = bt.X;
        a.tag = bt.tag;
        a.dis = dis;
        a.n = n;
        a.pstart = bt.pstart;
        a.plo = bt.plo;
        a.phi = bt.phi;
        a.cloud_piece = d_cpiece;
        a.cloud_off = d_coff;
        a.cloud_k = d_k;
        a.cloud_tag0 = d_tag0;
        a.out_off = d_ooff;
        a.Xref = bt.Xref;
        a.idmap = bt.idsnap;
        a.out = bc.d_out;
        a.counters = cnt;
        a.err = bt.err;
        a.out_pts = bc.d_out_pts;
        SamplerTimer timer;
        timer.begin(bc.stream);
        // both kinds at once: the clusters run on a side stream, concurrently
        // with the one-CTA sampler, and are launched first so they find SMs
        SideStream side;
        const bool both = !small.empty() && !clustered.empty();
        if (both && (rc = side.fork(bc.stream))) return rc;
        if (!clustered.empty()) {
            // one cluster per cloud, cl CTAs of at most cap_max pieces each
            BatchArgs b = a;
            b.order = d_order + small.size();
            b.n_items = (uint32_t)clustered.size();
            b.queue = d_queue + 1;
            b.cap = cap_max;
            b.mcap = 0;
            void* args[] = {&b};
            if ((rc = launch_clustered(cl_kern, (int)clustered.size(), cl, batch_threads(D), args,
                                       cl_smem, both ? side.s : bc.stream, bc.sms)))
                return rc;
        }
        if (!small.empty() && use_lead) {
            if constexpr (D <= 3) {
                if ((rc = launch_lead_sampler<D, FMA>(bc, bt, small, clustered, d_order, d_queue, d_coff,
                                                      d_cpiece, d_k, d_tag0, d_ooff, cnt, both, cl, maxc,
                                                      smem_optin, cap, sc)))
                    return rc;
            }
        } else if (!small.empty()) {
            a.order = d_order;
            a.n_items = (uint32_t)small.size();
            a.queue = d_queue;
            a.cap = cap;
            // what the piece starts and max coordinates leave of shared memory
            // holds small clouds' points
            uint64_t max_nc = 0;
            for (uint32_t c : small) max_nc = std::max<uint64_t>(max_nc, bc.off[c + 1] - bc.off[c]);
            const size_t left = avail - batch_smem_bytes(D, cap, 0);
            a.mcap = (uint32_t)std::min<uint64_t>(left / (4 * D + 8), max_nc);
            const size_t smem = batch_smem_bytes(D, cap, a.mcap);
            const void* kern = bc.kd ? (const void*)batch_sample<D, FMA, true, false>
                                     : (const void*)batch_sample<D, FMA, false, false>;
            if (int arc = allow_max_smem((const void*)kern)) return arc;
            int per_sm = 0;
            FPSGPU_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, batch_threads(D), smem));
            int slots = std::max(1, per_sm) * bc.sms;
            if (both) slots = std::max(1, slots - cl * std::min<int>((int)clustered.size(), maxc));
            const int G = (int)std::min<uint64_t>(small.size(), (uint64_t)slots);
            void* args[] = {&a};
            if ((rc = launch_persistent(kern, G, batch_threads(D), args, smem, bc.stream, false)))
                return rc;
        }
        if (both && (rc = side.join(bc.stream))) return rc;
        timer.end(bc.stream);
        unsigned long long h_cnt[2] = {0, 0};
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(h_cnt, cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, bc.stream));
        FPSGPU_CUDA_TRY(cudaStreamSynchronize(bc.stream));
        uint64_t ks = 0;
        for (uint32_t c : small) ks += bc.k[c];
        for (uint32_t c : clustered) ks += bc.k[c];
        const uint64_t cn[2] = {h_cnt[0], h_cnt[1]};
        timer.finish(ks, cn);
    }
    for (uint32_t c : big) {
        const uint64_t f = tag0[c];
        const uint32_t np = h_cpiece[c + 1] - h_cpiece[c];
        if ((rc = sample_grid<D, FMA>(bt, n, bc.kd, h_cpiece[c], np, bc.off[c + 1] - bc.off[c],
                                      bc.k[c], &f, 1, bc.off[c], bc.d_out + out_off[c], nullptr,
                                      bc.d_out_pts ? bc.d_out_pts + out_off[c] * D : nullptr,
                                      bc.stream, bc.sms, sc)))
            return rc;
    }
    return check_device_error(bt.err, bc.stream);
}

template <bool FMA>
int run_engine_dispatch(int dim, const EngineCall& c) {
    switch (dim) {
        case 1: return run_engine<1, FMA>(c);
        case 2: return run_engine<2, FMA>(c);
        case 3: return run_engine<3, FMA>(c);
        case 4: return run_engine<4, FMA>(c);
        case 5: return run_engine<5, FMA>(c);
        case 6: return run_engine<6, FMA>(c);
        case 7: return run_engine<7, FMA>(c);
        case 8: return run_engine<8, FMA>(c);
        default: return set_error(FPSGPU_ERR_DIM, "dim must be in [1, 8], got %d", dim);
    }
}

template <bool FMA>
int run_batch_dispatch(int dim, const BatchCall& c) {
    switch (dim) {
        case 1: return run_batch<1, FMA>(c);
        case 2: return run_batch<2, FMA>(c);
        case 3: return run_batch<3, FMA>(c);
        case 4: return run_batch<4, FMA>(c);
        case 5: return run_batch<5, FMA>(c);
        case 6: return run_batch<6, FMA>(c);
        case 7: return run_batch<7, FMA>(c);
        case 8: return run_batch<8, FMA>(c);
        default: return set_error(FPSGPU_ERR_DIM, "dim must be in [1, 8], got %d", dim);
    }
}

}  // namespace fpsgpu
