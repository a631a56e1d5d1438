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
//          [s+L, e); ranks from block-wide ballot scans; split point L clamped
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
// Sampling (fps_sample): a persistent cooperative grid; every warp owns a run
// of pieces and keeps each piece's max key (running distance, tag).  For a new
// reference point r, a piece whose box_bound(r) >= its max cannot change (see
// box_bound) and is skipped; other pieces recompute their points.  The grid
// argmax runs through exchange_max; the winner's coordinates come from Xref by
// tag.
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
};

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

// row-major points -> SoA, tag = original index, flags cleared, root node.
template <int D>
__global__ void build_prepare(const float* __restrict__ pts, BuildArgs a, uint32_t height,
                              int exact) {
    const uint64_t n = a.n;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n;
         p += (uint64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int d = 0; d < D; ++d) a.X[(uint64_t)d * n + p] = pts[p * D + d];
        a.tag[p] = (uint32_t)p;
        a.flag[p] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const uint4 root = make_uint4(0u, (uint32_t)n, 0u, height);
        const bool root_leaf = !exact || height == 0 || n == 1;
        if (root_leaf) {
            *a.cnt_cur = 0;
            if (n > kPiece) {
                a.refine[0] = root;
                *a.refine_cnt = 1;
            } else {
                *a.refine_cnt = 0;  // one piece; position 0 always starts one
            }
        } else {
            a.cur[0] = root;
            *a.cnt_cur = 1;
            *a.refine_cnt = 0;
        }
    }
}

// Splits the nodes of one level, one CTA per node.
// EXACT: the reference's kd-line rule (bit-exact permutation).
// !EXACT: refinement (any rule; mean of the widest dimension, or halving).
template <int D, bool EXACT>
__global__ void __launch_bounds__(EXACT ? kBuildThreads : kRefineThreads)
    split_kernel(BuildArgs a, int force_leaf) {
    constexpr int RING = EXACT ? kSumChunk : 4;
    __shared__ __align__(16) float s_ring[2][RING];
    __shared__ float s_lo[32][D], s_hi[32][D];
    __shared__ uint32_t s_w[2 * 32];
    __shared__ float s_fw[32];
    __shared__ float s_split;
    __shared__ int s_dim;
    __shared__ int s_degenerate;

    const uint32_t cnt = *a.cnt_cur;
    if (blockIdx.x >= cnt) return;
    const uint4 nd = a.cur[blockIdx.x];
    const uint32_t s = nd.x, e = nd.y, cntn = e - s;
    const uint64_t n = a.n;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const uint32_t T = blockDim.x;

    if (!EXACT && force_leaf) {  // last refinement level: everything left is a piece
        if (tid == 0) a.flag[s] = 1;
        return;
    }

    // 1. bounding box and split dimension
    {
        float lo[D], hi[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            lo[d] = FLT_MAX;
            hi[d] = -FLT_MAX;
        }
        for (uint32_t p = s + tid; p < e; p += T) {
#pragma unroll
            for (int d = 0; d < D; ++d) {
                float v = a.X[(uint64_t)d * n + p];
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
        float part = 0.0f;
        for (uint32_t p = s + tid; p < e; p += T) part += col[p];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(kFull, part, o);
        if (lane == 0) s_fw[warp] = part;
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
        for (uint32_t p = s + tid; p < e; p += T) {
            float v = col[p];
            mine += v < split ? 1u : 0u;
            if (EXACT) bad |= isnan(v);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(kFull, mine, o);
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
    //    k-th element < split counted from the right end of [s+L, e)
    if (!halve) {
        {
            uint32_t running = 0;
            const uint32_t rlen = e - (s + L);
            int par = 0;
            for (uint32_t c = 0; c < rlen; c += T) {
                const uint32_t i = c + tid;
                bool f = false;
                uint32_t p = 0;
                if (i < rlen) {
                    p = e - 1 - i;
                    f = col[p] < split;
                }
                uint32_t total;
                uint32_t r = block_rank(f, s_w, par, total);
                par ^= 1;
                if (f) a.sel[s + running + r] = p;
                running += total;
            }
        }
        __syncthreads();
        {
            uint32_t running = 0;
            int par = 0;
            for (uint32_t c = 0; c < L; c += T) {
                const uint32_t i = c + tid;
                bool f = false;
                uint32_t p = 0;
                if (i < L) {
                    p = s + i;
                    f = !(col[p] < split);
                }
                uint32_t total;
                uint32_t r = block_rank(f, s_w, par, total);
                par ^= 1;
                if (f) {
                    const uint32_t q = a.sel[s + running + r];
                    if (q >= s + L && q < e) {
#pragma unroll
                        for (int d = 0; d < D; ++d) {
                            float* cd = a.X + (uint64_t)d * n;
                            float u = cd[p], v = cd[q];
                            cd[p] = v;
                            cd[q] = u;
                        }
                        uint32_t ip = a.tag[p], iq = a.tag[q];
                        a.tag[p] = iq;
                        a.tag[q] = ip;
                    } else {  // unreachable: both sides count the same predicate
                        atomicOr(a.err, kErrBadIndex);
                    }
                }
                running += total;
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
        for (int ch = 0; ch < 2; ++ch) {
            const uint32_t len = ce[ch] - cs[ch];
            bool leaf;
            if (EXACT) leaf = nd.z + 1 >= nd.w || len == 1;  // KDLineTree.h:37-39
            else leaf = len <= kPiece;
            const uint4 child = make_uint4(cs[ch], ce[ch], nd.z + 1, nd.w);
            if (!leaf) {
                a.next[atomicAdd(a.cnt_next, 1u)] = child;
            } else if (EXACT && len > kPiece) {
                a.refine[atomicAdd(a.refine_cnt, 1u)] = child;
            } else {
                a.flag[cs[ch]] = 1;
            }
        }
    }
}

// After the exact phase: Xref/idsnap by permuted position, tag = position.
template <int D>
__global__ void build_snapshot(BuildArgs a, float* __restrict__ Xref, uint32_t* __restrict__ idsnap) {
    const uint64_t n = a.n;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n;
         p += (uint64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int d = 0; d < D; ++d) Xref[(uint64_t)d * n + p] = a.X[(uint64_t)d * n + p];
        if (idsnap) {
            idsnap[p] = a.tag[p];
            a.tag[p] = (uint32_t)p;
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
    const uint32_t* npieces;
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
    const uint32_t np = *a.npieces;
    const uint32_t total_warps = (uint32_t)G * nwarps;
    const uint32_t pw = (np + total_warps - 1) / total_warps;
    const uint32_t gw = blockIdx.x * nwarps + warp;
    const uint32_t q0 = gw * pw < np ? gw * pw : np;
    const uint32_t q1 = q0 + pw < np ? q0 + pw : np;

    const uint32_t tag0 = (uint32_t)a.forced[0];
    if (tid < D) s_ref[tid] = a.Xref[(uint64_t)tid * n + tag0];
    if (tid == 0) s_abort = 0;
    if (blockIdx.x == 0 && tid == 0 && a.k > 0) {
        a.out[0] = KD ? a.idmap[tag0] : tag0;
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
                if (G > 1) g = exchange_max(a.slots, G, xround++, g, a.err);
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
                if (lane < D) s_ref[lane] = a.Xref[(uint64_t)lane * n + tg];
                if (blockIdx.x == 0 && lane == 0) {
                    a.out[t + 1] = KD ? a.idmap[tg] : tg;
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

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
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
    // build-only mode (kd-line): host outputs
    uint64_t* h_perm;
    uint64_t* h_bucket_start;
    size_t* h_n_buckets;
};

template <int D, bool FMA>
int run_engine(const EngineCall& c) {
    Scratch sc(c.stream);
    const uint64_t n = c.n;
    int rc;
    BuildArgs b{};
    b.n = n;
    if ((rc = sc.alloc(&b.X, n * D))) return rc;
    if ((rc = sc.alloc(&b.tag, n))) return rc;
    if ((rc = sc.alloc(&b.sel, n))) return rc;
    if ((rc = sc.alloc(&b.flag, n))) return rc;
    if ((rc = sc.alloc(&b.err, 1))) return rc;
    const uint64_t node_cap = n / 2 + 1;
    uint4 *list_a, *list_b;
    if ((rc = sc.alloc(&list_a, node_cap))) return rc;
    if ((rc = sc.alloc(&list_b, node_cap))) return rc;
    if ((rc = sc.alloc(&b.refine, n / (kPiece + 1) + 2))) return rc;
    // counters: [0] refine count, then one per level (exact + refinement)
    const uint64_t levels = c.kd ? (c.height < n - 1 ? c.height : n - 1) : 0;
    const int refine_levels = 10 + (int)std::ceil(std::log2((double)n / kPiece + 1.0));
    const uint64_t ncounters = 1 + levels + 1 + refine_levels + 1;
    uint32_t* counters;
    if ((rc = sc.alloc(&counters, ncounters))) return rc;
    FPSGPU_CUDA_TRY(cudaMemsetAsync(counters, 0, ncounters * sizeof(uint32_t), c.stream));
    FPSGPU_CUDA_TRY(cudaMemsetAsync(b.err, 0, sizeof(int), c.stream));
    b.refine_cnt = counters;
    uint32_t* level_cnt = counters + 1;

    const unsigned elem_blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, 8192);
    b.cur = list_a;
    b.next = list_b;
    b.cnt_cur = level_cnt;
    stats_count_launch();
    build_prepare<D><<<elem_blocks, 256, 0, c.stream>>>(c.d_points, b, (uint32_t)c.height,
                                                         c.kd ? 1 : 0);
    FPSGPU_CUDA_TRY(cudaGetLastError());

    // exact phase (kd-line): one launch per level, grid = a bound on the nodes
    uint64_t bound = levels == 0 ? 0 : 1;
    uint32_t* cnt = level_cnt;
    for (uint64_t j = 0; j < levels && bound > 0; ++j) {
        b.cnt_cur = cnt;
        b.cnt_next = cnt + 1;
        stats_count_launch();
        split_kernel<D, true><<<(unsigned)bound, kBuildThreads, 0, c.stream>>>(b, 0);
        FPSGPU_CUDA_TRY(cudaGetLastError());
        std::swap(b.cur, b.next);
        ++cnt;
        bound = std::min<uint64_t>(2 * bound, node_cap);
        if (bound > 65536) {  // read the exact count instead of launching empty CTAs
            uint32_t h_cnt = 0;
            FPSGPU_CUDA_TRY(cudaMemcpyAsync(&h_cnt, cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                            c.stream));
            FPSGPU_CUDA_TRY(cudaStreamSynchronize(c.stream));
            bound = h_cnt;
        }
    }
    // In the exact phase nodes that reach the last level without becoming
    // leaves cannot exist: depth == height makes every child a leaf.

    float* Xref;
    uint32_t* idsnap = nullptr;
    if ((rc = sc.alloc(&Xref, n * D))) return rc;
    if (c.kd && (rc = sc.alloc(&idsnap, n))) return rc;
    stats_count_launch();
    build_snapshot<D><<<elem_blocks, 256, 0, c.stream>>>(b, Xref, idsnap);
    FPSGPU_CUDA_TRY(cudaGetLastError());

    if (c.h_perm) {  // build-only: reference permutation and buckets
        std::vector<uint32_t> h_id(n);
        int h_err = 0;
        uint32_t h_nref = 0;
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(h_id.data(), idsnap ? idsnap : b.tag, n * sizeof(uint32_t),
                                        cudaMemcpyDeviceToHost, c.stream));
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(&h_err, b.err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(&h_nref, b.refine_cnt, sizeof(uint32_t),
                                        cudaMemcpyDeviceToHost, c.stream));
        FPSGPU_CUDA_TRY(cudaStreamSynchronize(c.stream));
        if (h_err & kErrNonFiniteSplit)
            return set_error(FPSGPU_ERR_NONFINITE,
                             "kd-line build met a NaN coordinate in a split dimension");
        // buckets = exact leaves: the ones queued for refinement plus the small
        // ones already flagged as pieces
        std::vector<uint4> h_ref(h_nref);
        std::vector<uint8_t> h_flag(n);
        if (h_nref)
            FPSGPU_CUDA_TRY(cudaMemcpy(h_ref.data(), b.refine, h_nref * sizeof(uint4),
                                       cudaMemcpyDeviceToHost));
        FPSGPU_CUDA_TRY(cudaMemcpy(h_flag.data(), b.flag, n, cudaMemcpyDeviceToHost));
        for (const uint4& r : h_ref) h_flag[r.x] = 1;
        h_flag[0] = 1;
        size_t nb = 0;
        for (uint64_t p = 0; p < n; ++p)
            if (h_flag[p]) c.h_bucket_start[nb++] = p;
        for (uint64_t i = 0; i < n; ++i) c.h_perm[i] = h_id[i];
        *c.h_n_buckets = nb;
        return FPSGPU_OK;
    }

    // refinement phase
    {
        uint32_t* rcnt = level_cnt + levels + 1;
        b.cnt_cur = rcnt;
        stats_count_launch();
        build_seed_refine<<<64, 256, 0, c.stream>>>(b);  // refine list -> b.cur, *rcnt
        FPSGPU_CUDA_TRY(cudaGetLastError());
        uint64_t rbound = c.kd ? std::min<uint64_t>(levels < 40 ? (1ull << levels) : n,
                                                    n / (kPiece + 1) + 1)
                               : 1;
        const uint64_t rcap = n / (kPiece + 1) + 2;
        for (int j = 0; j < refine_levels && rbound > 0; ++j) {
            b.cnt_cur = rcnt + j;
            b.cnt_next = rcnt + j + 1;
            const int last = j + 1 == refine_levels;
            stats_count_launch();
            split_kernel<D, false><<<(unsigned)rbound, kRefineThreads, 0, c.stream>>>(b, last);
            FPSGPU_CUDA_TRY(cudaGetLastError());
            std::swap(b.cur, b.next);
            rbound = std::min<uint64_t>(2 * rbound, rcap);
        }
    }

    // pieces
    // pieces: exact leaves of <= kPiece points (<= 2^levels), two children per
    // refined node on every refinement level, everything left on the last one
    const uint64_t per_level = n / (kPiece + 1) + 1;
    const uint64_t np_cap = std::min<uint64_t>(
        n, (levels < 40 ? (1ull << levels) : n) + (2ull * refine_levels + 1) * per_level + 1);
    uint32_t* pstart;
    uint32_t* d_np;
    if ((rc = sc.alloc(&pstart, np_cap + 1))) return rc;
    if ((rc = sc.alloc(&d_np, 1))) return rc;
    if ((rc = compact_flags(b.flag, n, pstart, d_np, sc, c.stream))) return rc;
    float *plo, *phi, *dis;
    uint64_t* pkey;
    if ((rc = sc.alloc(&plo, np_cap * D))) return rc;
    if ((rc = sc.alloc(&phi, np_cap * D))) return rc;
    if ((rc = sc.alloc(&pkey, np_cap))) return rc;
    if ((rc = sc.alloc(&dis, n))) return rc;
    {
        const unsigned blocks = (unsigned)std::min<uint64_t>((np_cap * 32 + 255) / 256, 4096);
        stats_count_launch();
        piece_bbox<D><<<blocks, 256, 0, c.stream>>>(b.X, n, pstart, d_np, plo, phi);
        FPSGPU_CUDA_TRY(cudaGetLastError());
    }
    // grid: about two pieces per warp (pieces hold ~kPiece/2..kPiece points)
    uint64_t G = (n / (kPiece / 2) + 63) / 64;
    G = std::max<uint64_t>(1, std::min<uint64_t>(G, (uint64_t)c.sms));
    uint64_t* slots;
    if ((rc = sc.alloc(&slots, 3 * G))) return rc;
    FPSGPU_CUDA_TRY(cudaMemsetAsync(slots, 0, 3 * G * sizeof(uint64_t), c.stream));
    uint64_t* d_forced;
    if ((rc = sc.alloc(&d_forced, c.n_forced))) return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_forced, c.h_forced, c.n_forced * sizeof(uint64_t),
                                    cudaMemcpyHostToDevice, c.stream));
    unsigned long long* sc_counters;
    if ((rc = sc.alloc(&sc_counters, 2))) return rc;
    FPSGPU_CUDA_TRY(cudaMemsetAsync(sc_counters, 0, 2 * sizeof(unsigned long long), c.stream));

    SampleArgs s{};
    s.X = b.X;
    s.tag = b.tag;
    s.dis = dis;
    s.n = n;
    s.pstart = pstart;
    s.npieces = d_np;
    s.plo = plo;
    s.phi = phi;
    s.pkey = pkey;
    s.Xref = Xref;
    s.idmap = idsnap;
    s.k = c.k;
    s.forced = d_forced;
    s.n_forced = c.n_forced;
    s.out = c.d_out;
    s.trace = c.d_trace;
    s.slots = slots;
    s.err = b.err;
    s.counters = sc_counters;
    void* args[] = {&s};
    SamplerTimer timer;
    timer.begin(c.stream);
    const void* kern = c.kd ? (const void*)fps_sample<D, FMA, true> : (const void*)fps_sample<D, FMA, false>;
    if ((rc = launch_persistent(kern, (int)G, kSampleThreads, args, 0, c.stream, G > 1))) return rc;
    timer.end(c.stream);
    int h_err = 0;
    unsigned long long h_cnt[2] = {0, 0};
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(&h_err, b.err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(h_cnt, sc_counters, sizeof(h_cnt), cudaMemcpyDeviceToHost, c.stream));
    FPSGPU_CUDA_TRY(cudaStreamSynchronize(c.stream));
    {
        const uint64_t cn[2] = {h_cnt[0], h_cnt[1]};
        timer.finish(c.k, cn);
    }
    if (h_err & kErrNonFiniteSplit)
        return set_error(FPSGPU_ERR_NONFINITE,
                         "kd-line build met a NaN coordinate in a split dimension");
    if (h_err)
        return set_error(FPSGPU_ERR_DEVICE, "FPS sampler gave up (device error word 0x%x)", h_err);
    return FPSGPU_OK;
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

}  // namespace fpsgpu
