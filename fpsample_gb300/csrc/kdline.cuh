// kd-line QuickFPS on the GPU (reference: src/wrapper.hpp:45-60,
// src/_ext/KDTreeBase.h, KDLineTree.h, KDNode.h, Point.h).
//
// Contract.  The reference's bucket pruning never approximates, so its output
// equals plain FPS over the tree build's permuted order perm, started at
// position start_idx, with ties going to the LOWEST position and the running
// distance capped at FLT_MAX, mapped back through perm.  Only three things must
// therefore match the reference bit for bit: the permutation, the distance
// arithmetic and the tie rule.  Everything else is free.
//
// Build (exact).  Level-synchronous, one CTA per node of the level:
//   1. exact bounding box of the node (order-free min/max, NaN ignored,
//      KDTreeBase.h:181-207);
//   2. split dimension = first dimension with the strictly largest fp32 span
//      (KDTreeBase.h:160-179);
//   3. split value = SEQUENTIAL fp32 sum of that coordinate over the node in
//      its current order, divided by (float)count (KDTreeBase.h:151-158).
//      This chain is inherently serial; warps 1..31 stream the column into a
//      double-buffered shared-memory ring while thread 0 sums it;
//   4. the reference's two-pointer partition (KDTreeBase.h:123-149), computed
//      in parallel: with L = #(x < split), the k-th element >= split in
//      [s, s+L) trades places with the k-th element < split counted from the
//      right end of [s+L, e).  Ranks come from block-wide ballot scans.  The
//      split point is L clamped to [1, count-1].
//   A node is a leaf when its depth equals the height or it holds one point
//   (KDLineTree.h:37-39); a leaf marks its first position in a flag array.
//   Children and leaves keep position order, so buckets are the flagged runs.
//
// Sampling.  The permuted order is cut into "pieces": runs of at most kPiece
// positions that never cross a bucket boundary.  Each piece keeps its exact
// bounding box and the max key of its running distances.  Per sample, every
// piece whose box lies farther from the new reference point than its current
// max (box_bound >= max) provably keeps every distance and is skipped; the
// others recompute their points.  Pieces are owned by warps of a persistent
// cooperative grid; the global argmax runs through the same all-gather exchange
// as vanilla FPS.
#pragma once

#include "fpsgpu_device.cuh"
#include "fpsgpu_internal.h"

namespace fpsgpu {

constexpr int kBuildThreads = 1024;
constexpr int kSumChunk = 4096;   // floats per ring slot of the serial mean
constexpr int kSampleThreads = 1024;
constexpr uint32_t kPiece = 256;  // max positions per piece
constexpr int kCompactChunk = 8192;

struct KdBuildArgs {
    float* X;           // SoA [D][n], permuted in place
    uint32_t* id;       // [n] original index at each position
    uint32_t* sel;      // [n] scratch: partner positions
    uint8_t* flag;      // [n] 1 at the first position of every bucket
    uint2* nodes_cur;   // nodes to split at this level
    uint2* nodes_next;
    uint32_t* cnt;      // [levels + 1] node counts per level
    uint64_t n;
    uint64_t height;
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

template <int D>
__global__ void kd_prepare(const float* __restrict__ pts, KdBuildArgs a, int root_is_leaf) {
    const uint64_t n = a.n;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n;
         p += (uint64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int d = 0; d < D; ++d) a.X[(uint64_t)d * n + p] = pts[p * D + d];
        a.id[p] = (uint32_t)p;
        a.flag[p] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (root_is_leaf) {
            a.cnt[0] = 0;
        } else {
            a.nodes_cur[0] = make_uint2(0u, (uint32_t)n);
            a.cnt[0] = 1;
        }
    }
}

// flag[0] = 1 must happen after kd_prepare cleared the flags, so the root's
// leaf mark (height 0 or a single point) is left to the compaction predicate:
// position 0 always starts a bucket.

template <int D>
__global__ void __launch_bounds__(kBuildThreads, 1) kd_split_level(KdBuildArgs a, uint32_t level) {
    __shared__ __align__(16) float s_ring[2][kSumChunk];
    __shared__ float s_lo[32][D], s_hi[32][D];
    __shared__ uint32_t s_w[2 * 32];
    __shared__ float s_split;
    __shared__ int s_dim;

    const uint32_t cnt = a.cnt[level];
    if (blockIdx.x >= cnt) return;
    const uint2 nd = a.nodes_cur[blockIdx.x];
    const uint32_t s = nd.x, e = nd.y, cntn = e - s;
    const uint64_t n = a.n;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const uint32_t T = blockDim.x;

    // 1. bounding box
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
        }
        __syncthreads();
    }
    const int sd = s_dim;
    const float* col = a.X + (uint64_t)sd * n;

    // 2. split value: sequential fp32 sum in current order, / (float)count.
    // Warps 1..nwarps-1 fill ring slot c+1 while thread 0 sums slot c.
    {
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
    }
    const float split = s_split;

    // 3. L = #(x < split); any NaN among the values or as the split value
    //    makes the reference's two scans disagree, which the rank formulation
    //    below does not model: report it instead.
    uint32_t L = 0;
    bool bad_node = false;
    {
        uint32_t mine = 0;
        bool bad = isnan(split);
        for (uint32_t p = s + tid; p < e; p += T) {
            float v = col[p];
            mine += v < split ? 1u : 0u;
            bad |= isnan(v);
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
        // unordered values: the partition is undefined here; report and stop
        // splitting this node (its range becomes one bucket)
        if (tid == 0) {
            atomicOr(a.err, kErrNonFiniteSplit);
            a.flag[s] = 1;
        }
        return;
    }

    // 4a. right part [s+L, e): elements < split, ranked from the right end
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
    // 4b. left part [s, s+L): elements >= split trade places with their partner
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
                    uint32_t ip = a.id[p], iq = a.id[q];
                    a.id[p] = iq;
                    a.id[q] = ip;
                } else {  // cannot happen without NaN (excluded above); never touch memory out of range
                    atomicOr(a.err, kErrBadIndex);
                }
            }
            running += total;
        }
    }

    // 5. children (KDTreeBase.h:142-147 clamp; KDLineTree.h:37-39 leaf rule)
    if (tid == 0) {
        uint32_t lim = L;
        if (L == 0) lim = 1;
        if (L == cntn) lim = cntn - 1;
        const uint32_t cs[2] = {s, s + lim}, ce[2] = {s + lim, e};
        const bool leaf_depth = (uint64_t)level + 1 >= a.height;
        for (int ch = 0; ch < 2; ++ch) {
            if (leaf_depth || ce[ch] - cs[ch] == 1) {
                a.flag[cs[ch]] = 1;
            } else {
                uint32_t slot = atomicAdd(&a.cnt[level + 1], 1u);
                a.nodes_next[slot] = make_uint2(cs[ch], ce[ch]);
            }
        }
    }
}

// ---- compaction of boundary flags into an ordered start list -------------
// A position p starts a run if flag[p] != 0, p == 0, or (piece > 0 and
// p % piece == 0).  With piece == 0 the runs are the buckets; with
// piece == kPiece they are the sampling pieces.
__device__ __forceinline__ bool run_start(const uint8_t* flag, uint64_t p, uint32_t piece) {
    return p == 0 || flag[p] != 0 || (piece != 0 && p % piece == 0);
}

__global__ void compact_count(const uint8_t* flag, uint64_t n, uint32_t piece, uint32_t* bcount);
__global__ void compact_scan(uint32_t* bcount, uint32_t nblocks, uint32_t* total);
__global__ void compact_write(const uint8_t* flag, uint64_t n, uint32_t piece,
                              const uint32_t* boff, const uint32_t* total, uint32_t* starts);

// ---- pieces: bounding boxes -------------------------------------------------
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

// ---- sampling ---------------------------------------------------------------
struct KdSampleArgs {
    const float* X;         // SoA [D][n], permuted
    const uint32_t* id;     // [n]
    float* dis;             // [n]
    uint64_t n;
    const uint32_t* pstart; // [np + 1]
    const uint32_t* npieces;
    const float* plo;       // [np][D]
    const float* phi;
    uint64_t* pkey;         // [np]
    uint64_t k;
    uint32_t start_pos;
    uint64_t* out;
    float* trace;
    uint64_t* slots;
    int* err;
    unsigned long long* counters;  // [2]: boxes tested, distances recomputed
};

// Applies reference point r to the warp's pieces [q0, q1): INIT sets every
// running distance to min(FLT_MAX, d) (KDNode.h:84-103); otherwise only pieces
// whose box is nearer than their max are recomputed.  Returns the warp's best
// key over all its pieces (lowest position wins ties).
template <int D, bool FMA, bool INIT>
__device__ __forceinline__ uint64_t kd_apply(const KdSampleArgs& a, uint32_t q0, uint32_t q1,
                                             const float* r, unsigned long long& touched) {
    const int lane = threadIdx.x & 31;
    const uint64_t n = a.n;
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
                float dv = INIT ? FLT_MAX : a.dis[p];
                const float dd = sqdist<D, FMA>(x, r);
                if (dd < dv) {
                    dv = dd;
                    if (!INIT) a.dis[p] = dv;
                }
                if (INIT) a.dis[p] = dv;
                const uint64_t kk = key_low_wins(dv, p);
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

template <int D, bool FMA>
__global__ void __launch_bounds__(kSampleThreads, 1) kd_sample(KdSampleArgs a) {
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

    if (tid < D) s_ref[tid] = a.X[(uint64_t)tid * n + a.start_pos];
    if (tid == 0) s_abort = 0;
    if (blockIdx.x == 0 && tid == 0 && a.k > 0) {
        a.out[0] = a.id[a.start_pos];
        if (a.trace) a.trace[0] = FLT_MAX;
    }
    __syncthreads();

    uint32_t xround = 0;
    unsigned long long tested = 0, touched = 0;
    for (uint64_t t = 0; t + 1 < a.k; ++t) {
        float r[D];
#pragma unroll
        for (int d = 0; d < D; ++d) r[d] = s_ref[d];
        if (t > 0) tested += q1 - q0;
        const uint64_t wbest = t == 0 ? kd_apply<D, FMA, true>(a, q0, q1, r, touched)
                                      : kd_apply<D, FMA, false>(a, q0, q1, r, touched);
        if (lane == 0) s_wkey[warp] = wbest;
        __syncthreads();
        if (warp == 0) {
            uint64_t g = warp_max_key(lane < nwarps ? s_wkey[lane] : 0ull);
            if (G > 1) g = exchange_max(a.slots, G, xround++, g, a.err);
            if (g == 0) {
                if (lane == 0) s_abort = 1;
            } else {
                const uint32_t pos = key_pos<true>(g);
                if (pos >= n) {
                    if (lane == 0) {
                        s_abort = 1;
                        atomicOr(a.err, kErrBadIndex);
                    }
                } else {
                    if (lane < D) s_ref[lane] = a.X[(uint64_t)lane * n + pos];
                    if (blockIdx.x == 0 && lane == 0) {
                        a.out[t + 1] = a.id[pos];
                        if (a.trace) a.trace[t + 1] = key_dist(g);
                    }
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
// host launcher
// ---------------------------------------------------------------------------
int kd_compact(const uint8_t* flag, uint64_t n, uint32_t piece, uint32_t* starts,
               uint32_t* d_count, Scratch& sc, cudaStream_t stream);

template <int D, bool FMA>
int run_kdline_d(const KdlineCall& c) {
    Scratch sc(c.stream);
    const uint64_t n = c.n;
    int rc;
    KdBuildArgs b{};
    b.n = n;
    b.height = c.height;
    if ((rc = sc.alloc(&b.X, n * D))) return rc;
    if ((rc = sc.alloc(&b.id, n))) return rc;
    if ((rc = sc.alloc(&b.sel, n))) return rc;
    if ((rc = sc.alloc(&b.flag, n))) return rc;
    if ((rc = sc.alloc(&b.err, 1))) return rc;
    // Depth is bounded by the height and by n - 1 (every split leaves each
    // child at least one point smaller than its parent).
    const uint64_t levels = c.height < n - 1 ? c.height : n - 1;
    const uint64_t node_cap = n / 2 + 1;
    if ((rc = sc.alloc(&b.nodes_cur, node_cap))) return rc;
    if ((rc = sc.alloc(&b.nodes_next, node_cap))) return rc;
    if ((rc = sc.alloc(&b.cnt, levels + 2))) return rc;
    FPSGPU_CUDA_TRY(cudaMemsetAsync(b.cnt, 0, (levels + 2) * sizeof(uint32_t), c.stream));
    FPSGPU_CUDA_TRY(cudaMemsetAsync(b.err, 0, sizeof(int), c.stream));

    {
        uint64_t blocks = (n + 255) / 256;
        if (blocks > 8192) blocks = 8192;
        stats_count_launch();
        kd_prepare<D><<<(unsigned)blocks, 256, 0, c.stream>>>(c.d_points, b, levels == 0 ? 1 : 0);
        FPSGPU_CUDA_TRY(cudaGetLastError());
    }
    uint64_t known_cnt = levels == 0 ? 0 : 1;  // upper bound on nodes at this level
    for (uint64_t j = 0; j < levels; ++j) {
        uint64_t grid = known_cnt;
        if (grid == 0) break;
        stats_count_launch();
        kd_split_level<D><<<(unsigned)grid, kBuildThreads, 0, c.stream>>>(b, (uint32_t)j);
        FPSGPU_CUDA_TRY(cudaGetLastError());
        std::swap(b.nodes_cur, b.nodes_next);
        uint64_t next = 2 * known_cnt;
        if (next > node_cap) next = node_cap;
        if (next > 65536) {
            // large levels: read the exact count instead of launching empty CTAs
            uint32_t h_cnt = 0;
            FPSGPU_CUDA_TRY(cudaMemcpyAsync(&h_cnt, b.cnt + j + 1, sizeof(uint32_t),
                                            cudaMemcpyDeviceToHost, c.stream));
            FPSGPU_CUDA_TRY(cudaStreamSynchronize(c.stream));
            next = h_cnt;
        }
        known_cnt = next;
    }

    if (c.h_perm) {  // build-only mode
        uint32_t* starts;
        uint32_t* d_nb;
        if ((rc = sc.alloc(&starts, n + 1))) return rc;
        if ((rc = sc.alloc(&d_nb, 1))) return rc;
        if ((rc = kd_compact(b.flag, n, 0, starts, d_nb, sc, c.stream))) return rc;
        std::vector<uint32_t> h_id(n);
        uint32_t h_nb = 0;
        int h_err = 0;
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(h_id.data(), b.id, n * sizeof(uint32_t),
                                        cudaMemcpyDeviceToHost, c.stream));
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(&h_nb, d_nb, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                        c.stream));
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(&h_err, b.err, sizeof(int), cudaMemcpyDeviceToHost,
                                        c.stream));
        FPSGPU_CUDA_TRY(cudaStreamSynchronize(c.stream));
        if (h_err & kErrNonFiniteSplit)
            return set_error(FPSGPU_ERR_NONFINITE,
                             "kd-line build met a NaN coordinate in a split dimension");
        std::vector<uint32_t> h_st(h_nb);
        FPSGPU_CUDA_TRY(cudaMemcpy(h_st.data(), starts, h_nb * sizeof(uint32_t),
                                   cudaMemcpyDeviceToHost));
        for (uint64_t i = 0; i < n; ++i) c.h_perm[i] = h_id[i];
        for (uint32_t i = 0; i < h_nb; ++i) c.h_bucket_start[i] = h_st[i];
        *c.h_n_buckets = h_nb;
        return FPSGPU_OK;
    }

    // pieces
    // pieces <= n / kPiece + 1 + buckets, and buckets <= min(2^levels, n)
    const uint64_t nb_bound = levels < 40 ? (1ull << levels) : n;
    const uint64_t np_cap = n / kPiece + 1 + nb_bound;
    const uint64_t np_bound = np_cap < n ? np_cap : n;
    uint32_t* pstart;
    uint32_t* d_np;
    if ((rc = sc.alloc(&pstart, np_bound + 1))) return rc;
    if ((rc = sc.alloc(&d_np, 1))) return rc;
    if ((rc = kd_compact(b.flag, n, kPiece, pstart, d_np, sc, c.stream))) return rc;
    float *plo, *phi, *dis;
    uint64_t* pkey;
    if ((rc = sc.alloc(&plo, np_bound * D))) return rc;
    if ((rc = sc.alloc(&phi, np_bound * D))) return rc;
    if ((rc = sc.alloc(&pkey, np_bound))) return rc;
    if ((rc = sc.alloc(&dis, n))) return rc;
    {
        uint64_t blocks = (np_bound * 32 + 255) / 256;
        if (blocks > 4096) blocks = 4096;
        stats_count_launch();
        piece_bbox<D><<<(unsigned)blocks, 256, 0, c.stream>>>(b.X, n, pstart, d_np, plo, phi);
        FPSGPU_CUDA_TRY(cudaGetLastError());
    }
    // grid: about one piece per warp, at most one CTA per SM
    uint64_t G = (np_bound + 31) / 32;
    if (G > (uint64_t)c.sms) G = c.sms;
    if (G < 1) G = 1;
    uint64_t* slots;
    if ((rc = sc.alloc(&slots, 3 * G))) return rc;
    FPSGPU_CUDA_TRY(cudaMemsetAsync(slots, 0, 3 * G * sizeof(uint64_t), c.stream));

    KdSampleArgs s{};
    s.X = b.X;
    s.id = b.id;
    s.dis = dis;
    s.n = n;
    s.pstart = pstart;
    s.npieces = d_np;
    s.plo = plo;
    s.phi = phi;
    s.pkey = pkey;
    s.k = c.k;
    s.start_pos = (uint32_t)c.start;
    s.out = c.d_out;
    s.trace = c.d_trace;
    s.slots = slots;
    s.err = b.err;
    unsigned long long* counters;
    if ((rc = sc.alloc(&counters, 2))) return rc;
    FPSGPU_CUDA_TRY(cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned long long), c.stream));
    s.counters = counters;
    void* args[] = {&s};
    SamplerTimer timer;
    timer.begin(c.stream);
    if ((rc = launch_persistent((const void*)kd_sample<D, FMA>, (int)G, kSampleThreads, args, 0,
                                c.stream, G > 1)))
        return rc;
    timer.end(c.stream);
    int h_err = 0;
    unsigned long long h_cnt[2] = {0, 0};
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(&h_err, b.err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(h_cnt, counters, sizeof(h_cnt), cudaMemcpyDeviceToHost, c.stream));
    FPSGPU_CUDA_TRY(cudaStreamSynchronize(c.stream));
    {
        const uint64_t cnt[2] = {h_cnt[0], h_cnt[1]};
        timer.finish(c.k, cnt);
    }
    if (h_err & kErrNonFiniteSplit)
        return set_error(FPSGPU_ERR_NONFINITE,
                         "kd-line build met a NaN coordinate in a split dimension");
    if (h_err)
        return set_error(FPSGPU_ERR_DEVICE, "kd-line sampler gave up (device error word 0x%x)",
                         h_err);
    return FPSGPU_OK;
}

template <bool FMA>
int run_kdline_dispatch(const KdlineCall& c) {
    switch (c.dim) {
        case 1: return run_kdline_d<1, FMA>(c);
        case 2: return run_kdline_d<2, FMA>(c);
        case 3: return run_kdline_d<3, FMA>(c);
        case 4: return run_kdline_d<4, FMA>(c);
        case 5: return run_kdline_d<5, FMA>(c);
        case 6: return run_kdline_d<6, FMA>(c);
        case 7: return run_kdline_d<7, FMA>(c);
        case 8: return run_kdline_d<8, FMA>(c);
        default: return set_error(FPSGPU_ERR_DIM, "dim must be in [1, 8], got %d", c.dim);
    }
}

}  // namespace fpsgpu
