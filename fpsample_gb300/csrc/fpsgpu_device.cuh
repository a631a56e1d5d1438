// Device-side building blocks shared by the FPS kernels (sm_103a).
//
// * sqdist<D,FMA>: the reference's fp32 squared distance, bit for bit.
//   Reference: src/lib.cpp:214-221 (vanilla) and src/_ext/Point.h:48-53 with
//   utils.h:12-16 (kd-line).  Both sum (p_j - r_j)^2 over j = 0..D-1 in order.
//   FMA=false rounds every operation ((d0*d0 + d1*d1) + d2*d2); FMA=true is the
//   contracted chain fma(d2,d2,fma(d1,d1,d0*d0)) that a contracting host
//   compiler produces.  The explicit __f*_rn intrinsics stop nvcc from
//   contracting on its own.
// * 64-bit argmax keys: (valid bit 63) | (distance bits << 32) | tie field.
//   Distances are never negative or NaN, so their IEEE bits order like their
//   values.  The tie field is the position itself where the HIGHEST index wins
//   (vanilla, lib.cpp:226 uses >=) and its complement where the LOWEST position
//   wins (kd-line, KDNode.h:97,155 and KDLineTree.h:61 use strict >).
// * warp/block argmax via redux.sync, and the cross-CTA all-gather exchange
//   used by the persistent multi-CTA kernels.
#pragma once

#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

namespace fpsgpu {

constexpr uint64_t kKeyValid = 1ull << 63;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxDim = 8;

// error word bits (device -> host)
constexpr int kErrExchangeTimeout = 1;
constexpr int kErrNonFiniteSplit = 2;
constexpr int kErrBadIndex = 4;

// Upper bound on polls of one exchange slot before a CTA gives up, sets the
// error word and leaves the kernel (each poll is one L2 round trip, so this is
// a few seconds).
constexpr long long kSpinLimit = 1ll << 23;

template <int D, bool FMA>
__device__ __forceinline__ float sqdist(const float* p, const float* r) {
    float d = __fsub_rn(p[0], r[0]);
    float acc = __fmul_rn(d, d);
#pragma unroll
    for (int j = 1; j < D; ++j) {
        float e = __fsub_rn(p[j], r[j]);
        acc = FMA ? __fmaf_rn(e, e, acc) : __fadd_rn(acc, __fmul_rn(e, e));
    }
    return acc;
}

// Runtime-dimension variant (same operation order), for D > 8 in vanilla FPS.
template <bool FMA>
__device__ __forceinline__ float sqdist_rt(const float* __restrict__ X, uint64_t stride, uint64_t p,
                                           const float* r, int dim) {
    float d = __fsub_rn(X[p], r[0]);
    float acc = __fmul_rn(d, d);
    for (int j = 1; j < dim; ++j) {
        float e = __fsub_rn(X[(uint64_t)j * stride + p], r[j]);
        acc = FMA ? __fmaf_rn(e, e, acc) : __fadd_rn(acc, __fmul_rn(e, e));
    }
    return acc;
}

// Squared gap from r to the box [lo, hi], with the same operation structure as
// sqdist.  Rounding is monotone, so for every point p inside the box
// bound <= sqdist(p, r) in the same mode: a box whose bound is >= the largest
// running distance inside it cannot have any distance lowered by r.
template <int D, bool FMA>
__device__ __forceinline__ float box_bound(const float* lo, const float* hi, const float* r) {
    float acc = 0.0f;
#pragma unroll
    for (int j = 0; j < D; ++j) {
        // r above the box: r - hi > 0 > lo - r; below: lo - r > 0 > r - hi;
        // inside: both <= 0.  Same value as the branchy form, fewer steps.
        const float g = fmaxf(fmaxf(__fsub_rn(lo[j], r[j]), __fsub_rn(r[j], hi[j])), 0.0f);
        if (j == 0) acc = __fmul_rn(g, g);
        else acc = FMA ? __fmaf_rn(g, g, acc) : __fadd_rn(acc, __fmul_rn(g, g));
    }
    return acc;
}

__device__ __forceinline__ uint64_t key_high_wins(float dist, uint32_t pos) {
    return kKeyValid | ((uint64_t)__float_as_uint(dist) << 32) | pos;
}
__device__ __forceinline__ uint64_t key_low_wins(float dist, uint32_t pos) {
    return kKeyValid | ((uint64_t)__float_as_uint(dist) << 32) | (0xffffffffu - pos);
}
__device__ __forceinline__ float key_dist(uint64_t key) {
    return __uint_as_float((uint32_t)(key >> 32) & 0x7fffffffu);
}
template <bool LOW_WINS>
__device__ __forceinline__ uint32_t key_pos(uint64_t key) {
    uint32_t t = (uint32_t)key;
    return LOW_WINS ? 0xffffffffu - t : t;
}

// Max of a 64-bit key over the full warp: two redux.sync steps.
__device__ __forceinline__ uint64_t warp_max_key(uint64_t k) {
    uint32_t hi = (uint32_t)(k >> 32), lo = (uint32_t)k;
    uint32_t mh = __reduce_max_sync(kFull, hi);
    uint32_t ml = __reduce_max_sync(kFull, hi == mh ? lo : 0u);
    return ((uint64_t)mh << 32) | ml;
}

// ---- thread-block clusters: rank, barrier, distributed shared memory --------
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cluster_size() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
// Every thread of every CTA of the cluster: release what this thread wrote
// (shared, distributed shared and global), wait for all, acquire.
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::
                     : "memory");
}
// mbarrier-completed remote stores: st.async writes into CTA `rank`'s shared
// memory and counts its bytes on that CTA's mbarrier (no fence needed).
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"((uint32_t)__cvta_generic_to_shared(bar)),
                 "r"(count)
                 : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait_cluster(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"((uint32_t)__cvta_generic_to_shared(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void st_async_u64(uint32_t addr, uint64_t v, uint32_t bar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];" ::"r"(addr),
                 "l"(v), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ void st_async_f32(uint32_t addr, float v, uint32_t bar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];" ::"r"(addr),
                 "r"(__float_as_uint(v)), "r"(bar)
                 : "memory");
}
// Address of `p` (a shared variable of this CTA) in the shared memory of the
// cluster's CTA `rank`.
__device__ __forceinline__ uint32_t dsmem_addr(const void* p, uint32_t rank) {
    uint32_t out;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;"
                 : "=r"(out)
                 : "r"((uint32_t)__cvta_generic_to_shared(p)), "r"(rank));
    return out;
}
__device__ __forceinline__ uint32_t dsmem_ld_u32(uint32_t a) {
    uint32_t v;
    asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_gpu(uint64_t* p, uint64_t v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed_gpu(uint64_t* p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_acquire_gpu(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_relaxed_gpu_s32(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ uint64_t ld_relaxed_gpu(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// Largest grid exchange_max supports (slots polled per lane: kMaxGrid / 32).
constexpr int kMaxGrid = 256;

// Cross-CTA argmax for persistent kernels whose CTAs are all co-resident
// (cooperative launch).  Called by ONE full warp per CTA, once per round.
//
// slots: 3 * G u64, zeroed before the launch.  Round t uses row t % 3.  Every
// CTA publishes its key (never 0: bit 63 is set) with a release store, then
// polls the whole row until every entry is non-zero.  Each lane issues the
// loads of all its slots back to back (relaxed) so one poll costs one L2 round
// trip; a fence after the last poll makes it an acquire.  When a CTA has seen
// all of round t, every CTA has finished reading round t-1, so it clears its
// own round-(t-1) entry, which it will not publish into again before round
// t+2; the clear is ordered before its round t+1 release store, so a reader of
// round t+2 can never see the stale value.
//
// A CTA without candidates publishes kKeyValid alone, which never beats a
// real key of a valid point.  Returns 0 (and sets err) if the row is still
// incomplete after kSpinLimit polls.
__device__ __forceinline__ uint64_t exchange_max(uint64_t* slots, int G, uint32_t round,
                                                 uint64_t my_key, int* err) {
    constexpr int kPer = kMaxGrid / 32;
    const int lane = threadIdx.x & 31;
    uint64_t* row = slots + (uint64_t)(round % 3u) * G;
    if (lane == 0) st_release_gpu(row + blockIdx.x, my_key | kKeyValid);
    uint64_t v[kPer];
#pragma unroll
    for (int i = 0; i < kPer; ++i) v[i] = 0;
    long long spins = 0;
    for (;;) {
        bool mine = true;
#pragma unroll
        for (int i = 0; i < kPer; ++i) {
            const int j = lane + 32 * i;
            if (j < G && v[i] == 0) v[i] = ld_relaxed_gpu(row + j);
        }
#pragma unroll
        for (int i = 0; i < kPer; ++i) {
            const int j = lane + 32 * i;
            if (j < G && v[i] == 0) mine = false;
        }
        if (__all_sync(kFull, mine)) break;
        if (++spins > kSpinLimit) {
            if (lane == 0) atomicOr(err, kErrExchangeTimeout);
            return 0;
        }
    }
    fence_acq_rel_gpu();
    uint64_t best = 0;
#pragma unroll
    for (int i = 0; i < kPer; ++i) best = v[i] > best ? v[i] : best;
    best = warp_max_key(best);
    if (lane == 0) st_relaxed_gpu(slots + (uint64_t)((round + 2u) % 3u) * G + blockIdx.x, 0ull);
    return best;
}

// Largest grid exchange_leader supports (5 slots per polling lane).
constexpr int kMaxGridCoords = 160;

__device__ __forceinline__ uint64_t tagged(uint32_t tag, uint32_t payload) {
    return ((uint64_t)tag << 32) | payload;
}

// Words per exchange record: key (two tagged halves) + D tagged coordinates,
// padded to an even count for 16-byte loads.
template <int D>
constexpr int leader_words() { return (2 + D + 1) & ~1; }

__device__ __forceinline__ void ld_relaxed_gpu_v2(const uint64_t* p, uint64_t& a, uint64_t& b) {
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(p) : "memory");
}

// Cross-CTA argmax through a leader (CTA 0), for persistent cooperative grids.
// Called by ONE full warp per CTA, once per round; returns the winning key and
// (D > 0) the winner's coordinates in win_c, identical in every CTA.
//
// Every 64-bit word written here carries the round tag (round + 1) in its high
// half, and aligned 64-bit accesses are single-copy atomic, so a word showing
// this round's tag holds this round's payload: no fences or clearing needed.
//   1. every CTA writes its record (key hi, key lo, coordinates) into its slot;
//   2. CTA 0 polls all G slots until they show the tag, takes the max and
//      writes the winner's record into `bcast`;
//   3. every CTA polls `bcast` until it shows the tag.
// One slot row and one broadcast record suffice: a CTA rewrites its slot for
// round t+1 only after reading the round-t broadcast, which CTA 0 writes only
// after it has read every round-t slot; CTA 0 rewrites the broadcast for round
// t+1 only after every CTA has published round t+1, i.e. after every CTA has
// read the round-t broadcast.  L2 traffic per round is O(G) (the gather plus
// one record per CTA), not the O(G^2) of an all-to-all poll.
// Every poll loop gives up after `limit` rounds (kSpinLimit unless a self-test
// asks for fewer): err is set, 0 returned.
template <int D>
__device__ __forceinline__ uint64_t exchange_leader(uint64_t* slots, uint64_t* bcast, int G,
                                                    uint32_t round, uint64_t my_key,
                                                    const float* my_c, float* win_c, int* err,
                                                    long long limit = kSpinLimit) {
    constexpr int SW = leader_words<D>();
    constexpr int kPer = kMaxGridCoords / 32;
    const int lane = threadIdx.x & 31;
    const uint32_t rt = round + 1u;
    my_key |= kKeyValid;
    if (lane == 0) {
        uint64_t* mine = slots + (uint64_t)blockIdx.x * SW;
        st_relaxed_gpu(mine + 0, tagged(rt, (uint32_t)(my_key >> 32)));
        st_relaxed_gpu(mine + 1, tagged(rt, (uint32_t)my_key));
#pragma unroll
        for (int d = 0; d < D; ++d) st_relaxed_gpu(mine + 2 + d, tagged(rt, __float_as_uint(my_c[d])));
    }
    bool ok = true;
    if (blockIdx.x == 0) {
        uint64_t best = 0;
        float bc[D > 0 ? D : 1];
#pragma unroll
        for (int d = 0; d < (D > 0 ? D : 1); ++d) bc[d] = 0.0f;
        unsigned done = 0;
        long long spins = 0;
        for (;;) {
#pragma unroll
            for (int i = 0; i < kPer; ++i) {
                const int j = lane + 32 * i;
                if (j < G && !((done >> i) & 1u)) {
                    uint64_t w[SW];
#pragma unroll
                    for (int k = 0; k < SW; k += 2) ld_relaxed_gpu_v2(slots + (uint64_t)j * SW + k, w[k], w[k + 1]);
                    bool good = true;
#pragma unroll
                    for (int k = 0; k < 2 + D; ++k) good &= (uint32_t)(w[k] >> 32) == rt;
                    if (good) {
                        done |= 1u << i;
                        const uint64_t key = ((uint64_t)(uint32_t)w[0] << 32) | (uint32_t)w[1];
                        if (key > best) {
                            best = key;
#pragma unroll
                            for (int d = 0; d < D; ++d) bc[d] = __uint_as_float((uint32_t)w[2 + d]);
                        }
                    }
                }
            }
            bool all = true;
#pragma unroll
            for (int i = 0; i < kPer; ++i)
                if (lane + 32 * i < G && !((done >> i) & 1u)) all = false;
            if (__all_sync(kFull, all)) break;
            if (++spins > limit) {
                ok = false;
                break;
            }
        }
        if (__all_sync(kFull, ok)) {
            const uint64_t g = warp_max_key(best);
            const int owner = __ffs(__ballot_sync(kFull, best == g)) - 1;
            float wc[D > 0 ? D : 1];
#pragma unroll
            for (int d = 0; d < D; ++d) wc[d] = __shfl_sync(kFull, bc[d], owner);
            if (lane == 0) {
#pragma unroll
                for (int d = 0; d < D; ++d) st_relaxed_gpu(bcast + 2 + d, tagged(rt, __float_as_uint(wc[d])));
                st_relaxed_gpu(bcast + 1, tagged(rt, (uint32_t)g));
                st_relaxed_gpu(bcast + 0, tagged(rt, (uint32_t)(g >> 32)));
            }
        } else {
            ok = false;
        }
    }
    // every CTA reads the broadcast record
    uint64_t w[SW];
#pragma unroll
    for (int k = 0; k < SW; ++k) w[k] = 0;
    if (lane == 0 && ok) {
        long long spins = 0;
        for (;;) {
#pragma unroll
            for (int k = 0; k < SW; k += 2) ld_relaxed_gpu_v2(bcast + k, w[k], w[k + 1]);
            bool good = true;
#pragma unroll
            for (int k = 0; k < 2 + D; ++k) good &= (uint32_t)(w[k] >> 32) == rt;
            if (good) break;
            if (++spins > limit) {
                ok = false;
                break;
            }
        }
    }
    ok = __shfl_sync(kFull, ok ? 1 : 0, 0) != 0;
    if (!ok) {
        if (lane == 0) atomicOr(err, kErrExchangeTimeout);
        return 0;
    }
    const uint32_t hi = __shfl_sync(kFull, (uint32_t)w[0], 0);
    const uint32_t lo = __shfl_sync(kFull, (uint32_t)w[1], 0);
#pragma unroll
    for (int d = 0; d < D; ++d) win_c[d] = __uint_as_float(__shfl_sync(kFull, (uint32_t)w[2 + d], 0));
    return ((uint64_t)hi << 32) | lo;
}

}  // namespace fpsgpu
