// One CTA per cloud with a leader warp and worker warps: the batched engine's
// sampler for clouds of D <= 3 that one CTA holds (included by engine.cuh,
// inside namespace fpsgpu).
//
// Why.  A sample depends on the previous one, so a cloud's sampling time is
// K times the latency of one sample.  In the lockstep sampler (batch_sample)
// every sample waits for the whole CTA: every warp tests all its piece boxes,
// the warps holding dirty pieces recompute them one after the other, and one
// __syncthreads publishes the max.  Yet the next sample depends on very few
// pieces: keys only fall, so after sample t the argmax lies among the pieces
// whose old key beats the best key of the pieces that r_t left alone -- in
// practice the winner's own piece and the runner-up.
//
// Design.  Warp 0 (the leader) holds a hot table of 55 or 77 pieces in
// shared memory: at the start of an epoch every worker warp names its 5 or 7
// pieces of largest key; pieces that were hot already stay where they are,
// new ones are copied in, pieces that drop out are written back.  T = the
// largest key of the pieces left with the workers at that moment.  Keys only
// fall, so T bounds every non-hot piece for the whole epoch, and while the
// best hot key exceeds T the best hot piece holds the global argmax.  The
// leader then runs alone: take the best hot key, emit its point (into a
// shared output queue and the epoch's reference list), recompute its piece at
// once (the winner's piece is always dirty), then every other hot piece whose
// box is nearer than its key, repeat.  Workers (warps 1..11) apply the same
// references, in order and asynchronously, to the pieces they kept (box tests
// and recomputes as in batch_sample).  When the best hot key falls to T (or
// the reference list is full) the epoch ends at a CTA barrier.  No sample
// waits for the workers.
//
// Leader keys.  A hot record's low key word is position | record (7 bits) |
// entry (6 bits, 7 for the 77-entry table), with the cloud-local position in
// 18 bits (complemented for kd-line, like batch_key): the order is the
// reference's tie order (position first, and positions are unique), and the
// warp max itself names the winner's entry and record, so the next reference
// point is one shared load away.  Hot entries are padded to kPiece records
// with copies of their last record (same key), so a recompute needs no bounds.
//
// Exactness.  Hot pieces are kept exact (every sample applied, in order); a
// non-hot piece's stored key only ever over-states its true key, and the
// leader emits only while its best exact key is above T, so every emitted
// point is the global argmax of the running distances -- the same point the
// reference picks.  Running distances are lowered with the reference's strict
// "<" rule; min is order-free, so the workers' lag changes no value.
//
// Memory.  Points are float4 records {coordinates, running distance} (P4) plus
// a 32-bit low key word per point (LW, batch_key's low half), prepared once per
// call by lead_prepare, and stay in global memory (L1/L2) with their workers.

// 12 warps: at most three per SM sub-partition, so a thread may hold 168
// registers (the workers' boxes and keys stay in registers without spilling)
constexpr int kLeadThreads = 384;
constexpr int kLeadWorkers = kLeadThreads / 32 - 1;  // warps 1..11
constexpr int kLeadSlots = 5;                        // pieces per worker thread (<= 8: hent)
constexpr uint32_t kLeadCap = (uint32_t)kLeadWorkers * 32 * kLeadSlots;  // 1760 pieces
// Hot pieces per worker warp (HPW, a template parameter): 5 (a table of 55
// entries, two per leader lane) or 7 (77 entries, three per lane).  The wide
// table's longer epochs pay on large clouds (measured per sample: 0.694 vs
// 0.708 us at 65K points, 0.664 vs 0.677 at 124K); on clouds of 4K-32K points
// the narrow one is faster (0.65-0.70 vs 0.70-0.78 us), so a launch takes the
// wide table when its largest cloud has kLeadHotWideMin pieces or more.
constexpr int kLeadHotPerWarp = 7;                        // the wide table
constexpr int kLeadHot = kLeadWorkers * kLeadHotPerWarp;  // 77 entries at most
constexpr int kLeadHotSmall = 5;                          // the narrow table (55 entries)
constexpr uint32_t kLeadHotWideMin = 512;
// the layout of a table of HPW hot pieces per worker warp
template <int HPW>
struct LeadTable {
    static constexpr int kHot = kLeadWorkers * HPW;
    // leader key low word: position (18 bits) | record (7 bits) | entry (kEntryBits)
    static constexpr uint32_t kEntryBits = kHot <= 64 ? 6 : 7;
    static constexpr uint32_t kPosShift = kEntryBits + 7;
    static constexpr bool kThree = kHot > 64;  // three entries per leader lane
};
constexpr int kLeadRefs = 128;                            // samples per epoch at most
constexpr uint32_t kLeadDone = 0x80000000u;               // epoch-end bit of the reference count
constexpr uint32_t kLeadPosBits = 18;
constexpr uint32_t kLeadPosMask = (1u << kLeadPosBits) - 1;
// clouds the leader sampler takes: positions fit its keys
constexpr uint64_t kLeadMaxCloudPoints = 1ull << kLeadPosBits;

static_assert(kLeadHot <= 96, "entries fit 7 bits; the leader holds three per lane");
static_assert(kPiece == 128, "records of a piece fit 7 bits, four per lane");
static_assert(kLeadCap <= (1u << kBatchPieceBits), "piece index must fit batch_key");
static_assert(kLeadPosBits + 7 + 7 <= 32, "leader key low word");
static_assert((uint64_t)kLeadCap * kPiece <= kLeadMaxCloudPoints, "positions of a one-CTA cloud fit 18 bits");
static_assert(kLeadPosBits + 8 + 6 <= 32, "fill word: entry (6-bit entries) | piece start | length");

struct LeadArgs {
    float4* P4;             // [n] {x, y, z, running distance}, storage order
    const uint32_t* LW;     // [n] low key word of every point (batch_key format)
    const uint32_t* pstart;
    const float* plo;       // [np][D]
    const float* phi;
    const uint32_t* cloud_piece;  // [C + 1]
    const uint64_t* cloud_off;    // [C + 1]
    const uint64_t* cloud_k;      // [C]
    const uint64_t* cloud_tag0;   // [C]
    const uint64_t* out_off;      // [C]
    const uint32_t* order;        // [n_items] clouds in processing order
    uint32_t n_items;
    uint64_t n;
    const float* Xref;
    const uint32_t* idmap;  // kd-line: original index by tag; vanilla: null
    uint64_t* out;
    unsigned int* queue;
    unsigned long long* counters;
    int* err;
    float* out_pts;
    long long spin_limit;  // polls a worker makes for the next reference before giving up
    int mute;              // self-test of that bound: the leader publishes nothing
};

// shared region of a table of `entries` hot pieces: their records, then
// their leader low key words
constexpr size_t lead_smem_bytes(uint32_t entries) { return (size_t)entries * kPiece * 20; }

// P4 and LW for every point of every piece: coordinates from the SoA X, the
// low key word batch_key would build from the point's tag and cloud-local
// piece index.  One warp per piece.
template <int D, bool KD>
__global__ void lead_prepare(const float* __restrict__ X, const uint32_t* __restrict__ tag, uint64_t n,
                             const uint32_t* __restrict__ pstart, const uint32_t* __restrict__ cloud_piece,
                             const uint64_t* __restrict__ cloud_off, uint32_t n_clouds,
                             float4* __restrict__ P4, uint32_t* __restrict__ LW) {
    static_assert(D >= 1 && D <= 3, "float4 records hold at most three coordinates");
    const uint32_t np = cloud_piece[n_clouds];
    const uint32_t nwarps = gridDim.x * blockDim.x / 32;
    const int lane = threadIdx.x & 31;
    for (uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) / 32; g < np; g += nwarps) {
        uint32_t lo = 0, hi = n_clouds;  // last cloud whose first piece is <= g
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) / 2;
            if (cloud_piece[mid] <= g) lo = mid;
            else hi = mid;
        }
        const uint32_t q = (g - cloud_piece[lo]) & ((1u << kBatchPieceBits) - 1);
        const uint32_t base = (uint32_t)cloud_off[lo];
        const uint32_t pm = (1u << kBatchPosBits) - 1;
        for (uint32_t p = pstart[g] + lane; p < pstart[g + 1]; p += 32) {
            float4 v;
            v.x = X[p];
            v.y = D > 1 ? X[n + p] : 0.0f;
            v.z = D > 2 ? X[2 * n + p] : 0.0f;
            v.w = 0.0f;
            P4[p] = v;
            const uint32_t loc = (tag[p] - base) & pm;
            LW[p] = ((KD ? pm - loc : loc) << kBatchPieceBits) | q;
        }
    }
}

template <int D, bool FMA>
__device__ __forceinline__ float sqdist4(const float4& p, const float4& r) {
    const float pv[3] = {p.x, p.y, p.z}, rv[3] = {r.x, r.y, r.z};
    return sqdist<D, FMA>(pv, rv);
}

__device__ __forceinline__ uint32_t ld_acquire_cta_shared(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.cta.shared::cta.u32 %0, [%1];"
                 : "=r"(v)
                 : "r"((uint32_t)__cvta_generic_to_shared(p))
                 : "memory");
    return v;
}
__device__ __forceinline__ void st_release_cta_shared(uint32_t* p, uint32_t v) {
    asm volatile("st.release.cta.shared::cta.u32 [%0], %1;" ::"r"((uint32_t)__cvta_generic_to_shared(p)),
                 "r"(v)
                 : "memory");
}

// Cloud-local position of a low key word, worker (batch_key) or leader format.
template <bool KD>
__device__ __forceinline__ uint32_t lead_loc_worker(uint32_t lo) {
    const uint32_t pm = (1u << kBatchPosBits) - 1, f = (lo >> kBatchPieceBits) & pm;
    return KD ? pm - f : f;
}
template <bool KD, int HPW>
__device__ __forceinline__ uint32_t lead_loc_leader(uint32_t lo) {
    const uint32_t f = (lo >> LeadTable<HPW>::kPosShift) & kLeadPosMask;
    return KD ? kLeadPosMask - f : f;
}
template <bool KD, int HPW>
__device__ __forceinline__ uint32_t lead_pos_leader(uint32_t loc) {
    return (KD ? kLeadPosMask - loc : loc) << LeadTable<HPW>::kPosShift;
}
template <bool KD>
__device__ __forceinline__ uint32_t lead_pos_worker(uint32_t loc) {
    const uint32_t pm = (1u << kBatchPosBits) - 1;
    return (KD ? pm - loc : loc) << kBatchPieceBits;
}

// max of (h, l) pairs, h first
__device__ __forceinline__ void lead_pmax(uint32_t& h, uint32_t& l, uint32_t h2, uint32_t l2) {
    const bool gt = h2 > h || (h2 == h && l2 > l);
    h = gt ? h2 : h;
    l = gt ? l2 : l;
}

// Applies reference point r to the points [0, len) of one piece in global or
// shared memory (float4 records at pts, low key words at lw), with the
// reference's strict "<" rule, or the first reference (INIT: min(init, d)).
// Returns the piece's new max key to the whole warp.  Lanes past the end read
// the last record again (same key, same value stored): no branch.  Every
// load of the piece is issued before the first use (one round trip).
template <int D, bool FMA, bool INIT>
__device__ __forceinline__ uint64_t lead_update(float4* pts, const uint32_t* lw, uint32_t len, const float4 r,
                                                float init) {
    const uint32_t lane = threadIdx.x & 31;
    constexpr int PPL = kPiece / 32;
    float4 v[PPL];
    uint32_t w[PPL], pi[PPL];
#pragma unroll
    for (int j = 0; j < PPL; ++j) {
        const uint32_t p = lane + 32 * j;
        pi[j] = p < len ? p : len - 1;
        v[j] = pts[pi[j]];
        w[j] = lw[pi[j]];
    }
    uint32_t bh[PPL];
#pragma unroll
    for (int j = 0; j < PPL; ++j) {
        const float dd = sqdist4<D, FMA>(v[j], r);
        const float old = INIT ? init : v[j].w;
        const bool lower = dd < old;
        const float nv = lower ? dd : old;
        if (INIT || lower) reinterpret_cast<float*>(pts + pi[j])[3] = nv;
        bh[j] = __float_as_uint(nv) | 0x80000000u;
    }
    lead_pmax(bh[0], w[0], bh[1], w[1]);
    lead_pmax(bh[2], w[2], bh[3], w[3]);
    lead_pmax(bh[0], w[0], bh[2], w[2]);
    const uint32_t mh = __reduce_max_sync(kFull, bh[0]);
    const uint32_t ml = __reduce_max_sync(kFull, bh[0] == mh ? w[0] : 0u);
    return ((uint64_t)mh << 32) | ml;
}

// The leader's recompute of one hot entry: kPiece records in shared memory
// (padded), leader low key words.
template <int D, bool FMA>
__device__ __forceinline__ uint64_t lead_update_hot(float4* pts, const uint32_t* lw, const float4 r) {
    const uint32_t lane = threadIdx.x & 31;
    constexpr int PPL = kPiece / 32;
    float4 v[PPL];
    uint32_t w[PPL], bh[PPL];
#pragma unroll
    for (int j = 0; j < PPL; ++j) {
        v[j] = pts[lane + 32 * j];
        w[j] = lw[lane + 32 * j];
    }
#pragma unroll
    for (int j = 0; j < PPL; ++j) {
        const float dd = sqdist4<D, FMA>(v[j], r);
        const bool lower = dd < v[j].w;
        const float nv = lower ? dd : v[j].w;
        if (lower) reinterpret_cast<float*>(pts + lane + 32 * j)[3] = nv;
        bh[j] = __float_as_uint(nv) | 0x80000000u;
    }
    lead_pmax(bh[0], w[0], bh[1], w[1]);
    lead_pmax(bh[2], w[2], bh[3], w[3]);
    lead_pmax(bh[0], w[0], bh[2], w[2]);
    const uint32_t mh = __reduce_max_sync(kFull, bh[0]);
    const uint32_t ml = __reduce_max_sync(kFull, bh[0] == mh ? w[0] : 0u);
    return ((uint64_t)mh << 32) | ml;
}

// The CTA barrier that the leader's and the workers' routines both reach
// (named barrier 1 over the whole CTA; each routine reaches it the same number
// of times per cloud, from its own code).  The non-aligned form counts
// threads one by one, so lanes that arrive from different branches (a lane 0
// that just wrote shared state) are all counted; bar.sync, the aligned form,
// requires a converged warp.
__device__ __forceinline__ void lead_bar() {
    __syncwarp();
    asm volatile("barrier.sync 1, %0;" ::"r"(kLeadThreads) : "memory");
}

// Shared state of one CTA (besides the dynamic region of hot records), sized
// for the table: the narrow kernel's whole shared memory stays within the
// 164 KB carve-out, which leaves 92 KB of L1 to the workers' pieces.
template <int HPW>
struct LeadShared {
    static constexpr int kEnt = LeadTable<HPW>::kThree ? 96 : 64;  // 32 per leader lane slot
    uint64_t hkey[kEnt];         // hot table: key (leader format; 0: empty entry)
    float4 hlo[kEnt], hhi[kEnt];  // box
    uint32_t hlen[kEnt];         // records of the piece
    uint32_t hps[kEnt];          // piece start (cloud-local)
    uint8_t hmod[kEnt];          // the leader lowered a distance since the entry was filled
    float4 ref[kLeadRefs];     // this epoch's references, in order (their coordinates are the outputs' points)
    uint32_t outq[kLeadRefs];  // this epoch's outputs (cloud-local position), written out after the epoch
    uint32_t nref;             // references published | kLeadDone at the epoch's end
    uint64_t T[kLeadWorkers];  // best non-hot key of every worker warp (worker format)
    uint32_t wlo[kLeadWorkers][kLeadSlots][32];  // workers: low word of every slot's key
    uint32_t wpr[kLeadWorkers][kLeadSlots][32];  // workers: piece start (cloud-local) << 8 | length
    uint32_t fill[kLeadWorkers][HPW];  // workers: pieces to copy in: [entry << 26 |] piece start << 8 | length
    uint8_t fent[kLeadWorkers][LeadTable<HPW>::kEntryBits == 6 ? 1 : HPW];  // and their entries (7-bit entries)
    uint64_t fkey[kLeadWorkers][HPW];  // and their keys (worker format)
    uint32_t item;
    uint32_t emitted;
    int stall;
};

// What the leader and the workers both know about the current cloud.
struct LeadCloud {
    uint32_t P0, np, nc;
    uint64_t K, coff, ooff;
};

// Worker warp w (0..kLeadWorkers-1) on one cloud: its pieces' boxes and key
// distances in registers (low key words and piece ranges in shared memory),
// the first reference, then per epoch the hot selection and the epoch's
// references on the pieces it kept.  Reaches lead_bar() once after the first
// reference and twice per epoch, like lead_leader.
template <int D, bool FMA, bool KD, int HPW>
__device__ __forceinline__ void lead_worker(const LeadArgs& a, LeadShared<HPW>& S, float4* s_pt, uint32_t* s_lw,
                                            const LeadCloud& cc, float4 r, int w, unsigned long long& tested,
                                            unsigned long long& touched, bool& gave_up) {
    const uint32_t lane = threadIdx.x & 31;
    const float init = KD ? FLT_MAX : INFINITY;
    float4* const gP = a.P4 + cc.coff;  // my pieces' points (global memory)
    const uint32_t* const gL = a.LW + cc.coff;
    uint32_t(&wlo)[kLeadSlots][32] = S.wlo[w];  // low word of every slot's key
    uint32_t(&wpr)[kLeadSlots][32] = S.wpr[w];  // cloud-local start << 8 | length
    using Tab = LeadTable<HPW>;
    const uint32_t e0 = (uint32_t)w * HPW;  // my hot entries: e0 .. e0 + HPW - 1

    // slot j of lane l holds cloud piece (j * 32 + l) * kLeadWorkers + w
    // (neighbours in storage order go to different warps)
    float lo[kLeadSlots][D], hi[kLeadSlots][D];
    float kd[kLeadSlots];  // key distance (0 for an empty slot: never dirty)
    uint32_t valid = 0;    // slots holding a piece (bit j)
#pragma unroll
    for (int j = 0; j < kLeadSlots; ++j) {
        const uint32_t q = ((uint32_t)j * 32 + lane) * kLeadWorkers + (uint32_t)w;
        const bool have = q < cc.np;
        const uint64_t g = (uint64_t)cc.P0 + q;
        kd[j] = 0.0f;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            lo[j][d] = have ? a.plo[g * D + d] : INFINITY;
            hi[j][d] = have ? a.phi[g * D + d] : -INFINITY;
        }
        uint32_t v = 0;
        if (have) {
            const uint32_t ps = a.pstart[g], pe = a.pstart[g + 1];
            v = ((ps - (uint32_t)cc.coff) << 8) | (pe - ps);
            valid |= 1u << j;
        }
        wpr[j][lane] = v;
        wlo[j][lane] = 0;
    }
    __syncwarp();
    // full key of slot j (0 for an empty slot)
    auto full_key = [&](int j) -> uint64_t {
        return ((valid >> j) & 1u)
                   ? ((uint64_t)(__float_as_uint(kd[j]) | 0x80000000u) << 32) | wlo[j][lane]
                   : 0ull;
    };
    // recomputes the pieces of the slots set in `pend` (per lane, bit j) for
    // reference rr, one piece at a time (one call site)
    auto recompute = [&](uint32_t pend, const float4 rr, bool first) {
        while (__any_sync(kFull, pend != 0u)) {
            const int j = __ffs(__reduce_or_sync(kFull, pend)) - 1;
            const int l = __ffs(__ballot_sync(kFull, (pend >> j) & 1u)) - 1;
            const uint32_t v = wpr[j][l];
            const uint32_t ps = v >> 8, len = v & 0xffu;
            if (lane == 0) touched += len;
            const uint64_t k = first ? lead_update<D, FMA, true>(gP + ps, gL + ps, len, rr, init)
                                     : lead_update<D, FMA, false>(gP + ps, gL + ps, len, rr, init);
            if (lane == (uint32_t)l) {
#pragma unroll
                for (int jj = 0; jj < kLeadSlots; ++jj)
                    if (jj == j) kd[jj] = key_dist(k);
                wlo[j][l] = (uint32_t)k;
                pend &= ~(1u << j);
            }
        }
    };
    // the first reference reaches every piece
    recompute(valid, r, true);
    lead_bar();

    uint32_t hotm = 0;  // slots in the hot table (bit j)
    uint64_t hent = 0;  // their entries, 8 bits per slot
    uint32_t emitted = 1;
    while (emitted < cc.K) {
        // ---- my hot slots' keys come back (leader format -> mine)
#pragma unroll
        for (int j = 0; j < kLeadSlots; ++j) {
            if ((hotm >> j) & 1u) {
                const uint64_t k = S.hkey[(uint32_t)(hent >> (8 * j)) & 0xffu];
                const uint32_t q = ((uint32_t)j * 32 + lane) * kLeadWorkers + (uint32_t)w;
                kd[j] = key_dist(k);
                wlo[j][lane] = lead_pos_worker<KD>(lead_loc_leader<KD, HPW>((uint32_t)k)) | q;
            }
        }
        // ---- the new hot set: my HPW pieces of largest key
        uint32_t picked = 0;
        uint64_t fk[kLeadSlots];  // every slot's key, for the picks
#pragma unroll
        for (int j = 0; j < kLeadSlots; ++j) fk[j] = full_key(j);
        for (int i = 0; i < HPW; ++i) {
            uint64_t lk = 0;
            int lj = 0;
#pragma unroll
            for (int j = 0; j < kLeadSlots; ++j) {
                const uint64_t kj = ((picked >> j) & 1u) ? 0ull : fk[j];
                if (kj > lk) {
                    lk = kj;
                    lj = j;
                }
            }
            const uint64_t wk = warp_max_key(lk);
            const int owner = __ffs(__ballot_sync(kFull, wk != 0 && lk == wk)) - 1;
            if (lane == (uint32_t)owner) picked |= 1u << lj;
        }
        // entries: a slot that stays hot keeps its entry; the others free theirs
        uint32_t kept = 0;  // my entries (bit e - e0) still in use
#pragma unroll
        for (int j = 0; j < kLeadSlots; ++j)
            if ((hotm & picked) >> j & 1u) kept |= 1u << (((uint32_t)(hent >> (8 * j)) & 0xffu) - e0);
        kept = __reduce_or_sync(kFull, kept);
        // write back the freed entries the leader changed
        uint32_t freed = 0;
#pragma unroll
        for (int j = 0; j < kLeadSlots; ++j)
            if ((hotm & ~picked) >> j & 1u) freed |= 1u << (((uint32_t)(hent >> (8 * j)) & 0xffu) - e0);
        freed = __reduce_or_sync(kFull, freed);
        for (uint32_t fm = freed; fm; fm &= fm - 1) {
            const uint32_t e = e0 + __ffs(fm) - 1;
            if (!S.hmod[e]) continue;
            const uint32_t len = S.hlen[e], ps = S.hps[e];
            for (uint32_t p = lane; p < len; p += 32)
                reinterpret_cast<float*>(gP + ps + p)[3] = s_pt[e * kPiece + p].w;
        }
        // new picks take the free entries, lowest first
        uint32_t nfill = 0;
        {
            uint32_t freem = ~kept & ((1u << HPW) - 1);
            uint32_t nh = hotm & picked;
            uint64_t ne = 0;
#pragma unroll
            for (int j = 0; j < kLeadSlots; ++j)
                if ((hotm & picked) >> j & 1u) ne |= hent & (0xffull << (8 * j));
            uint32_t fresh = picked & ~hotm;  // per lane
            while (__any_sync(kFull, fresh != 0u)) {
                const int j = __ffs(__reduce_or_sync(kFull, fresh)) - 1;
                const int l = __ffs(__ballot_sync(kFull, (fresh >> j) & 1u)) - 1;
                const uint32_t ei = __ffs(freem) - 1;
                freem &= freem - 1;
                const uint32_t e = e0 + ei;
                if (lane == (uint32_t)l) {
                    nh |= 1u << j;
                    ne |= (uint64_t)e << (8 * j);
                    fresh &= ~(1u << j);
                    float4 l4 = make_float4(INFINITY, INFINITY, INFINITY, 0.0f);
                    float4 h4 = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.0f);
#pragma unroll
                    for (int jj = 0; jj < kLeadSlots; ++jj) {
                        if (jj == j) {
                            l4.x = lo[jj][0];
                            h4.x = hi[jj][0];
                            if (D > 1) {
                                l4.y = lo[jj][D > 1 ? 1 : 0];
                                h4.y = hi[jj][D > 1 ? 1 : 0];
                            }
                            if (D > 2) {
                                l4.z = lo[jj][D > 2 ? 2 : 0];
                                h4.z = hi[jj][D > 2 ? 2 : 0];
                            }
                        }
                    }
                    S.hlo[e] = l4;
                    S.hhi[e] = h4;
                    if constexpr (Tab::kEntryBits == 6) {
                        S.fill[w][nfill] = (e << 26) | wpr[j][l];
                    } else {
                        S.fill[w][nfill] = wpr[j][l];
                        S.fent[w][nfill] = (uint8_t)e;
                    }
                    S.fkey[w][nfill] = full_key(j);
                    S.hkey[e] = 0ull;  // set by the copy below
                }
                ++nfill;
            }
            // entries nobody holds now are empty
            for (uint32_t em = freem; em; em &= em - 1)
                if (lane == 0) S.hkey[e0 + __ffs(em) - 1] = 0ull;
            hotm = nh;
            hent = ne;
        }
        __syncwarp();
        // copy the new entries in, padded to kPiece with the last record, low
        // words in leader format (every load of an entry issued before the
        // first use: one round trip per entry); the record whose key is the
        // piece's key gives the entry its leader key
        for (uint32_t fi = 0; fi < nfill; ++fi) {
            const uint32_t f = S.fill[w][fi];
            const uint64_t fkey = S.fkey[w][fi];
            uint32_t e;
            if constexpr (Tab::kEntryBits == 6)
                e = f >> 26;
            else
                e = S.fent[w][fi];
            const uint32_t ps = (f >> 8) & kLeadPosMask, len = f & 0xffu;
            float4 x[kPiece / 32];
            uint32_t lw[kPiece / 32];
#pragma unroll
            for (int j = 0; j < kPiece / 32; ++j) {
                const uint32_t i = lane + 32 * j, ri = i < len ? i : len - 1;
                x[j] = gP[ps + ri];
                lw[j] = gL[ps + ri];
            }
#pragma unroll
            for (int j = 0; j < kPiece / 32; ++j) {
                const uint32_t i = lane + 32 * j, ri = i < len ? i : len - 1;
                const uint32_t ll = lead_pos_leader<KD, HPW>(lead_loc_worker<KD>(lw[j])) | (ri << Tab::kEntryBits) | e;
                s_pt[e * kPiece + i] = x[j];
                s_lw[e * kPiece + i] = ll;
                const uint64_t kk = ((uint64_t)(__float_as_uint(x[j].w) | 0x80000000u) << 32) | lw[j];
                if (i < len && kk == fkey) S.hkey[e] = (kk & 0xffffffff00000000ull) | ll;
            }
            if (lane == 0) {
                S.hlen[e] = len;
                S.hps[e] = ps;
                S.hmod[e] = 0;
            }
        }
        {
            uint64_t lt = 0;
#pragma unroll
            for (int j = 0; j < kLeadSlots; ++j) {
                const uint64_t kj = ((hotm >> j) & 1u) ? 0ull : full_key(j);
                lt = kj > lt ? kj : lt;
            }
            const uint64_t tw = warp_max_key(lt);
            if (lane == 0) S.T[w] = tw;
        }
        lead_bar();

        // ---- the epoch's references, in order, on the pieces I kept
        const uint32_t live = valid & ~hotm;
        if (__any_sync(kFull, live != 0u)) {
            uint32_t s = 0;
            for (;;) {
                uint32_t v = 0;
                long long spins = 0;
                for (;;) {
                    v = ld_acquire_cta_shared(&S.nref);
                    if ((v & ~kLeadDone) > s || (v & kLeadDone)) break;
                    if (++spins > a.spin_limit) {
                        gave_up = true;
                        break;
                    }
                    // the leader shares issue slots with the waiting warps
                    __nanosleep(64);
                }
                v = __shfl_sync(kFull, v, 0);
                if (__any_sync(kFull, gave_up)) break;
                const uint32_t cnt = v & ~kLeadDone;
                tested += (unsigned long long)__popc(live) * (cnt - s);
                for (; s < cnt; ++s) {
                    const float4 rr = S.ref[s];
                    const float rv[3] = {rr.x, rr.y, rr.z};
                    uint32_t dm = 0;
#pragma unroll
                    for (int j = 0; j < kLeadSlots; ++j)
                        if ((live >> j) & 1u) dm |= (uint32_t)(box_bound<D, FMA>(lo[j], hi[j], rv) < kd[j]) << j;
                    recompute(dm, rr, false);
                }
                if (v & kLeadDone) break;
            }
        }
        lead_bar();
        emitted = S.emitted;
        if (S.stall) break;
    }
}

// The leader warp on one cloud: per epoch, emit samples from the hot table
// while its best key beats T.  Reaches lead_bar() as often as lead_worker.
template <int D, bool FMA, bool KD, int HPW>
__device__ __forceinline__ void lead_leader(const LeadArgs& a, LeadShared<HPW>& S, float4* s_pt, uint32_t* s_lw,
                                            const LeadCloud& cc, unsigned long long& tested,
                                            unsigned long long& touched) {
    const uint32_t lane = threadIdx.x & 31;
    using Tab = LeadTable<HPW>;
    const bool has1 = lane + 32 < (uint32_t)Tab::kHot, has2 = Tab::kThree && lane + 64 < (uint32_t)Tab::kHot;
    S.hkey[lane] = 0ull;  // every entry starts empty
    S.hkey[lane + 32] = 0ull;
    if constexpr (Tab::kThree) S.hkey[lane + 64] = 0ull;
    if (lane == 0) S.stall = 0;
    lead_bar();  // the workers' first reference

    uint32_t emitted = 1;
    while (emitted < cc.K) {
        if (lane == 0) S.nref = 0;  // no worker reads it before the barrier below
        lead_bar();                 // the hot table is ready
        // T in leader format: the position decides ties, the rest is all ones
        uint64_t Tb = warp_max_key(lane < (uint32_t)kLeadWorkers ? S.T[lane] : 0ull);
        if (Tb) Tb = (Tb & 0xffffffff00000000ull) | lead_pos_leader<KD, HPW>(lead_loc_worker<KD>((uint32_t)Tb)) |
                       ((1u << Tab::kPosShift) - 1);
        uint64_t k0 = S.hkey[lane], k1 = has1 ? S.hkey[lane + 32] : 0ull, k2 = has2 ? S.hkey[lane + 64] : 0ull;
        const float4 l0 = S.hlo[lane], h0 = S.hhi[lane];
        const float4 l1 = has1 ? S.hlo[lane + 32] : make_float4(INFINITY, INFINITY, INFINITY, 0.0f);
        const float4 h1 = has1 ? S.hhi[lane + 32] : make_float4(-INFINITY, -INFINITY, -INFINITY, 0.0f);
        const float4 l2 = has2 ? S.hlo[lane + 64] : make_float4(INFINITY, INFINITY, INFINITY, 0.0f);
        const float4 h2 = has2 ? S.hhi[lane + 64] : make_float4(-INFINITY, -INFINITY, -INFINITY, 0.0f);
        const float lo0[3] = {l0.x, l0.y, l0.z}, hi0[3] = {h0.x, h0.y, h0.z};
        const float lo1[3] = {l1.x, l1.y, l1.z}, hi1[3] = {h1.x, h1.y, h1.z};
        const float lo2[3] = {l2.x, l2.y, l2.z}, hi2[3] = {h2.x, h2.y, h2.z};
        bool mod0 = false, mod1 = false, mod2 = false;
        uint32_t s = 0;
        // this lane's largest entry key
        auto lane_max = [&]() {
            const uint64_t m = k0 > k1 ? k0 : k1;
            if constexpr (Tab::kThree) return m > k2 ? m : k2;
            return m;
        };
        uint64_t wk = warp_max_key(lane_max());  // the best hot key (warp-uniform)
        while (!a.mute && emitted < cc.K && s < (uint32_t)kLeadRefs) {
            if (wk <= Tb) break;
            const uint32_t e = (uint32_t)wk & ((1u << Tab::kEntryBits) - 1), rec = ((uint32_t)wk >> Tab::kEntryBits) & 127u;
            float4* const ep = s_pt + e * kPiece;
            const uint32_t* const el = s_lw + e * kPiece;
            const float4 r = ep[rec];
            // the winner's entry is always dirty (its max point is r): its
            // loads go first, everything else below overlaps them
            float4 v[kPiece / 32];
            uint32_t w[kPiece / 32];
#pragma unroll
            for (int j = 0; j < kPiece / 32; ++j) {
                v[j] = ep[lane + 32 * j];
                w[j] = el[lane + 32 * j];
            }
            // publish (every lane stores the same values: no branch)
            S.outq[s] = lead_loc_leader<KD, HPW>((uint32_t)wk);
            S.ref[s] = r;
            st_release_cta_shared(&S.nref, s + 1);
            tested += lane == 0 ? (uint32_t)Tab::kHot : 0u;
            touched += lane == 0 ? kPiece : 0u;
            ++emitted;
            ++s;
            // the other entries' box tests do not depend on the winner's
            // recompute (branch-free, so they share its basic block)
            const bool o0 = lane != e, o1 = lane + 32 != e, o2 = lane + 64 != e;
            const uint64_t x0 = o0 ? k0 : 0ull, x1 = o1 ? k1 : 0ull, x2 = o2 ? k2 : 0ull;
            const float rv[3] = {r.x, r.y, r.z};
            const bool d0 = (x0 != 0) & (box_bound<D, FMA>(lo0, hi0, rv) < key_dist(x0));
            const bool d1 = (x1 != 0) & (box_bound<D, FMA>(lo1, hi1, rv) < key_dist(x1));
            const bool d2 = Tab::kThree && (x2 != 0) & (box_bound<D, FMA>(lo2, hi2, rv) < key_dist(x2));
            // the winner's recompute
            uint32_t bh[kPiece / 32];
#pragma unroll
            for (int j = 0; j < kPiece / 32; ++j) {
                const float dd = sqdist4<D, FMA>(v[j], r);
                const bool lower = dd < v[j].w;
                const float nv = lower ? dd : v[j].w;
                if (lower) reinterpret_cast<float*>(ep + lane + 32 * j)[3] = nv;
                bh[j] = __float_as_uint(nv) | 0x80000000u;
            }
            lead_pmax(bh[0], w[0], bh[1], w[1]);
            lead_pmax(bh[2], w[2], bh[3], w[3]);
            lead_pmax(bh[0], w[0], bh[2], w[2]);
            // One warp max over (the other entries' keys, this lane's best
            // record of the winner's entry) gives the next winner; an
            // independent one gives the winner entry's new key.  Their
            // reductions issue side by side.
            uint32_t ch = (uint32_t)(x0 >> 32), cl = (uint32_t)x0;
            lead_pmax(ch, cl, (uint32_t)(x1 >> 32), (uint32_t)x1);
            if constexpr (Tab::kThree) lead_pmax(ch, cl, (uint32_t)(x2 >> 32), (uint32_t)x2);
            lead_pmax(ch, cl, bh[0], w[0]);
            const uint32_t ah = __reduce_max_sync(kFull, ch);
            const uint32_t nh = __reduce_max_sync(kFull, bh[0]);
            const uint32_t al = __reduce_max_sync(kFull, ch == ah ? cl : 0u);
            const uint32_t nl = __reduce_max_sync(kFull, bh[0] == nh ? w[0] : 0u);
            const uint64_t nk = ((uint64_t)nh << 32) | nl;
            k0 = o0 ? k0 : nk;
            k1 = o1 ? k1 : nk;
            mod0 |= !o0;
            mod1 |= !o1;
            if constexpr (Tab::kThree) {
                k2 = o2 ? k2 : nk;
                mod2 |= !o2;
            }
            if (__any_sync(kFull, d0 || d1 || d2)) {
                // every other hot entry whose box is nearer than its key
                uint32_t m = __ballot_sync(kFull, d0);
                while (m) {
                    const uint32_t l = __ffs(m) - 1;
                    m &= m - 1;
                    touched += lane == 0 ? kPiece : 0u;
                    const uint64_t k = lead_update_hot<D, FMA>(s_pt + l * kPiece, s_lw + l * kPiece, r);
                    if (lane == l) {
                        k0 = k;
                        mod0 = true;
                    }
                }
                m = __ballot_sync(kFull, d1);
                while (m) {
                    const uint32_t l = __ffs(m) - 1;
                    m &= m - 1;
                    touched += lane == 0 ? kPiece : 0u;
                    const uint64_t k = lead_update_hot<D, FMA>(s_pt + (l + 32) * kPiece, s_lw + (l + 32) * kPiece, r);
                    if (lane == l) {
                        k1 = k;
                        mod1 = true;
                    }
                }
                if constexpr (Tab::kThree) {
                    m = __ballot_sync(kFull, d2);
                    while (m) {
                        const uint32_t l = __ffs(m) - 1;
                        m &= m - 1;
                        touched += lane == 0 ? kPiece : 0u;
                        const uint64_t k =
                            lead_update_hot<D, FMA>(s_pt + (l + 64) * kPiece, s_lw + (l + 64) * kPiece, r);
                        if (lane == l) {
                            k2 = k;
                            mod2 = true;
                        }
                    }
                }
                wk = warp_max_key(lane_max());
            } else {
                wk = ((uint64_t)ah << 32) | al;  // nothing else changed
            }
            __syncwarp();  // the lowered distances are visible to every lane
        }
        // this epoch's outputs: samples emitted - s .. emitted - 1
        for (uint32_t i = lane; i < s; i += 32) {
            const uint64_t o = cc.ooff + emitted - s + i;
            a.out[o] = KD ? S.outq[i] + cc.coff : S.outq[i];
            if (a.out_pts) {
                const float4 p = S.ref[i];
                a.out_pts[o * D] = p.x;
                if (D > 1) a.out_pts[o * D + (D > 1 ? 1 : 0)] = p.y;
                if (D > 2) a.out_pts[o * D + (D > 2 ? 2 : 0)] = p.z;
            }
        }
        S.hkey[lane] = k0;
        if (has1) {
            S.hkey[lane + 32] = k1;
            if (mod1) S.hmod[lane + 32] = 1;
        }
        if constexpr (Tab::kThree) {
            if (has2) {
                S.hkey[lane + 64] = k2;
                if (mod2) S.hmod[lane + 64] = 1;
            }
        }
        if (mod0) S.hmod[lane] = 1;
        if (lane == 0) {
            S.emitted = emitted;
            if (s == 0) S.stall = 1;  // cannot happen (but in the self-test): the best piece is always hot
            if (!a.mute) st_release_cta_shared(&S.nref, s | kLeadDone);
        }
        lead_bar();  // the workers have applied the epoch
        if (S.stall) break;
    }
}

template <int D, bool FMA, bool KD, int HPW>
__global__ void __launch_bounds__(kLeadThreads, 1) lead_sample(LeadArgs a) {
    constexpr uint32_t kHotPoints = (uint32_t)LeadTable<HPW>::kHot * kPiece;
    extern __shared__ __align__(16) unsigned char s_dyn[];
    __shared__ LeadShared<HPW> S;
    float4* s_pt = reinterpret_cast<float4*>(s_dyn);                  // [kHotPoints]
    uint32_t* s_lw = reinterpret_cast<uint32_t*>(s_pt + kHotPoints);  // [kHotPoints]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned long long tested = 0, touched = 0;
    bool gave_up = false;

    for (;;) {
        if (tid == 0) S.item = atomicAdd(a.queue, 1u);
        lead_bar();
        const uint32_t item = S.item;
        if (item >= a.n_items) break;
        const uint32_t c = a.order[item];
        LeadCloud cc;
        cc.P0 = a.cloud_piece[c];
        cc.np = a.cloud_piece[c + 1] - cc.P0;
        cc.K = a.cloud_k[c];
        cc.coff = a.cloud_off[c];
        cc.nc = (uint32_t)(a.cloud_off[c + 1] - cc.coff);
        cc.ooff = a.out_off[c];
        float4 r;
        {
            const uint32_t tag0 = (uint32_t)a.cloud_tag0[c];
            r.x = a.Xref[tag0];
            r.y = D > 1 ? a.Xref[a.n + tag0] : 0.0f;
            r.z = D > 2 ? a.Xref[2 * a.n + tag0] : 0.0f;
            r.w = 0.0f;
            if (tid == 0) a.out[cc.ooff] = KD ? tag0 : tag0 - cc.coff;
            if (a.out_pts && tid < D) a.out_pts[cc.ooff * D + tid] = tid == 0 ? r.x : tid == 1 ? r.y : r.z;
        }
        if (warp == 0)
            lead_leader<D, FMA, KD, HPW>(a, S, s_pt, s_lw, cc, tested, touched);
        else
            lead_worker<D, FMA, KD, HPW>(a, S, s_pt, s_lw, cc, r, warp - 1, tested, touched, gave_up);
        if (S.stall && tid == 0) atomicOr(a.err, kErrBadIndex);
        lead_bar();  // the leader's output writes are visible to the CTA
        if (KD) {
            // tags of this cloud map to its original indices; anything else is
            // reported, never dereferenced
            for (uint64_t i = tid; i < cc.K; i += kLeadThreads) {
                const uint64_t t = a.out[cc.ooff + i];
                const bool ok = t >= cc.coff && t < cc.coff + cc.nc;
                if (!ok) atomicOr(a.err, kErrBadIndex);
                a.out[cc.ooff + i] = ok ? a.idmap[t] - cc.coff : 0ull;
            }
        }
        lead_bar();  // nobody reads this cloud's state any more
    }
    if (gave_up && lane == 0 && a.err) atomicOr(a.err, kErrExchangeTimeout);
    if (a.counters) {
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
