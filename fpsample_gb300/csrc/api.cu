// C ABI of libfpsgpu (declared in include/fpsgpu.h) and the non-template
// device helpers shared by the kernel translation units.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "fpsgpu_device.cuh"
#include "fpsgpu_internal.h"
#include "engine.cuh"

static_assert(sizeof(size_t) == sizeof(uint64_t), "size_t must be 64-bit");

#define FPSGPU_VERSION_STRING "1.0.2+gb300.0.1"

// vanilla FPS on at most this many points runs the single-CTA brute-force
// kernel; larger clouds (dim <= 8) go through the pruned engine
constexpr uint64_t kVanillaBruteMax = 8192;

namespace fpsgpu {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
namespace {
thread_local std::string t_last_error;
}

int set_error(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_last_error = buf;
    return code;
}

void clear_error() { t_last_error.clear(); }

// ---------------------------------------------------------------------------
// device context: SM count and one non-blocking stream per device
// ---------------------------------------------------------------------------
namespace {
std::mutex g_ctx_mu;
std::vector<DevCtx> g_ctx;  // indexed by device ordinal; stream == nullptr until set up
}

int current_ctx(DevCtx* out) {
    int dev = 0;
    FPSGPU_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    if ((int)g_ctx.size() <= dev) g_ctx.resize(dev + 1);
    DevCtx& c = g_ctx[dev];
    if (c.stream == nullptr) {
        int sms = 0;
        FPSGPU_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        cudaStream_t s;
        FPSGPU_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        c.device = dev;
        c.sms = sms;
        c.stream = s;
    }
    *out = c;
    return FPSGPU_OK;
}

int launch_persistent(const void* func, int grid, int block, void** args, size_t smem,
                      cudaStream_t stream, bool cooperative) {
    stats_count_launch();
    if (cooperative && grid > kMaxGrid)
        return set_error(FPSGPU_ERR_ARG, "persistent grid of %d CTAs exceeds %d", grid, kMaxGrid);
    if (cooperative) {
        int dev = 0, sms = 0, per_sm = 0;
        FPSGPU_CUDA_TRY(cudaGetDevice(&dev));
        FPSGPU_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        FPSGPU_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, func, block, smem));
        if ((long long)per_sm * sms < grid)
            return set_error(FPSGPU_ERR_CUDA,
                             "persistent grid of %d CTAs cannot be co-resident (%d per SM x %d SMs)",
                             grid, per_sm, sms);
        FPSGPU_CUDA_TRY(cudaLaunchCooperativeKernel(func, dim3(grid), dim3(block), args, smem, stream));
    } else {
        FPSGPU_CUDA_TRY(cudaLaunchKernel(func, dim3(grid), dim3(block), args, smem, stream));
    }
    return FPSGPU_OK;
}

namespace {
thread_local cudaMemPool_t t_pool = nullptr;
std::mutex g_attr_mu;
std::set<std::pair<int, const void*>> g_smem_raised, g_cluster16;
}

// Kernel attributes are set once per (device, kernel) and never changed again:
// the dynamic shared-memory limit goes straight to the device's opt-in maximum,
// so concurrent calls (server workers) never change an attribute of a kernel
// that another stream is running.
int allow_max_smem(const void* func) {
    int dev = 0;
    FPSGPU_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_attr_mu);
    if (g_smem_raised.count({dev, func})) return FPSGPU_OK;
    int optin = 0;
    FPSGPU_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa{};
    FPSGPU_CUDA_TRY(cudaFuncGetAttributes(&fa, func));
    FPSGPU_CUDA_TRY(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         optin - (int)fa.sharedSizeBytes));
    g_smem_raised.insert({dev, func});
    return FPSGPU_OK;
}

int allow_cluster16(const void* func) {
    int dev = 0;
    FPSGPU_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_attr_mu);
    if (g_cluster16.count({dev, func})) return FPSGPU_OK;
    FPSGPU_CUDA_TRY(cudaFuncSetAttribute(func, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    g_cluster16.insert({dev, func});
    return FPSGPU_OK;
}
void set_thread_pool(cudaMemPool_t pool) { t_pool = pool; }

namespace {
// Scratch memory the library keeps mapped between calls on each device.  The
// device's default pool releases freed memory back to the system at every
// synchronisation (release threshold 0), so each call would map its scratch
// again: about 2 GB for a 16.7M-point cloud, several ms per call.
constexpr uint64_t kKeepMappedBytes = 8ull << 30;
std::mutex g_pool_mu;
std::vector<cudaMemPool_t> g_pools;  // per device; null until first use
}  // namespace

cudaMemPool_t thread_pool() {
    if (t_pool) return t_pool;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if ((int)g_pools.size() <= dev) g_pools.resize(dev + 1, nullptr);
    if (!g_pools[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
            (void)cudaGetLastError();
            return nullptr;  // fall back to the device's default pool
        }
        uint64_t keep = kKeepMappedBytes;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        g_pools[dev] = pool;
    }
    return g_pools[dev];
}

// Cluster size of the batched engine's cluster sampler: FPSGPU_CLUSTER_SIZE
// (1 turns clusters off; 2, 4, 8 or 16), default 8; clouds that need more CTAs
// get the next power of two up to 16.
bool lead_sampler_enabled() {
    static const bool v = [] {
        const char* e = std::getenv("FPSGPU_ONECTA_SAMPLER");
        return !(e && std::strcmp(e, "lockstep") == 0);
    }();
    return v;
}

int lead_hot_per_warp() {
    static const int v = [] {
        const char* e = std::getenv("FPSGPU_LEAD_HOT");
        if (!e) return 0;
        const int x = std::atoi(e);
        return x == 5 || x == 7 ? x : 0;
    }();
    return v;
}

int cluster_size_for_batch() {
    static const int v = [] {
        const char* e = std::getenv("FPSGPU_CLUSTER_SIZE");
        if (!e) return 8;
        const int x = std::atoi(e);
        return (x == 1 || x == 2 || x == 4 || x == 8 || x == 16) ? x : 8;
    }();
    return v;
}

// True when FPSGPU_CLUSTER_SIZE fixes the cluster size.  Otherwise a call whose
// clustered clouds all fit the GPU at 16 CTAs each takes 16: the SMs would sit
// idle anyway, and a 16-CTA cluster samples a 1M-point cloud about 4% faster
// than an 8-CTA one (fewer pieces per CTA; the exchange costs the same).
bool cluster_size_fixed() {
    static const bool v = std::getenv("FPSGPU_CLUSTER_SIZE") != nullptr;
    return v;
}

// FPSGPU_CLUSTER_MIN_PIECES: clouds with at least this many pieces run on a
// cluster even when one CTA could hold them (0, the default: only clouds that
// need it).  A tuning knob for batches whose largest clouds set the makespan.
uint32_t cluster_min_pieces() {
    static const uint32_t v = [] {
        const char* e = std::getenv("FPSGPU_CLUSTER_MIN_PIECES");
        if (!e) return 0u;
        const long x = std::atol(e);
        return x > 0 ? (uint32_t)x : 0u;
    }();
    return v;
}

// How many clusters of `cl` CTAs of `func` can be resident at once (0: none).
int cluster_capacity(const void* func, int cl, int block, size_t smem, int* out) {
    *out = 0;
    int rc;
    if (cl > 8 && (rc = allow_cluster16(func))) return rc;
    if ((rc = allow_max_smem(func))) return rc;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)cl;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)cl);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    const cudaError_t e = cudaOccupancyMaxActiveClusters(&n, func, &cfg);
    if (e != cudaSuccess) {  // e.g. a cluster size the device does not allow
        cudaGetLastError();
        return FPSGPU_OK;
    }
    *out = n;
    return FPSGPU_OK;
}

// Persistent cluster launch: min(items, resident clusters, max_ctas / cl)
// clusters of `cl` CTAs; the kernel's clusters take items from a queue.
int launch_clustered(const void* func, int items, int cl, int block, void** args, size_t smem,
                     cudaStream_t stream, int max_ctas) {
    int maxc = 0;
    int rc = cluster_capacity(func, cl, block, smem, &maxc);
    if (rc) return rc;
    if (maxc < 1) return set_error(FPSGPU_ERR_CUDA, "no cluster of %d CTAs fits on this GPU", cl);
    stats_count_launch();
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)cl;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    const int ncl = std::max(1, std::min({items, maxc, max_ctas > 0 ? max_ctas / cl : maxc}));
    cfg.gridDim = dim3((unsigned)(ncl * cl));
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    FPSGPU_CUDA_TRY(cudaLaunchKernelExC(&cfg, func, args));
    return FPSGPU_OK;
}

// ---------------------------------------------------------------------------
// measurement counters
// ---------------------------------------------------------------------------
namespace {
std::mutex g_stats_mu;
fpsgpu_stats g_stats{};
std::atomic<int> g_timing{0};
}  // namespace

void stats_count_launch(uint64_t n) {
    std::lock_guard<std::mutex> lk(g_stats_mu);
    g_stats.kernel_launches += n;
}

bool stats_timing_enabled() { return g_timing.load() != 0; }

void SamplerTimer::begin(cudaStream_t s) {
    on = stats_timing_enabled();
    if (!on) return;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        on = false;
        return;
    }
    cudaEventRecord(e0, s);
}

void SamplerTimer::end(cudaStream_t s) {
    if (on) cudaEventRecord(e1, s);
}

void SamplerTimer::finish(uint64_t samples, const uint64_t* c) {
    float ms = 0.0f;
    if (on) {
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
    }
    std::lock_guard<std::mutex> lk(g_stats_mu);
    g_stats.sampler_launches += 1;
    g_stats.sampler_ms += ms;
    g_stats.samples += samples;
    if (c) {
        g_stats.pieces_tested += c[0];
        g_stats.points_touched += c[1];
    }
}

SamplerTimer::~SamplerTimer() {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
}

// ---------------------------------------------------------------------------
// shared kernels
// ---------------------------------------------------------------------------
__global__ void transpose_to_soa(const float* __restrict__ pts, float* __restrict__ X, uint64_t n,
                                 int dim) {
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n;
         p += (uint64_t)gridDim.x * blockDim.x)
        for (int d = 0; d < dim; ++d) X[(uint64_t)d * n + p] = pts[p * dim + d];
}

__global__ void compact_count(const uint8_t* flag, uint64_t n, uint32_t* bcount) {
    const uint64_t lo = (uint64_t)blockIdx.x * kCompactChunk;
    uint64_t hi = lo + kCompactChunk;
    if (hi > n) hi = n;
    uint32_t c = 0;
    for (uint64_t p = lo + threadIdx.x; p < hi; p += blockDim.x) c += run_start(flag, p);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(kFull, c, o);
    __shared__ uint32_t s[32];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[w];
        bcount[blockIdx.x] = t;
    }
}

// single block: exclusive scan of bcount in place, total to *total
__global__ void compact_scan(uint32_t* bcount, uint32_t nblocks, uint32_t* total) {
    __shared__ uint32_t s_w[64];
    uint32_t carry = 0;
    int par = 0;
    for (uint32_t base = 0; base < nblocks; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < nblocks ? bcount[i] : 0u;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
        uint32_t x = v;  // inclusive scan within the warp
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t u = __shfl_up_sync(kFull, x, o);
            if (lane >= o) x += u;
        }
        uint32_t* w = s_w + par * 32;
        if (lane == 31) w[warp] = x;
        __syncthreads();
        const uint32_t c = lane < nwarps ? w[lane] : 0u;
        uint32_t y = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t u = __shfl_up_sync(kFull, y, o);
            if (lane >= o) y += u;
        }
        const uint32_t block_total = __shfl_sync(kFull, y, 31);
        const uint32_t warp_excl = __shfl_sync(kFull, y - c, warp);
        if (i < nblocks) bcount[i] = carry + warp_excl + (x - v);
        carry += block_total;
        par ^= 1;
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void compact_write(const uint8_t* flag, uint64_t n, const uint32_t* boff,
                              const uint32_t* total, uint32_t* starts) {
    __shared__ uint32_t s_w[64];
    const uint64_t lo = (uint64_t)blockIdx.x * kCompactChunk;
    uint64_t hi = lo + kCompactChunk;
    if (hi > n) hi = n;
    uint32_t running = boff[blockIdx.x];
    int par = 0;
    for (uint64_t base = lo; base < hi; base += blockDim.x) {
        const uint64_t p = base + threadIdx.x;
        const bool f = p < hi && run_start(flag, p);
        uint32_t tot;
        const uint32_t r = block_rank(f, s_w, par, tot);
        par ^= 1;
        if (f) starts[running + r] = (uint32_t)p;
        running += tot;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) starts[*total] = (uint32_t)n;
}

int compact_flags(const uint8_t* flag, uint64_t n, uint32_t* starts, uint32_t* d_count,
                  Scratch& sc, cudaStream_t stream) {
    const uint64_t nblocks = (n + kCompactChunk - 1) / kCompactChunk;
    uint32_t* bcount;
    int rc;
    if ((rc = sc.alloc(&bcount, nblocks))) return rc;
    stats_count_launch(3);
    compact_count<<<(unsigned)nblocks, 1024, 0, stream>>>(flag, n, bcount);
    FPSGPU_CUDA_TRY(cudaGetLastError());
    compact_scan<<<1, 1024, 0, stream>>>(bcount, (uint32_t)nblocks, d_count);
    FPSGPU_CUDA_TRY(cudaGetLastError());
    compact_write<<<(unsigned)nblocks, 1024, 0, stream>>>(flag, n, bcount, d_count, starts);
    FPSGPU_CUDA_TRY(cudaGetLastError());
    return FPSGPU_OK;
}

__global__ void map_tags(uint64_t* out, uint64_t k, const uint32_t* idmap, uint64_t id_offset) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < k;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = idmap[out[i]] - id_offset;
}

__global__ void cloud_piece_ranges(const uint32_t* pstart, const uint32_t* npieces,
                                   const uint64_t* cloud_off, uint32_t n_clouds, uint32_t* out) {
    const uint32_t np = *npieces;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c <= n_clouds;
         c += gridDim.x * blockDim.x) {
        const uint64_t key = cloud_off[c];
        uint32_t lo = 0, hi = np;  // first piece whose start >= key
        while (lo < hi) {
            const uint32_t mid = (lo + hi) / 2;
            if ((uint64_t)pstart[mid] < key) lo = mid + 1;
            else hi = mid;
        }
        out[c] = lo;
    }
}

__global__ void build_seed_refine(BuildArgs a) {
    const uint32_t m = *a.refine_cnt;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
        a.cur[i] = a.refine[i];
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.cnt_cur = m;
}

// ---------------------------------------------------------------------------
// floating-point mode
// ---------------------------------------------------------------------------
namespace {
std::once_flag g_mode_once;
// The default matches the reference as its own build recipe compiles it on
// this host's architecture: GCC fuses a*b+c by default and aarch64 has a fused
// multiply-add, so an aarch64 build contracts; the x86-64 baseline has no FMA
// instruction, so an x86-64 build cannot.
#if defined(__aarch64__)
int g_fp_mode = FPSGPU_FP_FMA;
#else
int g_fp_mode = FPSGPU_FP_NOFMA;
#endif
std::mutex g_mode_mu;

int fp_mode() {
    std::call_once(g_mode_once, [] {
        const char* e = std::getenv("FPSAMPLE_FP_MODE");
        if (e && (std::strcmp(e, "fma") == 0 || std::strcmp(e, "FMA") == 0)) g_fp_mode = FPSGPU_FP_FMA;
        if (e && (std::strcmp(e, "nofma") == 0 || std::strcmp(e, "NOFMA") == 0))
            g_fp_mode = FPSGPU_FP_NOFMA;
    });
    std::lock_guard<std::mutex> lk(g_mode_mu);
    return g_fp_mode;
}
}  // namespace

// Whether kernels on device `dev` may read pageable host memory through the
// host's page tables (hardware-coherent hosts such as Grace): then a kernel can
// gather host buffers itself.  Queried once per device.
int reads_host_page_tables(int dev, int* out) {
    static std::mutex mu;
    static std::vector<int> cache;  // -1: not queried yet
    std::lock_guard<std::mutex> lk(mu);
    if ((int)cache.size() <= dev) cache.resize(dev + 1, -1);
    if (cache[dev] < 0) {
        int pageable = 0, tables = 0;
        FPSGPU_CUDA_TRY(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev));
        FPSGPU_CUDA_TRY(
            cudaDeviceGetAttribute(&tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev));
        cache[dev] = pageable && tables ? 1 : 0;
    }
    *out = cache[dev];
    return FPSGPU_OK;
}

// dst[foff[c] + i] = src[c][i]: every cloud from its own host buffer into one
// device buffer (y: clouds, x: chunks of a cloud).
__global__ void gather_host_clouds(const float* const* src, const uint64_t* foff, uint32_t n_clouds,
                                   float* __restrict__ dst) {
    for (uint32_t c = blockIdx.y; c < n_clouds; c += gridDim.y) {
        const float* sc = src[c];
        const uint64_t b = foff[c], m = foff[c + 1] - b;
        for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
             i += (uint64_t)gridDim.x * blockDim.x)
            dst[b + i] = sc[i];
    }
}

namespace {
std::atomic<long long> g_alloc_budget{-1};
}  // namespace

bool scratch_alloc_refused() {
    long long v = g_alloc_budget.load();
    while (v >= 0) {
        if (v == 0) return true;
        if (g_alloc_budget.compare_exchange_weak(v, v - 1)) return false;
    }
    return false;
}

// Self-test of the grid exchange's bounded wait: ONE CTA runs exchange_leader
// for a grid of two, so the record of CTA 1 never arrives; the leader must give
// up after `limit` polls, set the error word and return.
__global__ void selftest_exchange_timeout(uint64_t* slots, int* err, long long limit) {
    if (threadIdx.x < 32) {
        const float c[3] = {0.0f, 0.0f, 0.0f};
        float w[3];
        (void)exchange_leader<3>(slots, slots + 2 * leader_words<3>(), 2, 0u, 1ull, c, w, err, limit);
    }
}

}  // namespace fpsgpu

using namespace fpsgpu;

namespace {

int resolve_stream(void* stream, DevCtx* ctx, cudaStream_t* out) {
    int rc = current_ctx(ctx);
    if (rc) return rc;
    *out = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    return FPSGPU_OK;
}

// One cloud, one start, no trace: the batched engine with a single cloud.  A
// cloud whose pieces fit one CTA's registers is sampled by one CTA with a
// __syncthreads per sample instead of a grid-wide exchange (about 1.6x less time
// per sample up to ~250K points); a larger cloud falls through to the same
// multi-CTA sampler run_engine uses.  Results are identical either way.
int single_via_batch(const float* d_points, size_t n, size_t dim, size_t k, size_t start,
                     size_t height, bool kd, uint64_t* d_out, cudaStream_t stream, int sms,
                     bool tie_last = false, float* d_out_pts = nullptr) {
    BatchCall b;
    b.tie_last = tie_last;
    b.d_out_pts = d_out_pts;
    b.d_points = d_points;
    b.off = {0, (uint64_t)n};
    b.k = {(uint64_t)k};
    b.start = {(uint64_t)start};
    b.height = {(uint64_t)height};
    b.kd = kd;
    b.d_out = d_out;
    b.stream = stream;
    b.sms = sms;
    return fp_mode() == FPSGPU_FP_FMA ? run_batch_fma((int)dim, b) : run_batch_nofma((int)dim, b);
}

int fps_device_impl(const float* d_points, size_t n, size_t dim, size_t k, const size_t* h_start,
                    size_t n_start, uint64_t* d_out, float* d_trace, cudaStream_t stream, int sms,
                    float* d_out_pts = nullptr) {
    VanillaCall c{};
    c.d_out_pts = d_out_pts;
    c.d_points = d_points;
    c.n = n;
    c.dim = (int)dim;
    c.k = k;
    c.h_starts = reinterpret_cast<const uint64_t*>(h_start);
    c.n_starts = (uint32_t)n_start;
    c.d_out = d_out;
    c.d_trace = d_trace;
    c.stream = stream;
    c.sms = sms;
    if (dim <= 8 && n > kVanillaBruteMax) {
        if (n_start == 1 && d_trace == nullptr)
            return single_via_batch(d_points, n, dim, k, h_start[0], 0, false, d_out, stream, sms,
                                    false, d_out_pts);
        EngineCall e{};
        e.d_out_pts = d_out_pts;
        e.d_points = d_points;
        e.n = n;
        e.k = k;
        e.kd = false;
        e.h_forced = reinterpret_cast<const uint64_t*>(h_start);
        e.n_forced = (uint32_t)n_start;
        e.d_out = d_out;
        e.d_trace = d_trace;
        e.stream = stream;
        e.sms = sms;
        return fp_mode() == FPSGPU_FP_FMA ? run_engine_fma((int)dim, e) : run_engine_nofma((int)dim, e);
    }
    return fp_mode() == FPSGPU_FP_FMA ? run_vanilla_fma(c) : run_vanilla_nofma(c);
}

int check_fps_args(size_t n, size_t dim, size_t k, const size_t* start, size_t n_start) {
    if (n == 0) return set_error(FPSGPU_ERR_ARG, "n_points must be >= 1");
    if (dim == 0) return set_error(FPSGPU_ERR_DIM, "dim must be >= 1");
    if (dim > 4096) return set_error(FPSGPU_ERR_DIM, "dim must be <= 4096, got %zu", dim);
    if (n > 0xfffffffeull) return set_error(FPSGPU_ERR_ARG, "n_points must be < 2^32 - 1");
    if (n_start == 0 || start == nullptr) return set_error(FPSGPU_ERR_ARG, "need at least one start index");
    if (k > 0 && n_start > k)
        return set_error(FPSGPU_ERR_ARG, "more start indices (%zu) than samples (%zu)", n_start, k);
    if (n_start > 0xffffffffull) return set_error(FPSGPU_ERR_ARG, "too many start indices");
    for (size_t i = 0; i < n_start; ++i)
        if (start[i] >= n)
            return set_error(FPSGPU_ERR_START, "start index %zu out of range (n_points=%zu)", start[i], n);
    return FPSGPU_OK;
}

int check_kdline_args(size_t n, size_t dim, size_t start) {
    if (dim == 0 || dim > 8) return set_error(FPSGPU_ERR_DIM, "dim must be in [1, 8], got %zu", dim);
    if (start >= n) return set_error(FPSGPU_ERR_START, "start_idx %zu out of range (n_points=%zu)", start, n);
    if (n > 0xfffffffeull) return set_error(FPSGPU_ERR_ARG, "n_points must be < 2^32 - 1");
    return FPSGPU_OK;
}

// tie_last: bucket_fps_kdtree, the same engine with no height limit and ties
// to the last position of the tree's order.
int kdline_device_impl(const float* d_points, size_t n, size_t dim, size_t k, size_t start,
                       size_t height, uint64_t* d_out, float* d_trace, cudaStream_t stream, int sms,
                       bool tie_last = false, float* d_out_pts = nullptr) {
    if (d_trace == nullptr)
        return single_via_batch(d_points, n, dim, k, start, height, true, d_out, stream, sms,
                                tie_last, d_out_pts);
    const uint64_t forced = start;
    EngineCall c{};
    c.tie_last = tie_last;
    c.d_out_pts = d_out_pts;
    c.d_points = d_points;
    c.n = n;
    c.k = k;
    c.kd = true;
    c.height = height;
    c.h_forced = &forced;
    c.n_forced = 1;
    c.d_out = d_out;
    c.d_trace = d_trace;
    c.stream = stream;
    c.sms = sms;
    return fp_mode() == FPSGPU_FP_FMA ? run_engine_fma((int)dim, c) : run_engine_nofma((int)dim, c);
}

}  // namespace

extern "C" {

void fpsgpu_stats_reset(void) {
    std::lock_guard<std::mutex> lk(g_stats_mu);
    g_stats = fpsgpu_stats{};
}

void fpsgpu_stats_get(fpsgpu_stats* out) {
    std::lock_guard<std::mutex> lk(g_stats_mu);
    *out = g_stats;
}

void fpsgpu_stats_timing(int enable) { g_timing.store(enable ? 1 : 0); }

const char* fpsgpu_last_error(void) { return t_last_error.c_str(); }

const char* fpsgpu_version(void) { return FPSGPU_VERSION_STRING; }

int fpsgpu_set_fp_mode(int mode) {
    if (mode != FPSGPU_FP_NOFMA && mode != FPSGPU_FP_FMA)
        return set_error(FPSGPU_ERR_ARG, "unknown fp mode %d", mode);
    fp_mode();  // consume the environment default first
    std::lock_guard<std::mutex> lk(g_mode_mu);
    g_fp_mode = mode;
    return FPSGPU_OK;
}

int fpsgpu_get_fp_mode(void) { return fp_mode(); }

int fpsgpu_fps_device(const float* d_points, size_t n_points, size_t dim, size_t n_samples,
                      const size_t* h_start, size_t n_start, uint64_t* d_out, float* d_trace,
                      void* stream) {
    clear_error();
    int rc = check_fps_args(n_points, dim, n_samples, h_start, n_start);
    if (rc) return rc;
    if (n_samples == 0) return FPSGPU_OK;
    DevCtx ctx;
    cudaStream_t s;
    if ((rc = resolve_stream(stream, &ctx, &s))) return rc;
    return fps_device_impl(d_points, n_points, dim, n_samples, h_start, n_start, d_out, d_trace, s,
                           ctx.sms);
}

int fpsgpu_fps(const float* raw_data, size_t n_points, size_t dim, size_t n_samples,
               const size_t* start_idx, size_t n_start, size_t* sampled_point_indices) {
    clear_error();
    int rc = check_fps_args(n_points, dim, n_samples, start_idx, n_start);
    if (rc) return rc;
    if (n_samples == 0) return FPSGPU_OK;
    DevCtx ctx;
    if ((rc = current_ctx(&ctx))) return rc;
    Scratch sc(ctx.stream);
    float* d_pts;
    uint64_t* d_out;
    if ((rc = sc.alloc(&d_pts, n_points * dim))) return rc;
    if ((rc = sc.alloc(&d_out, n_samples))) return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_pts, raw_data, n_points * dim * sizeof(float),
                                    cudaMemcpyHostToDevice, ctx.stream));
    if ((rc = fps_device_impl(d_pts, n_points, dim, n_samples, start_idx, n_start, d_out, nullptr,
                              ctx.stream, ctx.sms)))
        return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(sampled_point_indices, d_out, n_samples * sizeof(uint64_t),
                                    cudaMemcpyDeviceToHost, ctx.stream));
    FPSGPU_CUDA_TRY(cudaStreamSynchronize(ctx.stream));
    return FPSGPU_OK;
}

int fpsgpu_kdline_device(const float* d_points, size_t n_points, size_t dim, size_t n_samples,
                         size_t start_idx, size_t height, uint64_t* d_out, float* d_trace,
                         void* stream) {
    clear_error();
    int rc = check_kdline_args(n_points, dim, start_idx);
    if (rc) return rc;
    if (n_samples == 0) return FPSGPU_OK;
    DevCtx ctx;
    cudaStream_t s;
    if ((rc = resolve_stream(stream, &ctx, &s))) return rc;
    return kdline_device_impl(d_points, n_points, dim, n_samples, start_idx, height, d_out, d_trace,
                              s, ctx.sms);
}

int bucket_fps_kdline(const float* raw_data, size_t n_points, size_t dim, size_t n_samples,
                      size_t start_idx, size_t height, size_t* sampled_point_indices) {
    clear_error();
    int rc = check_kdline_args(n_points, dim, start_idx);
    if (rc) return rc;
    if (n_samples == 0) return FPSGPU_OK;
    DevCtx ctx;
    if ((rc = current_ctx(&ctx))) return rc;
    Scratch sc(ctx.stream);
    float* d_pts;
    uint64_t* d_out;
    if ((rc = sc.alloc(&d_pts, n_points * dim))) return rc;
    if ((rc = sc.alloc(&d_out, n_samples))) return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_pts, raw_data, n_points * dim * sizeof(float),
                                    cudaMemcpyHostToDevice, ctx.stream));
    if ((rc = kdline_device_impl(d_pts, n_points, dim, n_samples, start_idx, height, d_out, nullptr,
                                 ctx.stream, ctx.sms)))
        return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(sampled_point_indices, d_out, n_samples * sizeof(uint64_t),
                                    cudaMemcpyDeviceToHost, ctx.stream));
    FPSGPU_CUDA_TRY(cudaStreamSynchronize(ctx.stream));
    return FPSGPU_OK;
}

int fpsgpu_kdtree_device(const float* d_points, size_t n_points, size_t dim, size_t n_samples,
                         size_t start_idx, uint64_t* d_out, float* d_trace, void* stream) {
    clear_error();
    int rc = check_kdline_args(n_points, dim, start_idx);
    if (rc) return rc;
    if (n_samples == 0) return FPSGPU_OK;
    DevCtx ctx;
    cudaStream_t s;
    if ((rc = resolve_stream(stream, &ctx, &s))) return rc;
    return kdline_device_impl(d_points, n_points, dim, n_samples, start_idx, ~(size_t)0, d_out,
                              d_trace, s, ctx.sms, true);
}

int bucket_fps_kdtree(const float* raw_data, size_t n_points, size_t dim, size_t n_samples,
                      size_t start_idx, size_t* sampled_point_indices) {
    clear_error();
    int rc = check_kdline_args(n_points, dim, start_idx);
    if (rc) return rc;
    if (n_samples == 0) return FPSGPU_OK;
    DevCtx ctx;
    if ((rc = current_ctx(&ctx))) return rc;
    Scratch sc(ctx.stream);
    float* d_pts;
    uint64_t* d_out;
    if ((rc = sc.alloc(&d_pts, n_points * dim))) return rc;
    if ((rc = sc.alloc(&d_out, n_samples))) return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_pts, raw_data, n_points * dim * sizeof(float),
                                    cudaMemcpyHostToDevice, ctx.stream));
    if ((rc = kdline_device_impl(d_pts, n_points, dim, n_samples, start_idx, ~(size_t)0, d_out,
                                 nullptr, ctx.stream, ctx.sms, true)))
        return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(sampled_point_indices, d_out, n_samples * sizeof(uint64_t),
                                    cudaMemcpyDeviceToHost, ctx.stream));
    FPSGPU_CUDA_TRY(cudaStreamSynchronize(ctx.stream));
    return FPSGPU_OK;
}

int fpsgpu_kdline_batch_device(const float* d_points, const size_t* h_offsets, size_t n_clouds,
                               size_t dim, const size_t* h_n_samples, const size_t* h_start_idx,
                               const size_t* h_height, uint64_t* d_out, void* stream) {
    return fpsgpu::kdline_batch_device_capped(d_points, h_offsets, n_clouds, dim, h_n_samples,
                                              h_start_idx, h_height, d_out, stream, 0, nullptr);
}

int fpsgpu_kdline_batch_points_device(const float* d_points, const size_t* h_offsets,
                                      size_t n_clouds, size_t dim, const size_t* h_n_samples,
                                      const size_t* h_start_idx, const size_t* h_height,
                                      uint64_t* d_out, float* d_out_points, void* stream) {
    return fpsgpu::kdline_batch_device_capped(d_points, h_offsets, n_clouds, dim, h_n_samples,
                                              h_start_idx, h_height, d_out, stream, 0, d_out_points);
}

int fpsgpu_sample_points_device(int algo, const float* d_points, size_t n_points, size_t dim,
                                size_t n_samples, const size_t* h_start, size_t n_start,
                                size_t height, uint64_t* d_out, float* d_out_points, void* stream) {
    clear_error();
    int rc;
    if (algo == FPSGPU_ALGO_FPS) {
        if ((rc = check_fps_args(n_points, dim, n_samples, h_start, n_start))) return rc;
    } else if (algo == FPSGPU_ALGO_KDLINE || algo == FPSGPU_ALGO_KDTREE) {
        if (!h_start || n_start != 1)
            return set_error(FPSGPU_ERR_ARG, "kd-line and kd-tree take exactly one start index");
        if ((rc = check_kdline_args(n_points, dim, h_start[0]))) return rc;
    } else {
        return set_error(FPSGPU_ERR_ARG, "unknown algorithm %d", algo);
    }
    if (n_samples == 0) return FPSGPU_OK;
    DevCtx ctx;
    cudaStream_t s;
    if ((rc = resolve_stream(stream, &ctx, &s))) return rc;
    if (algo == FPSGPU_ALGO_FPS)
        return fps_device_impl(d_points, n_points, dim, n_samples, h_start, n_start, d_out, nullptr,
                               s, ctx.sms, d_out_points);
    const bool tree = algo == FPSGPU_ALGO_KDTREE;
    return kdline_device_impl(d_points, n_points, dim, n_samples, h_start[0],
                              tree ? ~(size_t)0 : height, d_out, nullptr, s, ctx.sms, tree,
                              d_out_points);
}

int fpsgpu_sample_points(int algo, const float* raw_data, size_t n_points, size_t dim,
                         size_t n_samples, const size_t* start_idx, size_t n_start, size_t height,
                         size_t* sampled_point_indices, float* sampled_points) {
    clear_error();
    if (n_samples == 0) return FPSGPU_OK;
    if (!raw_data || !sampled_point_indices) return set_error(FPSGPU_ERR_ARG, "null argument");
    DevCtx ctx;
    int rc;
    if ((rc = current_ctx(&ctx))) return rc;
    Scratch sc(ctx.stream);
    float* d_pts;
    uint64_t* d_out;
    float* d_xyz = nullptr;
    if ((rc = sc.alloc(&d_pts, n_points * (dim ? dim : 1)))) return rc;
    if ((rc = sc.alloc(&d_out, n_samples))) return rc;
    if (sampled_points && (rc = sc.alloc(&d_xyz, n_samples * (dim ? dim : 1)))) return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_pts, raw_data, n_points * dim * sizeof(float),
                                    cudaMemcpyHostToDevice, ctx.stream));
    if ((rc = fpsgpu_sample_points_device(algo, d_pts, n_points, dim, n_samples, start_idx, n_start,
                                          height, d_out, d_xyz, ctx.stream)))
        return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(sampled_point_indices, d_out, n_samples * sizeof(uint64_t),
                                    cudaMemcpyDeviceToHost, ctx.stream));
    if (sampled_points)
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(sampled_points, d_xyz, n_samples * dim * sizeof(float),
                                        cudaMemcpyDeviceToHost, ctx.stream));
    FPSGPU_CUDA_TRY(cudaStreamSynchronize(ctx.stream));
    return FPSGPU_OK;
}

}  // extern "C"

namespace fpsgpu {
int kdline_batch_device_capped(const float* d_points, const size_t* h_offsets, size_t n_clouds,
                               size_t dim, const size_t* h_n_samples, const size_t* h_start_idx,
                               const size_t* h_height, uint64_t* d_out, void* stream,
                               int max_grid, float* d_out_pts, int min_cluster) {
    clear_error();
    if (n_clouds == 0) return FPSGPU_OK;
    if (!h_offsets || !h_n_samples || !h_start_idx || !h_height)
        return set_error(FPSGPU_ERR_ARG, "null argument");
    if (dim == 0 || dim > 8) return set_error(FPSGPU_ERR_DIM, "dim must be in [1, 8], got %zu", dim);
    if (h_offsets[0] != 0) return set_error(FPSGPU_ERR_ARG, "offsets[0] must be 0");
    if (h_offsets[n_clouds] > 0xfffffffeull)
        return set_error(FPSGPU_ERR_ARG, "at most 2^32 - 2 points in one batch");
    for (size_t c = 0; c < n_clouds; ++c) {
        const size_t nc = h_offsets[c + 1] - h_offsets[c];
        if (h_offsets[c + 1] < h_offsets[c] || nc == 0)
            return set_error(FPSGPU_ERR_ARG, "cloud %zu is empty or offsets decrease", c);
        if (h_start_idx[c] >= nc)
            return set_error(FPSGPU_ERR_START, "cloud %zu: start_idx %zu out of range (n=%zu)", c,
                             h_start_idx[c], nc);
    }
    DevCtx ctx;
    cudaStream_t s;
    int rc;
    if ((rc = resolve_stream(stream, &ctx, &s))) return rc;
    BatchCall b;
    b.d_points = d_points;
    b.off.assign(h_offsets, h_offsets + n_clouds + 1);
    b.k.assign(h_n_samples, h_n_samples + n_clouds);
    b.start.assign(h_start_idx, h_start_idx + n_clouds);
    b.height.assign(h_height, h_height + n_clouds);
    b.kd = true;
    b.d_out = d_out;
    b.d_out_pts = d_out_pts;
    b.min_cluster = min_cluster;
    b.stream = s;
    b.sms = max_grid > 0 && max_grid < ctx.sms ? max_grid : ctx.sms;
    return fp_mode() == FPSGPU_FP_FMA ? run_batch_fma((int)dim, b) : run_batch_nofma((int)dim, b);
}
}  // namespace fpsgpu

extern "C" {

int fpsgpu_kdline_batch(const float* raw_data, const size_t* offsets, size_t n_clouds, size_t dim,
                        const size_t* n_samples, const size_t* start_idx, const size_t* height,
                        size_t* sampled_point_indices) {
    clear_error();
    if (n_clouds == 0) return FPSGPU_OK;
    if (!offsets || !n_samples) return set_error(FPSGPU_ERR_ARG, "null argument");
    DevCtx ctx;
    int rc;
    if ((rc = current_ctx(&ctx))) return rc;
    Scratch sc(ctx.stream);
    const size_t n = offsets[n_clouds];
    size_t ktot = 0;
    for (size_t c = 0; c < n_clouds; ++c) ktot += n_samples[c];
    float* d_pts;
    uint64_t* d_out;
    if ((rc = sc.alloc(&d_pts, n * (dim ? dim : 1)))) return rc;
    if ((rc = sc.alloc(&d_out, ktot))) return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_pts, raw_data, n * dim * sizeof(float),
                                    cudaMemcpyHostToDevice, ctx.stream));
    if ((rc = fpsgpu_kdline_batch_device(d_pts, offsets, n_clouds, dim, n_samples, start_idx,
                                         height, d_out, ctx.stream)))
        return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(sampled_point_indices, d_out, ktot * sizeof(uint64_t),
                                    cudaMemcpyDeviceToHost, ctx.stream));
    FPSGPU_CUDA_TRY(cudaStreamSynchronize(ctx.stream));
    return FPSGPU_OK;
}

int fpsgpu_kdline_batch_list(const float* const* clouds, const size_t* n_points, size_t n_clouds,
                             size_t dim, const size_t* n_samples, const size_t* start_idx,
                             const size_t* height, size_t* sampled_point_indices) {
    clear_error();
    if (n_clouds == 0) return FPSGPU_OK;
    if (!clouds || !n_points || !n_samples) return set_error(FPSGPU_ERR_ARG, "null argument");
    if (dim == 0 || dim > 8) return set_error(FPSGPU_ERR_DIM, "dim must be in [1, 8], got %zu", dim);
    std::vector<size_t> off(n_clouds + 1, 0);
    std::vector<uint64_t> foff(n_clouds + 1, 0);  // in floats
    size_t ktot = 0, max_f = 0;
    for (size_t c = 0; c < n_clouds; ++c) {
        if (n_points[c] > 0 && clouds[c] == nullptr)
            return set_error(FPSGPU_ERR_ARG, "cloud %zu has points but a null buffer", c);
        off[c + 1] = off[c] + n_points[c];
        foff[c + 1] = foff[c] + (uint64_t)n_points[c] * dim;
        max_f = std::max<size_t>(max_f, n_points[c] * dim);
        ktot += n_samples[c];
    }
    DevCtx ctx;
    int rc;
    if ((rc = current_ctx(&ctx))) return rc;
    Scratch sc(ctx.stream);
    const size_t n = off[n_clouds];
    float* d_pts;
    uint64_t* d_out;
    if ((rc = sc.alloc(&d_pts, n * dim))) return rc;
    if ((rc = sc.alloc(&d_out, ktot))) return rc;
    int host_tables = 0;
    if ((rc = reads_host_page_tables(ctx.device, &host_tables))) return rc;
    if (host_tables) {
        // one kernel reads every cloud from its own host buffer
        const float** d_src;
        uint64_t* d_foff;
        if ((rc = sc.alloc(&d_src, n_clouds))) return rc;
        if ((rc = sc.alloc(&d_foff, n_clouds + 1))) return rc;
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_src, clouds, n_clouds * sizeof(float*), cudaMemcpyHostToDevice,
                                        ctx.stream));
        FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_foff, foff.data(), (n_clouds + 1) * sizeof(uint64_t),
                                        cudaMemcpyHostToDevice, ctx.stream));
        const unsigned gx = (unsigned)std::min<size_t>((max_f + 2047) / 2048, 512);
        const unsigned gy = (unsigned)std::min<size_t>(n_clouds, 65535);
        stats_count_launch();
        gather_host_clouds<<<dim3(std::max(1u, gx), gy), 256, 0, ctx.stream>>>(d_src, d_foff,
                                                                            (uint32_t)n_clouds, d_pts);
        FPSGPU_CUDA_TRY(cudaGetLastError());
    } else {
        for (size_t c = 0; c < n_clouds; ++c)
            if (n_points[c] > 0)
                FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_pts + foff[c], clouds[c],
                                                n_points[c] * dim * sizeof(float),
                                                cudaMemcpyHostToDevice, ctx.stream));
    }
    if ((rc = fpsgpu_kdline_batch_device(d_pts, off.data(), n_clouds, dim, n_samples, start_idx,
                                         height, d_out, ctx.stream)))
        return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(sampled_point_indices, d_out, ktot * sizeof(uint64_t),
                                    cudaMemcpyDeviceToHost, ctx.stream));
    FPSGPU_CUDA_TRY(cudaStreamSynchronize(ctx.stream));
    return FPSGPU_OK;
}

int fpsgpu_selftest_exchange_timeout(void) {
    clear_error();
    DevCtx ctx;
    int rc;
    if ((rc = current_ctx(&ctx))) return rc;
    Scratch sc(ctx.stream);
    uint64_t* slots;
    int* err;
    const size_t nslots = 2 * leader_words<3>() + leader_words<3>();
    if ((rc = sc.alloc(&slots, nslots))) return rc;
    if ((rc = sc.alloc(&err, 1))) return rc;
    FPSGPU_CUDA_TRY(cudaMemsetAsync(slots, 0, nslots * sizeof(uint64_t), ctx.stream));
    FPSGPU_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), ctx.stream));
    stats_count_launch();
    selftest_exchange_timeout<<<1, 32, 0, ctx.stream>>>(slots, err, 4096);
    FPSGPU_CUDA_TRY(cudaGetLastError());
    return check_device_error(err, ctx.stream);
}

int fpsgpu_selftest_lead_timeout(void) {
    clear_error();
    DevCtx ctx;
    int rc;
    if ((rc = current_ctx(&ctx))) return rc;
    // one 20,000-point cloud: more pieces than the hot table, so that the
    // workers keep some and wait for the (muted) leader
    const size_t n = 20000, dim = 3;
    std::vector<float> pts(n * dim);
    uint32_t x = 12345u;
    for (float& v : pts) {
        x = x * 1664525u + 1013904223u;
        v = (float)(x >> 8) * (1.0f / 16777216.0f);
    }
    Scratch sc(ctx.stream);
    float* d_pts;
    uint64_t* d_out;
    if ((rc = sc.alloc(&d_pts, n * dim))) return rc;
    if ((rc = sc.alloc(&d_out, n / 4))) return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_pts, pts.data(), n * dim * sizeof(float), cudaMemcpyHostToDevice,
                                    ctx.stream));
    BatchCall b;
    b.d_points = d_pts;
    b.off = {0, n};
    b.k = {n / 4};
    b.start = {0};
    b.height = {5};
    b.kd = true;
    b.d_out = d_out;
    b.stream = ctx.stream;
    b.sms = ctx.sms;
    b.lead_selftest = true;
    rc = fp_mode() == FPSGPU_FP_FMA ? run_batch_fma((int)dim, b) : run_batch_nofma((int)dim, b);
    FPSGPU_CUDA_TRY(cudaStreamSynchronize(ctx.stream));
    return rc;
}

void fpsgpu_debug_fail_allocations(long long after) { g_alloc_budget.store(after < 0 ? -1 : after); }

int fpsgpu_kdline_build(const float* raw_data, size_t n_points, size_t dim, size_t height,
                        uint64_t* h_perm, uint64_t* h_bucket_start, size_t* n_buckets) {
    clear_error();
    int rc = check_kdline_args(n_points, dim, 0);
    if (rc) return rc;
    if (!h_perm || !h_bucket_start || !n_buckets) return set_error(FPSGPU_ERR_ARG, "null output");
    DevCtx ctx;
    if ((rc = current_ctx(&ctx))) return rc;
    Scratch sc(ctx.stream);
    float* d_pts;
    if ((rc = sc.alloc(&d_pts, n_points * dim))) return rc;
    FPSGPU_CUDA_TRY(cudaMemcpyAsync(d_pts, raw_data, n_points * dim * sizeof(float),
                                    cudaMemcpyHostToDevice, ctx.stream));
    const uint64_t forced = 0;
    EngineCall c{};
    c.d_points = d_pts;
    c.n = n_points;
    c.kd = true;
    c.height = height;
    c.h_forced = &forced;
    c.n_forced = 1;
    c.stream = ctx.stream;
    c.sms = ctx.sms;
    c.h_perm = h_perm;
    c.h_bucket_start = h_bucket_start;
    c.h_n_buckets = n_buckets;
    return fp_mode() == FPSGPU_FP_FMA ? run_engine_fma((int)dim, c) : run_engine_nofma((int)dim, c);
}

}  // extern "C"
