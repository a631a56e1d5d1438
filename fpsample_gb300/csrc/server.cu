// Request server: QuickFPS as a service with continuous batching.
//
// Clients submit one cloud per request (host buffers) at any time.  Worker
// threads, each with its own CUDA stream, repeatedly take every request that is
// waiting in their size class -- as long as it fits in the device-memory
// budget -- and run them as one batch through the batched engine
// (fpsgpu_kdline_batch_device); requests that arrive while a batch is on the
// GPU are picked up by the next free worker, so work from different batches
// overlaps on the device.  Each request's points, running distances and piece
// state stay on the device until its K samples are done; then its indices are
// copied back and the request completes.  Results are identical to one
// bucket_fps_kdline call per request: the batched engine is exact per cloud.
//
// Size classes keep small requests from waiting behind very large ones:
// requests of at most kSmallPoints points go to the "small" workers, the rest
// to the "large" workers, and a batch only gathers requests of similar sample
// counts.  Each worker has its own stream; the streams only run side by side if
// the device has enough hardware work queues (CUDA_DEVICE_MAX_CONNECTIONS, 8
// unless set before the process first uses CUDA; the Python package sets 32),
// otherwise a small batch can wait behind a large batch's kernel that shares
// its queue.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "fpsgpu_internal.h"

namespace fpsgpu {
namespace {

// at most 131072 points: every small request fits one CTA of the batched
// sampler (2048 pieces), so no small batch ever waits for a cluster
constexpr size_t kSmallPoints = 131072;
constexpr size_t kMaxBatch = 64;

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// Device bytes a request may need at peak: the input and the engine's scratch
// (coordinates twice, tags, ids, partner scratch, flags, distances, pieces).
size_t request_bytes(size_t n, size_t dim, size_t k) {
    return n * (dim * 4 * 3 + 4 * 6 + 1) + k * 8 + (n / 32 + 1024) * (8 * dim + 16) + (1u << 16);
}

struct Request {
    uint64_t id = 0;
    const float* pts = nullptr;
    size_t n = 0, dim = 0, k = 0, start = 0, height = 0;
    uint64_t* out = nullptr;
    size_t bytes = 0;
    double t_submit = 0, t_admit = 0, t_done = 0;
    int rc = 0;
    bool done = false;
    bool claimed = false;  // a caller is waiting on it (one waiter per ticket)
};

// What one worker thread runs on: its stream and its memory pool, both made by
// fpsgpu_server_create so that a failure is reported there.
struct WorkerRes {
    int cls = 0;
    cudaStream_t stream = nullptr;
    cudaMemPool_t pool = nullptr;
};

}  // namespace

struct Server {
    int device = 0;
    std::vector<WorkerRes> res;
    size_t budget = 0, in_use = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> pending[2];  // [0] small, [1] large
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    uint64_t next_id = 1;
    bool stopping = false;
    std::vector<std::thread> workers;
    std::atomic<uint64_t> batches{0};
    int grid_cap = 0;  // CTAs a multi-CTA sampler may use, so batches can overlap

    void worker(WorkerRes res) {
        cudaSetDevice(device);
        const int cls = res.cls;
        cudaStream_t stream = res.stream;
        cudaMemPool_t pool = res.pool;
        set_thread_pool(pool);
        for (;;) {
            std::vector<Request*> batch;
            size_t bytes = 0;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_work.wait(lk, [&] { return stopping || !pending[cls].empty(); });
                if (stopping && pending[cls].empty()) break;
                // the oldest waiting request opens the batch (a request larger
                // than the whole budget still runs alone once nothing else is
                // on the device); others join, in arrival order, while the
                // memory budget allows and only if their sample count is
                // within a factor of two of its own: a batch completes with its
                // longest cloud, so no request waits long for a much longer one
                {
                    Request* r0 = pending[cls].front();
                    if (in_use + r0->bytes <= budget || in_use == 0) {
                        pending[cls].pop_front();
                        bytes += r0->bytes;
                        batch.push_back(r0);
                        for (auto it = pending[cls].begin();
                             it != pending[cls].end() && batch.size() < kMaxBatch;) {
                            Request* r = *it;
                            if (r->dim == r0->dim && r->k <= 2 * r0->k && 2 * r->k >= r0->k &&
                                in_use + bytes + r->bytes <= budget) {
                                bytes += r->bytes;
                                batch.push_back(r);
                                it = pending[cls].erase(it);
                            } else {
                                ++it;
                            }
                        }
                    }
                }
                if (batch.empty()) {  // nothing fits now: wait for memory to free up
                    cv_done.wait(lk);
                    continue;
                }
                in_use += bytes;
                const double t = now_ms();
                for (Request* r : batch) r->t_admit = t;
            }
            // upload every request straight from its caller's buffer into the
            // batch's device buffer: no pinned staging, whose cudaFreeHost on
            // growth would wait for every other worker's kernels
            const size_t dim = batch[0]->dim;
            std::vector<size_t> off(batch.size() + 1, 0), koff(batch.size() + 1, 0), ks, starts,
                heights;
            for (size_t i = 0; i < batch.size(); ++i) {
                off[i + 1] = off[i] + batch[i]->n;
                koff[i + 1] = koff[i] + batch[i]->k;
                ks.push_back(batch[i]->k);
                starts.push_back(batch[i]->start);
                heights.push_back(batch[i]->height);
            }
            int rc = FPSGPU_OK;
            const size_t npts = off.back(), ktot = koff.back();
            float* d_pts = nullptr;
            uint64_t* d_out = nullptr;
            auto dev_alloc = [&](void** p, size_t bytes) {
                return pool ? cudaMallocFromPoolAsync(p, bytes, pool, stream)
                            : cudaMallocAsync(p, bytes, stream);
            };
            if (dev_alloc((void**)&d_pts, npts * dim * sizeof(float)) != cudaSuccess ||
                dev_alloc((void**)&d_out, ktot * sizeof(uint64_t)) != cudaSuccess)
                rc = set_error(FPSGPU_ERR_CUDA, "device allocation for a batch failed");
            for (size_t i = 0; i < batch.size() && !rc; ++i)
                if (cudaMemcpyAsync(d_pts + off[i] * dim, batch[i]->pts,
                                    batch[i]->n * dim * sizeof(float), cudaMemcpyHostToDevice,
                                    stream) != cudaSuccess)
                    rc = set_error(FPSGPU_ERR_CUDA, "upload failed");
            if (!rc)
                rc = kdline_batch_device_capped(d_pts, off.data(), batch.size(), dim, ks.data(),
                                                starts.data(), heights.data(), d_out, stream,
                                                grid_cap, nullptr, /*min_cluster=*/1);
            for (size_t i = 0; i < batch.size() && !rc; ++i)
                if (cudaMemcpyAsync(batch[i]->out, d_out + koff[i], batch[i]->k * sizeof(uint64_t),
                                    cudaMemcpyDeviceToHost, stream) != cudaSuccess)
                    rc = set_error(FPSGPU_ERR_CUDA, "download failed");
            if (d_pts) cudaFreeAsync(d_pts, stream);
            if (d_out) cudaFreeAsync(d_out, stream);
            if (cudaStreamSynchronize(stream) != cudaSuccess && !rc)
                rc = set_error(FPSGPU_ERR_CUDA, "batch failed on the device");
            batches.fetch_add(1);
            {
                std::lock_guard<std::mutex> lk(mu);
                const double t = now_ms();
                for (Request* r : batch) {
                    r->rc = rc;
                    r->t_done = t;
                    r->done = true;
                }
                in_use -= bytes;
            }
            cv_done.notify_all();
            cv_work.notify_all();
        }
        cudaStreamSynchronize(stream);
        set_thread_pool(nullptr);
    }
};

// Frees what make_worker_res made.
void free_worker_res(std::vector<WorkerRes>& rs) {
    for (WorkerRes& r : rs) {
        if (r.stream) {
            cudaStreamSynchronize(r.stream);
            cudaStreamDestroy(r.stream);
        }
        if (r.pool) cudaMemPoolDestroy(r.pool);
    }
    rs.clear();
}

// One stream and one memory pool per worker.  Small requests first: their
// streams get the device's highest priority, so their CTAs are scheduled ahead
// of the large class's as SMs free up.  Each worker allocates from a pool of
// its own, so no allocation of one worker waits for another worker's batch;
// a pool keeps up to budget / n_workers of freed memory for its next batch, so
// the server never holds more than the admitted requests' memory plus one
// budget.
int make_worker_res(int device, size_t budget, int small_workers, int large_workers,
                    std::vector<WorkerRes>& out) {
    int lo_prio = 0, hi_prio = 0;
    FPSGPU_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio));
    const int n = small_workers + large_workers;
    for (int i = 0; i < n; ++i) {
        WorkerRes r;
        r.cls = i < small_workers ? 0 : 1;
        out.push_back(r);
        cudaError_t e = cudaStreamCreateWithPriority(&out.back().stream, cudaStreamNonBlocking,
                                                     r.cls == 0 ? hi_prio : lo_prio);
        if (e != cudaSuccess) {
            out.back().stream = nullptr;
            free_worker_res(out);
            return set_error(FPSGPU_ERR_CUDA, "cannot create a worker stream: %s",
                             cudaGetErrorString(e));
        }
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        e = cudaMemPoolCreate(&out.back().pool, &props);
        if (e != cudaSuccess) {
            out.back().pool = nullptr;
            free_worker_res(out);
            return set_error(FPSGPU_ERR_CUDA, "cannot create a worker memory pool: %s",
                             cudaGetErrorString(e));
        }
        uint64_t keep = budget / (uint64_t)n;
        cudaMemPoolSetAttribute(out.back().pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    return FPSGPU_OK;
}

}  // namespace fpsgpu

using fpsgpu::Request;
using fpsgpu::Server;

extern "C" {

int fpsgpu_server_create(size_t max_device_bytes, int small_workers, int large_workers,
                         void** out) {
    fpsgpu::clear_error();
    if (!out || small_workers < 1 || large_workers < 1)
        return fpsgpu::set_error(FPSGPU_ERR_ARG, "need an output handle and >= 1 worker per class");
    int dev = 0;
    FPSGPU_CUDA_TRY(cudaGetDevice(&dev));
    auto* s = new Server();
    s->device = dev;
    s->budget = max_device_bytes;
    int sms = 0;
    FPSGPU_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    s->grid_cap = std::max(1, sms / (large_workers + 1));
    if (int rc = fpsgpu::make_worker_res(dev, s->budget, small_workers, large_workers, s->res)) {
        delete s;
        return rc;
    }
    for (const fpsgpu::WorkerRes& r : s->res) s->workers.emplace_back(&Server::worker, s, r);
    *out = s;
    return FPSGPU_OK;
}

int fpsgpu_server_submit(void* server, const float* points, size_t n_points, size_t dim,
                         size_t n_samples, size_t start_idx, size_t height,
                         size_t* sampled_point_indices, uint64_t* ticket) {
    fpsgpu::clear_error();
    auto* s = static_cast<Server*>(server);
    if (!s || !points || !sampled_point_indices || !ticket)
        return fpsgpu::set_error(FPSGPU_ERR_ARG, "null argument");
    if (dim == 0 || dim > 8) return fpsgpu::set_error(FPSGPU_ERR_DIM, "dim must be in [1, 8]");
    if (start_idx >= n_points) return fpsgpu::set_error(FPSGPU_ERR_START, "start_idx out of range");
    if (n_samples == 0 || height == 0)
        return fpsgpu::set_error(FPSGPU_ERR_ARG, "n_samples and height must be >= 1");
    auto r = std::make_unique<Request>();
    r->pts = points;
    r->n = n_points;
    r->dim = dim;
    r->k = n_samples;
    r->start = start_idx;
    r->height = height;
    r->out = reinterpret_cast<uint64_t*>(sampled_point_indices);
    r->bytes = fpsgpu::request_bytes(n_points, dim, n_samples);
    r->t_submit = fpsgpu::now_ms();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->id = s->next_id++;
        *ticket = r->id;
        s->pending[n_points > fpsgpu::kSmallPoints ? 1 : 0].push_back(r.get());
        s->reqs.emplace(r->id, std::move(r));
    }
    s->cv_work.notify_all();
    return FPSGPU_OK;
}

int fpsgpu_server_wait(void* server, uint64_t ticket, double* queue_ms, double* total_ms) {
    auto* s = static_cast<Server*>(server);
    if (!s) return fpsgpu::set_error(FPSGPU_ERR_ARG, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return fpsgpu::set_error(FPSGPU_ERR_ARG, "unknown ticket");
    Request* r = it->second.get();
    // one waiter per ticket: the waiter erases the request when it returns
    if (r->claimed) return fpsgpu::set_error(FPSGPU_ERR_ARG, "ticket already waited on");
    r->claimed = true;
    s->cv_done.wait(lk, [&] { return r->done; });
    const int rc = r->rc;
    if (queue_ms) *queue_ms = r->t_admit - r->t_submit;
    if (total_ms) *total_ms = r->t_done - r->t_submit;
    s->reqs.erase(it);
    if (rc) return fpsgpu::set_error(rc, "request %llu failed", (unsigned long long)ticket);
    return FPSGPU_OK;
}

int fpsgpu_server_destroy(void* server) {
    auto* s = static_cast<Server*>(server);
    if (!s) return FPSGPU_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv_work.notify_all();
    s->cv_done.notify_all();
    for (auto& t : s->workers) t.join();
    fpsgpu::free_worker_res(s->res);
    delete s;
    return FPSGPU_OK;
}

}  // extern "C"
