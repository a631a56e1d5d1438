/*
 * fpsgpu.h -- C ABI of libfpsgpu, the GB300 (sm_103a) farthest-point-sampling
 * library behind fpsample_gb300.
 *
 * Conventions (all entry points):
 *   - plain pointers and sizes only; the caller owns every buffer;
 *   - points are row-major float32 [n_points][dim];
 *   - sampled indices are uint64 (size_t on LP64 hosts), original point ids;
 *   - return 0 on success, a positive FPSGPU_ERR_* code otherwise, with a
 *     message for the calling thread in fpsgpu_last_error();
 *   - every call runs on the CUDA device that is current on the calling thread;
 *   - scratch memory is stream-ordered and comes from a memory pool the library
 *     keeps per device, which holds up to 8 GB mapped between calls (the
 *     device's default pool would unmap it at every synchronisation); it is
 *     given back when the process exits;
 *   - there is no CPU fallback: without a usable GPU the calls fail with
 *     FPSGPU_ERR_CUDA.
 *
 * Floating point: distances are computed exactly as the reference computes
 * them (fp32, dimensions summed in order).  Whether a*b+c is fused into an FMA
 * changes results, so the library has two modes (fpsgpu_set_fp_mode):
 * FPSGPU_FP_NOFMA matches a reference build that does not contract (the
 * default x86-64 build); FPSGPU_FP_FMA matches a contracting build (GCC's
 * default on aarch64, or x86-64 with -mfma).  The default is the mode of the
 * reference's stock build on the CPU architecture the library runs on: FMA on
 * aarch64 hosts (Grace), NOFMA elsewhere.
 */
#ifndef FPSGPU_H
#define FPSGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* error codes; 1 and 2 are the reference's own (src/wrapper.hpp:105-111,121-127) */
#define FPSGPU_OK 0
#define FPSGPU_ERR_DIM 1          /* dim outside the supported range            */
#define FPSGPU_ERR_START 2        /* a start index >= n_points                  */
#define FPSGPU_ERR_ARG 3          /* any other invalid argument                 */
#define FPSGPU_ERR_CUDA 4         /* CUDA runtime error (no device, OOM, ...)   */
#define FPSGPU_ERR_DEVICE 5       /* a kernel gave up waiting (bounded spin)    */
#define FPSGPU_ERR_NONFINITE 6    /* NaN met by the kd-line build's partition   */

#define FPSGPU_FP_NOFMA 0
#define FPSGPU_FP_FMA 1

/* algorithm selector of fpsgpu_sample_points* */
#define FPSGPU_ALGO_FPS 0      /* vanilla FPS (fpsgpu_fps), any number of starts */
#define FPSGPU_ALGO_KDLINE 1   /* bucket_fps_kdline, one start, `height`         */
#define FPSGPU_ALGO_KDTREE 2   /* bucket_fps_kdtree, one start                    */

/*
 * Replaces the reference's C ABI of the same name and signature
 * (src/wrapper.hpp:118-132): QuickFPS with a kd-line bucket tree of `height`.
 * The first sample is the point at position start_idx of the tree build's
 * permuted order, exactly as the reference (wrapper.hpp:54-55).
 * Host buffers in and out; synchronous.  dim must be in [1, 8] (returns 1),
 * start_idx < n_points (returns 2).
 */
int bucket_fps_kdline(const float *raw_data, size_t n_points, size_t dim,
                      size_t n_samples, size_t start_idx, size_t height,
                      size_t *sampled_point_indices);

/*
 * Replaces the reference's C ABI of the same name and signature
 * (src/wrapper.hpp:102-116, kdtree_sample :29-43): QuickFPS on a full kd-tree
 * (split until every leaf holds one point, KDTree.h:26).  Same start rule and
 * return codes as bucket_fps_kdline.  Subtree maxima are combined with
 * KDNode::updateMaxPoint (KDNode.h:41-46), which keeps the left child only when
 * it is strictly farther, so among equal distances the LAST position of the
 * tree's order wins (bucket_fps_kdline: the first).
 */
int bucket_fps_kdtree(const float *raw_data, size_t n_points, size_t dim,
                      size_t n_samples, size_t start_idx,
                      size_t *sampled_point_indices);

/*
 * Vanilla FPS with one or more start indices.  The reference has no C ABI for
 * this path; this is the C form of _fps_sampling (src/lib.cpp:249-270), which
 * dispatches to fps_sampling (lib.cpp:188-246, n_start == 1) and
 * fps_sampling_multi_start_index (lib.cpp:111-186).  The first n_start outputs
 * are the given starts; later ties go to the highest index.
 * Host buffers; synchronous.  Any dim >= 1.
 */
int fpsgpu_fps(const float *raw_data, size_t n_points, size_t dim,
               size_t n_samples, const size_t *start_idx, size_t n_start,
               size_t *sampled_point_indices);

/*
 * Device-buffer forms of the two calls above (same semantics as
 * bucket_fps_kdline / fpsgpu_fps).  d_points and d_out (n_samples uint64) are
 * device pointers; d_trace is NULL or n_samples floats receiving the running
 * min-distance of every chosen point when it was chosen (the max-min trace;
 * FLT_MAX / +inf for the first and forced samples).  h_start is a HOST array.
 * stream is a cudaStream_t (NULL: the library's own stream).  The call
 * returns when the result is in d_out.
 */
int fpsgpu_kdline_device(const float *d_points, size_t n_points, size_t dim,
                         size_t n_samples, size_t start_idx, size_t height,
                         uint64_t *d_out, float *d_trace, void *stream);

/* bucket_fps_kdtree on device buffers; d_trace as in fpsgpu_kdline_device. */
int fpsgpu_kdtree_device(const float *d_points, size_t n_points, size_t dim,
                         size_t n_samples, size_t start_idx, uint64_t *d_out,
                         float *d_trace, void *stream);

int fpsgpu_fps_device(const float *d_points, size_t n_points, size_t dim,
                      size_t n_samples, const size_t *h_start, size_t n_start,
                      uint64_t *d_out, float *d_trace, void *stream);

/*
 * Vanilla FPS that allocates no GPU memory (no counterpart in the reference;
 * same semantics and results as fpsgpu_fps_device).  For callers that cannot
 * call cudaMalloc -- memory owned by another allocator or pool, a loop with a
 * no-allocation rule, a device already fully reserved.  Its scratch is a fixed
 * 4.4 KB __device__ array inside the library: at most 65536 points, 512 start
 * indices, dim in [1, 8] (larger requests return FPSGPU_ERR_ARG).  All calls
 * share that array, so calls whose GPU work overlaps (two streams, two host
 * threads) race and must be serialised.  The first call on a device looks up
 * the array's address; make it before any stream capture.  stream NULL means
 * the legacy default stream.
 */
int fpsgpu_fps_device_noalloc(const float *d_points, size_t n_points, size_t dim,
                              size_t n_samples, const size_t *h_start, size_t n_start,
                              uint64_t *d_out, float *d_trace, void *stream);

/*
 * Many clouds in one call: the batched form of bucket_fps_kdline.  Cloud c is
 * rows [offsets[c], offsets[c+1]) of raw_data (offsets[0] == 0, n_clouds + 1
 * entries); n_samples[c], start_idx[c] and height[c] mean what they mean in
 * bucket_fps_kdline for that cloud alone, and the result is identical to
 * calling it once per cloud.  Cloud c's indices (local to the cloud) are
 * written at sampled_point_indices[n_samples[0] + ... + n_samples[c-1]].
 * The reference has no batched entry point; its per-cloud equivalent is
 * src/wrapper.hpp:118-132 called in a loop.  Host buffers; synchronous.
 */
int fpsgpu_kdline_batch(const float *raw_data, const size_t *offsets, size_t n_clouds,
                        size_t dim, const size_t *n_samples, const size_t *start_idx,
                        const size_t *height, size_t *sampled_point_indices);

/*
 * fpsgpu_kdline_batch with every cloud in its own host buffer: cloud c is
 * clouds[c], row-major n_points[c] x dim float.  The caller does not have to
 * concatenate the clouds first (for 256 clouds of 83 MB in all that copy cost
 * more host time than moving the data to the GPU).  Where the GPU reads
 * pageable host memory through the host's page tables (Grace), one kernel
 * gathers the clouds straight from the buffers; elsewhere each cloud is one
 * host-to-device copy.  Same checks, codes and results as fpsgpu_kdline_batch;
 * the reference's per-cloud equivalent is src/wrapper.hpp:118-132 called in a
 * loop.  Host buffers; synchronous.
 */
int fpsgpu_kdline_batch_list(const float *const *clouds, const size_t *n_points,
                             size_t n_clouds, size_t dim, const size_t *n_samples,
                             const size_t *start_idx, const size_t *height,
                             size_t *sampled_point_indices);

/* Device-buffer form of fpsgpu_kdline_batch: d_points and d_out are device
   pointers, the per-cloud arrays are HOST arrays; stream as above. */
int fpsgpu_kdline_batch_device(const float *d_points, const size_t *h_offsets,
                               size_t n_clouds, size_t dim, const size_t *h_n_samples,
                               const size_t *h_start_idx, const size_t *h_height,
                               uint64_t *d_out, void *stream);

/*
 * Request server (no counterpart in the reference): bucket_fps_kdline as a
 * service with continuous batching.  Worker threads, one CUDA stream each,
 * repeatedly take the oldest waiting request of their size class (at most
 * 131072 points: "small" workers; larger: "large" workers) together with the
 * other waiting requests whose sample counts are within a factor of two of
 * its own, as far as the device-memory budget allows, and run them as one
 * batch; requests arriving meanwhile go to the next free worker, so batches
 * overlap on the GPU.  Every result is identical to one bucket_fps_kdline call
 * on that cloud.  The workers' streams only run side by side if the process
 * has enough hardware work queues: set CUDA_DEVICE_MAX_CONNECTIONS=32 before
 * the process first uses CUDA (the default, 8, let a small batch wait behind
 * a large batch's kernel: p99 latency of clouds up to 64K points 533 ms
 * instead of 21 ms in one measurement).
 *   create : budget in bytes of device memory for admitted requests; the
 *            workers' streams and memory pools are made here (an error code if
 *            any cannot be).  Freed memory kept for reuse is capped at one
 *            budget over all workers, so the server holds at most the admitted
 *            requests' memory plus one budget.
 *   submit : host buffers; `points` and `sampled_point_indices` must stay valid
 *            until fpsgpu_server_wait returns for the ticket
 *   wait   : blocks until the request is done; queue_ms = time until its
 *            batch started, total_ms = submit-to-result latency (either may be
 *            NULL).  One waiter per ticket: a second wait on a ticket that is
 *            being waited on returns FPSGPU_ERR_ARG.
 *   destroy: finishes the requests already submitted, then stops the workers
 */
int fpsgpu_server_create(size_t max_device_bytes, int small_workers, int large_workers,
                         void **server);
int fpsgpu_server_submit(void *server, const float *points, size_t n_points, size_t dim,
                         size_t n_samples, size_t start_idx, size_t height,
                         size_t *sampled_point_indices, uint64_t *ticket);
int fpsgpu_server_wait(void *server, uint64_t ticket, double *queue_ms, double *total_ms);
int fpsgpu_server_destroy(void *server);

/*
 * The kd-line tree build alone (KDTreeBase.h:84-207 of the reference), for
 * inspection and tests: h_perm (n_points, HOST) receives the original index of
 * the point at every position of the permuted order, h_bucket_start (HOST,
 * capacity n_points) the first position of every bucket in order, and
 * *n_buckets their number.
 */
int fpsgpu_kdline_build(const float *raw_data, size_t n_points, size_t dim,
                        size_t height, uint64_t *h_perm, uint64_t *h_bucket_start,
                        size_t *n_buckets);

/* floating-point mode for subsequent calls from any thread (FPSGPU_FP_*).
   Initial value: environment variable FPSAMPLE_FP_MODE ("fma" / "nofma"),
   else the host architecture's stock reference build (FPSGPU_FP_FMA on
   aarch64, FPSGPU_FP_NOFMA elsewhere). */
int fpsgpu_set_fp_mode(int mode);
int fpsgpu_get_fp_mode(void);

/*
 * Process-wide counters for measurement (all calls, all threads).
 *   kernel_launches : kernels this library launched
 *   sampler_launches: launches of the sampling kernels (the hot loop)
 *   sampler_ms      : their summed device time, from CUDA events recorded on
 *                     the launching stream; only while timing is enabled
 *   samples         : points chosen by the sampling kernels
 *   pieces_tested   : bounding-box tests made by the pruned sampler
 *   points_touched  : running distances recomputed by the sampling kernels
 */
typedef struct {
    uint64_t kernel_launches;
    uint64_t sampler_launches;
    double sampler_ms;
    uint64_t samples;
    uint64_t pieces_tested;
    uint64_t points_touched;
} fpsgpu_stats;

void fpsgpu_stats_reset(void);
void fpsgpu_stats_get(fpsgpu_stats *out);
/* 1: record CUDA events around every sampler launch (adds a stream sync per call) */
void fpsgpu_stats_timing(int enable);

/* message describing the last failure on the calling thread ("" if none) */
const char *fpsgpu_last_error(void);

/*
 * Failure handling checks (no counterpart in the reference, whose C ABI only
 * returns argument codes).  Every wait of the multi-CTA samplers on another
 * CTA is bounded: past its limit the kernel sets an error word and exits, and
 * the call returns FPSGPU_ERR_DEVICE instead of hanging.
 *   fpsgpu_selftest_exchange_timeout: runs the samplers' grid exchange on one
 *     CTA for a grid of two, so the partner never arrives, with a limit of 4096
 *     polls; returns FPSGPU_ERR_DEVICE when the bounded wait works.  The GPU
 *     stays usable afterwards.
 *   fpsgpu_selftest_lead_timeout: runs the one-CTA leader/worker sampler on a
 *     20,000-point cloud with the leader muted, so its worker warps wait for
 *     a sample that never comes, with a limit of 4096 polls; returns
 *     FPSGPU_ERR_DEVICE when that bounded wait works (FPSGPU_ERR_ARG when
 *     FPSGPU_ONECTA_SAMPLER=lockstep turned the sampler off).  The GPU stays
 *     usable afterwards.
 *   fpsgpu_debug_fail_allocations: host-side fault injection.  After `after`
 *     more successful scratch allocations (any thread) every scratch
 *     allocation fails with FPSGPU_ERR_CUDA, until called with -1.
 */
int fpsgpu_selftest_exchange_timeout(void);
int fpsgpu_selftest_lead_timeout(void);
void fpsgpu_debug_fail_allocations(long long after);

/* library version string */
const char *fpsgpu_version(void);

/* ---- sampled points: the gather that callers do next, fused -------------
 * What callers of FPS do next is the gather pc[idx]: the sampled coordinates
 * are what the next stage consumes.  These calls return, beside
 * the indices, the sampled points themselves as n_samples x dim floats,
 * row-major like the input, written by the sampler at the moment each point
 * is chosen (it holds the winner's coordinates anyway): no second pass over
 * the cloud, no extra launch.  sampled_points / d_out_points may be NULL.
 * Indices are the same as from the calls above for the same algorithm. */
int fpsgpu_sample_points(int algo, const float *raw_data, size_t n_points, size_t dim,
                         size_t n_samples, const size_t *start_idx, size_t n_start,
                         size_t height, size_t *sampled_point_indices, float *sampled_points);
int fpsgpu_sample_points_device(int algo, const float *d_points, size_t n_points, size_t dim,
                                size_t n_samples, const size_t *h_start, size_t n_start,
                                size_t height, uint64_t *d_out, float *d_out_points,
                                void *stream);
/* fpsgpu_kdline_batch_device plus the sampled points ([sum n_samples][dim],
 * cloud c's rows after the rows of clouds 0..c-1). */
int fpsgpu_kdline_batch_points_device(const float *d_points, const size_t *h_offsets,
                                      size_t n_clouds, size_t dim, const size_t *h_n_samples,
                                      const size_t *h_start_idx, const size_t *h_height,
                                      uint64_t *d_out, float *d_out_points, void *stream);


#ifdef __cplusplus
}
#endif

#endif /* FPSGPU_H */
