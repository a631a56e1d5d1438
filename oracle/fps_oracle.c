/*
 * fps_oracle.c -- CPU restatement of fpsample's farthest-point-sampling path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: it is loaded by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline /
 * reference arm, and only as the answer GPU results are compared with (or the
 * timed CPU baseline).  The
 * product (libfpsgpu + fpsample_gb300) never links, loads or calls it and
 * has no CPU fallback.
 *
 * Parity is pinned against the real reference: tests/golden/ holds vectors
 * produced by the unmodified reference library (compiled from its own
 * sources by oracle/Makefile) and the CPU test suite checks this oracle
 * against every one of them.
 *
 * What is restated (file:line in the reference project):
 *   - vanilla FPS, single start           src/lib.cpp:188-246
 *   - vanilla FPS, list of start indices  src/lib.cpp:111-186
 *   - kd-line tree build                  src/_ext/KDTreeBase.h:84-207
 *       widest dimension                  KDTreeBase.h:160-179
 *       split value = serial fp32 mean    KDTreeBase.h:151-158
 *       two-pointer partition + clamp     KDTreeBase.h:123-149
 *       leaf rule                         src/_ext/KDLineTree.h:37-39
 *   - kd-line sampling with the bucket
 *     max cache and deferred references   KDLineTree.h:56-85, KDNode.h:84-166
 *   - start point = point at the PERMUTED
 *     position start_idx after the build  src/wrapper.hpp:45-60
 *
 * Floating point.  Distances are fp32 sums of squared differences over the
 * dimensions in order 0..D-1 (lib.cpp:214-221, Point.h:48-53).  The result
 * depends on whether the compiler contracts a*b+c into an FMA, so every
 * entry point takes fma_mode:
 *   0: every operation rounded on its own  ((d0*d0 + d1*d1) + d2*d2)
 *   1: contracted chain                   fma(d2,d2,fma(d1,d1,d0*d0))
 * The file must be compiled with -ffp-contract=off so that mode 0 stays
 * uncontracted on compilers whose default contracts (GCC on aarch64).
 */
#define _POSIX_C_SOURCE 200809L /* pthread barriers under -std=c11 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_OK 0
#define ORACLE_BAD_DIM 1
#define ORACLE_BAD_START 2
#define ORACLE_BAD_ARG 3
#define ORACLE_NO_MEMORY 4

static inline float sqdist(const float *a, const float *b, size_t dim, int fma_mode) {
    float acc = 0.0f;
    if (fma_mode) {
        for (size_t j = 0; j < dim; ++j) {
            float d = a[j] - b[j];
            acc = fmaf(d, d, acc);
        }
    } else {
        for (size_t j = 0; j < dim; ++j) {
            float d = a[j] - b[j];
            float sq = d * d;
            acc = acc + sq;
        }
    }
    return acc;
}

/* ------------------------------------------------------------------------ */
/* Vanilla FPS                                                                */
/* ------------------------------------------------------------------------ */

/*
 * Vanilla FPS over row-major pts[n][dim].  The first n_starts outputs are the
 * given starts (lib.cpp:171-176, 151-155); every later output is the point
 * with the largest running min-distance, ties going to the HIGHEST index
 * because the scan uses >= (lib.cpp:223-230, 160-165).  The running
 * min-distance starts at +inf and is lowered with a strict < (lib.cpp:220).
 *
 * trace (optional, k floats): trace[t] = the running min-distance of the
 * point chosen at step t (the max-min value); +inf for forced starts.
 */
int oracle_fps(const float *pts, size_t n, size_t dim, size_t k,
               const uint64_t *starts, size_t n_starts, int fma_mode,
               uint64_t *out, float *trace) {
    if (n == 0 || dim == 0) return ORACLE_BAD_ARG;
    if (n_starts == 0 || n_starts > (k ? k : 1)) return ORACLE_BAD_ARG;
    for (size_t s = 0; s < n_starts; ++s)
        if (starts[s] >= n) return ORACLE_BAD_START;
    if (k == 0) return ORACLE_OK;

    float *dmin = (float *)malloc(n * sizeof(float));
    if (!dmin) return ORACLE_NO_MEMORY;
    for (size_t i = 0; i < n; ++i) dmin[i] = INFINITY;

    out[0] = starts[0];
    if (trace) trace[0] = INFINITY;
    for (size_t t = 1; t < k; ++t) {
        const float *ref = pts + (size_t)out[t - 1] * dim;
        for (size_t i = 0; i < n; ++i) {
            float d = sqdist(pts + i * dim, ref, dim, fma_mode);
            if (d < dmin[i]) dmin[i] = d;
        }
        if (t < n_starts) {
            out[t] = starts[t];
            if (trace) trace[t] = INFINITY;
            continue;
        }
        size_t best = 0;
        float best_v = -1.0f;
        for (size_t i = 0; i < n; ++i) {
            if (dmin[i] >= best_v) {
                best_v = dmin[i];
                best = i;
            }
        }
        out[t] = best;
        if (trace) trace[t] = best_v;
    }
    free(dmin);
    return ORACLE_OK;
}

/* ------------------------------------------------------------------------ */
/* kd-line tree build                                                         */
/* ------------------------------------------------------------------------ */

typedef struct {
    float *w;        /* working coordinates, row-major, permuted in place */
    uint64_t *id;    /* original index of the point at each position      */
    size_t dim;
    size_t height;
    uint64_t *bstart;  /* bucket start positions, DFS (= position) order  */
    size_t nb;
} kd_build_t;

static void swap_points(kd_build_t *b, size_t i, size_t j) {
    float *wi = b->w + i * b->dim, *wj = b->w + j * b->dim;
    for (size_t d = 0; d < b->dim; ++d) {
        float t = wi[d];
        wi[d] = wj[d];
        wj[d] = t;
    }
    uint64_t t = b->id[i];
    b->id[i] = b->id[j];
    b->id[j] = t;
}

/*
 * One node [left, right) at depth `depth`.  Iterative over the right spine
 * (recursion only into the left child) so that a degenerate comb-shaped tree
 * of large height does not exhaust the stack.
 */
static void kd_divide(kd_build_t *b, size_t left, size_t right, size_t depth) {
    const size_t dim = b->dim;
    for (;;) {
        size_t count = right - left;
        if (depth == b->height || count == 1) {  /* KDLineTree.h:37-39 */
            b->bstart[b->nb++] = left;
            return;
        }
        /* exact bounding box: min/max, NaN ignored (KDTreeBase.h:181-207) */
        size_t split_dim = 0;
        {
            float span_best = 0.0f;
            for (size_t d = 0; d < dim; ++d) {
                float lo = FLT_MAX, hi = -FLT_MAX;
                for (size_t i = left; i < right; ++i) {
                    float v = b->w[i * dim + d];
                    if (v < lo) lo = v;
                    if (hi < v) hi = v;
                }
                float span = hi - lo;
                if (span > span_best) {  /* first strictly widest, KDTreeBase.h:160-179 */
                    span_best = span;
                    split_dim = d;
                }
            }
        }
        /* split value: sequential fp32 sum in current order, then / (float)count
           (KDTreeBase.h:151-158; the accumulator is rounded to float each step) */
        float sum = 0.0f;
        for (size_t i = left; i < right; ++i) sum = sum + b->w[i * dim + split_dim];
        float split = sum / (float)count;

        /* two-pointer partition: left scan passes x < split, right scan passes
           x >= split, stuck pairs are swapped (KDTreeBase.h:123-149) */
        ptrdiff_t s = (ptrdiff_t)left, e = (ptrdiff_t)right - 1;
        for (;;) {
            while (s <= e && b->w[(size_t)s * dim + split_dim] < split) ++s;
            while (s <= e && b->w[(size_t)e * dim + split_dim] >= split) --e;
            if (s > e) break;
            swap_points(b, (size_t)s, (size_t)e);
            ++s;
            --e;
        }
        size_t lim = (size_t)s - left;
        if ((size_t)s == left) lim = 1;
        if ((size_t)s == right) lim = count - 1;

        kd_divide(b, left, left + lim, depth + 1);
        left = left + lim;
        depth = depth + 1;
    }
}

/*
 * Build the kd-line tree of `height` over pts[n][dim].
 *   perm   (n)       : perm[p] = original index of the point at position p
 *   bstart (<= n)    : start position of every bucket, in position order
 *   *nb              : number of buckets
 */
int oracle_kdline_build(const float *pts, size_t n, size_t dim, size_t height,
                        uint64_t *perm, uint64_t *bstart, size_t *nb) {
    if (n == 0 || dim == 0) return ORACLE_BAD_ARG;
    kd_build_t b;
    b.w = (float *)malloc(n * dim * sizeof(float));
    if (!b.w) return ORACLE_NO_MEMORY;
    memcpy(b.w, pts, n * dim * sizeof(float));
    b.id = perm;
    for (size_t i = 0; i < n; ++i) perm[i] = i;
    b.dim = dim;
    b.height = height;
    b.bstart = bstart;
    b.nb = 0;
    kd_divide(&b, 0, n, 0);
    *nb = b.nb;
    free(b.w);
    return ORACLE_OK;
}

/* ------------------------------------------------------------------------ */
/* kd-line sampling                                                           */
/* ------------------------------------------------------------------------ */

typedef struct {
    size_t lo_pos, hi_pos;  /* [lo_pos, hi_pos) */
    size_t max_pos;
    float max_dis;          /* dis of max_pos when it was cached (KDNode max_point copy) */
    size_t *delay;          /* deferred reference positions */
    size_t n_delay, cap_delay;
} bucket_t;

static float bbox_bound(const float *lo, const float *hi, const float *r, size_t dim, int fma_mode) {
    /* squared gap from r to the box, same operation structure as sqdist
       (KDNode.h:105-118) */
    float acc = 0.0f;
    for (size_t d = 0; d < dim; ++d) {
        float g = 0.0f;
        if (r[d] > hi[d]) g = r[d] - hi[d];
        else if (r[d] < lo[d]) g = lo[d] - r[d];
        if (fma_mode) acc = fmaf(g, g, acc);
        else {
            float sq = g * g;
            acc = acc + sq;
        }
    }
    return acc;
}

static int push_delay(bucket_t *bk, size_t pos) {
    if (bk->n_delay == bk->cap_delay) {
        size_t cap = bk->cap_delay ? 2 * bk->cap_delay : 8;
        size_t *p = (size_t *)realloc(bk->delay, cap * sizeof(size_t));
        if (!p) return ORACLE_NO_MEMORY;
        bk->delay = p;
        bk->cap_delay = cap;
    }
    bk->delay[bk->n_delay++] = pos;
    return ORACLE_OK;
}

/*
 * bucket_fps_kdline(pts, n, dim, k, start_idx, height) -> out[k] original ids.
 * Error codes follow src/wrapper.hpp:118-132: 1 = dim outside [1, 8],
 * 2 = start_idx >= n.
 * trace (optional): dis value of each chosen point when it was chosen
 * (FLT_MAX-capped; trace[0] = FLT_MAX).
 * perm_out (optional, n): the build permutation.
 */
/* The body below is instantiated per (dim, fma_mode) by oracle_kdline, so the
   distance loops unroll as they do in the reference, whose buckets are
   templated on the dimension (wrapper.hpp:45-60 dispatches DIM 1..8); the
   arithmetic is the same in every instance. */
static inline __attribute__((always_inline)) int kdline_sample(
    const float *pts, size_t n, const size_t dim, size_t k, size_t start_idx, size_t height,
    const int fma_mode, uint64_t *out, float *trace, uint64_t *perm_out) {
    int rc = ORACLE_OK;
    uint64_t *perm = (uint64_t *)malloc(n * sizeof(uint64_t));
    uint64_t *bstart = (uint64_t *)malloc(n * sizeof(uint64_t));
    float *w = (float *)malloc(n * dim * sizeof(float));
    float *dis = (float *)malloc(n * sizeof(float));
    if (!perm || !bstart || !w || !dis) {
        free(perm); free(bstart); free(w); free(dis);
        return ORACLE_NO_MEMORY;
    }
    size_t nb = 0;
    rc = oracle_kdline_build(pts, n, dim, height, perm, bstart, &nb);
    if (rc) goto done;
    for (size_t p = 0; p < n; ++p)
        memcpy(w + p * dim, pts + (size_t)perm[p] * dim, dim * sizeof(float));
    if (perm_out) memcpy(perm_out, perm, n * sizeof(uint64_t));

    bucket_t *bk = (bucket_t *)calloc(nb, sizeof(bucket_t));
    float *blo = (float *)malloc(nb * dim * sizeof(float));
    float *bhi = (float *)malloc(nb * dim * sizeof(float));
    if (!bk || !blo || !bhi) {
        free(bk); free(blo); free(bhi);
        rc = ORACLE_NO_MEMORY;
        goto done;
    }
    for (size_t b = 0; b < nb; ++b) {
        bk[b].lo_pos = bstart[b];
        bk[b].hi_pos = (b + 1 < nb) ? bstart[b + 1] : n;
        for (size_t d = 0; d < dim; ++d) {
            float lo = FLT_MAX, hi = -FLT_MAX;
            for (size_t p = bk[b].lo_pos; p < bk[b].hi_pos; ++p) {
                float v = w[p * dim + d];
                if (v < lo) lo = v;
                if (hi < v) hi = v;
            }
            blo[b * dim + d] = lo;
            bhi[b * dim + d] = hi;
        }
    }

    /* init with the point at PERMUTED position start_idx (wrapper.hpp:54-55,
       KDNode.h:84-103): dis = min(FLT_MAX, d), first strict max per bucket */
    const float *ref = w + start_idx * dim;
    for (size_t b = 0; b < nb; ++b) {
        float mx = -FLT_MAX;
        for (size_t p = bk[b].lo_pos; p < bk[b].hi_pos; ++p) {
            float d = sqdist(w + p * dim, ref, dim, fma_mode);
            dis[p] = FLT_MAX;
            if (d < dis[p]) dis[p] = d;
            if (dis[p] > mx) {
                mx = dis[p];
                bk[b].max_pos = p;
            }
        }
        bk[b].max_dis = mx;
    }
    if (k > 0) {
        out[0] = perm[start_idx];
        if (trace) trace[0] = FLT_MAX;
    }

    for (size_t t = 1; t < k; ++t) {
        /* max_point(): strict > over buckets in order (KDLineTree.h:56-67) */
        float best = -FLT_MAX;
        size_t pick = bk[0].max_pos;
        for (size_t b = 0; b < nb; ++b) {
            if (bk[b].max_dis > best) {
                best = bk[b].max_dis;
                pick = bk[b].max_pos;
            }
        }
        out[t] = perm[pick];
        if (trace) trace[t] = best;
        const float *r = w + pick * dim;

        /* update_distance(ref) for every bucket (KDLineTree.h:69-75, KDNode.h:120-166) */
        for (size_t b = 0; b < nb; ++b) {
            float last = bk[b].max_dis;
            float cur = sqdist(w + bk[b].max_pos * dim, r, dim, fma_mode);
            if (cur > last) {
                if (bbox_bound(blo + b * dim, bhi + b * dim, r, dim, fma_mode) < last) {
                    if ((rc = push_delay(&bk[b], pick))) goto free_buckets;
                }
            } else {
                if ((rc = push_delay(&bk[b], pick))) goto free_buckets;
                for (size_t q = 0; q < bk[b].n_delay; ++q) {
                    const float *rr = w + bk[b].delay[q] * dim;
                    float mx = -FLT_MAX;
                    for (size_t p = bk[b].lo_pos; p < bk[b].hi_pos; ++p) {
                        float d = sqdist(w + p * dim, rr, dim, fma_mode);
                        if (d < dis[p]) dis[p] = d;
                        if (dis[p] > mx) {
                            mx = dis[p];
                            bk[b].max_pos = p;
                        }
                    }
                    bk[b].max_dis = mx;
                }
                bk[b].n_delay = 0;
            }
        }
    }

free_buckets:
    for (size_t b = 0; b < nb; ++b) free(bk[b].delay);
    free(bk); free(blo); free(bhi);
done:
    free(perm); free(bstart); free(w); free(dis);
    return rc;
}

int oracle_kdline(const float *pts, size_t n, size_t dim, size_t k, size_t start_idx,
                  size_t height, int fma_mode, uint64_t *out, float *trace,
                  uint64_t *perm_out) {
    if (dim == 0 || dim > 8) return ORACLE_BAD_DIM;
    if (start_idx >= n) return ORACLE_BAD_START;
#define ORACLE_KDLINE_CASE(D)                                                                  \
    case D:                                                                                    \
        return fma_mode ? kdline_sample(pts, n, D, k, start_idx, height, 1, out, trace, perm_out) \
                        : kdline_sample(pts, n, D, k, start_idx, height, 0, out, trace, perm_out);
    switch (dim) {
        ORACLE_KDLINE_CASE(1)
        ORACLE_KDLINE_CASE(2)
        ORACLE_KDLINE_CASE(3)
        ORACLE_KDLINE_CASE(4)
        ORACLE_KDLINE_CASE(5)
        ORACLE_KDLINE_CASE(6)
        ORACLE_KDLINE_CASE(7)
        ORACLE_KDLINE_CASE(8)
    }
#undef ORACLE_KDLINE_CASE
    return ORACLE_BAD_DIM;
}

/*
 * The same result computed the direct way: plain FPS over the permuted
 * array with first-position ties and a FLT_MAX-capped initial distance.
 * O(n*k); used by the tests to check that the bucket pruning above and on
 * the GPU never changes a value.
 */
int oracle_kdline_direct(const float *pts, size_t n, size_t dim, size_t k, size_t start_idx,
                         size_t height, int fma_mode, uint64_t *out) {
    if (dim == 0 || dim > 8) return ORACLE_BAD_DIM;
    if (start_idx >= n) return ORACLE_BAD_START;
    uint64_t *perm = (uint64_t *)malloc(n * sizeof(uint64_t));
    uint64_t *bstart = (uint64_t *)malloc(n * sizeof(uint64_t));
    float *w = (float *)malloc(n * dim * sizeof(float));
    float *dis = (float *)malloc(n * sizeof(float));
    int rc = ORACLE_OK;
    if (!perm || !bstart || !w || !dis) {
        rc = ORACLE_NO_MEMORY;
        goto done;
    }
    size_t nb;
    rc = oracle_kdline_build(pts, n, dim, height, perm, bstart, &nb);
    if (rc) goto done;
    for (size_t p = 0; p < n; ++p) {
        memcpy(w + p * dim, pts + (size_t)perm[p] * dim, dim * sizeof(float));
        dis[p] = FLT_MAX;
    }
    size_t cur = start_idx;
    for (size_t t = 0; t < k; ++t) {
        out[t] = perm[cur];
        if (t + 1 == k) break;
        const float *r = w + cur * dim;
        float best = -FLT_MAX;
        size_t pick = 0;
        for (size_t p = 0; p < n; ++p) {
            float d = sqdist(w + p * dim, r, dim, fma_mode);
            if (d < dis[p]) dis[p] = d;
            if (dis[p] > best) {
                best = dis[p];
                pick = p;
            }
        }
        cur = pick;
    }
done:
    free(perm); free(bstart); free(w); free(dis);
    return rc;
}

/* bucket_fps_kdtree (wrapper.hpp:29-43, KDTree.h:13-51, KDNode.h:41-46 and
 * :105-166): the same build with no height limit (KDTree::leftNode: a node is a
 * leaf when it holds one point), started at permuted position start_idx, and
 * FPS in which subtree maxima are combined by KDNode::updateMaxPoint, which
 * keeps the left child only when it is strictly farther.  Among equal running
 * distances the LAST position of the tree's order therefore wins; the
 * deferred-reference scheme never changes a value (as for kd-line).  Checked
 * against the reference's own output (tests/golden), including integer grids
 * full of ties. */
int oracle_kdtree(const float *pts, size_t n, size_t dim, size_t k, size_t start_idx,
                  int fma_mode, uint64_t *out) {
    if (dim == 0 || dim > 8) return ORACLE_BAD_DIM;
    if (start_idx >= n) return ORACLE_BAD_START;
    uint64_t *perm = (uint64_t *)malloc(n * sizeof(uint64_t));
    uint64_t *bstart = (uint64_t *)malloc(n * sizeof(uint64_t));
    float *w = (float *)malloc(n * dim * sizeof(float));
    float *dis = (float *)malloc(n * sizeof(float));
    int rc = ORACLE_OK;
    if (!perm || !bstart || !w || !dis) {
        rc = ORACLE_NO_MEMORY;
        goto done;
    }
    size_t nb;
    rc = oracle_kdline_build(pts, n, dim, (size_t)-1, perm, bstart, &nb);
    if (rc) goto done;
    for (size_t p = 0; p < n; ++p) {
        memcpy(w + p * dim, pts + (size_t)perm[p] * dim, dim * sizeof(float));
        dis[p] = FLT_MAX;
    }
    size_t cur = start_idx;
    for (size_t t = 0; t < k; ++t) {
        out[t] = perm[cur];
        if (t + 1 == k) break;
        const float *r = w + cur * dim;
        float best = -FLT_MAX;
        size_t pick = 0;
        for (size_t p = 0; p < n; ++p) {
            float d = sqdist(w + p * dim, r, dim, fma_mode);
            if (d < dis[p]) dis[p] = d;
            if (dis[p] >= best) {  /* updateMaxPoint: ties go right */
                best = dis[p];
                pick = p;
            }
        }
        cur = pick;
    }
done:
    free(perm); free(bstart); free(w); free(dis);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Vanilla FPS on several host threads                                       */
/* ------------------------------------------------------------------------ */

/*
 * The same answer as oracle_fps (src/lib.cpp:111-246), computed by n_threads
 * threads so that clouds of tens of millions of points can be sampled to full
 * K on the CPU.  Exactness rests on two facts:
 *   - every running min-distance update (lib.cpp:214-221) reads only its own
 *     point and the reference point, so the points can be split into
 *     contiguous chunks, one per thread, with the same arithmetic per point;
 *   - the reference's argmax scan with >= (lib.cpp:223-230) returns the LAST
 *     index holding the largest value.  Each thread scans its chunk in index
 *     order with >=, and the chunk results are folded in chunk order, again
 *     with >=, which is that same sequential scan cut into pieces.
 * Points are copied into one array per dimension so each thread streams them.
 */

typedef struct {
    float v;
    int valid;
    size_t i;
} mt_best_t;

typedef struct {
    const float *const *col; /* col[j][i]: coordinate j of point i */
    float *dmin;
    size_t n, dim, k, n_starts;
    const uint64_t *starts;
    int fma_mode;
    size_t n_threads;
    mt_best_t *slot;         /* [2][n_threads], double-buffered by step parity */
    pthread_barrier_t *bar;
    uint64_t *out;
    float *trace;
} mt_job_t;

typedef struct {
    mt_job_t *job;
    size_t tid;
} mt_arg_t;

/* Running min-distance update of points [lo, hi) against ref, the
   arithmetic of lib.cpp:214-221 per point (one column per dimension). */
static inline __attribute__((always_inline)) void mt_update_body(
    const float *const *col, float *dmin, size_t lo, size_t hi, size_t dim, const float *ref,
    int fma_mode) {
    if (fma_mode) {
        for (size_t i = lo; i < hi; ++i) {
            float acc = 0.0f;
            for (size_t j = 0; j < dim; ++j) {
                float d = col[j][i] - ref[j];
                acc = fmaf(d, d, acc);
            }
            dmin[i] = acc < dmin[i] ? acc : dmin[i];
        }
    } else {
        for (size_t i = lo; i < hi; ++i) {
            float acc = 0.0f;
            for (size_t j = 0; j < dim; ++j) {
                float d = col[j][i] - ref[j];
                float sq = d * d;
                acc = acc + sq;
            }
            dmin[i] = acc < dmin[i] ? acc : dmin[i];
        }
    }
}

#if defined(__x86_64__) && defined(__GNUC__) && !defined(__clang__)
/* The x86-64 baseline has no FMA instruction, so fmaf() is a library call per
   point and dimension.  GCC also emits a clone for CPUs that have one, where
   fmaf is a single instruction and the loop vectorises; fmaf's result is fully
   specified by IEEE 754, so every clone computes the same values. */
#define MT_CLONES __attribute__((target_clones("default", "fma")))
#else
#define MT_CLONES
#endif

MT_CLONES static void mt_update(const float *const *col, float *dmin, size_t lo, size_t hi,
                                size_t dim, const float *ref, int fma_mode) {
    switch (dim) {
#define MT_CASE(D) \
    case D: mt_update_body(col, dmin, lo, hi, D, ref, fma_mode); return;
        MT_CASE(1) MT_CASE(2) MT_CASE(3) MT_CASE(4) MT_CASE(5) MT_CASE(6) MT_CASE(7) MT_CASE(8)
#undef MT_CASE
    default: mt_update_body(col, dmin, lo, hi, dim, ref, fma_mode);
    }
}

static void *mt_worker(void *p) {
    mt_arg_t *a = (mt_arg_t *)p;
    mt_job_t *J = a->job;
    const size_t T = J->n_threads, tid = a->tid;
    const size_t lo = J->n * tid / T, hi = J->n * (tid + 1) / T;
    float *dmin = J->dmin;
    float ref[64];
    size_t cur = (size_t)J->starts[0];
    for (size_t t = 1; t < J->k; ++t) {
        for (size_t j = 0; j < J->dim; ++j) ref[j] = J->col[j][cur];
        mt_update(J->col, dmin, lo, hi, J->dim, ref, J->fma_mode);
        mt_best_t b = {-1.0f, 0, 0};
        for (size_t i = lo; i < hi; ++i) {
            if (dmin[i] >= b.v) {
                b.v = dmin[i];
                b.i = i;
                b.valid = 1;
            }
        }
        mt_best_t *slots = J->slot + (t & 1) * T;
        slots[tid] = b;
        pthread_barrier_wait(J->bar);
        /* every thread folds the chunk results in chunk order (the slots of
           this parity are next written two steps later, after another barrier) */
        mt_best_t g = {-1.0f, 0, 0};
        for (size_t c = 0; c < T; ++c)
            if (slots[c].valid && slots[c].v >= g.v) g = slots[c];
        if (t < J->n_starts) {
            cur = (size_t)J->starts[t];
            if (tid == 0) {
                J->out[t] = J->starts[t];
                if (J->trace) J->trace[t] = INFINITY;
            }
        } else {
            cur = g.i;  /* no valid chunk (all NaN): index 0, as the reference */
            if (tid == 0) {
                J->out[t] = g.i;
                if (J->trace) J->trace[t] = g.v;
            }
        }
    }
    return NULL;
}

int oracle_fps_mt(const float *pts, size_t n, size_t dim, size_t k,
                  const uint64_t *starts, size_t n_starts, int fma_mode,
                  size_t n_threads, uint64_t *out, float *trace) {
    if (n == 0 || dim == 0 || dim > 64) return ORACLE_BAD_ARG;
    if (n_starts == 0 || n_starts > (k ? k : 1)) return ORACLE_BAD_ARG;
    for (size_t s = 0; s < n_starts; ++s)
        if (starts[s] >= n) return ORACLE_BAD_START;
    if (k == 0) return ORACLE_OK;
    if (n_threads == 0) n_threads = 1;
    if (n_threads > n) n_threads = n;

    int rc = ORACLE_OK;
    float **col = (float **)calloc(dim, sizeof(float *));
    float *dmin = (float *)malloc(n * sizeof(float));
    mt_best_t *slot = (mt_best_t *)calloc(2 * n_threads, sizeof(mt_best_t));
    pthread_t *th = (pthread_t *)calloc(n_threads, sizeof(pthread_t));
    mt_arg_t *args = (mt_arg_t *)calloc(n_threads, sizeof(mt_arg_t));
    pthread_barrier_t bar;
    if (!col || !dmin || !slot || !th || !args) {
        rc = ORACLE_NO_MEMORY;
        goto done;
    }
    for (size_t j = 0; j < dim; ++j) {
        col[j] = (float *)malloc(n * sizeof(float));
        if (!col[j]) {
            rc = ORACLE_NO_MEMORY;
            goto done;
        }
        for (size_t i = 0; i < n; ++i) col[j][i] = pts[i * dim + j];
    }
    for (size_t i = 0; i < n; ++i) dmin[i] = INFINITY;
    out[0] = starts[0];
    if (trace) trace[0] = INFINITY;

    mt_job_t job = {(const float *const *)col, dmin, n, dim, k, n_starts, starts, fma_mode,
                    n_threads, slot, &bar, out, trace};
    pthread_barrier_init(&bar, NULL, (unsigned)n_threads);
    size_t started = 0;
    for (; started < n_threads; ++started) {
        args[started].job = &job;
        args[started].tid = started;
        if (pthread_create(&th[started], NULL, mt_worker, &args[started])) break;
    }
    if (started < n_threads) {
        /* the barrier counts n_threads parties: the threads already running
           would wait forever, so this cannot be recovered */
        abort();
    }
    for (size_t t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
    pthread_barrier_destroy(&bar);
done:
    if (col)
        for (size_t j = 0; j < dim; ++j) free(col[j]);
    free(col); free(dmin); free(slot); free(th); free(args);
    return rc;
}
