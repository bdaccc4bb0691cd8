/*
 * fuel_oracle.c -- CPU restatement of kno10/fuel's linear-scan kNN / range
 * search and Lloyd k-means, used ONLY as the test checker and as the timed
 * CPU baseline ("restated fuel CPU path", not the fuel binary).
 *
 * This file is test infrastructure.  Nothing in the product library links,
 * loads or calls it; tests, the smoke check and the CPU-baseline leg of the
 * benchmark do.
 *
 * Every routine restates the reference's arithmetic in the reference's own
 * operation order, so that the result is bit-identical to what fuel computes
 * on the same host ISA.  Two summation profiles exist because fuel selects
 * its kernels at compile time:
 *   FO_ORDER_ARM  non-x86 builds (the Grace host): src/math/unroll.rs,
 *                 src/math/scalar.rs and the portable fallback in
 *                 src/distance/squared_euclidean.rs:99-133;
 *   FO_ORDER_X86  x86_64 builds with AVX2+FMA: src/math/avx2.rs and
 *                 src/distance/squared_euclidean.rs:16-67.
 * Rust never contracts a*b+c into an FMA, so this file must be compiled with
 * -ffp-contract=off; every FMA the reference performs is an explicit fma().
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define FO_ORDER_ARM 0
#define FO_ORDER_X86 1

#define FO_KIND_KNN 0      /* DistanceFunction<SquaredEuclidean>::distance   */
#define FO_KIND_SQDIST 1   /* math::sqdist -> VecOps::vec_sqdist              */
#define FO_KIND_PAIRWISE 2 /* per-pair order of VecOps::vec_pairwise_sqdist   */
#define FO_KIND_DOT 3      /* math::dot (only used by the tol>0 stop rule)    */

#define FO_METRIC_SQEUCLIDEAN 0
#define FO_METRIC_EUCLIDEAN 1

#define FO_EXCLUDE_NONE 0
#define FO_EXCLUDE_LINEAR 1 /* python/search.rs:485-488: search k, drop self   */
#define FO_EXCLUDE_KPLUS1 2 /* python/search.rs:1163-1170: search k+1, drop self */

/* ------------------------------------------------------------------------ */
/* Per-pair distance kernels, f32                                            */
/* ------------------------------------------------------------------------ */

/* src/distance/squared_euclidean.rs:16-39: one 8-lane FMA accumulator over
 * d&~7, lanes stored and summed in lane order, FMA tail. */
static float knn_x86_f32(const float *a, const float *b, int64_t d) {
    int64_t sd = d & ~(int64_t)7;
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t i = 0; i < sd; i += 8)
        for (int l = 0; l < 8; l++) {
            float df = a[i + l] - b[i + l];
            acc[l] = fmaf(df, df, acc[l]);
        }
    float sum = -0.0f;
    for (int l = 0; l < 8; l++) sum = sum + acc[l];
    for (int64_t i = sd; i < d; i++) {
        float df = a[i] - b[i];
        sum = fmaf(df, df, sum);
    }
    return sum;
}

/* src/distance/squared_euclidean.rs:99-133 (fallback) and
 * src/math/unroll.rs:16-38 (sqdist): 8 lanes of mul-then-add, folded in lane
 * order, mul-then-add tail.  The two are the same arithmetic. */
static float lane8_muladd_f32(const float *a, const float *b, int64_t d) {
    int64_t sd = d & ~(int64_t)7;
    float vs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t i = 0; i < sd; i += 8)
        for (int l = 0; l < 8; l++) {
            float df = a[i + l] - b[i + l];
            float sq = df * df;
            vs[l] = sq + vs[l];
        }
    float sum = -0.0f;
    for (int l = 0; l < 8; l++) sum = sum + vs[l];
    for (int64_t i = sd; i < d; i++) {
        float df = a[i] - b[i];
        float sq = df * df;
        sum = sum + sq;
    }
    return sum;
}

/* src/math/scalar.rs:10-16: sequential mul-then-add chain. */
static float scalar_f32(const float *a, const float *b, int64_t d) {
    float sum = -0.0f;
    for (int64_t i = 0; i < d; i++) {
        float df = a[i] - b[i];
        float sq = df * df;
        sum = sum + sq;
    }
    return sum;
}

/* src/math/avx2.rs:69-81 horizontal_sum_f32: ((v0+v4)+(v1+v5))+((v2+v6)+(v3+v7)). */
static float hsum8_x86_f32(const float v[8]) {
    float s0 = v[0] + v[4], s1 = v[1] + v[5], s2 = v[2] + v[6], s3 = v[3] + v[7];
    float t0 = s0 + s1, t2 = s2 + s3;
    return t0 + t2;
}

/* src/math/avx2.rs:103-151 sqdist_f32: four 8-lane FMA accumulators over
 * 32-blocks, combined (acc0+acc1)+(acc2+acc3), then 8-blocks into the
 * combined accumulator, horizontal sum, FMA tail. */
static float sqdist_x86_f32(const float *a, const float *b, int64_t d) {
    float acc[4][8];
    memset(acc, 0, sizeof(acc));
    int64_t i = 0;
    for (; i + 32 <= d; i += 32)
        for (int u = 0; u < 4; u++)
            for (int l = 0; l < 8; l++) {
                float df = a[i + u * 8 + l] - b[i + u * 8 + l];
                acc[u][l] = fmaf(df, df, acc[u][l]);
            }
    float c[8];
    for (int l = 0; l < 8; l++) c[l] = (acc[0][l] + acc[1][l]) + (acc[2][l] + acc[3][l]);
    for (; i + 8 <= d; i += 8)
        for (int l = 0; l < 8; l++) {
            float df = a[i + l] - b[i + l];
            c[l] = fmaf(df, df, c[l]);
        }
    float sum = hsum8_x86_f32(c);
    for (; i < d; i++) {
        float df = a[i] - b[i];
        sum = fmaf(df, df, sum);
    }
    return sum;
}

/* src/math/avx2.rs:903-975 micro_sqdist_f32: one FMA chain per pair over k. */
static float fmachain_f32(const float *a, const float *b, int64_t d) {
    float acc = 0.0f;
    for (int64_t i = 0; i < d; i++) {
        float df = a[i] - b[i];
        acc = fmaf(df, df, acc);
    }
    return acc;
}

/* src/math/unroll.rs:227-303: per pair tile[i][j] += diff*diff over k. */
static float muladdchain_f32(const float *a, const float *b, int64_t d) {
    float acc = 0.0f;
    for (int64_t i = 0; i < d; i++) {
        float df = a[i] - b[i];
        float sq = df * df;
        acc = acc + sq;
    }
    return acc;
}

/* src/math/avx2.rs:787-835 dot_f32 and src/math/unroll.rs:201-221 dot. */
static float dot_x86_f32(const float *a, const float *b, int64_t d) {
    float acc[4][8];
    memset(acc, 0, sizeof(acc));
    int64_t i = 0;
    for (; i + 32 <= d; i += 32)
        for (int u = 0; u < 4; u++)
            for (int l = 0; l < 8; l++) acc[u][l] = fmaf(a[i + u * 8 + l], b[i + u * 8 + l], acc[u][l]);
    float c[8];
    for (int l = 0; l < 8; l++) c[l] = (acc[0][l] + acc[1][l]) + (acc[2][l] + acc[3][l]);
    for (; i + 8 <= d; i += 8)
        for (int l = 0; l < 8; l++) c[l] = fmaf(a[i + l], b[i + l], c[l]);
    float sum = hsum8_x86_f32(c);
    for (; i < d; i++) sum = fmaf(a[i], b[i], sum);
    return sum;
}
static float dot_arm_f32(const float *a, const float *b, int64_t d) {
    int64_t sd = d & ~(int64_t)7;
    float vs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t i = 0; i < sd; i += 8)
        for (int l = 0; l < 8; l++) {
            float p = a[i + l] * b[i + l];
            vs[l] = vs[l] + p;
        }
    float sum = -0.0f;
    for (int l = 0; l < 8; l++) sum = sum + vs[l];
    for (int64_t i = sd; i < d; i++) {
        float p = a[i] * b[i];
        sum = sum + p;
    }
    return sum;
}
static float dot_scalar_f32(const float *a, const float *b, int64_t d) {
    float sum = -0.0f;
    for (int64_t i = 0; i < d; i++) {
        float p = a[i] * b[i];
        sum = sum + p;
    }
    return sum;
}

/* VecOps dispatch, src/math/mod.rs:51-63 (UNROLL_SIZE = 4, line 20). */
float fo_dist_f32(int kind, int order, const float *a, const float *b, int64_t d) {
    switch (kind) {
    case FO_KIND_KNN:
        return order == FO_ORDER_X86 ? knn_x86_f32(a, b, d) : lane8_muladd_f32(a, b, d);
    case FO_KIND_SQDIST:
        if (d < 4) return scalar_f32(a, b, d);
        return order == FO_ORDER_X86 ? sqdist_x86_f32(a, b, d) : lane8_muladd_f32(a, b, d);
    case FO_KIND_PAIRWISE:
        if (d < 4) return scalar_f32(a, b, d);
        return order == FO_ORDER_X86 ? fmachain_f32(a, b, d) : muladdchain_f32(a, b, d);
    case FO_KIND_DOT:
        if (d < 4) return dot_scalar_f32(a, b, d);
        return order == FO_ORDER_X86 ? dot_x86_f32(a, b, d) : dot_arm_f32(a, b, d);
    }
    return NAN;
}

/* ------------------------------------------------------------------------ */
/* Per-pair distance kernels, f64                                            */
/* ------------------------------------------------------------------------ */

/* src/distance/squared_euclidean.rs:44-67: 4-lane FMA accumulator. */
static double knn_x86_f64(const double *a, const double *b, int64_t d) {
    int64_t sd = d & ~(int64_t)3;
    double acc[4] = {0, 0, 0, 0};
    for (int64_t i = 0; i < sd; i += 4)
        for (int l = 0; l < 4; l++) {
            double df = a[i + l] - b[i + l];
            acc[l] = fma(df, df, acc[l]);
        }
    double sum = -0.0;
    for (int l = 0; l < 4; l++) sum = sum + acc[l];
    for (int64_t i = sd; i < d; i++) {
        double df = a[i] - b[i];
        sum = fma(df, df, sum);
    }
    return sum;
}
static double lane8_muladd_f64(const double *a, const double *b, int64_t d) {
    int64_t sd = d & ~(int64_t)7;
    double vs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t i = 0; i < sd; i += 8)
        for (int l = 0; l < 8; l++) {
            double df = a[i + l] - b[i + l];
            double sq = df * df;
            vs[l] = sq + vs[l];
        }
    double sum = -0.0;
    for (int l = 0; l < 8; l++) sum = sum + vs[l];
    for (int64_t i = sd; i < d; i++) {
        double df = a[i] - b[i];
        double sq = df * df;
        sum = sum + sq;
    }
    return sum;
}
static double scalar_f64(const double *a, const double *b, int64_t d) {
    double sum = -0.0;
    for (int64_t i = 0; i < d; i++) {
        double df = a[i] - b[i];
        double sq = df * df;
        sum = sum + sq;
    }
    return sum;
}
/* src/math/avx2.rs:158-204 sqdist_f64: four 4-lane accumulators over
 * 16-blocks, (acc0+acc1)+(acc2+acc3), 4-blocks, horizontal_sum_f64
 * (src/math/avx2.rs:85-94: (v0+v2)+(v1+v3)), FMA tail. */
static double sqdist_x86_f64(const double *a, const double *b, int64_t d) {
    double acc[4][4];
    memset(acc, 0, sizeof(acc));
    int64_t i = 0;
    for (; i + 16 <= d; i += 16)
        for (int u = 0; u < 4; u++)
            for (int l = 0; l < 4; l++) {
                double df = a[i + u * 4 + l] - b[i + u * 4 + l];
                acc[u][l] = fma(df, df, acc[u][l]);
            }
    double c[4];
    for (int l = 0; l < 4; l++) c[l] = (acc[0][l] + acc[1][l]) + (acc[2][l] + acc[3][l]);
    for (; i + 4 <= d; i += 4)
        for (int l = 0; l < 4; l++) {
            double df = a[i + l] - b[i + l];
            c[l] = fma(df, df, c[l]);
        }
    double sum = (c[0] + c[2]) + (c[1] + c[3]);
    for (; i < d; i++) {
        double df = a[i] - b[i];
        sum = fma(df, df, sum);
    }
    return sum;
}
static double fmachain_f64(const double *a, const double *b, int64_t d) {
    double acc = 0.0;
    for (int64_t i = 0; i < d; i++) {
        double df = a[i] - b[i];
        acc = fma(df, df, acc);
    }
    return acc;
}
static double muladdchain_f64(const double *a, const double *b, int64_t d) {
    double acc = 0.0;
    for (int64_t i = 0; i < d; i++) {
        double df = a[i] - b[i];
        double sq = df * df;
        acc = acc + sq;
    }
    return acc;
}

double fo_dist_f64(int kind, int order, const double *a, const double *b, int64_t d) {
    switch (kind) {
    case FO_KIND_KNN:
        return order == FO_ORDER_X86 ? knn_x86_f64(a, b, d) : lane8_muladd_f64(a, b, d);
    case FO_KIND_SQDIST:
        if (d < 4) return scalar_f64(a, b, d);
        return order == FO_ORDER_X86 ? sqdist_x86_f64(a, b, d) : lane8_muladd_f64(a, b, d);
    case FO_KIND_PAIRWISE:
        if (d < 4) return scalar_f64(a, b, d);
        return order == FO_ORDER_X86 ? fmachain_f64(a, b, d) : muladdchain_f64(a, b, d);
    }
    return NAN;
}

/* src/math/mod.rs:558-660 free pairwise_sqdist (matrix of all pairs). */
void fo_pairwise_sqdist_f32(int order, const float *p1, int64_t n1, const float *p2, int64_t n2, int64_t d,
                            float *out) {
    for (int64_t i = 0; i < n1; i++)
        for (int64_t j = 0; j < n2; j++) out[i * n2 + j] = fo_dist_f32(FO_KIND_PAIRWISE, order, p1 + i * d, p2 + j * d, d);
}
void fo_pairwise_sqdist_f64(int order, const double *p1, int64_t n1, const double *p2, int64_t n2, int64_t d,
                            double *out) {
    for (int64_t i = 0; i < n1; i++)
        for (int64_t j = 0; j < n2; j++) out[i * n2 + j] = fo_dist_f64(FO_KIND_PAIRWISE, order, p1 + i * d, p2 + j * d, d);
}

/* ------------------------------------------------------------------------ */
/* Tiny parallel-for over [0, count) with a fixed number of workers.         */
/* ------------------------------------------------------------------------ */

typedef void (*fo_task_fn)(void *ctx, int64_t item);
typedef struct {
    fo_task_fn fn;
    void *ctx;
    int64_t count;
    int nworkers;
    int wid;
} fo_worker;

static void *fo_worker_main(void *p) {
    fo_worker *w = (fo_worker *)p;
    /* static interleaved schedule: deterministic, no shared counters */
    for (int64_t it = w->wid; it < w->count; it += w->nworkers) w->fn(w->ctx, it);
    return NULL;
}

static void fo_parallel_for(int threads, int64_t count, fo_task_fn fn, void *ctx) {
    if (threads <= 1 || count <= 1) {
        for (int64_t i = 0; i < count; i++) fn(ctx, i);
        return;
    }
    if (threads > count) threads = (int)count;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    fo_worker *ws = (fo_worker *)malloc(sizeof(fo_worker) * threads);
    for (int t = 0; t < threads; t++) {
        ws[t].fn = fn;
        ws[t].ctx = ctx;
        ws[t].count = count;
        ws[t].nworkers = threads;
        ws[t].wid = t;
    }
    char *spawned = (char *)calloc(threads, 1);
    for (int t = 1; t < threads; t++) spawned[t] = pthread_create(&th[t], NULL, fo_worker_main, &ws[t]) == 0;
    fo_worker_main(&ws[0]);
    for (int t = 1; t < threads; t++) {
        if (spawned[t]) pthread_join(th[t], NULL);
        else fo_worker_main(&ws[t]); /* thread creation failed: run that share inline */
    }
    free(spawned);
    free(th);
    free(ws);
}

/* ------------------------------------------------------------------------ */
/* DistPair + KNNHeap, src/api/search.rs:9-151                              */
/* ------------------------------------------------------------------------ */

typedef struct {
    double dist; /* holds the f32 or f64 distance exactly */
    int64_t idx;
} fo_pair;

/* DistPair::cmp, src/api/search.rs:23-30: distance partial_cmp (unordered ->
 * Equal), then index. */
static int fo_pair_cmp(const fo_pair *a, const fo_pair *b) {
    if (a->dist < b->dist) return -1;
    if (a->dist > b->dist) return 1;
    if (a->idx < b->idx) return -1;
    if (a->idx > b->idx) return 1;
    return 0;
}
static int fo_pair_qcmp(const void *a, const void *b) { return fo_pair_cmp((const fo_pair *)a, (const fo_pair *)b); }

typedef struct {
    int64_t k;
    fo_pair *heap; /* binary max-heap by fo_pair_cmp, capacity k */
    int64_t hlen;
    fo_pair *ties;
    int64_t tlen, tcap;
    double kdist;
} fo_knnheap;

static void heap_sift_up(fo_pair *h, int64_t i) {
    while (i > 0) {
        int64_t p = (i - 1) / 2;
        if (fo_pair_cmp(&h[i], &h[p]) <= 0) break;
        fo_pair t = h[i];
        h[i] = h[p];
        h[p] = t;
        i = p;
    }
}
static void heap_sift_down(fo_pair *h, int64_t n, int64_t i) {
    for (;;) {
        int64_t l = 2 * i + 1, r = l + 1, m = i;
        if (l < n && fo_pair_cmp(&h[l], &h[m]) > 0) m = l;
        if (r < n && fo_pair_cmp(&h[r], &h[m]) > 0) m = r;
        if (m == i) break;
        fo_pair t = h[i];
        h[i] = h[m];
        h[m] = t;
        i = m;
    }
}
static void ties_push(fo_knnheap *s, fo_pair p) {
    if (s->tlen == s->tcap) {
        s->tcap = s->tcap ? s->tcap * 2 : 16;
        s->ties = (fo_pair *)realloc(s->ties, sizeof(fo_pair) * s->tcap);
    }
    s->ties[s->tlen++] = p;
}

/* KNNHeap::insert, src/api/search.rs:105-135. */
static void knnheap_insert(fo_knnheap *s, fo_pair p) {
    if (s->k == 0) return;
    if (s->hlen < s->k) {
        s->heap[s->hlen++] = p;
        heap_sift_up(s->heap, s->hlen - 1);
        if (s->hlen == s->k) s->kdist = s->heap[0].dist;
        return;
    }
    int less = p.dist < s->kdist, greater = p.dist > s->kdist;
    if (less) {
        fo_pair removed = s->heap[0];
        s->heap[0] = s->heap[s->hlen - 1];
        s->hlen--;
        heap_sift_down(s->heap, s->hlen, 0);
        s->heap[s->hlen++] = p;
        heap_sift_up(s->heap, s->hlen - 1);
        double nk = s->heap[0].dist;
        if (nk < s->kdist) s->tlen = 0;
        else if (removed.dist == nk) ties_push(s, removed);
        s->kdist = nk;
    } else if (!greater) {
        ties_push(s, p); /* Equal (or unordered) */
    }
}

/* ------------------------------------------------------------------------ */
/* linear_scan_knn / linear_scan_range batches                               */
/* ------------------------------------------------------------------------ */

typedef struct {
    int is64;
    const void *X, *Q;
    int64_t n, d, m, k;
    int metric, order, exclude_mode;
    int64_t *out_idx;
    void *out_dist;
} fo_knn_ctx;

static double fo_query_distance(const fo_knn_ctx *c, const void *q, int64_t i) {
    if (c->is64) {
        double v = fo_dist_f64(FO_KIND_KNN, c->order, (const double *)q, (const double *)c->X + i * c->d, c->d);
        if (c->metric == FO_METRIC_EUCLIDEAN) v = sqrt(v); /* src/distance/euclidean.rs:7-9 */
        return v;
    }
    float v = fo_dist_f32(FO_KIND_KNN, c->order, (const float *)q, (const float *)c->X + i * c->d, c->d);
    if (c->metric == FO_METRIC_EUCLIDEAN) v = sqrtf(v);
    return (double)v;
}

/* One query row: linear_scan_knn (src/api/search.rs:169-184), the exclude-self
 * retain (python/search.rs:485-488 or 1163-1170) and knn_results_to_arrays
 * truncation + padding (python/search.rs:1195-1216). */
static void fo_knn_task(void *vctx, int64_t qi) {
    fo_knn_ctx *c = (fo_knn_ctx *)vctx;
    const void *q = c->is64 ? (const void *)((const double *)c->Q + qi * c->d)
                            : (const void *)((const float *)c->Q + qi * c->d);
    int64_t k = c->k;
    int64_t qk = (c->exclude_mode == FO_EXCLUDE_KPLUS1) ? k + 1 : k;
    int64_t nres = 0;
    fo_pair *res = NULL;
    if (qk > 0 && c->n > 0) {
        fo_knnheap h;
        memset(&h, 0, sizeof(h));
        h.k = qk;
        h.heap = (fo_pair *)malloc(sizeof(fo_pair) * qk);
        h.kdist = INFINITY;
        for (int64_t i = 0; i < c->n; i++) {
            fo_pair p = {fo_query_distance(c, q, i), i};
            knnheap_insert(&h, p);
        }
        nres = h.hlen + h.tlen;
        res = (fo_pair *)malloc(sizeof(fo_pair) * (nres ? nres : 1));
        memcpy(res, h.heap, sizeof(fo_pair) * h.hlen);
        if (h.tlen) memcpy(res + h.hlen, h.ties, sizeof(fo_pair) * h.tlen);
        qsort(res, nres, sizeof(fo_pair), fo_pair_qcmp); /* KNNHeap::into_vec */
        free(h.heap);
        free(h.ties);
    }
    if (c->exclude_mode != FO_EXCLUDE_NONE) {
        int64_t w = 0;
        for (int64_t r = 0; r < nres; r++)
            if (res[r].idx != qi) res[w++] = res[r];
        nres = w;
    }
    for (int64_t j = 0; j < k; j++) {
        int have = j < nres;
        c->out_idx[qi * k + j] = have ? res[j].idx : -1;
        if (c->is64) ((double *)c->out_dist)[qi * k + j] = have ? res[j].dist : INFINITY;
        else ((float *)c->out_dist)[qi * k + j] = have ? (float)res[j].dist : INFINITY;
    }
    free(res);
}

static int fo_knn_any(int is64, const void *X, int64_t n, int64_t d, const void *Q, int64_t m, int64_t k, int metric,
                      int order, int exclude_mode, int threads, int64_t *out_idx, void *out_dist) {
    if (n < 0 || d < 0 || m < 0 || k < 0) return 1;
    fo_knn_ctx c = {is64, X, Q, n, d, m, k, metric, order, exclude_mode, out_idx, out_dist};
    fo_parallel_for(threads, m, fo_knn_task, &c);
    return 0;
}
int fo_knn_f32(const float *X, int64_t n, int64_t d, const float *Q, int64_t m, int64_t k, int metric, int order,
               int exclude_mode, int threads, int64_t *out_idx, float *out_dist) {
    return fo_knn_any(0, X, n, d, Q, m, k, metric, order, exclude_mode, threads, out_idx, out_dist);
}
int fo_knn_f64(const double *X, int64_t n, int64_t d, const double *Q, int64_t m, int64_t k, int metric, int order,
               int exclude_mode, int threads, int64_t *out_idx, double *out_dist) {
    return fo_knn_any(1, X, n, d, Q, m, k, metric, order, exclude_mode, threads, out_idx, out_dist);
}

typedef struct {
    fo_knn_ctx base;
    double radius;
    int exclude_self;
    fo_pair **rows;
    int64_t *counts;
} fo_range_ctx;

/* linear_scan_range, src/api/search.rs:154-166, plus the exclude-self retain
 * of linear_scan_range_batch, python/search.rs:494-514. */
static void fo_range_task(void *vctx, int64_t qi) {
    fo_range_ctx *rc = (fo_range_ctx *)vctx;
    fo_knn_ctx *c = &rc->base;
    const void *q = c->is64 ? (const void *)((const double *)c->Q + qi * c->d)
                            : (const void *)((const float *)c->Q + qi * c->d);
    int64_t cap = 16, cnt = 0;
    fo_pair *out = (fo_pair *)malloc(sizeof(fo_pair) * cap);
    for (int64_t i = 0; i < c->n; i++) {
        double v = fo_query_distance(c, q, i);
        if (v <= rc->radius) {
            if (rc->exclude_self && i == qi) continue;
            if (cnt == cap) {
                cap *= 2;
                out = (fo_pair *)realloc(out, sizeof(fo_pair) * cap);
            }
            out[cnt].dist = v;
            out[cnt].idx = i;
            cnt++;
        }
    }
    qsort(out, cnt, sizeof(fo_pair), fo_pair_qcmp);
    rc->rows[qi] = out;
    rc->counts[qi] = cnt;
}

/* The radius arrives as f64 and is cast to the index dtype
 * (python/search.rs:781-783: radius as f32). Output is CSR. */
static int fo_range_any(int is64, const void *X, int64_t n, int64_t d, const void *Q, int64_t m, double radius,
                        int metric, int order, int exclude_self, int threads, int64_t **offsets, int64_t **idx,
                        void **dist) {
    fo_range_ctx rc;
    memset(&rc, 0, sizeof(rc));
    fo_knn_ctx c = {is64, X, Q, n, d, m, 0, metric, order, 0, NULL, NULL};
    rc.base = c;
    rc.radius = is64 ? radius : (double)(float)radius;
    rc.exclude_self = exclude_self;
    rc.rows = (fo_pair **)calloc(m ? m : 1, sizeof(fo_pair *));
    rc.counts = (int64_t *)calloc(m ? m : 1, sizeof(int64_t));
    fo_parallel_for(threads, m, fo_range_task, &rc);
    int64_t *off = (int64_t *)malloc(sizeof(int64_t) * (m + 1));
    off[0] = 0;
    for (int64_t i = 0; i < m; i++) off[i + 1] = off[i] + rc.counts[i];
    int64_t tot = off[m];
    int64_t *oi = (int64_t *)malloc(sizeof(int64_t) * (tot ? tot : 1));
    void *od = malloc((is64 ? 8 : 4) * (tot ? tot : 1));
    for (int64_t i = 0; i < m; i++) {
        for (int64_t j = 0; j < rc.counts[i]; j++) {
            oi[off[i] + j] = rc.rows[i][j].idx;
            if (is64) ((double *)od)[off[i] + j] = rc.rows[i][j].dist;
            else ((float *)od)[off[i] + j] = (float)rc.rows[i][j].dist;
        }
        free(rc.rows[i]);
    }
    free(rc.rows);
    free(rc.counts);
    *offsets = off;
    *idx = oi;
    *dist = od;
    return 0;
}
int fo_range_f32(const float *X, int64_t n, int64_t d, const float *Q, int64_t m, double radius, int metric, int order,
                 int exclude_self, int threads, int64_t **offsets, int64_t **idx, float **dist) {
    return fo_range_any(0, X, n, d, Q, m, radius, metric, order, exclude_self, threads, offsets, idx, (void **)dist);
}
int fo_range_f64(const double *X, int64_t n, int64_t d, const double *Q, int64_t m, double radius, int metric,
                 int order, int exclude_self, int threads, int64_t **offsets, int64_t **idx, double **dist) {
    return fo_range_any(1, X, n, d, Q, m, radius, metric, order, exclude_self, threads, offsets, idx, (void **)dist);
}
/* ------------------------------------------------------------------------ */
/* Pairwise distance matrix of one point set (fuel.search.pairwise_distances */
/* for raw f32 points): compute_pairwise_condensed,                         */
/* src/api/condensed_distance_matrix.rs:22-48 -- rows i = 1..n-1, j = 0..i-1 */
/* in order, out[i*(i-1)/2 + j] = distance(points[i], points[j]) -- and     */
/* compute_pairwise_dense, src/api/square_distance_matrix.rs:11-40 --      */
/* row[j] = distance(points[i], points[j]) for j >= i, mirrored to (j, i).  */
/* distance = DistanceFunction<SquaredEuclidean> (FO_KIND_KNN order), sqrt  */
/* for Euclidean (src/distance/euclidean.rs:7-9).                           */
/* ------------------------------------------------------------------------ */
typedef struct {
    const float *X;
    int64_t n, d;
    int metric, order, square;
    float *out;
} fo_pw_ctx;

static float fo_pw_value(const fo_pw_ctx *c, int64_t i, int64_t j) {
    float v = fo_dist_f32(FO_KIND_KNN, c->order, c->X + i * c->d, c->X + j * c->d, c->d);
    if (c->metric == FO_METRIC_EUCLIDEAN) v = sqrtf(v);
    return v;
}

static void fo_pw_task(void *ctx, int64_t i) {
    const fo_pw_ctx *c = (const fo_pw_ctx *)ctx;
    if (!c->square) {
        for (int64_t j = 0; j < i; j++) c->out[i * (i - 1) / 2 + j] = fo_pw_value(c, i, j);
        return;
    }
    for (int64_t j = i; j < c->n; j++) {
        const float v = fo_pw_value(c, i, j);
        c->out[i * c->n + j] = v;
        if (j > i) c->out[j * c->n + i] = v;
    }
}

int fo_pairwise_dist_f32(const float *X, int64_t n, int64_t d, int metric, int order, int square, int threads,
                         float *out) {
    if (n < 0 || d < 0) return 1;
    fo_pw_ctx c = {X, n, d, metric, order, square, out};
    fo_parallel_for(threads, n, fo_pw_task, &c);
    return 0;
}

void fo_free(void *p) { free(p); }

/* ------------------------------------------------------------------------ */
/* Lloyd k-means, src/cluster/kmeans/lloyd.rs:12-202                         */
/* ------------------------------------------------------------------------ */

#define FO_SUMS_REFERENCE 0 /* fuel: f32 running sums updated by f32 per-chunk deltas */
#define FO_SUMS_FP64 1      /* fp64 sums of member rows; centre = (f32)(sum / count)  */

typedef struct {
    const float *X;
    int64_t n, d, k;
    const float *cent;
    int kind, order;
    int64_t chunk;
    int64_t *assign;   /* in: old labels (iteration >= 2); out: new labels */
    float *best;       /* out: per-point best distance */
    /* per-chunk outputs (reference mode) */
    int64_t *dcsize;   /* [nchunks][k] */
    float *dsums;      /* [nchunks][k*d] */
    float *lsum;       /* [nchunks] */
    int64_t *lchanged; /* [nchunks] */
    int initial;
} fo_lloyd_ctx;

/* One rayon chunk of par_chunks_map_mut (src/api/parallel.rs:116-125):
 * initial assignment lloyd.rs:77-102, later iterations lloyd.rs:155-184. */
static void fo_lloyd_chunk(void *vctx, int64_t ci) {
    fo_lloyd_ctx *c = (fo_lloyd_ctx *)vctx;
    int64_t i0 = ci * c->chunk, i1 = i0 + c->chunk;
    if (i1 > c->n) i1 = c->n;
    int64_t k = c->k, d = c->d;
    int64_t *dc = c->dcsize ? c->dcsize + ci * k : NULL;
    float *ds = c->dsums ? c->dsums + ci * k * d : NULL;
    if (dc) memset(dc, 0, sizeof(int64_t) * k);
    if (ds) memset(ds, 0, sizeof(float) * k * d);
    float local = 0.0f;
    int64_t changed = 0;
    for (int64_t i = i0; i < i1; i++) {
        const float *pt = c->X + i * d;
        int64_t a = 0;
        float s = fo_dist_f32(c->kind, c->order, c->kind == FO_KIND_PAIRWISE ? pt : c->cent, c->kind == FO_KIND_PAIRWISE ? c->cent : pt, d);
        for (int64_t j = 1; j < k; j++) {
            float t = c->kind == FO_KIND_PAIRWISE ? fo_dist_f32(c->kind, c->order, pt, c->cent + j * d, d)
                                                  : fo_dist_f32(c->kind, c->order, c->cent + j * d, pt, d);
            if (t < s) {
                a = j;
                s = t;
            }
        }
        c->best[i] = s;
        local = local + s;
        if (c->initial) {
            c->assign[i] = a;
            if (dc) {
                dc[a] += 1;
                for (int64_t t = 0; t < d; t++) ds[a * d + t] = ds[a * d + t] + pt[t];
            }
        } else {
            int64_t old = c->assign[i];
            if (a != old) {
                c->assign[i] = a;
                if (dc) {
                    dc[old] -= 1;
                    dc[a] += 1;
                    for (int64_t t = 0; t < d; t++) ds[old * d + t] = ds[old * d + t] - pt[t];
                    for (int64_t t = 0; t < d; t++) ds[a * d + t] = ds[a * d + t] + pt[t];
                }
                changed++;
            }
        }
    }
    c->lsum[ci] = local;
    c->lchanged[ci] = changed;
}

/* Exact fp64 inertia of (centres, labels): sum_i ||x_i - c_{l_i}||^2 with the
 * squared differences formed and summed in double. */
static double fo_inertia_fp64(const float *X, int64_t n, int64_t d, const float *cent, const int64_t *lab) {
    double tot = 0.0;
    for (int64_t i = 0; i < n; i++) {
        const float *p = X + i * d, *c = cent + lab[i] * d;
        double s = 0.0;
        for (int64_t t = 0; t < d; t++) {
            double df = (double)p[t] - (double)c[t];
            s += df * df;
        }
        tot += s;
    }
    return tot;
}

/* One assignment pass against fixed centres, without any centre update: the
 * per-iteration parity check ("same centres in -> same labels out").
 * initial != 0 selects the initial-assignment order (pairwise kernel). */
int fo_lloyd_assign_f32(const float *X, int64_t n, int64_t d, int64_t k, const float *cent, int initial, int order,
                        int threads, int64_t *labels, float *best) {
    if (threads < 1) threads = 1;
    int64_t chunk = (n + threads - 1) / threads;
    if (chunk < 1) chunk = 1;
    int64_t nch = n ? (n + chunk - 1) / chunk : 0;
    fo_lloyd_ctx c;
    memset(&c, 0, sizeof(c));
    c.X = X, c.n = n, c.d = d, c.k = k, c.cent = cent;
    c.kind = initial ? FO_KIND_PAIRWISE : FO_KIND_SQDIST;
    c.order = order, c.chunk = chunk, c.assign = labels, c.best = best, c.initial = initial;
    c.lsum = (float *)calloc(nch ? nch : 1, sizeof(float));
    c.lchanged = (int64_t *)calloc(nch ? nch : 1, sizeof(int64_t));
    if (initial) memset(labels, 0, sizeof(int64_t) * n);
    fo_parallel_for(threads, nch, fo_lloyd_chunk, &c);
    free(c.lsum);
    free(c.lchanged);
    return 0;
}

/* lloyd(), src/cluster/kmeans/lloyd.rs:118-202, with InitMethod::Fixed
 * (python/kmeans.rs:111-130) as the initialisation.  `threads` is the rayon
 * thread count that sets the chunk size ceil(n/threads)
 * (src/api/parallel.rs:119) and hence the f32 summation order of the
 * reference sums.  sums_mode FO_SUMS_FP64 replaces the f32 running sums by
 * fp64 sums of each cluster's rows (centre = (f32)(sum / count)) and reports
 * the fp64 inertia of the returned (centres, labels). */
int fo_lloyd_f32(const float *X, int64_t n, int64_t d, int64_t k, const float *init, int64_t maxiter, double tol,
                 int order, int threads, int sums_mode, float *out_centers, int64_t *out_labels, int64_t *out_iters,
                 double *out_inertia, int64_t *out_changed_last) {
    if (n <= 0 || d <= 0 || k <= 0 || k > n) return 1;
    if (threads < 1) threads = 1;
    int64_t chunk = (n + threads - 1) / threads;
    if (chunk < 1) chunk = 1;
    int64_t nch = (n + chunk - 1) / chunk;
    float *cent = out_centers;
    memcpy(cent, init, sizeof(float) * k * d);
    float *sums = (float *)calloc(k * d, sizeof(float));
    double *sums64 = (double *)calloc(k * d, sizeof(double));
    int64_t *csize = (int64_t *)calloc(k, sizeof(int64_t));
    float *best = (float *)malloc(sizeof(float) * n);
    float *scratch = (float *)malloc(sizeof(float) * d);
    fo_lloyd_ctx c;
    memset(&c, 0, sizeof(c));
    c.X = X, c.n = n, c.d = d, c.k = k, c.cent = cent, c.order = order, c.chunk = chunk;
    c.assign = out_labels, c.best = best;
    c.lsum = (float *)calloc(nch, sizeof(float));
    c.lchanged = (int64_t *)calloc(nch, sizeof(int64_t));
    if (sums_mode == FO_SUMS_REFERENCE) {
        c.dcsize = (int64_t *)calloc(nch * k, sizeof(int64_t));
        c.dsums = (float *)calloc(nch * k * d, sizeof(float));
    }
    /* initial assignment, lloyd.rs:63-110 (the pairwise-matrix branch) */
    memset(out_labels, 0, sizeof(int64_t) * n);
    c.kind = FO_KIND_PAIRWISE;
    c.initial = 1;
    fo_parallel_for(threads, nch, fo_lloyd_chunk, &c);
    float lastsum = 0.0f;
    int64_t changed = n;
    if (sums_mode == FO_SUMS_REFERENCE) {
        for (int64_t ci = 0; ci < nch; ci++) {
            for (int64_t j = 0; j < k; j++) {
                csize[j] += c.dcsize[ci * k + j];
                for (int64_t t = 0; t < d; t++) sums[j * d + t] = sums[j * d + t] + c.dsums[(ci * k + j) * d + t];
            }
            lastsum = lastsum + c.lsum[ci];
        }
    } else {
        for (int64_t i = 0; i < n; i++) {
            int64_t a = out_labels[i];
            csize[a] += 1;
            for (int64_t t = 0; t < d; t++) sums64[a * d + t] += (double)X[i * d + t];
        }
    }
    int64_t iter = 1;
    c.kind = FO_KIND_SQDIST;
    c.initial = 0;
    while (iter < maxiter) {
        iter++;
        float old_norm = 0.0f, diff_sq = 0.0f;
        if (tol > 0) {
            /* Centers::frobenius_norm, src/cluster/kmeans/util.rs:182-190 */
            for (int64_t j = 0; j < k; j++)
                old_norm = old_norm + fo_dist_f32(FO_KIND_DOT, order, cent + j * d, cent + j * d, d);
            old_norm = sqrtf(old_norm);
        }
        for (int64_t j = 0; j < k; j++) {
            if (csize[j] > 0) {
                if (sums_mode == FO_SUMS_REFERENCE) {
                    float r = 1.0f / (float)csize[j]; /* N::from(csize_j).recip(), lloyd.rs:140 */
                    for (int64_t t = 0; t < d; t++) scratch[t] = sums[j * d + t] * r;
                } else {
                    for (int64_t t = 0; t < d; t++) scratch[t] = (float)(sums64[j * d + t] / (double)csize[j]);
                }
                if (tol > 0) diff_sq = diff_sq + fo_dist_f32(FO_KIND_SQDIST, order, cent + j * d, scratch, d);
                memcpy(cent + j * d, scratch, sizeof(float) * d);
            }
        }
        if (tol > 0) {
            float diff = sqrtf(diff_sq);
            float rel = old_norm == 0.0f ? diff : diff / old_norm;
            if (rel <= (float)tol) break;
        }
        fo_parallel_for(threads, nch, fo_lloyd_chunk, &c);
        changed = 0;
        float total = 0.0f;
        if (sums_mode == FO_SUMS_REFERENCE) {
            for (int64_t ci = 0; ci < nch; ci++) {
                changed += c.lchanged[ci];
                total = total + c.lsum[ci];
                for (int64_t j = 0; j < k; j++) {
                    for (int64_t t = 0; t < d; t++)
                        sums[j * d + t] = sums[j * d + t] + c.dsums[(ci * k + j) * d + t];
                    csize[j] = csize[j] + c.dcsize[ci * k + j];
                }
            }
        } else {
            for (int64_t ci = 0; ci < nch; ci++) {
                changed += c.lchanged[ci];
                total = total + c.lsum[ci];
            }
            memset(sums64, 0, sizeof(double) * k * d);
            memset(csize, 0, sizeof(int64_t) * k);
            for (int64_t i = 0; i < n; i++) {
                int64_t a = out_labels[i];
                csize[a] += 1;
                for (int64_t t = 0; t < d; t++) sums64[a * d + t] += (double)X[i * d + t];
            }
        }
        lastsum = total;
        if (changed == 0) break;
    }
    *out_iters = iter;
    if (out_changed_last) *out_changed_last = changed;
    if (sums_mode == FO_SUMS_REFERENCE) *out_inertia = (double)lastsum;
    else *out_inertia = fo_inertia_fp64(X, n, d, cent, out_labels);
    free(sums);
    free(sums64);
    free(csize);
    free(best);
    free(scratch);
    free(c.lsum);
    free(c.lchanged);
    free(c.dcsize);
    free(c.dsums);
    return 0;
}

/* linear_scan_knn for one query row WITHOUT the marshaller's truncation: the
 * full tie-inclusive KNNHeap::into_vec list (src/api/search.rs:145-150).
 * Writes up to `cap` pairs, returns the list length. */
static int64_t fo_knn_ties_any(int is64, const void *X, int64_t n, int64_t d, const void *q, int64_t k, int metric,
                               int order, int64_t cap, int64_t *out_idx, void *out_dist) {
    fo_knn_ctx c = {is64, X, q, n, d, 1, k, metric, order, 0, NULL, NULL};
    if (k <= 0 || n <= 0) return 0;
    fo_knnheap h;
    memset(&h, 0, sizeof(h));
    h.k = k;
    h.heap = (fo_pair *)malloc(sizeof(fo_pair) * k);
    h.kdist = INFINITY;
    for (int64_t i = 0; i < n; i++) {
        fo_pair p = {fo_query_distance(&c, q, i), i};
        knnheap_insert(&h, p);
    }
    int64_t nres = h.hlen + h.tlen;
    fo_pair *res = (fo_pair *)malloc(sizeof(fo_pair) * (nres ? nres : 1));
    memcpy(res, h.heap, sizeof(fo_pair) * h.hlen);
    if (h.tlen) memcpy(res + h.hlen, h.ties, sizeof(fo_pair) * h.tlen);
    qsort(res, nres, sizeof(fo_pair), fo_pair_qcmp);
    for (int64_t j = 0; j < nres && j < cap; j++) {
        out_idx[j] = res[j].idx;
        if (is64) ((double *)out_dist)[j] = res[j].dist;
        else ((float *)out_dist)[j] = (float)res[j].dist;
    }
    free(res);
    free(h.heap);
    free(h.ties);
    return nres;
}
int64_t fo_knn_ties_f32(const float *X, int64_t n, int64_t d, const float *q, int64_t k, int metric, int order,
                        int64_t cap, int64_t *out_idx, float *out_dist) {
    return fo_knn_ties_any(0, X, n, d, q, k, metric, order, cap, out_idx, out_dist);
}
int64_t fo_knn_ties_f64(const double *X, int64_t n, int64_t d, const double *q, int64_t k, int metric, int order,
                        int64_t cap, int64_t *out_idx, double *out_dist) {
    return fo_knn_ties_any(1, X, n, d, q, k, metric, order, cap, out_idx, out_dist);
}
