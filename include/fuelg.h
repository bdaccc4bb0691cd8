/*
 * fuelg.h -- C ABI of the GB300 engine for kno10/fuel's linear-scan kNN /
 * range search and Lloyd k-means hot path.
 *
 * Plain C: pointers, sizes and status codes; no C++ or torch types.  Every
 * pointer argument may be a host pointer or a CUDA device pointer (unified
 * addressing); host buffers are staged through the device by the call.
 * Every call is synchronous: when it returns, outputs are written.
 * Calls return FUELG_OK (0) or a status code; fuelg_last_error() then gives a
 * message for the calling thread.
 *
 * Semantics follow the reference exactly:
 *  - distances use fuel's own summation order for the chosen host profile
 *    (FUELG_ORDER_ARM = non-x86 builds: src/math/unroll.rs and the portable
 *    fallback of src/distance/squared_euclidean.rs:99-133;
 *    FUELG_ORDER_X86 = x86_64 AVX2+FMA builds: src/math/avx2.rs and
 *    src/distance/squared_euclidean.rs:16-39), so the returned f32 distances
 *    are bit-identical to fuel's;
 *  - neighbours are ordered by (distance, index) as DistPair orders them
 *    (src/api/search.rs:23-30), rows are truncated to k and padded with
 *    -1 / +inf as knn_results_to_arrays does (python/search.rs:1195-1216).
 */
#ifndef FUELG_H
#define FUELG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define FUELG_OK 0
#define FUELG_EINVAL 1     /* bad argument (Python: ValueError)               */
#define FUELG_ENOMEM 2     /* device or host allocation failed                 */
#define FUELG_ECUDA 3      /* CUDA runtime error (Python: RuntimeError)        */
#define FUELG_ECANCELLED 4 /* fuelg_cancel() was called (Python: KeyboardInterrupt) */
#define FUELG_ENOTSUP 5    /* shape or option outside the supported envelope   */
#define FUELG_ENODEV 6     /* no CUDA device                                   */
#define FUELG_ETIMEOUT 7   /* a bounded device wait gave up                    */

/* ---- enums --------------------------------------------------------------- */
#define FUELG_METRIC_SQEUCLIDEAN 0 /* "sqeuclidean" / "squared_euclidean"  */
#define FUELG_METRIC_EUCLIDEAN 1   /* "euclidean" / "l2": sqrt of the above */

#define FUELG_ORDER_ARM 0 /* fuel built for a non-x86 host (e.g. Grace) */
#define FUELG_ORDER_X86 1 /* fuel built for x86_64 with AVX2+FMA        */

#define FUELG_EXCLUDE_NONE 0   /* keep self matches                                         */
#define FUELG_EXCLUDE_LINEAR 1 /* linear-scan index: search k, drop self (python/search.rs:485-488) */
#define FUELG_EXCLUDE_KPLUS1 2 /* tree / precomputed path: search k+1, drop self (python/search.rs:1163-1170) */

#define FUELG_PREC_FP32 0       /* plain FP32 CUDA-core distances (exact reference order)  */
#define FUELG_PREC_BF16 1       /* tcgen05 BF16 screen + exact FP32 re-score (d >= 32)     */
#define FUELG_PREC_SPLIT_BF16 2 /* tcgen05 split-BF16 (hi+lo) screen + exact FP32 re-score */
/* Reported in fuelg_stats.precision_used only: the split-BF16 tier found the
   data to be small integers times one scale (e.g. 8-bit values / 255), so the
   point operand is exact in BF16 and its lo half (zero) is neither stored nor
   read.  Requested as FUELG_PREC_SPLIT_BF16.                                  */
#define FUELG_PREC_SPLIT_BF16_SCALED 3
/* kNN / range only: tcgen05 FP16 screen (one product, ~2^-11 operand rounding,
   a wider proof margin) + exact FP32 re-score; values must lie within the FP16
   range (|v| <= 65504), otherwise the plain FP32 tier answers.               */
#define FUELG_PREC_F16 4
/* Let the engine pick the tier (every tier returns the same bits).  kNN /
   range / serving: d outside [32, 256] -> FP32; integer data with |v| <= 256
   -> BF16 (its screen is exact); otherwise the fastest of the eligible
   tensor-core tiers, timed on the call's first (up to) 4096 query rows the
   first time a (d, log2 n, log2 k, value class) bucket is seen, and kept for
   the process -- and in the file named by FUELG_TUNE_CACHE when that variable
   is set, one line per bucket.  k-means: the split-BF16 tier where its screen
   serves the shape (d >= 32) and the problem is large enough (n >= 16384),
   else FP32; batched k-means: split-BF16 for the problems it serves.
   fuelg_stats.precision_used reports what ran. */
#define FUELG_PREC_AUTO (-1)
/* Reported in fuelg_stats.precision_used by the float64 calls (the exact FP64
   scan); not a request value. */
#define FUELG_PREC_FP64 5

#define FUELG_LLOYD_FIXED_ITERS 1 /* run exactly max_iter iterations (ignore changed==0 stop) */

typedef struct fuelg_index fuelg_index;
typedef struct fuelg_range_result fuelg_range_result;

/* Per-call measurements, filled when a non-NULL pointer is passed. */
typedef struct {
    double device_ms;       /* device time of the call's kernels (CUDA events)      */
    int64_t h2d_bytes;      /* host->device bytes copied by the call                */
    int64_t d2h_bytes;      /* device->host bytes copied by the call                */
    int64_t distance_evals; /* (query, point) distances formed                       */
    int64_t rescored;       /* rows re-scored exactly after a tensor-core screen    */
    int32_t iterations;     /* Lloyd iterations run                                 */
    int32_t precision_used; /* FUELG_PREC_* actually used                           */
    double hot_kernel_ms;   /* summed device time of the dominant kernel's launches,
                               CUDA events on the stream it runs on               */
    int32_t hot_kernel_launches; /* launches of the dominant kernel               */
    int32_t kernel_launches;     /* launches of this library's own kernels        */
} fuelg_stats;

/* Message for the last failing call on this thread ("" if none). */
const char *fuelg_last_error(void);
/* Library version string. */
const char *fuelg_version(void);
/* Number of visible CUDA devices. */
int fuelg_device_count(int32_t *out_count);

/* ---- linear-scan index ---------------------------------------------------
 * Replaces build_linear_scan_f32 (python/search.rs:1353-1370).  Unlike the
 * reference (whose LinearScanSearcher holds only the distance function,
 * python/search.rs:516-518) the handle OWNS a device copy of the data, so
 * repeated queries do not re-upload it. */
int fuelg_index_create(const float *data, int64_t n, int32_t d, int32_t metric, int32_t order, fuelg_index **out);
int fuelg_index_destroy(fuelg_index *index);
int fuelg_index_info(const fuelg_index *index, int64_t *n, int32_t *d, int32_t *metric, int32_t *order);

/* k nearest neighbours of every query row.  Replaces SearchIndex::knn for a
 * linear index (python/search.rs:560-568 -> linear_scan_knn_batch :471-491 ->
 * linear_scan_knn, src/api/search.rs:169-184).  out_idx / out_dist are
 * [m, k] row-major (int64 / f32).  exclude_mode selects the exclude-self rule
 * (FUELG_EXCLUDE_*), which drops index i from query row i.  queries may be
 * NULL when m equals the index size: the index's own rows are then the
 * queries (an all-points self-join with no upload). */
int fuelg_knn(fuelg_index *index, const float *queries, int64_t m, int32_t k, int32_t exclude_mode, int32_t precision,
              int64_t *out_idx, float *out_dist, fuelg_stats *stats);

/* Tie-inclusive k nearest neighbours: for every query row the k nearest
 * points plus every point tied with the k-th distance, sorted by (distance,
 * index) -- the list KNNHeap::into_vec returns (src/api/search.rs:80-151) and
 * fuel's KnnSearch::search_knn contract (src/api/search.rs:268-270) promises.
 * exclude_mode as for fuelg_knn: FUELG_EXCLUDE_LINEAR searches k and then
 * drops index i from row i (python/search.rs:485-488), FUELG_EXCLUDE_KPLUS1
 * searches k+1 and drops self (python/search.rs:1163-1170).  With k = max_k
 * over the index's own rows (queries NULL, m = n, FUELG_EXCLUDE_NONE) this is
 * the table PrecomputedKnnSearcher::new builds (src/search/precomputed.rs:36-55).
 * The lists are CSR, owned by *out (fuelg_range_size / _copy / _free).  Rows
 * with more ties than the call's spare ranks are completed by an exact range
 * scan at their k-th distance. */
int fuelg_knn_ties(fuelg_index *index, const float *queries, int64_t m, int32_t k, int32_t exclude_mode,
                   int32_t precision, fuelg_range_result **out, fuelg_stats *stats);

/* Many independent kNN query sets in one call.  No single counterpart in the
 * reference (fuel answers one SearchIndex::knn at a time,
 * python/search.rs:560-568); each set gets exactly what fuelg_knn returns for
 * a linear index built from its `data` (same metric and summation order,
 * FUELG_PREC_FP32) with its queries, k and exclude rule -- bit-identical
 * indices and distances.  All sets are scanned by one launch over a list of
 * (set, query block, index split) items with their own n, d and k, then
 * merged and finalized by a second launch.  Inputs and outputs are host or
 * device arrays.  precision: FUELG_PREC_FP32 or FUELG_PREC_AUTO (both run the
 * exact CUDA-core scan; the tensor-core tiers serve one index per fuelg_knn
 * call).  Per-set failures (bad shape, d beyond the scan's limit) are written
 * to the set's status and the call returns FUELG_EINVAL; nothing is computed
 * then. */
typedef struct {
  const float *data;    /* [n, d] */
  int64_t n;
  int32_t d;
  int32_t metric;       /* FUELG_METRIC_* */
  const float *queries; /* [m, d] */
  int64_t m;
  int32_t k;
  int32_t exclude_mode; /* FUELG_EXCLUDE_*: query row i vs point i of this set */
  int64_t *out_idx;     /* [m, k] */
  float *out_dist;      /* [m, k] */
  int32_t status;       /* FUELG_OK or the set's error */
  int32_t reserved;
} fuelg_knn_set;
int fuelg_knn_batched(fuelg_knn_set *sets, int32_t count, int32_t order, int32_t precision, fuelg_stats *stats);

/* Accuracy of returned kNN rows against FP64.  No counterpart in the
 * reference (fuel's distances are f32 throughout); it checks results of
 * fuelg_knn / fuelg_server_* against distances formed in double: for every
 * returned pair (idx >= 0) of rows [m, k] (host or device arrays; queries NULL
 * = the index's own rows, as for fuelg_knn) the f32 distance is compared with
 * the FP64 one, adjacent neighbours whose f32 distances are equal or one ulp
 * apart are counted as near_ties, and adjacent neighbours that the FP64
 * distances (index breaking exact ties, DistPair order, src/api/search.rs:23-30)
 * rank the other way are counted as order_flips -- the only places where the
 * reference's f32 lists can differ from an FP64 ranking. */
typedef struct {
    double max_abs_err;  /* max |d_f32 - d_fp64| over the returned pairs            */
    double max_rel_err;  /* max |d_f32 - d_fp64| / d_fp64 (pairs with d_fp64 > 0)   */
    int64_t pairs;       /* returned (query, neighbour) pairs checked               */
    int64_t near_ties;   /* adjacent neighbours within one f32 ulp (or equal)       */
    int64_t order_flips; /* adjacent neighbours ranked the other way by FP64        */
} fuelg_error_report;
int fuelg_knn_error(fuelg_index *index, const float *queries, int64_t m, int32_t k, const int64_t *idx,
                    const float *dist, fuelg_error_report *out);

/* Sustained FP32 FMA issue rate of the current GPU in 10^12 FMA/s (an FMA is
 * one lane operation; two flops): the denominator of the plain FP32 tiers'
 * roofline.  No counterpart in the reference. */
int fuelg_fp32_rate(double *tera_fma_per_s);

/* All points with distance <= radius (radius is cast to f32 as
 * python/search.rs:781-783 does), sorted by (distance, index).  Replaces
 * SearchIndex::radius_search (python/search.rs:776-790 -> linear_scan_range,
 * src/api/search.rs:154-166).  The result is CSR, owned by the handle *out. */
int fuelg_range(fuelg_index *index, const float *queries, int64_t m, double radius, int32_t exclude_self,
                fuelg_range_result **out, fuelg_stats *stats);
int fuelg_range_size(const fuelg_range_result *res, int64_t *m, int64_t *total);
/* offsets: [m+1]; idx / dist: [total]. */
int fuelg_range_copy(const fuelg_range_result *res, int64_t *offsets, int64_t *idx, float *dist);
int fuelg_range_free(fuelg_range_result *res);

/* All pairwise distances of one point set.  Replaces
 * fuel.search.pairwise_distances for raw f32 points (python/fuel/search.py:
 * 92-150 -> _compute_pairwise_distances[_condensed]_f32, python/mod.rs:74-124
 * -> compute_pairwise_condensed / compute_pairwise_dense,
 * src/api/condensed_distance_matrix.rs:16-48, square_distance_matrix.rs:11-40).
 * form FUELG_PAIRWISE_CONDENSED: out[i*(i-1)/2 + j] for j < i (n*(n-1)/2
 * values); FUELG_PAIRWISE_SQUARE: out[i*n + j], n*n values.  Values are
 * bit-identical to the reference distance in the given summation order.
 * X and out may be host or device pointers. */
#define FUELG_PAIRWISE_CONDENSED 0
#define FUELG_PAIRWISE_SQUARE 1
int fuelg_pairwise(const float *X, int64_t n, int32_t d, int32_t metric, int32_t order, int32_t form, float *out,
                   fuelg_stats *stats);

/* ---- float64 data ----------------------------------------------------------
 * fuel builds a float64 index for every input that is not float32
 * (python/fuel/_dispatch.py:8-19; build_linear_scan_f64, python/search.rs:
 * 1371-1389) and compares f64 distances in its f64 operation order
 * (src/distance/squared_euclidean.rs:44-67 on x86 AVX + FMA builds, :99-133
 * elsewhere; Euclidean = f64 sqrt).  These calls run the exact FP64 scan:
 * every (query, point) distance in that order, (distance, index) order and
 * the same tie, exclude and padding rules as the float32 calls.  A float64
 * index (n <= 2^32 - 2) serves only the _f64 calls, a float32 index only the
 * float32 calls (FUELG_EINVAL otherwise).  Distances are f64 (+inf padding);
 * fuelg_stats.precision_used reports FUELG_PREC_FP64. */
int fuelg_index_create_f64(const double *data, int64_t n, int32_t d, int32_t metric, int32_t order,
                           fuelg_index **out);
/* As fuelg_knn: out_idx / out_dist [m, k] (int64 / f64); queries NULL = the
 * index's own rows (m = n). */
int fuelg_knn_f64(fuelg_index *index, const double *queries, int64_t m, int32_t k, int32_t exclude_mode,
                  int64_t *out_idx, double *out_dist, fuelg_stats *stats);
/* As fuelg_knn_ties; read the lists with fuelg_range_copy_f64. */
int fuelg_knn_ties_f64(fuelg_index *index, const double *queries, int64_t m, int32_t k, int32_t exclude_mode,
                       fuelg_range_result **out, fuelg_stats *stats);
/* As fuelg_range with an f64 radius (linear_scan_range on f64 data); read the
 * lists with fuelg_range_copy_f64. */
int fuelg_range_f64(fuelg_index *index, const double *queries, int64_t m, double radius, int32_t exclude_self,
                    fuelg_range_result **out, fuelg_stats *stats);
/* offsets [m+1]; idx / dist [total] of a float64 result. */
int fuelg_range_copy_f64(const fuelg_range_result *res, int64_t *offsets, int64_t *idx, double *dist);
/* As fuelg_pairwise on float64 points (_compute_pairwise_distances[_condensed]_f64,
 * python/mod.rs:74-124). */
int fuelg_pairwise_f64(const double *X, int64_t n, int32_t d, int32_t metric, int32_t order, int32_t form,
                       double *out, fuelg_stats *stats);

/* Lloyd k-means with fixed initial centres.  Replaces lloyd_f32
 * (python/kmeans.rs:188-218, 355) -> cluster::kmeans::lloyd
 * (src/cluster/kmeans/lloyd.rs:118-202) with InitMethod::Fixed
 * (python/kmeans.rs:111-130).  Centre sums are exact integer sums (every
 * f32 coordinate is an integer multiple of a common power of two; FP64 sums
 * when the exponent range is too wide), means are rounded to nearest f32,
 * and inertia is the FP64 sum of squared distances of the final pass.
 * out_centers [k, d] f32, out_labels [n] int64. */
int fuelg_kmeans_lloyd(const float *data, int64_t n, int32_t d, int32_t k, const float *init_centers,
                       int32_t max_iter, double tol, int32_t precision, int32_t order, int32_t flags,
                       float *out_centers, int64_t *out_labels, int32_t *out_iters, double *out_inertia,
                       fuelg_stats *stats);

/* One Lloyd assignment pass against fixed centres: for every point the
 * nearest centre, the first index winning ties (strict < over centres in
 * order).  initial != 0 uses the initial pass's arithmetic
 * (lloyd_initial_assignment, src/cluster/kmeans/lloyd.rs:12-112, through
 * vec_pairwise_sqdist), initial == 0 that of the iteration loop
 * (lloyd.rs:140-158, math::sqdist).  It is the per-shard compute of a
 * sharded Lloyd (points split across devices, exact sums all-reduced).
 * out_labels [n] int64; out_best [n] f32 squared distance (may be NULL). */
int fuelg_lloyd_assign(const float *data, int64_t n, int32_t d, const float *centers, int32_t k, int32_t initial,
                       int32_t order, int64_t *out_labels, float *out_best, fuelg_stats *stats);

/* Many independent Lloyd k-means problems in one call.  No single
 * counterpart in the reference (fuel runs one lloyd() at a time,
 * src/cluster/kmeans/lloyd.rs:118-202); each problem gets exactly what
 * fuelg_kmeans_lloyd (same order, same flags) returns for it: all problems'
 * points are assigned by one persistent kernel per iteration over a work
 * queue of 256-row items, sums of changed points are kept exactly, and the
 * middle iterations run as one replayed CUDA graph.  Inputs are host or
 * device arrays; per-problem results and status are written into the
 * descriptors (status FUELG_ENOTSUP: data whose exponent range exceeds the
 * exact 128-bit sums, or non-finite values). */
typedef struct {
  const float *data;   /* [n, d] */
  int64_t n;
  int32_t d;
  int32_t k;
  const float *init;   /* [k, d] initial centres */
  float *out_centers;  /* [k, d] */
  int64_t *out_labels; /* [n] */
  int32_t out_iters;
  int32_t status;
  double out_inertia;
} fuelg_kmeans_problem;
/* precision: FUELG_PREC_FP32 = exact CUDA-core assignment everywhere; BF16 or
 * SPLIT_BF16 = problems with 32 <= d <= 64 and k <= 256 are screened with
 * split-BF16 tensor-core products and re-scored exactly where the screen
 * cannot decide (identical results). */
int fuelg_kmeans_batched(fuelg_kmeans_problem *problems, int32_t count, int32_t max_iter, int32_t order,
                         int32_t precision, int32_t flags, fuelg_stats *stats);

/* kNN serving with continuous batching over a resident index.  No
 * counterpart in the reference (fuel answers one call at a time); it serves
 * streams of independent query batches.  `workers` threads each own a CUDA
 * stream; a free worker takes every queued request that fits
 * max_batch_queries rows and the device-memory budget (budget_bytes, charged
 * per request while its batch runs) and runs them as one batch, so requests
 * that arrive while others are on the GPU are admitted as memory frees up and
 * their device work overlaps.  Each request gets exactly what fuelg_knn
 * (exclude_mode FUELG_EXCLUDE_NONE, same precision tier) returns for its rows.
 * The index must outlive the server and must not be used by other calls while
 * the server runs. */
typedef struct fuelg_server fuelg_server;
int fuelg_server_create(fuelg_index *ix, int32_t precision, int64_t max_batch_queries, int64_t budget_bytes,
                        int32_t workers, fuelg_server **out);
/* Queues m query rows (copied before returning); out_idx [m, k] / out_dist
 * [m, k] are host memory written when the request completes (keep them alive
 * until fuelg_server_wait returns).  Fails with FUELG_ENOMEM when the request
 * alone exceeds the budget. */
int fuelg_server_submit(fuelg_server *s, const float *queries, int64_t m, int32_t k, int64_t *out_idx,
                        float *out_dist, int64_t *request_id);
/* Blocks until the request finished (timeout_ms < 0: no limit; on expiry
 * FUELG_ETIMEOUT and the request stays pending); returns its status and the
 * submit-to-completion latency.  Each id can be waited for once. */
int fuelg_server_wait(fuelg_server *s, int64_t request_id, int32_t timeout_ms, double *latency_ms);
int fuelg_server_stats(fuelg_server *s, int64_t *batches, int64_t *queries, int64_t *max_batch_rows,
                       int64_t *max_batch_requests, double *device_ms);
/* Finishes every queued request, then stops the workers. */
int fuelg_server_destroy(fuelg_server *s);

/* Allocation-free exact kNN.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory -- hosts whose GPU memory belongs
 * to another allocator (a framework's caching pool) or is budgeted up front,
 * and embedded callers that must not grow their footprint after start-up.
 * Same results as fuelg_knn on a linear index built from `data` with the same
 * metric and order.
 *  - data [n, d], queries [m, d], out_idx / out_dist [m, k] must be memory of
 *    the current device (or managed / mapped memory): host buffers and device
 *    memory of another GPU are rejected with FUELG_EINVAL, since staging them
 *    would need an allocation.
 *  - every temporary lives in one static 32 MiB device array of the library,
 *    held by each GPU that loads it until the process exits; queries are
 *    processed in batches that fit it; k <= 4095 (FUELG_ENOTSUP beyond).
 *  - the first call on a device (and the first call in a different CUDA
 *    context) resolves that array's address with cudaGetSymbolAddress.
 *  - all calls share the array and leave their contents in it, so calls that
 *    overlap on the GPU (different streams, host threads) race: serialise them.
 *  - work is ordered on `stream` (a cudaStream_t, NULL = legacy default); the
 *    call waits for that stream to finish and reads a device status word back
 *    before it returns; no cancellation. */
int fuelg_knn_noalloc(const float *data, int64_t n, int32_t d, const float *queries, int64_t m, int32_t k,
                      int32_t metric, int32_t order, int32_t exclude_mode, int64_t *out_idx, float *out_dist,
                      void *stream);

/* Cooperative cancellation (src/api/mod.rs:29 SHUTDOWN_REQUESTED): running
 * kernels poll a host-mapped word and stop; the call returns
 * FUELG_ECANCELLED.  Each call clears the word when it starts, as
 * py_interruptible does (src/api/parallel.rs:145-173). */
int fuelg_cancel(void);
int fuelg_reset_cancel(void);

/* Frees what the library keeps between calls: its stream-ordered memory pool
 * of temporaries (up to 16 GB cached per device), the instantiated CUDA graphs
 * of the Lloyd loop (kept per host thread), the host-mapped cancellation word
 * and the resolved scratch addresses of fuelg_knn_noalloc.  Later calls set
 * them up again.  Indexes and range results stay valid across a release
 * (they own their device memory); FUELG_EINVAL while a server is open.  Call
 * it with no library call in flight on any thread: before cudaDeviceReset, or
 * before destroying a CUDA context the library ran in (after destroying the
 * handles made in it). */
int fuelg_release(void);

#ifdef __cplusplus
}
#endif
#endif /* FUELG_H */
