// fuelg_internal.h -- host-side declarations shared by the engine's
// translation units (not part of the public C ABI; see include/fuelg.h).
#pragma once
#include <cstdint>
#include <cstdio>
#include <string>
#include <utility>
#include <vector>
#include <cuda.h>
#include <cuda_runtime.h>

namespace fuelg {

// Status codes mirrored by include/fuelg.h.
enum Status : int {
  ST_OK = 0,
  ST_EINVAL = 1,
  ST_ENOMEM = 2,
  ST_ECUDA = 3,
  ST_ECANCELLED = 4,
  ST_ENOTSUP = 5,
  ST_ENODEV = 6,
  ST_ETIMEOUT = 7,
};

void set_error(const char* fmt, ...);
const char* last_error();

#define FUELG_CUDA(call)                                                                               \
  do {                                                                                                 \
    cudaError_t e_ = (call);                                                                           \
    if (e_ != cudaSuccess) {                                                                           \
      ::fuelg::set_error("CUDA error %s at %s:%d: %s", cudaGetErrorName(e_), __FILE__, __LINE__,       \
                         cudaGetErrorString(e_));                                                      \
      return ::fuelg::ST_ECUDA;                                                                        \
    }                                                                                                  \
  } while (0)

#define FUELG_TRY(expr)            \
  do {                             \
    int s_ = (expr);               \
    if (s_ != ::fuelg::ST_OK) return s_; \
  } while (0)

// The stream-ordered memory pool of this library's temporaries on the current
// device: it keeps up to 16 GB cached between calls, where the device's default
// pool hands its memory back at every synchronisation and the next call maps it
// again.
cudaMemPool_t lib_pool();

// The calling thread's current CUDA context (nullptr when it has none), read
// through the driver's cuCtxGetCurrent.
CUcontext current_context();

// State kept between calls is released by fuelg_release.  The Lloyd loop's
// instantiated graphs are kept per host thread: keep_graph registers one so
// that a release destroys every thread's, drop_graph destroys a registered one
// (once), and cache_generation() changes at every release, after which a
// thread's own handles are stale and must be forgotten, not destroyed.
void keep_graph(cudaGraphExec_t g);
void drop_graph(cudaGraphExec_t g);
uint64_t cache_generation();
// Forgets the allocation-free kNN path's resolved scratch addresses.
void noalloc_forget();
// Open serving handles (a release is refused while one is open).
void server_opened();
void server_closed();

// Stream-ordered scratch allocations (from lib_pool) freed on scope exit.
struct Scratch {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  Scratch() = default;
  Scratch(const Scratch&) = delete;
  Scratch& operator=(const Scratch&) = delete;
  ~Scratch() {
    if (p) cudaFreeAsync(p, s);
  }
  int alloc(size_t bytes, cudaStream_t stream) {
    s = stream;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMallocFromPoolAsync(&p, bytes, lib_pool(), stream);
    if (e != cudaSuccess) {
      p = nullptr;
      set_error("device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
      return ST_ENOMEM;
    }
    return ST_OK;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

// Per-thread accounting of this library's own kernel launches, and optional
// CUDA-event timing of the dominant ("hot") kernel of a call, recorded on the
// stream that kernel is launched on.
void note_launch(int count = 1);
int64_t launch_count();
struct HotTimer {
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
  void begin(cudaStream_t s) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
    ev.emplace_back(a, b);
  }
  void end(cudaStream_t s) { cudaEventRecord(ev.back().second, s); }
  double total_ms() const {
    double t = 0;
    for (auto& e : ev) {
      float ms = 0.f;
      cudaEventSynchronize(e.second);
      cudaEventElapsedTime(&ms, e.first, e.second);
      t += ms;
    }
    return t;
  }
  int count() const { return (int)ev.size(); }
  ~HotTimer() {
    for (auto& e : ev) {
      cudaEventDestroy(e.first);
      cudaEventDestroy(e.second);
    }
  }
};
// The timer the current call installed for its hot kernel (or nullptr).
HotTimer*& hot_timer();

// Launch with programmatic stream serialisation (see griddep_wait()).
template <typename... KArgs, typename... Args>
int launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  note_launch();
  cudaError_t e = cudaLaunchKernelEx(&cfg, kern, ((KArgs)args)...);
  if (e != cudaSuccess) {
    set_error("kernel launch failed: %s", cudaGetErrorString(e));
    return ST_ECUDA;
  }
  return ST_OK;
}

// Host-mapped cancel word (pinned, device-visible); set by fuelg_cancel().
int* cancel_word_device();
bool cancel_requested();

// Device status word helpers (per call).
struct DevStatus {
  int* d = nullptr;
};

// -------- exact linear-scan top-k (fuelg_knn.cu) ----------------------------
struct ExactScanParams {
  const float* A = nullptr;  // queries [m, d] (device)
  int64_t m = 0;
  const float* B = nullptr;  // points [n, d] (device)
  int64_t n = 0;
  int d = 0;
  int kind = 0;    // Kind
  int order = 0;   // Order
  int metric = 0;  // Metric
  int kk = 0;      // keys kept per query (k or k+1)
};

// Top-kk (distance, index) keys per query, sorted ascending, written to
// out_keys [m, kk] (device).  Unused slots hold ~0ull.
int exact_topk(const ExactScanParams& p, uint64_t* out_keys, int* dev_status, cudaStream_t stream);

// Turn sorted keys [m, kk] into the reference's (int64 idx, float dist) rows
// with the given exclude-self mode and -1/+inf padding.
int finalize_knn(const uint64_t* keys, int64_t m, int kk, int k, int exclude_mode, int64_t* out_idx, float* out_dist,
                 cudaStream_t stream);

// Many independent kNN query sets (device buffers), each with its own data,
// n, d, k, metric and exclude rule, scanned in one launch over a list of
// (set, query block, index split) items, merged and finalized in a second.
struct KnnSetDev {
  const float* A;  // queries [m, d]
  int64_t m;
  const float* B;  // points [n, d]
  int64_t n;
  int d, metric, k, mode;
  int64_t* out_idx;  // [m, k]
  float* out_dist;
};
struct KnnSetOut {
  int64_t* out_idx;
  float* out_dist;
  int32_t k, mode;
};
int exact_knn_sets(const KnnSetDev* sets, int count, int order, int* dev_status, cudaStream_t stream);

// Top-k + finalize with every temporary inside the caller-provided scratch
// region (no allocation; queries are batched to fit; no cancellation).
int exact_knn_in_scratch(const ExactScanParams& p, int k, int exclude_mode, int64_t* out_idx, float* out_dist,
                         void* scratch, size_t scratch_bytes, cudaStream_t stream);

// The exact FP64 scan (fuelg_f64.cu) over a float64 index X [n, d] (n <= 2^32 - 2).
struct F64Scan {
  const double* X = nullptr;
  int64_t n = 0;
  int d = 0;
  int metric = 0;
  int order = 0;
};
// Truncated kNN rows [m, k] (device outputs) under an exclude rule (FUELG_EXCLUDE_*).
int f64_knn(const F64Scan& x, const double* Q, int64_t m, int k, int mode, int64_t* out_idx, double* out_dist,
            cudaStream_t s);
// CSR lists in host memory: tie-inclusive kNN lists of kq (range false), or
// every point within radius (range true); drop_self leaves point i out of row i.
int f64_lists(const F64Scan& x, const double* Q, int64_t m, bool range, int64_t kq, bool drop_self, double radius,
              std::vector<int64_t>* off, std::vector<int64_t>* idx, std::vector<double>* dist, int64_t* d2h,
              cudaStream_t s);
// All pairwise distances of X (FUELG_PAIRWISE_* layouts), device output.
int f64_pairwise(const double* X, int64_t n, int d, int metric, int order, int form, double* out, cudaStream_t s);

// Tensor-core kNN (fuelg_knn_tc.cu): top-kk keys per query [m, kk] via a
// tcgen05 screen; exact for integer data, otherwise re-scored and proven.
// Operand tiers: BF16 (one product, error ~2^-8), split BF16 (hi + lo, three
// products, ~2^-16), FP16 (one product, ~2^-11; values within the FP16 range).
constexpr int TC_BF16 = 0, TC_SPLIT = 1, TC_F16 = 2;
bool knn_tc_supported(int64_t n, int d, int kk, int tier);
// Resident tensor-core form of an index: BF16 copy padded to whole tiles, FP32
// norms, integer census and the index-side bounds; built once per handle.
struct TcIndex;
int knn_tc_index_build(const float* X32, int64_t n, int d, cudaStream_t stream, TcIndex** out);
void knn_tc_index_free(TcIndex* t);
// Value class of an index's data, which decides the cheapest exact tier:
// integers with |v| <= 256 (the BF16 screen is exact), values within the FP16
// range, or wider values.
constexpr int TC_CLASS_INTEGER = 0, TC_CLASS_F16_RANGE = 1, TC_CLASS_WIDE = 2;
int knn_tc_index_class(const TcIndex* t);
int knn_tc_index_add_lo(TcIndex* t, const float* X32, cudaStream_t stream);
// FP16 copy of the index; ST_ENOTSUP when a value lies outside the FP16 range.
int knn_tc_index_add_f16(TcIndex* t, const float* X32, cudaStream_t stream);
// tier: TC_BF16 / TC_SPLIT / TC_F16 operands; integer data whose BF16 screen
// is exact always use BF16 (no margin, no re-score); FP16 falls back to the
// split tier when the queries leave the FP16 range.  row_k (device, m entries, or
// nullptr): a smaller k per query row -- row q's first row_k[q] keys (of the
// kk per row written) are its exact top row_k[q]; the rest are unspecified.
int knn_tc_topk(const TcIndex* ti, const float* Q32, int64_t m, const float* X32, int kk, int order, int metric,
                int tier, uint64_t* out_keys, int* dev_status, cudaStream_t stream, int64_t* rescored,
                int* exact_out, const int32_t* row_k = nullptr);

// Read-only view of an index handle for concurrent users (the serving loop);
// with want_tc the tensor-core form is built first when the shape allows it.
struct IndexView {
  int device = 0;
  int64_t n = 0;
  int d = 0;
  int metric = 0;
  int order = 0;
  const float* X = nullptr;
  const TcIndex* tc = nullptr;
  bool f16 = false;  // the index has its FP16 copy (FP16 tier)
};
}  // namespace fuelg
struct fuelg_index;
namespace fuelg {
// want_tier (TC_*, or -1 for none): build that tensor-core form of the index.
int index_view_get(fuelg_index* ix, int want_tier, IndexView* out);

// All pairwise distances (fuelg_pairwise.cu): condensed or square form, out on the device.
int pairwise_launch(const float* X, int64_t n, int d, int metric, int order, int form, float* out,
                    cudaStream_t stream);

// Range search, CSR output on the device.  Allocates *off/*idx/*dist with cudaMalloc.
// radii (device, p.m entries, or nullptr): a radius per query row instead of `radius`.
int exact_range(const ExactScanParams& p, float radius, int exclude_self, int64_t** d_off, int64_t** d_idx,
                float** d_dist, int64_t* total, int* dev_status, cudaStream_t stream, const float* radii = nullptr);

// -------- tie-inclusive kNN lists (fuelg_ties.cu) ------------------------------
// Keys kept per query for tie-inclusive lists of kq neighbours (kq plus spare ranks).
int ties_spare_kk(int kq, int64_t n);
// From sorted top-kk keys [m, kk] (device; kk from ties_spare_kk), the lists
// {i : dist(q, i) <= D_kq} of every query row, sorted by (distance, index),
// index r dropped from row r when drop_self; rows with more ties than spare
// ranks are answered by an exact range scan of base (queries base.A, index
// base.B).  CSR output allocated with cudaMalloc (freed by the caller, also on
// error); *range_rows = rows that took the range scan.
int knn_ties_lists(const uint64_t* keys, int64_t m, int kk, int kq, int drop_self, const ExactScanParams& base,
                   int64_t** d_off, int64_t** d_idx, float** d_dist, int64_t* total, int64_t* range_rows,
                   int* dev_status, cudaStream_t s);

// -------- accuracy report and FP32 issue rate (fuelg_check.cu) ----------------
// FP64 check of returned kNN rows (Q [m, d], X the index, idx / dist [m, k],
// all device): max |d - D| and max |d - D| / D over the returned pairs, the
// number of pairs, adjacent neighbours within one f32 ulp, and adjacent
// neighbours that FP64 distances order the other way.
int knn_error_report(const float* Q, const float* X, int64_t m, int d, int k, int metric, const int64_t* idx,
                     const float* dist, double* max_abs, double* max_rel, int64_t* pairs, int64_t* near_ties,
                     int64_t* flips, cudaStream_t s);
// Sustained FP32 FMA issue rate of the current device (10^12 FMA/s; one FMA
// is one lane operation, two flops), best of five CUDA-event-timed launches.
int fp32_issue_rate(double* tera_fma_per_s, double* ms);

// -------- Lloyd (fuelg_lloyd.cu) -------------------------------------------
struct LloydParams {
  const float* X = nullptr;  // [n, d] device
  int64_t n = 0;
  int d = 0;
  int k = 0;
  const float* init = nullptr;  // [k, d] device
  int max_iter = 0;
  double tol = 0.0;
  int order = 0;
  int precision = 0;
  int fixed_iters = 0;  // 1: ignore the changed==0 stop (benchmark mode)
};
struct LloydResult {
  float* centers = nullptr;   // [k, d] device (caller-provided)
  int32_t* labels = nullptr;  // [n] device (caller-provided)
  int32_t iters = 0;
  double inertia = 0.0;
  int64_t rescored = 0;       // points re-scored exactly (tensor-core tiers)
  int precision_used = 0;     // tier that actually ran
  bool exact_sums = false;    // centroid sums exact (integer) rather than FP64
  double kernel_ms = 0.0;
};
int lloyd_run(const LloydParams& p, LloydResult* r, int* dev_status, cudaStream_t stream);

}  // namespace fuelg
