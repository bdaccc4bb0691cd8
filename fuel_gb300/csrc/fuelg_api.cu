// fuelg_api.cu -- the C ABI (include/fuelg.h): handles, staging of host
// buffers, status codes, cancellation and per-call measurements.
#include <cstdarg>
#include <cstring>
#include <atomic>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "../../include/fuelg.h"
#include "fuelg_common.cuh"
#include "fuelg_internal.h"

namespace fuelg {

namespace {
thread_local std::string g_err;
thread_local int64_t g_launches = 0;
thread_local HotTimer* g_hot = nullptr;
std::mutex g_cancel_mu;
int* g_cancel_host = nullptr;  // pinned + mapped
int* g_cancel_dev = nullptr;
}  // namespace

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
}
const char* last_error() { return g_err.c_str(); }
void note_launch(int count) { g_launches += count; }
int64_t launch_count() { return g_launches; }
HotTimer*& hot_timer() { return g_hot; }

namespace {
// Memory pools made by lib_pool, per device (a device whose pool could not be
// made uses its default pool, which is not destroyed on release).
struct PoolEntry {
  cudaMemPool_t pool = nullptr;
  bool created = false;
};
std::mutex g_pool_mu;
std::map<int, PoolEntry>& pools() {
  static auto* m = new std::map<int, PoolEntry>();  // never destroyed: threads may outlive static teardown
  return *m;
}

// Every thread's kept graph executables, and the release generation.
struct GraphRegistry {
  std::mutex mu;
  std::set<cudaGraphExec_t> graphs;
  std::atomic<uint64_t> gen{1};
};
GraphRegistry& graph_registry() {
  static auto* r = new GraphRegistry();
  return *r;
}

std::atomic<int> g_open_servers{0};
}  // namespace

cudaMemPool_t lib_pool() {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_pool_mu);
  auto it = pools().find(dev);
  if (it != pools().end()) return it->second.pool;
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.handleTypes = cudaMemHandleTypeNone;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  PoolEntry e;
  if (cudaMemPoolCreate(&e.pool, &props) == cudaSuccess) {
    uint64_t keep = 16ull << 30;
    cudaMemPoolSetAttribute(e.pool, cudaMemPoolAttrReleaseThreshold, &keep);
    e.created = true;
  } else {
    cudaGetLastError();
    e.pool = nullptr;
    cudaDeviceGetDefaultMemPool(&e.pool, dev);
  }
  pools()[dev] = e;
  return e.pool;
}

CUcontext current_context() {
  using Fn = CUresult (*)(CUcontext*);
  static Fn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<Fn>(p);
    cudaGetLastError();
    return (Fn) nullptr;
  }();
  CUcontext ctx = nullptr;
  if (!fn || fn(&ctx) != CUDA_SUCCESS) return nullptr;
  return ctx;
}

void keep_graph(cudaGraphExec_t g) {
  GraphRegistry& r = graph_registry();
  std::lock_guard<std::mutex> lk(r.mu);
  r.graphs.insert(g);
}
void drop_graph(cudaGraphExec_t g) {
  GraphRegistry& r = graph_registry();
  std::lock_guard<std::mutex> lk(r.mu);
  if (r.graphs.erase(g)) cudaGraphExecDestroy(g);
}
uint64_t cache_generation() { return graph_registry().gen.load(); }

void server_opened() { g_open_servers++; }
void server_closed() { g_open_servers--; }

static int ensure_cancel_word() {
  std::lock_guard<std::mutex> lk(g_cancel_mu);
  if (g_cancel_host) return ST_OK;
  int* h = nullptr;
  cudaError_t e = cudaHostAlloc(&h, sizeof(int), cudaHostAllocMapped | cudaHostAllocPortable);
  if (e != cudaSuccess) {
    set_error("cannot allocate the cancel word: %s", cudaGetErrorString(e));
    return ST_ECUDA;
  }
  *h = 0;
  int* dptr = nullptr;
  e = cudaHostGetDevicePointer(&dptr, h, 0);
  if (e != cudaSuccess) {
    cudaFreeHost(h);
    set_error("cannot map the cancel word: %s", cudaGetErrorString(e));
    return ST_ECUDA;
  }
  g_cancel_dev = dptr;
  g_cancel_host = h;
  return ST_OK;
}
int* cancel_word_device() { return g_cancel_dev; }
bool cancel_requested() { return g_cancel_host && *(volatile int*)g_cancel_host; }

__global__ void widen_labels_kernel(const int32_t* __restrict__ a, int64_t* __restrict__ b, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}
void widen_labels(const int32_t* a, int64_t* b, int64_t n, cudaStream_t s) {
  if (n > 0) widen_labels_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, b, n); ::fuelg::note_launch();
}

}  // namespace fuelg

using namespace fuelg;

struct fuelg_index {
  int device = 0;
  int64_t n = 0;
  int32_t d = 0;
  int32_t metric = 0;
  int32_t order = 0;
  float* X = nullptr;  // device copy [n, d]
  TcIndex* tc = nullptr;  // tensor-core form, built on the first tensor-core call
  bool f64 = false;       // a float64 index (fuelg_index_create_f64): X64 instead of X
  double* X64 = nullptr;  // device copy [n, d]
  cudaStream_t stream = nullptr;
  std::mutex mu;  // calls on one handle are serialised
};

struct fuelg_range_result {
  int64_t m = 0, total = 0;
  int64_t* off = nullptr;  // device
  int64_t* idx = nullptr;
  float* dist = nullptr;
  // float64 lists (fuelg_knn_ties_f64 / fuelg_range_f64) are kept in host memory
  bool f64 = false;
  std::vector<int64_t> h_off, h_idx;
  std::vector<double> h_dist;
};

namespace {

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// A read-only input view: device pointer used in place, host pointer staged.
struct InBuf {
  const void* dptr = nullptr;
  Scratch own;
  int64_t h2d = 0;
  int init(const void* src, size_t bytes, cudaStream_t s) {
    if (bytes == 0) {
      dptr = nullptr;
      return ST_OK;
    }
    if (is_device_ptr(src)) {
      dptr = src;
      return ST_OK;
    }
    FUELG_TRY(own.alloc(bytes, s));
    FUELG_CUDA(cudaMemcpyAsync(own.p, src, bytes, cudaMemcpyHostToDevice, s));
    dptr = own.p;
    h2d = (int64_t)bytes;
    return ST_OK;
  }
};

// An output view: device pointer written in place, host pointer written back.
struct OutBuf {
  void* user = nullptr;
  void* dptr = nullptr;
  Scratch own;
  size_t bytes = 0;
  bool staged = false;
  int init(void* dst, size_t b, cudaStream_t s) {
    user = dst;
    bytes = b;
    if (b == 0) return ST_OK;
    if (is_device_ptr(dst)) {
      dptr = dst;
      return ST_OK;
    }
    FUELG_TRY(own.alloc(b, s));
    dptr = own.p;
    staged = true;
    return ST_OK;
  }
  int flush(cudaStream_t s, int64_t* d2h) {
    if (staged && bytes) {
      FUELG_CUDA(cudaMemcpyAsync(user, dptr, bytes, cudaMemcpyDeviceToHost, s));
      if (d2h) *d2h += (int64_t)bytes;
    }
    return ST_OK;
  }
};

int check_device() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    set_error("no CUDA device is visible; the GB300 engine has no CPU fallback");
    return ST_ENODEV;
  }
  return ST_OK;
}

int begin_call() {
  FUELG_TRY(check_device());
  FUELG_TRY(ensure_cancel_word());
  *(volatile int*)g_cancel_host = 0;  // py_interruptible resets before running
  return ST_OK;
}

int read_dev_status(const int* dstat, cudaStream_t s) {
  int h = 0;
  FUELG_CUDA(cudaMemcpyAsync(&h, dstat, sizeof(int), cudaMemcpyDeviceToHost, s));
  FUELG_CUDA(cudaStreamSynchronize(s));
  if (h & DEV_CANCELLED) {
    set_error("interrupted");
    return ST_ECANCELLED;
  }
  if (h & DEV_TIMEOUT) {
    set_error("a bounded device wait timed out");
    return ST_ETIMEOUT;
  }
  if (h & DEV_BADARG) {
    set_error("a kernel rejected its arguments");
    return ST_EINVAL;
  }
  return ST_OK;
}

// Installs a HotTimer for the current call and snapshots the launch counter.
struct CallMeter {
  HotTimer ht;
  int64_t launches0;
  CallMeter() : launches0(launch_count()) { hot_timer() = &ht; }
  ~CallMeter() { hot_timer() = nullptr; }
  void fill(fuelg_stats* st) {
    if (!st) return;
    st->hot_kernel_ms = ht.total_ms();
    st->hot_kernel_launches = ht.count();
    st->kernel_launches = (int32_t)(launch_count() - launches0);
  }
};

struct Timer {
  cudaEvent_t a = nullptr, b = nullptr;
  cudaStream_t s;
  explicit Timer(cudaStream_t st) : s(st) {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
  }
  double stop() {
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
  }
  ~Timer() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

}  // namespace

extern "C" {

const char* fuelg_last_error(void) { return fuelg::last_error(); }
const char* fuelg_version(void) { return "fuel-gb300 0.1.0 (sm_103a)"; }

int fuelg_device_count(int32_t* out_count) {
  if (!out_count) {
    set_error("out_count is NULL");
    return ST_EINVAL;
  }
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  *out_count = n;
  return ST_OK;
}

int fuelg_cancel(void) {
  if (g_cancel_host) *(volatile int*)g_cancel_host = 1;
  return ST_OK;
}
int fuelg_reset_cancel(void) {
  if (g_cancel_host) *(volatile int*)g_cancel_host = 0;
  return ST_OK;
}

int fuelg_release(void) {
  if (g_open_servers.load() > 0) {
    set_error("%d serving handle(s) still open: destroy them before fuelg_release", g_open_servers.load());
    return ST_EINVAL;
  }
  {
    GraphRegistry& r = graph_registry();
    std::lock_guard<std::mutex> lk(r.mu);
    for (cudaGraphExec_t g : r.graphs) cudaGraphExecDestroy(g);
    r.graphs.clear();
    r.gen++;
  }
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    // a pool with allocations still out is freed once they are returned
    for (auto& kv : pools())
      if (kv.second.created) cudaMemPoolDestroy(kv.second.pool);
    pools().clear();
  }
  {
    std::lock_guard<std::mutex> lk(g_cancel_mu);
    int* h = g_cancel_host;
    g_cancel_host = nullptr;
    g_cancel_dev = nullptr;
    if (h) cudaFreeHost(h);
  }
  noalloc_forget();
  cudaGetLastError();  // a context already gone makes the destroys fail: nothing is left to free then
  return ST_OK;
}

}  // extern "C"

namespace {

int index_create_impl(const void* data, bool f64, int64_t n, int32_t d, int32_t metric, int32_t order,
                      fuelg_index** out) {
  if (!out) {
    set_error("out is NULL");
    return ST_EINVAL;
  }
  *out = nullptr;
  if (n < 0 || d <= 0 || (n > 0 && !data)) {
    set_error("invalid index shape n=%lld d=%d", (long long)n, d);
    return ST_EINVAL;
  }
  if (metric != FUELG_METRIC_SQEUCLIDEAN && metric != FUELG_METRIC_EUCLIDEAN) {
    set_error("unsupported metric %d (the GPU path serves sqeuclidean and euclidean)", metric);
    return ST_EINVAL;
  }
  if (order != FUELG_ORDER_ARM && order != FUELG_ORDER_X86) {
    set_error("unknown summation order %d", order);
    return ST_EINVAL;
  }
  if (f64 && n > (1ll << 32) - 2) {
    set_error("float64 index too large: n=%lld (limit 2^32-2)", (long long)n);
    return ST_ENOTSUP;
  }
  FUELG_TRY(begin_call());
  fuelg_index* ix = new fuelg_index();
  cudaGetDevice(&ix->device);
  ix->f64 = f64;
  ix->n = n;
  ix->d = d;
  ix->metric = metric;
  ix->order = order;
  if (cudaStreamCreateWithFlags(&ix->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ix;
    set_error("cannot create a stream");
    return ST_ECUDA;
  }
  const size_t bytes = (size_t)n * d * (f64 ? sizeof(double) : sizeof(float));
  if (bytes) {
    void* dst = nullptr;
    if (cudaMalloc(&dst, bytes) != cudaSuccess) {
      cudaGetLastError();
      cudaStreamDestroy(ix->stream);
      delete ix;
      set_error("cannot allocate %zu bytes for the index", bytes);
      return ST_ENOMEM;
    }
    if (f64) ix->X64 = static_cast<double*>(dst);
    else ix->X = static_cast<float*>(dst);
    cudaError_t e = cudaMemcpyAsync(dst, data, bytes, cudaMemcpyDefault, ix->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ix->stream);
    if (e != cudaSuccess) {
      cudaFree(dst);
      cudaStreamDestroy(ix->stream);
      delete ix;
      set_error("index upload failed: %s", cudaGetErrorString(e));
      return ST_ECUDA;
    }
  }
  *out = ix;
  return ST_OK;
}

}  // namespace

extern "C" {

int fuelg_index_create(const float* data, int64_t n, int32_t d, int32_t metric, int32_t order, fuelg_index** out) {
  return index_create_impl(data, false, n, d, metric, order, out);
}

int fuelg_index_create_f64(const double* data, int64_t n, int32_t d, int32_t metric, int32_t order,
                           fuelg_index** out) {
  return index_create_impl(data, true, n, d, metric, order, out);
}

}  // extern "C"

namespace fuelg {
int index_view_get(fuelg_index* ix, int want_tier, IndexView* out) {
  if (ix->f64) {
    set_error("the index holds float64 data: this call serves float32 indexes");
    return ST_EINVAL;
  }
  std::lock_guard<std::mutex> lk(ix->mu);
  cudaSetDevice(ix->device);
  if (want_tier >= 0 && !ix->tc && ix->n > 0 && knn_tc_supported(ix->n, ix->d, 1, TC_BF16))
    FUELG_TRY(knn_tc_index_build(ix->X, ix->n, ix->d, ix->stream, &ix->tc));
  if (want_tier == TC_SPLIT && ix->tc) FUELG_TRY(knn_tc_index_add_lo(ix->tc, ix->X, ix->stream));
  out->f16 = false;
  if (want_tier == TC_F16 && ix->tc) {
    const int rc = knn_tc_index_add_f16(ix->tc, ix->X, ix->stream);
    if (rc != ST_OK && rc != ST_ENOTSUP) return rc;
    out->f16 = rc == ST_OK;  // else values outside the FP16 range: the plain tier serves
  }
  out->device = ix->device;
  out->n = ix->n;
  out->d = ix->d;
  out->metric = ix->metric;
  out->order = ix->order;
  out->X = ix->X;
  out->tc = ix->tc;
  return ST_OK;
}
}  // namespace fuelg

extern "C" {

int fuelg_index_destroy(fuelg_index* ix) {
  if (!ix) return ST_OK;
  cudaSetDevice(ix->device);
  if (ix->stream) cudaStreamSynchronize(ix->stream);
  knn_tc_index_free(ix->tc);
  if (ix->X) cudaFree(ix->X);
  if (ix->X64) cudaFree(ix->X64);
  if (ix->stream) cudaStreamDestroy(ix->stream);
  delete ix;
  return ST_OK;
}

int fuelg_index_info(const fuelg_index* ix, int64_t* n, int32_t* d, int32_t* metric, int32_t* order) {
  if (!ix) {
    set_error("index is NULL");
    return ST_EINVAL;
  }
  if (n) *n = ix->n;
  if (d) *d = ix->d;
  if (metric) *metric = ix->metric;
  if (order) *order = ix->order;
  return ST_OK;
}

}  // extern "C"

namespace {

// Top-kk (distance, index) keys of m query rows against the index, by the
// requested precision tier (the plain FP32 scan where the tensor-core tier does
// not serve the shape or the value range).  *used: the tier that ran.
int index_topk(fuelg_index* ix, const float* Q, int64_t m, int kk, int precision, uint64_t* keys, int* dstat,
               cudaStream_t s, int* used, int64_t* rescored) {
  ExactScanParams p;
  p.A = Q;
  p.m = m;
  p.B = ix->X;
  p.n = ix->n;
  p.d = ix->d;
  p.kind = KIND_KNN;
  p.order = ix->order;
  p.metric = ix->metric;
  p.kk = kk;
  *used = FUELG_PREC_FP32;
  *rescored = 0;
  const int tier = precision == FUELG_PREC_SPLIT_BF16 ? TC_SPLIT : precision == FUELG_PREC_F16 ? TC_F16 : TC_BF16;
  if (precision != FUELG_PREC_FP32 && knn_tc_supported(ix->n, ix->d, kk, tier) && ix->n > 0) {
    int exact = 0;
    if (!ix->tc) FUELG_TRY(knn_tc_index_build(ix->X, ix->n, ix->d, s, &ix->tc));
    if (tier == TC_SPLIT) FUELG_TRY(knn_tc_index_add_lo(ix->tc, ix->X, s));
    int rc = tier == TC_F16 ? knn_tc_index_add_f16(ix->tc, ix->X, s) : ST_OK;
    // values outside the FP16 range (index or queries): the plain tier answers
    if (rc == ST_OK)
      rc = knn_tc_topk(ix->tc, Q, m, ix->X, kk, ix->order, ix->metric, tier, keys, dstat, s, rescored, &exact);
    if (rc != ST_OK && rc != ST_ENOTSUP) return rc;
    if (rc == ST_OK) {
      // integer data run the exact one-product screen whatever the split request
      *used = tier == TC_F16 ? FUELG_PREC_F16 : (tier == TC_SPLIT && !exact) ? FUELG_PREC_SPLIT_BF16 : FUELG_PREC_BF16;
      return ST_OK;
    }
    *rescored = 0;
  }
  return exact_topk(p, keys, dstat, s);
}

// ---- precision autotuner ---------------------------------------------------
// Buckets (d, floor(log2 n), ceil(log2 kk), value class) -> tier, shared by all
// indexes of the process, loaded from / appended to FUELG_TUNE_CACHE.
struct TuneKey {
  int d, nb, kb, cls;
  bool operator<(const TuneKey& o) const {
    return d != o.d ? d < o.d : nb != o.nb ? nb < o.nb : kb != o.kb ? kb < o.kb : cls < o.cls;
  }
};
std::mutex g_tune_mu;
std::map<TuneKey, int> g_tune;
bool g_tune_loaded = false;

int ilog2_floor(int64_t v) {
  int r = 0;
  while (v > 1) {
    v >>= 1;
    r++;
  }
  return r;
}

void tune_load_locked() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const char* path = getenv("FUELG_TUNE_CACHE");
  if (!path) return;
  FILE* f = fopen(path, "r");
  if (!f) return;
  char kind[16];
  TuneKey key;
  int tier;
  while (fscanf(f, "%15s %d %d %d %d %d", kind, &key.d, &key.nb, &key.kb, &key.cls, &tier) == 6)
    if (strcmp(kind, "knn") == 0 && (tier == FUELG_PREC_BF16 || tier == FUELG_PREC_SPLIT_BF16 ||
                                     tier == FUELG_PREC_F16 || tier == FUELG_PREC_FP32))
      g_tune[key] = tier;
  fclose(f);
}

void tune_store_locked(const TuneKey& key, int tier) {
  g_tune[key] = tier;
  const char* path = getenv("FUELG_TUNE_CACHE");
  if (!path) return;
  if (FILE* f = fopen(path, "a")) {
    fprintf(f, "knn %d %d %d %d %d\n", key.d, key.nb, key.kb, key.cls, tier);
    fclose(f);
  }
}

// The tier a FUELG_PREC_AUTO kNN call runs.  Called with ix->mu held.
int resolve_knn_precision(fuelg_index* ix, const float* Q, int64_t m, int kk, int* dstat, cudaStream_t s,
                          int* out) {
  *out = FUELG_PREC_FP32;
  if (ix->n == 0 || !knn_tc_supported(ix->n, ix->d, kk, TC_BF16)) return ST_OK;
  if (!ix->tc) FUELG_TRY(knn_tc_index_build(ix->X, ix->n, ix->d, s, &ix->tc));
  const int cls = knn_tc_index_class(ix->tc);
  if (cls == TC_CLASS_INTEGER) {
    *out = FUELG_PREC_BF16;  // exact screen, no margin, no re-score
    return ST_OK;
  }
  const TuneKey key{ix->d, ilog2_floor(ix->n), ilog2_floor(2 * (int64_t)kk - 1), cls};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_load_locked();
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      *out = it->second;
      return ST_OK;
    }
  }
  // time the eligible tiers on the first rows of this call (each run twice:
  // the first builds the tier's index copy and warms up)
  const int64_t mt = std::min<int64_t>(m, 4096);
  Scratch keys;
  FUELG_TRY(keys.alloc((size_t)mt * kk * sizeof(uint64_t), s));
  const int cand_f16[3] = {FUELG_PREC_F16, FUELG_PREC_SPLIT_BF16, FUELG_PREC_BF16};
  const int cand_wide[2] = {FUELG_PREC_SPLIT_BF16, FUELG_PREC_BF16};
  const int* cand = cls == TC_CLASS_F16_RANGE ? cand_f16 : cand_wide;
  const int nc = cls == TC_CLASS_F16_RANGE ? 3 : 2;
  int best = FUELG_PREC_SPLIT_BF16;
  float best_ms = 1e30f;
  for (int c = 0; c < nc; c++) {
    int used = 0;
    int64_t resc = 0;
    FUELG_TRY(index_topk(ix, Q, mt, kk, cand[c], keys.as<uint64_t>(), dstat, s, &used, &resc));
    Timer tm(s);
    FUELG_TRY(index_topk(ix, Q, mt, kk, cand[c], keys.as<uint64_t>(), dstat, s, &used, &resc));
    const float ms = (float)tm.stop();
    if (used == cand[c] && ms < best_ms) {
      best_ms = ms;
      best = cand[c];
    }
  }
  std::lock_guard<std::mutex> lk(g_tune_mu);
  tune_store_locked(key, best);
  *out = best;
  return ST_OK;
}

int check_knn_args(fuelg_index* ix, const float* queries, int64_t m, int32_t k, int32_t exclude_mode,
                   int32_t precision) {
  if (!ix) {
    set_error("index is NULL");
    return ST_EINVAL;
  }
  if (ix->f64) {
    set_error("the index holds float64 data: use the _f64 calls");
    return ST_EINVAL;
  }
  if (m < 0 || k < 0 || (m > 0 && !queries && m != ix->n)) {
    set_error("invalid knn arguments m=%lld k=%d (queries may be NULL only for the index's own %lld rows)",
              (long long)m, k, (long long)ix->n);
    return ST_EINVAL;
  }
  if (exclude_mode < FUELG_EXCLUDE_NONE || exclude_mode > FUELG_EXCLUDE_KPLUS1) {
    set_error("unknown exclude mode %d", exclude_mode);
    return ST_EINVAL;
  }
  if (precision < FUELG_PREC_AUTO || precision > FUELG_PREC_F16 || precision == FUELG_PREC_SPLIT_BF16_SCALED) {
    set_error("unknown precision tier %d", precision);
    return ST_EINVAL;
  }
  if (k > 4095) {
    set_error("k=%d exceeds the supported maximum of 4095", k);
    return ST_ENOTSUP;
  }
  return ST_OK;
}

}  // namespace

extern "C" {

int fuelg_knn(fuelg_index* ix, const float* queries, int64_t m, int32_t k, int32_t exclude_mode, int32_t precision,
              int64_t* out_idx, float* out_dist, fuelg_stats* stats) {
  FUELG_TRY(check_knn_args(ix, queries, m, k, exclude_mode, precision));
  if (m > 0 && k > 0 && (!out_idx || !out_dist)) {
    set_error("invalid knn arguments: output buffers are NULL");
    return ST_EINVAL;
  }
  std::lock_guard<std::mutex> lk(ix->mu);
  FUELG_TRY(begin_call());
  cudaSetDevice(ix->device);
  if (stats) memset(stats, 0, sizeof(*stats));
  if (m == 0 || k == 0) return ST_OK;
  cudaStream_t s = ix->stream;
  const int kk = exclude_mode == FUELG_EXCLUDE_NONE ? k : k + 1;
  CallMeter meter;
  Timer tm(s);
  InBuf q;
  if (queries) FUELG_TRY(q.init(queries, (size_t)m * ix->d * sizeof(float), s));
  const float* Q = queries ? static_cast<const float*>(q.dptr) : ix->X;
  OutBuf oi, od;
  FUELG_TRY(oi.init(out_idx, (size_t)m * k * sizeof(int64_t), s));
  FUELG_TRY(od.init(out_dist, (size_t)m * k * sizeof(float), s));
  Scratch keys, dstat;
  FUELG_TRY(keys.alloc((size_t)m * kk * sizeof(uint64_t), s));
  FUELG_TRY(dstat.alloc(sizeof(int), s));
  FUELG_CUDA(cudaMemsetAsync(dstat.p, 0, sizeof(int), s));
  int used = FUELG_PREC_FP32;
  int64_t rescored = 0;
  if (precision == FUELG_PREC_AUTO)
    FUELG_TRY(resolve_knn_precision(ix, Q, m, kk, dstat.as<int>(), s, &precision));
  FUELG_TRY(index_topk(ix, Q, m, kk, precision, keys.as<uint64_t>(), dstat.as<int>(), s, &used, &rescored));
  FUELG_TRY(finalize_knn(keys.as<uint64_t>(), m, kk, k, exclude_mode, static_cast<int64_t*>(oi.dptr),
                         static_cast<float*>(od.dptr), s));
  int64_t d2h = 0;
  FUELG_TRY(oi.flush(s, &d2h));
  FUELG_TRY(od.flush(s, &d2h));
  const double ms = tm.stop();
  FUELG_TRY(read_dev_status(dstat.as<int>(), s));
  if (stats) {
    stats->device_ms = ms;
    stats->h2d_bytes = q.h2d;
    stats->d2h_bytes = d2h;
    stats->distance_evals = m * ix->n;
    stats->precision_used = used;
    stats->rescored = rescored;
    meter.fill(stats);
  }
  return ST_OK;
}

int fuelg_knn_ties(fuelg_index* ix, const float* queries, int64_t m, int32_t k, int32_t exclude_mode,
                   int32_t precision, fuelg_range_result** out, fuelg_stats* stats) {
  if (!out) {
    set_error("out is NULL");
    return ST_EINVAL;
  }
  *out = nullptr;
  FUELG_TRY(check_knn_args(ix, queries, m, k, exclude_mode, precision));
  std::lock_guard<std::mutex> lk(ix->mu);
  FUELG_TRY(begin_call());
  cudaSetDevice(ix->device);
  if (stats) memset(stats, 0, sizeof(*stats));
  cudaStream_t s = ix->stream;
  fuelg_range_result* r = new fuelg_range_result();
  r->m = m;
  // linear-index rule searches k, the k+1 rule k+1; both drop self afterwards
  const int kq = exclude_mode == FUELG_EXCLUDE_KPLUS1 ? k + 1 : k;
  if (m == 0 || kq == 0 || ix->n == 0) {
    int st = ST_OK;
    if (cudaMalloc(&r->off, sizeof(int64_t) * (m + 1)) != cudaSuccess ||
        cudaMemset(r->off, 0, sizeof(int64_t) * (m + 1)) != cudaSuccess) {
      cudaGetLastError();
      set_error("cannot allocate the result offsets");
      st = ST_ENOMEM;
    }
    if (st != ST_OK) {
      fuelg_range_free(r);
      return st;
    }
    *out = r;
    return ST_OK;
  }
  CallMeter meter;
  Timer tm(s);
  auto run = [&]() -> int {
    InBuf q;
    if (queries) FUELG_TRY(q.init(queries, (size_t)m * ix->d * sizeof(float), s));
    const float* Q = queries ? static_cast<const float*>(q.dptr) : ix->X;
    const int kk = ties_spare_kk(kq, ix->n);
    Scratch keys, dstat;
    FUELG_TRY(keys.alloc((size_t)m * kk * sizeof(uint64_t), s));
    FUELG_TRY(dstat.alloc(sizeof(int), s));
    FUELG_CUDA(cudaMemsetAsync(dstat.p, 0, sizeof(int), s));
    int used = FUELG_PREC_FP32;
    int64_t rescored = 0, range_rows = 0;
    int prec = precision;
    if (prec == FUELG_PREC_AUTO) FUELG_TRY(resolve_knn_precision(ix, Q, m, kk, dstat.as<int>(), s, &prec));
    FUELG_TRY(index_topk(ix, Q, m, kk, prec, keys.as<uint64_t>(), dstat.as<int>(), s, &used, &rescored));
    ExactScanParams base;
    base.A = Q;
    base.m = m;
    base.B = ix->X;
    base.n = ix->n;
    base.d = ix->d;
    base.kind = KIND_KNN;
    base.order = ix->order;
    base.metric = ix->metric;
    FUELG_TRY(knn_ties_lists(keys.as<uint64_t>(), m, kk, kq, exclude_mode != FUELG_EXCLUDE_NONE, base, &r->off,
                             &r->idx, &r->dist, &r->total, &range_rows, dstat.as<int>(), s));
    const double ms = tm.stop();
    FUELG_TRY(read_dev_status(dstat.as<int>(), s));
    if (stats) {
      stats->device_ms = ms;
      stats->h2d_bytes = q.h2d;
      stats->distance_evals = m * ix->n + range_rows * ix->n;
      stats->precision_used = used;
      stats->rescored = rescored;
      meter.fill(stats);
    }
    return ST_OK;
  };
  const int st = run();
  if (st != ST_OK) {
    fuelg_range_free(r);
    return st;
  }
  *out = r;
  return ST_OK;
}

int fuelg_knn_batched(fuelg_knn_set* sets, int32_t count, int32_t order, int32_t precision, fuelg_stats* stats) {
  if (count < 0 || (count > 0 && !sets)) {
    set_error("invalid batched kNN arguments count=%d", count);
    return ST_EINVAL;
  }
  if (order != FUELG_ORDER_ARM && order != FUELG_ORDER_X86) {
    set_error("unknown summation order %d", order);
    return ST_EINVAL;
  }
  if (precision != FUELG_PREC_FP32 && precision != FUELG_PREC_AUTO) {
    set_error("batched kNN runs the exact FP32 scan (precision %d requested)", precision);
    return ST_ENOTSUP;
  }
  int bad = 0;
  for (int i = 0; i < count; i++) {
    fuelg_knn_set& t = sets[i];
    t.status = ST_OK;
    const bool ok = t.n >= 0 && t.d >= 1 && t.d <= 1024 && t.m >= 0 && t.k >= 0 && t.k <= 4095 &&
                    (t.metric == FUELG_METRIC_SQEUCLIDEAN || t.metric == FUELG_METRIC_EUCLIDEAN) &&
                    t.exclude_mode >= FUELG_EXCLUDE_NONE && t.exclude_mode <= FUELG_EXCLUDE_KPLUS1 &&
                    (t.n == 0 || t.data) && (t.m == 0 || t.queries) &&
                    (t.m == 0 || t.k == 0 || (t.out_idx && t.out_dist));
    if (!ok) {
      t.status = ST_EINVAL;
      if (!bad) set_error("set %d: invalid shape or arguments (n=%lld d=%d m=%lld k=%d)", i, (long long)t.n, t.d,
                          (long long)t.m, t.k);
      bad = 1;
    }
  }
  if (bad) return ST_EINVAL;
  FUELG_TRY(begin_call());
  if (stats) memset(stats, 0, sizeof(*stats));
  cudaStream_t s;
  FUELG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{s};
  CallMeter meter;
  Timer tm(s);
  std::vector<InBuf> xs(count), qs(count);
  std::vector<OutBuf> ois(count), ods(count);
  std::vector<KnnSetDev> dev(count);
  Scratch dstat;
  FUELG_TRY(dstat.alloc(sizeof(int), s));
  FUELG_CUDA(cudaMemsetAsync(dstat.p, 0, sizeof(int), s));
  int64_t h2d = 0, evals = 0;
  for (int i = 0; i < count; i++) {
    const fuelg_knn_set& t = sets[i];
    const int64_t mk = (t.m > 0 && t.k > 0) ? t.m : 0;
    FUELG_TRY(xs[i].init(t.data, mk ? (size_t)t.n * t.d * sizeof(float) : 0, s));
    FUELG_TRY(qs[i].init(t.queries, mk ? (size_t)t.m * t.d * sizeof(float) : 0, s));
    FUELG_TRY(ois[i].init(t.out_idx, (size_t)mk * t.k * sizeof(int64_t), s));
    FUELG_TRY(ods[i].init(t.out_dist, (size_t)mk * t.k * sizeof(float), s));
    h2d += xs[i].h2d + qs[i].h2d;
    evals += mk * t.n;
    dev[i] = KnnSetDev{static_cast<const float*>(qs[i].dptr), mk, static_cast<const float*>(xs[i].dptr), t.n, t.d,
                       t.metric, t.k, t.exclude_mode, static_cast<int64_t*>(ois[i].dptr),
                       static_cast<float*>(ods[i].dptr)};
  }
  FUELG_TRY(exact_knn_sets(dev.data(), count, order, dstat.as<int>(), s));
  int64_t d2h = 0;
  for (int i = 0; i < count; i++) {
    FUELG_TRY(ois[i].flush(s, &d2h));
    FUELG_TRY(ods[i].flush(s, &d2h));
  }
  const double ms = tm.stop();
  FUELG_TRY(read_dev_status(dstat.as<int>(), s));
  if (stats) {
    stats->device_ms = ms;
    stats->h2d_bytes = h2d;
    stats->d2h_bytes = d2h;
    stats->distance_evals = evals;
    stats->precision_used = FUELG_PREC_FP32;
    meter.fill(stats);
  }
  return ST_OK;
}

int fuelg_knn_error(fuelg_index* ix, const float* queries, int64_t m, int32_t k, const int64_t* idx,
                    const float* dist, fuelg_error_report* out) {
  if (!ix || !out || m < 0 || k < 0 || (m > 0 && k > 0 && (!idx || !dist)) || (m > 0 && !queries && m != ix->n)) {
    set_error("invalid knn_error arguments");
    return ST_EINVAL;
  }
  if (ix->f64) {
    set_error("the index holds float64 data: the error report serves float32 indexes");
    return ST_EINVAL;
  }
  memset(out, 0, sizeof(*out));
  std::lock_guard<std::mutex> lk(ix->mu);
  FUELG_TRY(begin_call());
  cudaSetDevice(ix->device);
  if (m == 0 || k == 0 || ix->n == 0) return ST_OK;
  cudaStream_t s = ix->stream;
  InBuf q, bi, bd;
  if (queries) FUELG_TRY(q.init(queries, (size_t)m * ix->d * sizeof(float), s));
  FUELG_TRY(bi.init(idx, (size_t)m * k * sizeof(int64_t), s));
  FUELG_TRY(bd.init(dist, (size_t)m * k * sizeof(float), s));
  const float* Q = queries ? static_cast<const float*>(q.dptr) : ix->X;
  return knn_error_report(Q, ix->X, m, ix->d, k, ix->metric, static_cast<const int64_t*>(bi.dptr),
                          static_cast<const float*>(bd.dptr), &out->max_abs_err, &out->max_rel_err, &out->pairs,
                          &out->near_ties, &out->order_flips, s);
}

int fuelg_fp32_rate(double* tera_fma_per_s) {
  if (!tera_fma_per_s) {
    set_error("tera_fma_per_s is NULL");
    return ST_EINVAL;
  }
  FUELG_TRY(begin_call());
  double ms = 0.0;
  return fp32_issue_rate(tera_fma_per_s, &ms);
}

int fuelg_pairwise(const float* X, int64_t n, int32_t d, int32_t metric, int32_t order, int32_t form, float* out,
                   fuelg_stats* stats) {
  if (n < 0 || d < 1 || (n > 0 && !X)) {
    set_error("invalid pairwise arguments n=%lld d=%d", (long long)n, d);
    return ST_EINVAL;
  }
  if (metric != FUELG_METRIC_SQEUCLIDEAN && metric != FUELG_METRIC_EUCLIDEAN) {
    set_error("unknown metric %d", metric);
    return ST_EINVAL;
  }
  if (order != FUELG_ORDER_ARM && order != FUELG_ORDER_X86) {
    set_error("unknown summation order %d", order);
    return ST_EINVAL;
  }
  if (form != FUELG_PAIRWISE_CONDENSED && form != FUELG_PAIRWISE_SQUARE) {
    set_error("unknown pairwise form %d", form);
    return ST_EINVAL;
  }
  const int64_t outs = form == FUELG_PAIRWISE_CONDENSED ? n * (n - 1) / 2 : n * n;
  if (outs > 0 && !out) {
    set_error("out is NULL");
    return ST_EINVAL;
  }
  FUELG_TRY(begin_call());
  if (stats) memset(stats, 0, sizeof(*stats));
  if (outs <= 0) return ST_OK;
  cudaStream_t s;
  FUELG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{s};
  CallMeter meter;
  Timer tm(s);
  InBuf xb;
  FUELG_TRY(xb.init(X, (size_t)n * d * sizeof(float), s));
  OutBuf ob;
  FUELG_TRY(ob.init(out, (size_t)outs * sizeof(float), s));
  FUELG_TRY(pairwise_launch(static_cast<const float*>(xb.dptr), n, d, metric, order, form,
                            static_cast<float*>(ob.dptr), s));
  int64_t d2h = 0;
  FUELG_TRY(ob.flush(s, &d2h));
  const double ms = tm.stop();
  FUELG_CUDA(cudaStreamSynchronize(s));
  if (stats) {
    stats->device_ms = ms;
    stats->h2d_bytes = xb.h2d;
    stats->d2h_bytes = d2h;
    stats->distance_evals = form == FUELG_PAIRWISE_CONDENSED ? outs : n * (n + 1) / 2;
    stats->precision_used = FUELG_PREC_FP32;
    meter.fill(stats);
  }
  return ST_OK;
}

int fuelg_range(fuelg_index* ix, const float* queries, int64_t m, double radius, int32_t exclude_self,
                fuelg_range_result** out, fuelg_stats* stats) {
  if (!ix || !out) {
    set_error("index or out is NULL");
    return ST_EINVAL;
  }
  *out = nullptr;
  if (m < 0 || (m > 0 && !queries)) {
    set_error("invalid range arguments m=%lld", (long long)m);
    return ST_EINVAL;
  }
  if (ix->f64) {
    set_error("the index holds float64 data: use fuelg_range_f64");
    return ST_EINVAL;
  }
  std::lock_guard<std::mutex> lk(ix->mu);
  FUELG_TRY(begin_call());
  cudaSetDevice(ix->device);
  if (stats) memset(stats, 0, sizeof(*stats));
  cudaStream_t s = ix->stream;
  CallMeter meter;
  Timer tm(s);
  InBuf q;
  FUELG_TRY(q.init(queries, (size_t)m * ix->d * sizeof(float), s));
  Scratch dstat;
  FUELG_TRY(dstat.alloc(sizeof(int), s));
  FUELG_CUDA(cudaMemsetAsync(dstat.p, 0, sizeof(int), s));
  ExactScanParams p;
  p.A = static_cast<const float*>(q.dptr);
  p.m = m;
  p.B = ix->X;
  p.n = ix->n;
  p.d = ix->d;
  p.kind = KIND_KNN;
  p.order = ix->order;
  p.metric = ix->metric;
  fuelg_range_result* r = new fuelg_range_result();
  r->m = m;
  int st = exact_range(p, (float)radius, exclude_self ? 1 : 0, &r->off, &r->idx, &r->dist, &r->total,
                       dstat.as<int>(), s);
  if (st == ST_OK) st = read_dev_status(dstat.as<int>(), s);
  const double ms = tm.stop();
  if (st != ST_OK) {
    fuelg_range_free(r);
    return st;
  }
  if (stats) {
    stats->device_ms = ms;
    stats->h2d_bytes = q.h2d;
    stats->distance_evals = 2 * m * ix->n;
    stats->precision_used = FUELG_PREC_FP32;
    meter.fill(stats);
  }
  *out = r;
  return ST_OK;
}

int fuelg_range_size(const fuelg_range_result* r, int64_t* m, int64_t* total) {
  if (!r) {
    set_error("range result is NULL");
    return ST_EINVAL;
  }
  if (m) *m = r->m;
  if (total) *total = r->total;
  return ST_OK;
}

int fuelg_range_copy(const fuelg_range_result* r, int64_t* offsets, int64_t* idx, float* dist) {
  if (!r) {
    set_error("range result is NULL");
    return ST_EINVAL;
  }
  if (r->f64) {
    set_error("float64 lists: read them with fuelg_range_copy_f64");
    return ST_EINVAL;
  }
  if (offsets) FUELG_CUDA(cudaMemcpy(offsets, r->off, sizeof(int64_t) * (r->m + 1), cudaMemcpyDefault));
  if (r->total) {
    if (idx) FUELG_CUDA(cudaMemcpy(idx, r->idx, sizeof(int64_t) * r->total, cudaMemcpyDefault));
    if (dist) FUELG_CUDA(cudaMemcpy(dist, r->dist, sizeof(float) * r->total, cudaMemcpyDefault));
  }
  return ST_OK;
}

int fuelg_range_free(fuelg_range_result* r) {
  if (!r) return ST_OK;
  if (r->off) cudaFree(r->off);
  if (r->idx) cudaFree(r->idx);
  if (r->dist) cudaFree(r->dist);
  delete r;
  return ST_OK;
}

}  // extern "C"

namespace {

int check_f64_index(fuelg_index* ix) {
  if (!ix) {
    set_error("index is NULL");
    return ST_EINVAL;
  }
  if (!ix->f64) {
    set_error("the index holds float32 data: use the float32 calls");
    return ST_EINVAL;
  }
  return ST_OK;
}

F64Scan f64_view(const fuelg_index* ix) {
  F64Scan x;
  x.X = ix->X64;
  x.n = ix->n;
  x.d = ix->d;
  x.metric = ix->metric;
  x.order = ix->order;
  return x;
}

// fuelg_knn_ties_f64 / fuelg_range_f64: host-side CSR lists into a result handle.
int f64_lists_call(fuelg_index* ix, const double* queries, int64_t m, bool range, int64_t kq, bool drop_self,
                   double radius, fuelg_range_result** out, fuelg_stats* stats) {
  std::lock_guard<std::mutex> lk(ix->mu);
  FUELG_TRY(begin_call());
  cudaSetDevice(ix->device);
  if (stats) memset(stats, 0, sizeof(*stats));
  cudaStream_t s = ix->stream;
  CallMeter meter;
  Timer tm(s);
  InBuf q;
  if (queries) FUELG_TRY(q.init(queries, (size_t)m * ix->d * sizeof(double), s));
  const double* Q = queries ? static_cast<const double*>(q.dptr) : ix->X64;
  fuelg_range_result* r = new fuelg_range_result();
  r->m = m;
  r->f64 = true;
  int64_t d2h = 0;
  const int st = f64_lists(f64_view(ix), Q, m, range, kq, drop_self, radius, &r->h_off, &r->h_idx, &r->h_dist,
                           &d2h, s);
  const double ms = tm.stop();
  if (st != ST_OK) {
    delete r;
    return st;
  }
  r->total = r->h_off.empty() ? 0 : r->h_off.back();
  if (stats) {
    stats->device_ms = ms;
    stats->h2d_bytes = q.h2d;
    stats->d2h_bytes = d2h;
    stats->distance_evals = m * ix->n;
    stats->precision_used = FUELG_PREC_FP64;
    meter.fill(stats);
  }
  *out = r;
  return ST_OK;
}

}  // namespace

extern "C" {

int fuelg_knn_f64(fuelg_index* ix, const double* queries, int64_t m, int32_t k, int32_t exclude_mode,
                  int64_t* out_idx, double* out_dist, fuelg_stats* stats) {
  FUELG_TRY(check_f64_index(ix));
  if (m < 0 || k < 0 || (m > 0 && !queries && m != ix->n)) {
    set_error("invalid knn arguments m=%lld k=%d (queries may be NULL only for the index's own %lld rows)",
              (long long)m, k, (long long)ix->n);
    return ST_EINVAL;
  }
  if (exclude_mode < FUELG_EXCLUDE_NONE || exclude_mode > FUELG_EXCLUDE_KPLUS1) {
    set_error("unknown exclude mode %d", exclude_mode);
    return ST_EINVAL;
  }
  if (k > 4095) {
    set_error("k=%d exceeds the supported maximum of 4095", k);
    return ST_ENOTSUP;
  }
  if (m > 0 && k > 0 && (!out_idx || !out_dist)) {
    set_error("invalid knn arguments: output buffers are NULL");
    return ST_EINVAL;
  }
  std::lock_guard<std::mutex> lk(ix->mu);
  FUELG_TRY(begin_call());
  cudaSetDevice(ix->device);
  if (stats) memset(stats, 0, sizeof(*stats));
  if (m == 0 || k == 0) return ST_OK;
  cudaStream_t s = ix->stream;
  CallMeter meter;
  Timer tm(s);
  InBuf q;
  if (queries) FUELG_TRY(q.init(queries, (size_t)m * ix->d * sizeof(double), s));
  const double* Q = queries ? static_cast<const double*>(q.dptr) : ix->X64;
  OutBuf oi, od;
  FUELG_TRY(oi.init(out_idx, (size_t)m * k * sizeof(int64_t), s));
  FUELG_TRY(od.init(out_dist, (size_t)m * k * sizeof(double), s));
  FUELG_TRY(f64_knn(f64_view(ix), Q, m, k, exclude_mode, static_cast<int64_t*>(oi.dptr),
                    static_cast<double*>(od.dptr), s));
  int64_t d2h = 0;
  FUELG_TRY(oi.flush(s, &d2h));
  FUELG_TRY(od.flush(s, &d2h));
  const double ms = tm.stop();
  FUELG_CUDA(cudaStreamSynchronize(s));
  if (stats) {
    stats->device_ms = ms;
    stats->h2d_bytes = q.h2d;
    stats->d2h_bytes = d2h;
    stats->distance_evals = m * ix->n;
    stats->precision_used = FUELG_PREC_FP64;
    meter.fill(stats);
  }
  return ST_OK;
}

int fuelg_knn_ties_f64(fuelg_index* ix, const double* queries, int64_t m, int32_t k, int32_t exclude_mode,
                       fuelg_range_result** out, fuelg_stats* stats) {
  if (!out) {
    set_error("out is NULL");
    return ST_EINVAL;
  }
  *out = nullptr;
  FUELG_TRY(check_f64_index(ix));
  if (m < 0 || k < 0 || (m > 0 && !queries && m != ix->n)) {
    set_error("invalid knn arguments m=%lld k=%d (queries may be NULL only for the index's own %lld rows)",
              (long long)m, k, (long long)ix->n);
    return ST_EINVAL;
  }
  if (exclude_mode < FUELG_EXCLUDE_NONE || exclude_mode > FUELG_EXCLUDE_KPLUS1) {
    set_error("unknown exclude mode %d", exclude_mode);
    return ST_EINVAL;
  }
  if (k > 4095) {
    set_error("k=%d exceeds the supported maximum of 4095", k);
    return ST_ENOTSUP;
  }
  // the linear-index rule searches k, the k+1 rule k+1; both drop self afterwards
  const int64_t kq = exclude_mode == FUELG_EXCLUDE_KPLUS1 ? (int64_t)k + 1 : k;
  return f64_lists_call(ix, queries, m, false, kq, exclude_mode != FUELG_EXCLUDE_NONE, 0.0, out, stats);
}

int fuelg_range_f64(fuelg_index* ix, const double* queries, int64_t m, double radius, int32_t exclude_self,
                    fuelg_range_result** out, fuelg_stats* stats) {
  if (!out) {
    set_error("out is NULL");
    return ST_EINVAL;
  }
  *out = nullptr;
  FUELG_TRY(check_f64_index(ix));
  if (m < 0 || (m > 0 && !queries)) {
    set_error("invalid range arguments m=%lld", (long long)m);
    return ST_EINVAL;
  }
  return f64_lists_call(ix, queries, m, true, 0, exclude_self != 0, radius, out, stats);
}

int fuelg_range_copy_f64(const fuelg_range_result* r, int64_t* offsets, int64_t* idx, double* dist) {
  if (!r) {
    set_error("range result is NULL");
    return ST_EINVAL;
  }
  if (!r->f64) {
    set_error("float32 lists: read them with fuelg_range_copy");
    return ST_EINVAL;
  }
  if (offsets && !r->h_off.empty())
    FUELG_CUDA(cudaMemcpy(offsets, r->h_off.data(), sizeof(int64_t) * r->h_off.size(), cudaMemcpyDefault));
  if (r->total) {
    if (idx) FUELG_CUDA(cudaMemcpy(idx, r->h_idx.data(), sizeof(int64_t) * r->total, cudaMemcpyDefault));
    if (dist) FUELG_CUDA(cudaMemcpy(dist, r->h_dist.data(), sizeof(double) * r->total, cudaMemcpyDefault));
  }
  return ST_OK;
}

int fuelg_pairwise_f64(const double* X, int64_t n, int32_t d, int32_t metric, int32_t order, int32_t form,
                       double* out, fuelg_stats* stats) {
  if (n < 0 || d < 1 || (n > 0 && !X)) {
    set_error("invalid pairwise arguments n=%lld d=%d", (long long)n, d);
    return ST_EINVAL;
  }
  if (metric != FUELG_METRIC_SQEUCLIDEAN && metric != FUELG_METRIC_EUCLIDEAN) {
    set_error("unknown metric %d", metric);
    return ST_EINVAL;
  }
  if (order != FUELG_ORDER_ARM && order != FUELG_ORDER_X86) {
    set_error("unknown summation order %d", order);
    return ST_EINVAL;
  }
  if (form != FUELG_PAIRWISE_CONDENSED && form != FUELG_PAIRWISE_SQUARE) {
    set_error("unknown pairwise form %d", form);
    return ST_EINVAL;
  }
  const int64_t outs = form == FUELG_PAIRWISE_CONDENSED ? n * (n - 1) / 2 : n * n;
  if (outs > 0 && !out) {
    set_error("out is NULL");
    return ST_EINVAL;
  }
  FUELG_TRY(begin_call());
  if (stats) memset(stats, 0, sizeof(*stats));
  if (outs <= 0) return ST_OK;
  cudaStream_t s;
  FUELG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{s};
  CallMeter meter;
  Timer tm(s);
  InBuf xb;
  FUELG_TRY(xb.init(X, (size_t)n * d * sizeof(double), s));
  OutBuf ob;
  FUELG_TRY(ob.init(out, (size_t)outs * sizeof(double), s));
  FUELG_TRY(f64_pairwise(static_cast<const double*>(xb.dptr), n, d, metric, order, form,
                         static_cast<double*>(ob.dptr), s));
  int64_t d2h = 0;
  FUELG_TRY(ob.flush(s, &d2h));
  const double ms = tm.stop();
  FUELG_CUDA(cudaStreamSynchronize(s));
  if (stats) {
    stats->device_ms = ms;
    stats->h2d_bytes = xb.h2d;
    stats->d2h_bytes = d2h;
    stats->distance_evals = form == FUELG_PAIRWISE_CONDENSED ? outs : n * n;
    stats->precision_used = FUELG_PREC_FP64;
    meter.fill(stats);
  }
  return ST_OK;
}

int fuelg_kmeans_lloyd(const float* data, int64_t n, int32_t d, int32_t k, const float* init_centers,
                       int32_t max_iter, double tol, int32_t precision, int32_t order, int32_t flags,
                       float* out_centers, int64_t* out_labels, int32_t* out_iters, double* out_inertia,
                       fuelg_stats* stats) {
  if (n <= 0 || d <= 0 || k <= 0 || !data || !init_centers || !out_centers || !out_labels) {
    set_error("invalid lloyd arguments n=%lld d=%d k=%d", (long long)n, d, k);
    return ST_EINVAL;
  }
  if (max_iter < 1) {
    set_error("max_iter must be >= 1");
    return ST_EINVAL;
  }
  if (!(tol >= 0.0)) {
    set_error("tol must be >= 0");
    return ST_EINVAL;
  }
  if (order != FUELG_ORDER_ARM && order != FUELG_ORDER_X86) {
    set_error("unknown summation order %d", order);
    return ST_EINVAL;
  }
  if (precision < FUELG_PREC_AUTO || precision > FUELG_PREC_SPLIT_BF16) {
    set_error("unknown precision tier %d", precision);
    return ST_EINVAL;
  }
  // automatic tier: the split-BF16 screen (which also finds scaled-integer
  // data) where it serves the shape and the pass is long enough to pay for
  // its set-up; the plain CUDA-core scan otherwise
  if (precision == FUELG_PREC_AUTO) precision = (d >= 32 && n >= 16384) ? FUELG_PREC_SPLIT_BF16 : FUELG_PREC_FP32;
  FUELG_TRY(begin_call());
  if (stats) memset(stats, 0, sizeof(*stats));
  cudaStream_t s;
  FUELG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{s};
  CallMeter meter;
  Timer tm(s);
  InBuf X, C0;
  FUELG_TRY(X.init(data, (size_t)n * d * sizeof(float), s));
  FUELG_TRY(C0.init(init_centers, (size_t)k * d * sizeof(float), s));
  OutBuf oc, ol;
  FUELG_TRY(oc.init(out_centers, (size_t)k * d * sizeof(float), s));
  FUELG_TRY(ol.init(out_labels, (size_t)n * sizeof(int64_t), s));
  Scratch lab32, dstat;
  FUELG_TRY(lab32.alloc(sizeof(int32_t) * n, s));
  FUELG_TRY(dstat.alloc(sizeof(int), s));
  FUELG_CUDA(cudaMemsetAsync(dstat.p, 0, sizeof(int), s));
  LloydParams p;
  p.X = static_cast<const float*>(X.dptr);
  p.n = n;
  p.d = d;
  p.k = k;
  p.init = static_cast<const float*>(C0.dptr);
  p.max_iter = max_iter;
  p.tol = tol;
  p.order = order;
  p.precision = precision;
  p.fixed_iters = (flags & FUELG_LLOYD_FIXED_ITERS) ? 1 : 0;
  LloydResult r;
  r.centers = static_cast<float*>(oc.dptr);
  r.labels = lab32.as<int32_t>();
  FUELG_TRY(lloyd_run(p, &r, dstat.as<int>(), s));
  // widen labels to int64 (python/kmeans.rs:20: `v as i64`)
  widen_labels(r.labels, static_cast<int64_t*>(ol.dptr), n, s);
  FUELG_CUDA(cudaGetLastError());
  int64_t d2h = 0;
  FUELG_TRY(oc.flush(s, &d2h));
  FUELG_TRY(ol.flush(s, &d2h));
  const double ms = tm.stop();
  FUELG_TRY(read_dev_status(dstat.as<int>(), s));
  if (out_iters) *out_iters = r.iters;
  if (out_inertia) *out_inertia = r.inertia;
  if (stats) {
    stats->device_ms = ms;
    stats->h2d_bytes = X.h2d + C0.h2d;
    stats->d2h_bytes = d2h;
    stats->distance_evals = (int64_t)r.iters * n * k;
    stats->rescored = r.rescored;
    stats->iterations = r.iters;
    stats->precision_used = r.precision_used;
    meter.fill(stats);
  }
  return ST_OK;
}

int fuelg_lloyd_assign(const float* data, int64_t n, int32_t d, const float* centers, int32_t k, int32_t initial,
                       int32_t order, int64_t* out_labels, float* out_best, fuelg_stats* stats) {
  if (n <= 0 || d <= 0 || k <= 0 || !data || !centers || !out_labels) {
    set_error("invalid lloyd_assign arguments n=%lld d=%d k=%d", (long long)n, d, k);
    return ST_EINVAL;
  }
  if (order != FUELG_ORDER_ARM && order != FUELG_ORDER_X86) {
    set_error("unknown summation order %d", order);
    return ST_EINVAL;
  }
  FUELG_TRY(begin_call());
  if (stats) memset(stats, 0, sizeof(*stats));
  cudaStream_t s;
  FUELG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{s};
  CallMeter meter;
  Timer tm(s);
  InBuf X, C;
  FUELG_TRY(X.init(data, (size_t)n * d * sizeof(float), s));
  FUELG_TRY(C.init(centers, (size_t)k * d * sizeof(float), s));
  OutBuf ol, ob;
  FUELG_TRY(ol.init(out_labels, (size_t)n * sizeof(int64_t), s));
  Scratch best_tmp, keys, dstat;
  float* best = nullptr;
  if (out_best) {
    FUELG_TRY(ob.init(out_best, (size_t)n * sizeof(float), s));
    best = static_cast<float*>(ob.dptr);
  } else {
    FUELG_TRY(best_tmp.alloc(sizeof(float) * n, s));
    best = best_tmp.as<float>();
  }
  FUELG_TRY(keys.alloc(sizeof(uint64_t) * n, s));
  FUELG_TRY(dstat.alloc(sizeof(int), s));
  FUELG_CUDA(cudaMemsetAsync(dstat.p, 0, sizeof(int), s));
  ExactScanParams p;
  p.A = static_cast<const float*>(X.dptr);
  p.m = n;
  p.B = static_cast<const float*>(C.dptr);
  p.n = k;
  p.d = d;
  p.kind = initial ? KIND_PAIRWISE : KIND_SQDIST;
  p.order = order;
  p.metric = METRIC_SQEUCLIDEAN;
  p.kk = 1;
  FUELG_TRY(exact_topk(p, keys.as<uint64_t>(), dstat.as<int>(), s));
  FUELG_TRY(finalize_knn(keys.as<uint64_t>(), n, 1, 1, FUELG_EXCLUDE_NONE, static_cast<int64_t*>(ol.dptr), best, s));
  int64_t d2h = 0;
  FUELG_TRY(ol.flush(s, &d2h));
  if (out_best) FUELG_TRY(ob.flush(s, &d2h));
  const double ms = tm.stop();
  FUELG_TRY(read_dev_status(dstat.as<int>(), s));
  if (stats) {
    stats->device_ms = ms;
    stats->h2d_bytes = X.h2d + C.h2d;
    stats->d2h_bytes = d2h;
    stats->distance_evals = n * (int64_t)k;
    stats->iterations = 1;
    meter.fill(stats);
  }
  return ST_OK;
}

}  // extern "C"

