// fuelg_server.cu -- kNN serving over a resident index with continuous
// batching.
//
// Requests (query rows + k) are queued on submit.  Each worker owns a CUDA
// stream and, whenever it is free, takes every queued request that fits its
// batch (query rows) and the server's device-memory budget, runs them as one
// kNN batch -- one tensor-core launch in which every query row selects only
// its own request's k (plus the proof margin); the plain tier computes
// top-max(k) -- exactly the keys each request would get alone: the k smallest
// (distance, index) keys are a prefix of the k' smallest for k' >= k -- and
// hands each request its own first k columns.  Requests that
// arrive while batches are on the GPU are admitted by the next free worker as
// memory frees up, so their device work overlaps.  Results are bit-identical
// to a single fuelg_knn call on the same rows.
#include <algorithm>
#include <condition_variable>
#include <chrono>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/fuelg.h"
#include "fuelg_common.cuh"
#include "fuelg_internal.h"

using namespace fuelg;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t id = 0;
  std::vector<float> q;  // [m, d], copied at submit
  int64_t m = 0;
  int k = 0;
  int64_t* out_idx = nullptr;  // caller memory [m, k]
  float* out_dist = nullptr;
  size_t bytes = 0;  // device bytes charged against the budget
  int status = -1;   // -1 pending / running, else a status code
  std::string error;
  Clock::time_point t_submit, t_done;
};

}  // namespace

struct fuelg_server {
  IndexView view;
  int precision = 0;
  int64_t max_batch = 0;
  int64_t budget = 0;
  std::vector<std::thread> workers;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> pending;
  std::unordered_map<int64_t, Request*> reqs;
  int64_t next_id = 1;
  int64_t inflight = 0;
  bool stop = false;
  // statistics
  int64_t batches = 0, queries = 0, max_rows = 0, max_reqs = 0;
  double device_ms = 0.0;
};

namespace {

// Device bytes a request holds while its batch runs: query rows (f32 and
// BF16), keys and outputs, and the tensor-core tier's per-query lists.
size_t request_bytes(int64_t m, int d, int k) {
  const int64_t kk2 = k + std::max(8, k / 8);
  return (size_t)m * ((size_t)d * 4 + (size_t)((d + 63) / 64) * 64 * 2 + 4 + (size_t)k * 20 +
                      (size_t)(3 * kk2 + 256) * 8 + 64);
}

int run_batch(fuelg_server* sv, std::vector<Request*>& batch, cudaStream_t s, float* pin_q, int32_t* pin_k,
              int64_t* pin_i, float* pin_d, double* ms_out) {
  const IndexView& ix = sv->view;
  int64_t m = 0;
  int kmax = 0;
  for (Request* r : batch) {
    memcpy(pin_q + m * ix.d, r->q.data(), sizeof(float) * r->m * ix.d);
    for (int64_t i = 0; i < r->m; i++) pin_k[m + i] = r->k;
    m += r->m;
    kmax = std::max(kmax, r->k);
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  struct EvGuard {
    cudaEvent_t a, b;
    ~EvGuard() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } eg{e0, e1};
  cudaEventRecord(e0, s);
  Scratch q, rk, keys, oi, od, dstat;
  FUELG_TRY(q.alloc(sizeof(float) * m * ix.d, s));
  FUELG_TRY(rk.alloc(sizeof(int32_t) * m, s));
  FUELG_TRY(keys.alloc(sizeof(uint64_t) * m * kmax, s));
  FUELG_TRY(oi.alloc(sizeof(int64_t) * m * kmax, s));
  FUELG_TRY(od.alloc(sizeof(float) * m * kmax, s));
  FUELG_TRY(dstat.alloc(sizeof(int), s));
  FUELG_CUDA(cudaMemsetAsync(dstat.p, 0, sizeof(int), s));
  FUELG_CUDA(cudaMemcpyAsync(q.p, pin_q, sizeof(float) * m * ix.d, cudaMemcpyHostToDevice, s));
  FUELG_CUDA(cudaMemcpyAsync(rk.p, pin_k, sizeof(int32_t) * m, cudaMemcpyHostToDevice, s));
  const int tier = sv->precision == FUELG_PREC_SPLIT_BF16 ? TC_SPLIT
                   : sv->precision == FUELG_PREC_F16    ? TC_F16
                                                        : TC_BF16;
  int rc = ST_ENOTSUP;
  if (sv->precision != FUELG_PREC_FP32 && ix.tc && (tier != TC_F16 || ix.f16) &&
      knn_tc_supported(ix.n, ix.d, kmax, tier)) {
    // one launch for the mixed batch: every row selects only its own k (plus margin)
    int64_t rescored = 0;
    int exact = 0;
    rc = knn_tc_topk(ix.tc, q.as<float>(), m, ix.X, kmax, ix.order, ix.metric, tier, keys.as<uint64_t>(),
                     dstat.as<int>(), s, &rescored, &exact, rk.as<int32_t>());
    if (rc != ST_OK && rc != ST_ENOTSUP) return rc;  // ENOTSUP: queries outside the FP16 range
  }
  if (rc != ST_OK) {
    ExactScanParams p;
    p.A = q.as<float>();
    p.m = m;
    p.B = ix.X;
    p.n = ix.n;
    p.d = ix.d;
    p.kind = KIND_KNN;
    p.order = ix.order;
    p.metric = ix.metric;
    p.kk = kmax;
    FUELG_TRY(exact_topk(p, keys.as<uint64_t>(), dstat.as<int>(), s));
  }
  FUELG_TRY(finalize_knn(keys.as<uint64_t>(), m, kmax, kmax, FUELG_EXCLUDE_NONE, oi.as<int64_t>(), od.as<float>(), s));
  FUELG_CUDA(cudaMemcpyAsync(pin_i, oi.p, sizeof(int64_t) * m * kmax, cudaMemcpyDeviceToHost, s));
  FUELG_CUDA(cudaMemcpyAsync(pin_d, od.p, sizeof(float) * m * kmax, cudaMemcpyDeviceToHost, s));
  cudaEventRecord(e1, s);
  FUELG_CUDA(cudaStreamSynchronize(s));
  int hst = 0;
  FUELG_CUDA(cudaMemcpy(&hst, dstat.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (hst & DEV_TIMEOUT) {
    set_error("a device wait timed out");
    return ST_ETIMEOUT;
  }
  if (hst & DEV_CANCELLED) {
    set_error("interrupted");
    return ST_ECANCELLED;
  }
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  *ms_out = ms;
  // each request's own first k columns
  int64_t r0 = 0;
  for (Request* r : batch) {
    for (int64_t i = 0; i < r->m; i++) {
      memcpy(r->out_idx + i * r->k, pin_i + (r0 + i) * kmax, sizeof(int64_t) * r->k);
      memcpy(r->out_dist + i * r->k, pin_d + (r0 + i) * kmax, sizeof(float) * r->k);
    }
    r0 += r->m;
  }
  return ST_OK;
}

void worker_main(fuelg_server* sv) {
  cudaSetDevice(sv->view.device);
  cudaStream_t s;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  const int64_t rows = sv->max_batch;
  const int d = sv->view.d;
  // pinned staging for one batch (kmax <= 4095 bounded by submit checks)
  float* pin_q = nullptr;
  int32_t* pin_k = nullptr;
  int64_t* pin_i = nullptr;
  float* pin_d = nullptr;
  cudaHostAlloc(&pin_q, sizeof(float) * rows * d, cudaHostAllocDefault);
  cudaHostAlloc(&pin_k, sizeof(int32_t) * rows, cudaHostAllocDefault);
  size_t out_cap = 0;
  for (;;) {
    std::vector<Request*> batch;
    size_t bytes = 0;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      sv->cv_work.wait(lk, [&] {
        return sv->stop || (!sv->pending.empty() && (sv->inflight == 0 ||
                                                    sv->inflight + (int64_t)sv->pending.front()->bytes <= sv->budget));
      });
      if (sv->stop && sv->pending.empty()) break;
      int64_t m = 0;
      while (!sv->pending.empty()) {
        Request* r = sv->pending.front();
        if (!batch.empty() && (m + r->m > rows || sv->inflight + (int64_t)(bytes + r->bytes) > sv->budget)) break;
        sv->pending.pop_front();
        batch.push_back(r);
        bytes += r->bytes;
        m += r->m;
      }
      sv->inflight += (int64_t)bytes;
    }
    int64_t m = 0;
    int kmax = 0;
    for (Request* r : batch) {
      m += r->m;
      kmax = std::max(kmax, r->k);
    }
    if ((size_t)(m * kmax) > out_cap) {
      if (pin_i) cudaFreeHost(pin_i);
      if (pin_d) cudaFreeHost(pin_d);
      out_cap = (size_t)(m * kmax);
      cudaHostAlloc(&pin_i, sizeof(int64_t) * out_cap, cudaHostAllocDefault);
      cudaHostAlloc(&pin_d, sizeof(float) * out_cap, cudaHostAllocDefault);
    }
    double ms = 0.0;
    const int st = (pin_q && pin_k && pin_i && pin_d) ? run_batch(sv, batch, s, pin_q, pin_k, pin_i, pin_d, &ms)
                                                      : ST_ENOMEM;
    const std::string err = st == ST_OK ? std::string() : std::string(fuelg_last_error());
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      sv->inflight -= (int64_t)bytes;
      const auto now = Clock::now();
      for (Request* r : batch) {
        r->status = st;
        r->error = err;
        r->t_done = now;
      }
      if (st == ST_OK) {
        sv->batches++;
        sv->queries += m;
        sv->max_rows = std::max(sv->max_rows, m);
        sv->max_reqs = std::max(sv->max_reqs, (int64_t)batch.size());
        sv->device_ms += ms;
      }
    }
    sv->cv_done.notify_all();
    sv->cv_work.notify_all();
  }
  if (pin_q) cudaFreeHost(pin_q);
  if (pin_k) cudaFreeHost(pin_k);
  if (pin_i) cudaFreeHost(pin_i);
  if (pin_d) cudaFreeHost(pin_d);
  cudaStreamDestroy(s);
}

}  // namespace

extern "C" {

int fuelg_server_create(fuelg_index* ix, int32_t precision, int64_t max_batch_queries, int64_t budget_bytes,
                        int32_t workers, fuelg_server** out) {
  if (!out || !ix) {
    set_error("index and out must be non-NULL");
    return ST_EINVAL;
  }
  *out = nullptr;
  if (precision < FUELG_PREC_AUTO || precision > FUELG_PREC_F16 || precision == FUELG_PREC_SPLIT_BF16_SCALED ||
      max_batch_queries < 1 ||
      budget_bytes < 1 || workers < 1 || workers > 16) {
    set_error("invalid server arguments (precision=%d max_batch=%lld budget=%lld workers=%d)", precision,
              (long long)max_batch_queries, (long long)budget_bytes, workers);
    return ST_EINVAL;
  }
  IndexView v;
  if (precision == FUELG_PREC_AUTO) {
    // by the index's value class: the exact BF16 screen for small integers,
    // FP16 (one product) within its range, split BF16 otherwise
    FUELG_TRY(index_view_get(ix, TC_BF16, &v));
    precision = !v.tc ? FUELG_PREC_FP32
                : knn_tc_index_class(v.tc) == TC_CLASS_INTEGER   ? FUELG_PREC_BF16
                : knn_tc_index_class(v.tc) == TC_CLASS_F16_RANGE ? FUELG_PREC_F16
                                                                 : FUELG_PREC_SPLIT_BF16;
  }
  const int want = precision == FUELG_PREC_FP32         ? -1
                   : precision == FUELG_PREC_SPLIT_BF16 ? TC_SPLIT
                   : precision == FUELG_PREC_F16        ? TC_F16
                                                        : TC_BF16;
  FUELG_TRY(index_view_get(ix, want, &v));
  fuelg_server* sv = new fuelg_server();
  sv->view = v;
  sv->precision = precision;
  sv->max_batch = max_batch_queries;
  sv->budget = budget_bytes;
  for (int i = 0; i < workers; i++) sv->workers.emplace_back(worker_main, sv);
  server_opened();
  *out = sv;
  return ST_OK;
}

int fuelg_server_submit(fuelg_server* sv, const float* queries, int64_t m, int32_t k, int64_t* out_idx,
                        float* out_dist, int64_t* request_id) {
  if (!sv || !request_id || m < 1 || k < 1 || !queries || !out_idx || !out_dist) {
    set_error("invalid submit arguments m=%lld k=%d", (long long)m, k);
    return ST_EINVAL;
  }
  if (k > 4095) {
    set_error("k=%d exceeds the supported maximum of 4095", k);
    return ST_ENOTSUP;
  }
  if (m > sv->max_batch) {
    set_error("request of %lld rows exceeds the server batch of %lld rows", (long long)m, (long long)sv->max_batch);
    return ST_EINVAL;
  }
  const size_t bytes = request_bytes(m, sv->view.d, k);
  if ((int64_t)bytes > sv->budget) {
    set_error("request needs %zu device bytes, above the server budget of %lld", bytes, (long long)sv->budget);
    return ST_ENOMEM;
  }
  Request* r = new Request();
  r->q.assign(queries, queries + m * sv->view.d);
  r->m = m;
  r->k = k;
  r->out_idx = out_idx;
  r->out_dist = out_dist;
  r->bytes = bytes;
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->stop) {
      delete r;
      set_error("server is shutting down");
      return ST_EINVAL;
    }
    r->id = sv->next_id++;
    sv->reqs[r->id] = r;
    sv->pending.push_back(r);
    *request_id = r->id;
  }
  sv->cv_work.notify_one();
  return ST_OK;
}

int fuelg_server_wait(fuelg_server* sv, int64_t request_id, int32_t timeout_ms, double* latency_ms) {
  if (!sv) {
    set_error("server is NULL");
    return ST_EINVAL;
  }
  std::unique_lock<std::mutex> lk(sv->mu);
  auto it = sv->reqs.find(request_id);
  if (it == sv->reqs.end()) {
    set_error("unknown request id %lld", (long long)request_id);
    return ST_EINVAL;
  }
  Request* r = it->second;
  auto done = [&] { return r->status != -1; };
  if (timeout_ms < 0) {
    sv->cv_done.wait(lk, done);
  } else if (!sv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) {
    set_error("request %lld not finished within %d ms", (long long)request_id, timeout_ms);
    return ST_ETIMEOUT;
  }
  const int st = r->status;
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  if (st != ST_OK) set_error("%s", r->error.c_str());
  sv->reqs.erase(it);
  delete r;
  return st;
}

int fuelg_server_stats(fuelg_server* sv, int64_t* batches, int64_t* queries, int64_t* max_batch_rows,
                       int64_t* max_batch_requests, double* device_ms) {
  if (!sv) {
    set_error("server is NULL");
    return ST_EINVAL;
  }
  std::lock_guard<std::mutex> lk(sv->mu);
  if (batches) *batches = sv->batches;
  if (queries) *queries = sv->queries;
  if (max_batch_rows) *max_batch_rows = sv->max_rows;
  if (max_batch_requests) *max_batch_requests = sv->max_reqs;
  if (device_ms) *device_ms = sv->device_ms;
  return ST_OK;
}

int fuelg_server_destroy(fuelg_server* sv) {
  if (!sv) return ST_OK;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  for (auto& t : sv->workers) t.join();
  for (auto& kv : sv->reqs) delete kv.second;
  delete sv;
  server_closed();
  return ST_OK;
}

}  // extern "C"
