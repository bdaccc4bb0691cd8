// fuelg_noalloc.cu -- an allocation-free variant of the exact linear-scan kNN.
//
// Some callers cannot allocate device memory at all: code running while a CUDA
// graph is being captured (where cudaMalloc is not permitted), callers whose
// GPU memory is owned by another allocator or budgeted up front, and embedded
// hosts that must not grow their footprint after start-up.  fuelg_knn_noalloc
// serves them: it takes device-resident inputs and outputs and keeps every
// temporary in one statically sized device array that lives in this module.
#include <cstring>
#include <mutex>

#include "../../include/fuelg.h"
#include "fuelg_common.cuh"
#include "fuelg_internal.h"

namespace fuelg {
namespace {

// Fixed scratch for the allocation-free entry point.  Every GPU that loads this
// library holds these bytes until the process exits.
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;  // 32 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device, looked up once per
// device (host code must not use the symbol itself: on the host it is only a
// stand-in, not a device address).
int noalloc_scratch(void** out) {
  int dev = 0;
  FUELG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device ordinal %d outside the supported range", dev);
    return ST_ENOTSUP;
  }
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (g_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      set_error("cannot resolve the static scratch on device %d: %s", dev, cudaGetErrorString(e));
      return ST_ECUDA;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return ST_OK;
}

bool device_accessible(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged ||
         (at.type == cudaMemoryTypeHost && at.devicePointer != nullptr);
}

}  // namespace
}  // namespace fuelg

using namespace fuelg;

extern "C" int fuelg_knn_noalloc(const float* data, int64_t n, int32_t d, const float* queries, int64_t m, int32_t k,
                                 int32_t metric, int32_t order, int32_t exclude_mode, int64_t* out_idx,
                                 float* out_dist, void* stream) {
  if (n < 0 || d <= 0 || m < 0 || k < 0) {
    set_error("invalid knn shape n=%lld d=%d m=%lld k=%d", (long long)n, d, (long long)m, k);
    return ST_EINVAL;
  }
  if (metric != FUELG_METRIC_SQEUCLIDEAN && metric != FUELG_METRIC_EUCLIDEAN) {
    set_error("unsupported metric %d", metric);
    return ST_EINVAL;
  }
  if (order != FUELG_ORDER_ARM && order != FUELG_ORDER_X86) {
    set_error("unknown summation order %d", order);
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
  if (m == 0 || k == 0) return ST_OK;
  // no staging: everything must already be reachable from the device
  if ((n > 0 && !device_accessible(data)) || !device_accessible(queries) || !device_accessible(out_idx) ||
      !device_accessible(out_dist)) {
    set_error("fuelg_knn_noalloc needs device-accessible data, queries and outputs (it cannot stage host buffers)");
    return ST_EINVAL;
  }
  void* scratch = nullptr;
  FUELG_TRY(noalloc_scratch(&scratch));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  ExactScanParams p;
  p.A = queries;
  p.m = m;
  p.B = data;
  p.n = n;
  p.d = d;
  p.kind = KIND_KNN;
  p.order = order;
  p.metric = metric;
  p.kk = exclude_mode == FUELG_EXCLUDE_NONE ? k : k + 1;
  FUELG_TRY(exact_knn_in_scratch(p, k, exclude_mode, out_idx, out_dist, scratch, kNoAllocScratchBytes, s));
  int h = 0;
  FUELG_CUDA(cudaMemcpyAsync(&h, scratch, sizeof(int), cudaMemcpyDeviceToHost, s));
  FUELG_CUDA(cudaStreamSynchronize(s));
  if (h != 0) {
    set_error("a kernel reported device status %d", h);
    return ST_ECUDA;
  }
  return ST_OK;
}
