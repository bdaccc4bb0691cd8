// fuelg_noalloc.cu -- an allocation-free variant of the exact linear-scan kNN.
//
// Some callers cannot allocate device memory: hosts whose GPU memory belongs to
// another allocator (a framework's caching pool, a memory budget fixed at
// start-up) and embedded users that must not grow their footprint once they are
// running.  fuelg_knn_noalloc serves them: it takes device-resident inputs and
// outputs and keeps every temporary in one statically sized device array that
// lives in this module.  The call waits for its stream to finish and reads a
// status word back before it returns.
#include <cstring>
#include <mutex>

#include <cuda.h>

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
struct ScratchSlot {
  CUcontext ctx = nullptr;  // context the address was resolved in
  void* ptr = nullptr;
};
ScratchSlot g_scratch[kMaxDevices];

// Device address of g_noalloc_scratch for the current device and context.  It
// is looked up with cudaGetSymbolAddress on the first call on a device (host
// code must not use the symbol itself: on the host it is only a stand-in, not a
// device address) and looked up again when the calling thread's current context
// is not the one the cached address came from (a context made through the
// driver API, or the primary context re-created after cudaDeviceReset).
int noalloc_scratch(void** out) {
  int dev = 0;
  FUELG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device ordinal %d outside the supported range", dev);
    return ST_ENOTSUP;
  }
  CUcontext ctx = current_context();
  if (ctx == nullptr) {
    // no context yet on this thread: cudaSetDevice makes the device's primary
    // context current (a context the caller made current is left alone)
    FUELG_CUDA(cudaSetDevice(dev));
    ctx = current_context();
  }
  if (ctx == nullptr) {
    set_error("no current CUDA context on device %d", dev);
    return ST_ECUDA;
  }
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  ScratchSlot& slot = g_scratch[dev];
  if (slot.ptr == nullptr || slot.ctx != ctx) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      slot = ScratchSlot{};
      set_error("cannot resolve the static scratch on device %d: %s", dev, cudaGetErrorString(e));
      return ST_ECUDA;
    }
    slot.ctx = ctx;
    slot.ptr = p;
  }
  *out = slot.ptr;
  return ST_OK;
}

// Memory the kernels on the current device can read and write without a copy:
// device memory of this device, managed memory, or mapped host memory.  Device
// memory of another GPU is refused (peer access is not assumed).
bool device_accessible(const void* p, int dev) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type == cudaMemoryTypeDevice) return at.device == dev;
  return at.type == cudaMemoryTypeManaged || (at.type == cudaMemoryTypeHost && at.devicePointer != nullptr);
}

}  // namespace

void noalloc_forget() {
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  for (ScratchSlot& slot : g_scratch) slot = ScratchSlot{};
}

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
  // no staging: everything must already be reachable from the current device
  int dev = 0;
  FUELG_CUDA(cudaGetDevice(&dev));
  if ((n > 0 && !device_accessible(data, dev)) || !device_accessible(queries, dev) ||
      !device_accessible(out_idx, dev) || !device_accessible(out_dist, dev)) {
    set_error("fuelg_knn_noalloc needs data, queries and outputs in memory of the current device (or managed / "
              "mapped memory); it cannot stage host buffers");
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
