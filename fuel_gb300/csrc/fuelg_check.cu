// fuelg_check.cu -- accuracy report of returned kNN results against FP64, and
// the FP32 issue-rate measurement that the plain tiers' roofline is quoted on.
//
// Report: for every returned (query, neighbour) pair the distance is formed
// again in FP64 (differences, squares and sums in double; sqrt in double for
// the euclidean metric) and compared with the returned f32 value; adjacent
// neighbours of a row whose f32 distances are equal or one ulp apart are
// counted as near-ties, and adjacent neighbours whose FP64 distances (index
// breaking exact ties, as DistPair does, src/api/search.rs:23-30) order them
// the other way are counted as order flips -- the only places where the f32
// list the reference returns can differ from an FP64 ranking.
#include <cstring>

#include "fuelg_common.cuh"
#include "fuelg_internal.h"

namespace fuelg {
namespace {

constexpr int kWarps = 8;

struct ReportAcc {
  unsigned long long max_abs_bits;  // non-negative doubles: bit order = value order
  unsigned long long max_rel_bits;
  unsigned long long pairs;
  unsigned long long near_ties;
  unsigned long long flips;
};

__device__ __forceinline__ double dist64(const float* __restrict__ q, const float* __restrict__ x, int d, bool vec4) {
  double s = 0.0;
  if (vec4) {
    const float4* q4 = reinterpret_cast<const float4*>(q);
    const float4* x4 = reinterpret_cast<const float4*>(x);
    for (int c = 0; c < (d >> 2); c++) {
      const float4 a = q4[c], b = __ldg(x4 + c);
      const double e0 = (double)a.x - (double)b.x, e1 = (double)a.y - (double)b.y;
      const double e2 = (double)a.z - (double)b.z, e3 = (double)a.w - (double)b.w;
      s = fma(e0, e0, s);
      s = fma(e1, e1, s);
      s = fma(e2, e2, s);
      s = fma(e3, e3, s);
    }
  } else {
    for (int c = 0; c < d; c++) {
      const double e = (double)q[c] - (double)__ldg(x + c);
      s = fma(e, e, s);
    }
  }
  return s;
}

// One warp per query row, one lane per neighbour (strided by 32).
__global__ void knn_error_kernel(const float* __restrict__ Q, const float* __restrict__ X, int64_t m, int d, int k,
                                 int euclid, int vec4, const int64_t* __restrict__ idx, const float* __restrict__ dist,
                                 ReportAcc* __restrict__ acc) {
  const int lane = threadIdx.x & 31;
  const int64_t r = (int64_t)blockIdx.x * kWarps + (threadIdx.x >> 5);
  if (r >= m) return;
  const float* q = Q + r * d;
  double max_abs = 0.0, max_rel = 0.0;
  unsigned long long pairs = 0, ties = 0, flips = 0;
  double prev_last = 0.0;  // FP64 distance of the previous chunk's last neighbour (lane 31)
  for (int b = 0; b < k; b += 32) {
    const int j = b + lane;
    const int64_t i = j < k ? idx[r * k + j] : -1;
    const float df = j < k ? dist[r * k + j] : 0.f;
    double D = 0.0;
    if (i >= 0) {
      D = dist64(q, X + i * (int64_t)d, d, vec4);
      if (euclid) D = sqrt(D);
      const double err = fabs((double)df - D);
      max_abs = fmax(max_abs, err);
      if (D > 0.0) max_rel = fmax(max_rel, err / D);
      else if (err > 0.0) max_rel = fmax(max_rel, 1.0);
      pairs++;
    }
    // compare with the previous neighbour (lane - 1, or the last lane of the previous chunk)
    double Dp = __shfl_up_sync(0xffffffffu, D, 1);
    if (lane == 0) Dp = prev_last;
    const int64_t ip = (j >= 1 && j < k) ? idx[r * k + j - 1] : -1;
    if (i >= 0 && ip >= 0) {
      const float dfp = dist[r * k + j - 1];
      const int32_t gap = (int32_t)(__float_as_uint(df) - __float_as_uint(dfp));
      if (gap >= 0 && gap <= 1) ties++;
      if (Dp > D || (Dp == D && ip > i)) flips++;
    }
    prev_last = __shfl_sync(0xffffffffu, D, 31);
  }
  for (int o = 16; o > 0; o >>= 1) {
    max_abs = fmax(max_abs, __shfl_xor_sync(0xffffffffu, max_abs, o));
    max_rel = fmax(max_rel, __shfl_xor_sync(0xffffffffu, max_rel, o));
    pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
    ties += __shfl_xor_sync(0xffffffffu, ties, o);
    flips += __shfl_xor_sync(0xffffffffu, flips, o);
  }
  if (lane == 0) {
    atomicMax(&acc->max_abs_bits, (unsigned long long)__double_as_longlong(max_abs));
    atomicMax(&acc->max_rel_bits, (unsigned long long)__double_as_longlong(max_rel));
    atomicAdd(&acc->pairs, pairs);
    atomicAdd(&acc->near_ties, ties);
    atomicAdd(&acc->flips, flips);
  }
}

// FP32 issue rate: eight independent FMA chains per thread.  The iteration
// count arrives at run time and the result is stored only under a condition
// the host never meets, so the chains cannot be folded away.
__global__ void __launch_bounds__(256) fp32_rate_kernel(int iters, float seed, float* __restrict__ sink) {
  float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
  float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
  const float b = 0.999999f, c = 1e-7f;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 16; u++) {
      a0 = fmaf(a0, b, c);
      a1 = fmaf(a1, b, c);
      a2 = fmaf(a2, b, c);
      a3 = fmaf(a3, b, c);
      a4 = fmaf(a4, b, c);
      a5 = fmaf(a5, b, c);
      a6 = fmaf(a6, b, c);
      a7 = fmaf(a7, b, c);
    }
  }
  const float s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == -1.f) sink[threadIdx.x] = s;
}

}  // namespace

int knn_error_report(const float* Q, const float* X, int64_t m, int d, int k, int metric, const int64_t* idx,
                     const float* dist, double* max_abs, double* max_rel, int64_t* pairs, int64_t* near_ties,
                     int64_t* flips, cudaStream_t s) {
  Scratch acc;
  FUELG_TRY(acc.alloc(sizeof(ReportAcc), s));
  FUELG_CUDA(cudaMemsetAsync(acc.p, 0, sizeof(ReportAcc), s));
  const int vec4 = (d % 4 == 0) && ((reinterpret_cast<uintptr_t>(Q) & 15) == 0) &&
                   ((reinterpret_cast<uintptr_t>(X) & 15) == 0);
  if (m > 0 && k > 0) {
    knn_error_kernel<<<(unsigned)((m + kWarps - 1) / kWarps), 32 * kWarps, 0, s>>>(
        Q, X, m, d, k, metric == METRIC_EUCLIDEAN, vec4, idx, dist, acc.as<ReportAcc>());
    note_launch();
    FUELG_CUDA(cudaGetLastError());
  }
  ReportAcc h;
  FUELG_CUDA(cudaMemcpyAsync(&h, acc.p, sizeof(h), cudaMemcpyDeviceToHost, s));
  FUELG_CUDA(cudaStreamSynchronize(s));
  long long ab = (long long)h.max_abs_bits, rb = (long long)h.max_rel_bits;
  memcpy(max_abs, &ab, sizeof(double));
  memcpy(max_rel, &rb, sizeof(double));
  *pairs = (int64_t)h.pairs;
  *near_ties = (int64_t)h.near_ties;
  *flips = (int64_t)h.flips;
  return ST_OK;
}

int fp32_issue_rate(double* tera_fma_per_s, double* ms_out) {
  int dev = 0, sms = 0;
  FUELG_CUDA(cudaGetDevice(&dev));
  FUELG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  cudaStream_t s;
  FUELG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct Guard {
    cudaStream_t s;
    cudaEvent_t a = nullptr, b = nullptr;
    float* sink = nullptr;
    ~Guard() {
      if (a) cudaEventDestroy(a);
      if (b) cudaEventDestroy(b);
      if (sink) cudaFree(sink);
      cudaStreamDestroy(s);
    }
  } g{s};
  FUELG_CUDA(cudaMalloc(&g.sink, 256 * sizeof(float)));
  FUELG_CUDA(cudaEventCreate(&g.a));
  FUELG_CUDA(cudaEventCreate(&g.b));
  const int blocks = sms * 8, threads = 256, iters = 4096;
  fp32_rate_kernel<<<blocks, threads, 0, s>>>(iters / 8, 1.f, g.sink);  // warm-up
  note_launch();
  float best = 1e30f;
  for (int rep = 0; rep < 5; rep++) {
    FUELG_CUDA(cudaEventRecord(g.a, s));
    fp32_rate_kernel<<<blocks, threads, 0, s>>>(iters, 1.f, g.sink);
    note_launch();
    FUELG_CUDA(cudaEventRecord(g.b, s));
    FUELG_CUDA(cudaEventSynchronize(g.b));
    float ms = 0.f;
    FUELG_CUDA(cudaEventElapsedTime(&ms, g.a, g.b));
    best = ms < best ? ms : best;
  }
  FUELG_CUDA(cudaGetLastError());
  const double fmas = (double)blocks * threads * iters * 16 * 8;
  *tera_fma_per_s = fmas / (best * 1e-3) / 1e12;
  *ms_out = best;
  return ST_OK;
}

}  // namespace fuelg
