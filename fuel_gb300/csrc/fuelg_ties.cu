// fuelg_ties.cu -- tie-inclusive kNN lists (KNNHeap::into_vec semantics).
//
// fuel's KNNHeap (src/api/search.rs:80-151) returns the k nearest points plus
// every point tied with the k-th distance, sorted by (distance, index).  That
// list is exactly {i : dist(q, i) <= D_k}, D_k being the k-th smallest distance
// (with multiplicity), so it is built here from a top-kk key list with kk > k
// spare ranks: a row whose tie run at D_k ends inside its kk keys is complete;
// a row whose kept keys all lie at or below D_k (more ties than spare ranks) is
// answered by an exact range scan with radius D_k.  The linear-index exclude
// rule (python/search.rs:485-488: search k, then drop self) and the k+1 rule of
// the tree / precomputed paths (:1163-1170) drop index i from row i afterwards,
// as `results.retain(|p| p.index != i)` does.
#include <algorithm>
#include <cub/device/device_scan.cuh>

#include "fuelg_common.cuh"
#include "fuelg_internal.h"

namespace fuelg {
namespace {

constexpr int kWarpsPerBlock = 8;

// One warp per row: run length at D_k, whether self lies in it, overflow.
// lim[r] = keys of row r that belong to its list (all of them when the row has
// fewer than kq valid keys); cnt[r] = the list length after dropping self;
// radius[r] = D_k (+inf when the row has fewer than kq points); rows whose
// every kept key lies at or below D_k while the index has more points are
// appended to ovf (their lists come from a range scan).
__global__ void ties_rows_kernel(const uint64_t* __restrict__ keys, int64_t m, int kk, int kq, int64_t n,
                                 int drop_self, int32_t* __restrict__ lim, int64_t* __restrict__ cnt,
                                 float* __restrict__ radius, int32_t* __restrict__ ovf, int32_t* __restrict__ n_ovf,
                                 int32_t* __restrict__ ovf_pos) {
  const int lane = threadIdx.x & 31;
  const int64_t r = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (r >= m) return;
  const uint64_t* row = keys + r * (int64_t)kk;
  // valid keys form a prefix (sorted ascending, KEY_NONE last)
  int valid = 0;
  for (int b = 0; b < kk; b += 32) {
    const int j = b + lane;
    const bool ok = j < kk && row[j] != KEY_NONE;
    const unsigned bal = __ballot_sync(0xffffffffu, ok);
    valid += __popc(bal);
    if (bal != 0xffffffffu) break;
  }
  int c;
  float D;
  if (valid < kq) {
    c = valid;
    D = __int_as_float(0x7f800000);
  } else {
    const uint32_t dbits = static_cast<uint32_t>(row[kq - 1] >> 32);
    D = __uint_as_float(dbits);
    // first key past the run: keys are sorted, so count those with distance bits <= dbits
    c = kq;
    for (int b = kq; b < valid; b += 32) {
      const int j = b + lane;
      const bool in = j < valid && static_cast<uint32_t>(row[j] >> 32) <= dbits;
      const unsigned bal = __ballot_sync(0xffffffffu, in);
      c += __popc(bal);
      if (bal != 0xffffffffu) break;
    }
  }
  const bool overflow = valid >= kq && c == kk && n > kk;
  int self = 0;
  if (drop_self && !overflow) {
    for (int b = 0; b < c; b += 32) {
      const int j = b + lane;
      const bool hit = j < c && (int64_t)key_idx(row[j]) == r;
      if (__any_sync(0xffffffffu, hit)) {
        self = 1;
        break;
      }
    }
  }
  if (lane == 0) {
    lim[r] = c;
    radius[r] = D;
    if (overflow) {
      const int slot = atomicAdd(n_ovf, 1);
      ovf[slot] = (int32_t)r;
      ovf_pos[r] = slot;
      cnt[r] = 0;  // set from the range result
    } else {
      ovf_pos[r] = -1;
      cnt[r] = c - self;
    }
  }
}

__global__ void gather_rows_kernel(const float* __restrict__ Q, int d, const int32_t* __restrict__ list, int o,
                                   const float* __restrict__ radius, float* __restrict__ out,
                                   float* __restrict__ out_radius) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)o * d) return;
  const int j = (int)(e / d);
  const int c = (int)(e - (int64_t)j * d);
  const int64_t r = list[j];
  out[e] = Q[r * d + c];
  if (c == 0) out_radius[j] = radius[r];
}

// List length of an overflow row after dropping self.
__global__ void ovf_count_kernel(const int32_t* __restrict__ list, int o, const int64_t* __restrict__ off,
                                 const int64_t* __restrict__ idx, int drop_self, int64_t* __restrict__ cnt) {
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (j >= o) return;
  const int64_t r = list[j];
  const int64_t b0 = off[j], b1 = off[j + 1];
  int self = 0;
  if (drop_self) {
    for (int64_t b = b0; b < b1; b += 32) {
      const int64_t e = b + lane;
      if (__any_sync(0xffffffffu, e < b1 && idx[e] == r)) {
        self = 1;
        break;
      }
    }
  }
  if (lane == 0) cnt[r] = (b1 - b0) - self;
}

// One warp per row: write the row's list (self dropped) at its CSR offset.
__global__ void ties_fill_kernel(const uint64_t* __restrict__ keys, int64_t m, int kk, int drop_self,
                                 const int32_t* __restrict__ lim, const int32_t* __restrict__ ovf_pos,
                                 const int64_t* __restrict__ roff, const int64_t* __restrict__ ridx,
                                 const float* __restrict__ rdist, const int64_t* __restrict__ off,
                                 int64_t* __restrict__ out_idx, float* __restrict__ out_dist) {
  const int lane = threadIdx.x & 31;
  const int64_t r = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (r >= m) return;
  int64_t w = off[r];
  const int pos = ovf_pos[r];
  if (pos < 0) {
    const uint64_t* row = keys + r * (int64_t)kk;
    const int c = lim[r];
    for (int b = 0; b < c; b += 32) {
      const int j = b + lane;
      uint64_t key = j < c ? row[j] : KEY_NONE;
      const bool keep = j < c && !(drop_self && (int64_t)key_idx(key) == r);
      const unsigned bal = __ballot_sync(0xffffffffu, keep);
      if (keep) {
        const int64_t at = w + __popc(bal & ((1u << lane) - 1u));
        out_idx[at] = key_idx(key);
        out_dist[at] = key_dist(key);
      }
      w += __popc(bal);
    }
  } else {
    const int64_t b0 = roff[pos], b1 = roff[pos + 1];
    for (int64_t b = b0; b < b1; b += 32) {
      const int64_t e = b + lane;
      const int64_t i = e < b1 ? ridx[e] : -1;
      const bool keep = e < b1 && !(drop_self && i == r);
      const unsigned bal = __ballot_sync(0xffffffffu, keep);
      if (keep) {
        const int64_t at = w + __popc(bal & ((1u << lane) - 1u));
        out_idx[at] = i;
        out_dist[at] = rdist[e];
      }
      w += __popc(bal);
    }
  }
}

}  // namespace

int ties_spare_kk(int kq, int64_t n) {
  // spare ranks past the k-th: enough for the tie runs of ordinary data; rows
  // with longer runs take the range-scan path
  int kk = kq + std::max(8, kq / 4);
  kk = std::min(kk, 4096);
  if ((int64_t)kk > n) kk = (int)std::max<int64_t>(kq, n);
  return std::max(kk, kq);
}

int knn_ties_lists(const uint64_t* keys, int64_t m, int kk, int kq, int drop_self, const ExactScanParams& base,
                   int64_t** d_off, int64_t** d_idx, float** d_dist, int64_t* total, int64_t* range_rows,
                   int* dev_status, cudaStream_t s) {
  *d_off = nullptr;
  *d_idx = nullptr;
  *d_dist = nullptr;
  *total = 0;
  *range_rows = 0;
  FUELG_CUDA(cudaMalloc(d_off, sizeof(int64_t) * (m + 1)));
  if (m == 0) {
    FUELG_CUDA(cudaMemsetAsync(*d_off, 0, sizeof(int64_t), s));
    return ST_OK;
  }
  Scratch lim, cnt, radius, ovf, n_ovf, ovf_pos;
  FUELG_TRY(lim.alloc(sizeof(int32_t) * m, s));
  FUELG_TRY(cnt.alloc(sizeof(int64_t) * (m + 1), s));
  FUELG_TRY(radius.alloc(sizeof(float) * m, s));
  FUELG_TRY(ovf.alloc(sizeof(int32_t) * m, s));
  FUELG_TRY(n_ovf.alloc(sizeof(int32_t), s));
  FUELG_TRY(ovf_pos.alloc(sizeof(int32_t) * m, s));
  FUELG_CUDA(cudaMemsetAsync(n_ovf.p, 0, sizeof(int32_t), s));
  FUELG_CUDA(cudaMemsetAsync(cnt.as<int64_t>() + m, 0, sizeof(int64_t), s));
  const unsigned rblocks = (unsigned)((m + kWarpsPerBlock - 1) / kWarpsPerBlock);
  ties_rows_kernel<<<rblocks, 32 * kWarpsPerBlock, 0, s>>>(keys, m, kk, kq, base.n, drop_self, lim.as<int32_t>(),
                                                           cnt.as<int64_t>(), radius.as<float>(), ovf.as<int32_t>(),
                                                           n_ovf.as<int32_t>(), ovf_pos.as<int32_t>());
  note_launch();
  FUELG_CUDA(cudaGetLastError());
  int o = 0;
  FUELG_CUDA(cudaMemcpyAsync(&o, n_ovf.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  FUELG_CUDA(cudaStreamSynchronize(s));
  *range_rows = o;
  // rows with more ties than spare ranks: exact range scan at radius D_k
  int64_t *roff = nullptr, *ridx = nullptr;
  float* rdist = nullptr;
  struct RangeOut {
    int64_t **a, **b;
    float** c;
    ~RangeOut() {
      if (*a) cudaFree(*a);
      if (*b) cudaFree(*b);
      if (*c) cudaFree(*c);
    }
  } guard{&roff, &ridx, &rdist};
  if (o > 0) {
    Scratch qo, ro;
    FUELG_TRY(qo.alloc(sizeof(float) * (size_t)o * base.d, s));
    FUELG_TRY(ro.alloc(sizeof(float) * o, s));
    const int64_t elems = (int64_t)o * base.d;
    gather_rows_kernel<<<(unsigned)((elems + 255) / 256), 256, 0, s>>>(base.A, base.d, ovf.as<int32_t>(), o,
                                                                      radius.as<float>(), qo.as<float>(),
                                                                      ro.as<float>());
    note_launch();
    FUELG_CUDA(cudaGetLastError());
    ExactScanParams rp = base;
    rp.A = qo.as<float>();
    rp.m = o;
    int64_t rtot = 0;
    FUELG_TRY(exact_range(rp, 0.0f, 0, &roff, &ridx, &rdist, &rtot, dev_status, s, ro.as<float>()));
    ovf_count_kernel<<<(unsigned)((o + kWarpsPerBlock - 1) / kWarpsPerBlock), 32 * kWarpsPerBlock, 0, s>>>(
        ovf.as<int32_t>(), o, roff, ridx, drop_self, cnt.as<int64_t>());
    note_launch();
    FUELG_CUDA(cudaGetLastError());
  }
  size_t tb = 0;
  FUELG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, cnt.as<int64_t>(), *d_off, m + 1, s));
  Scratch tmp;
  FUELG_TRY(tmp.alloc(tb, s));
  FUELG_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tb, cnt.as<int64_t>(), *d_off, m + 1, s));
  int64_t tot = 0;
  FUELG_CUDA(cudaMemcpyAsync(&tot, *d_off + m, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  FUELG_CUDA(cudaStreamSynchronize(s));
  *total = tot;
  if (tot == 0) return ST_OK;
  FUELG_CUDA(cudaMalloc(d_idx, sizeof(int64_t) * tot));
  FUELG_CUDA(cudaMalloc(d_dist, sizeof(float) * tot));
  ties_fill_kernel<<<rblocks, 32 * kWarpsPerBlock, 0, s>>>(keys, m, kk, drop_self, lim.as<int32_t>(),
                                                           ovf_pos.as<int32_t>(), roff, ridx, rdist, *d_off, *d_idx,
                                                           *d_dist);
  note_launch();
  FUELG_CUDA(cudaGetLastError());
  FUELG_CUDA(cudaStreamSynchronize(s));  // the range buffers are freed on return
  return ST_OK;
}

}  // namespace fuelg
