// fuelg_f64.cu -- the exact FP64 linear scan: fuel's float64 search path.
//
// fuel builds a float64 index for every input that is not float32
// (python/fuel/_dispatch.py:8-19, build_linear_scan_f64 python/search.rs:
// 1371-1389) and compares f64 distances: squared_euclidean_distance_f64_avx_fma
// on x86 builds with AVX + FMA (src/distance/squared_euclidean.rs:44-67: one
// 4-lane FMA accumulator, the lanes summed left to right, an FMA tail), the
// 8-lane fallback elsewhere (:99-133: separate multiply and add per lane, the
// lanes folded left to right, a multiply-add tail); Euclidean is the f64 sqrt
// of that (src/distance/euclidean.rs:7-9).
//
// Per batch of query rows one launch writes every (query, point) distance of
// the batch to HBM ([B, n] doubles, at most 1 GiB).  One block per query row
// then finds the row's kk-th smallest key by an 8-pass radix select over the
// 64-bit patterns of the distances (non-negative doubles order as their bits,
// NaN after +inf), and a pass in index order collects the keys below it and,
// still in index order, the keys equal to it -- the order in which
// KNNHeap::into_vec lists equal distances (DistPair order, src/api/search.rs:
// 23-30).  The keys below the threshold (fewer than kk <= 4096) are sorted in
// shared memory.  Range lists are collected in index order and sorted stably
// by distance.
#include <algorithm>
#include <cstring>
#include <vector>

#include <cub/device/device_segmented_sort.cuh>

#include "../../include/fuelg.h"
#include "fuelg_internal.h"

namespace fuelg {
namespace {

constexpr int kT = 256;                           // threads per block of every kernel here
constexpr size_t kBatchBytes = size_t(1) << 30;   // distance matrix of one query batch
constexpr int kMaxSortKeys = 4096;                // keys one block sorts in shared memory
constexpr unsigned kFull = 0xffffffffu;

// One (query, point) squared distance in fuel's f64 operation order.
template <int ORDER>
__device__ __forceinline__ double sqdist64(const double* __restrict__ q, const double* __restrict__ x, int d) {
  if (ORDER == FUELG_ORDER_X86) {
    const int sd = d & ~3;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    for (int i = 0; i < sd; i += 4) {
      const double e0 = __dsub_rn(q[i], x[i]), e1 = __dsub_rn(q[i + 1], x[i + 1]);
      const double e2 = __dsub_rn(q[i + 2], x[i + 2]), e3 = __dsub_rn(q[i + 3], x[i + 3]);
      a0 = __fma_rn(e0, e0, a0);
      a1 = __fma_rn(e1, e1, a1);
      a2 = __fma_rn(e2, e2, a2);
      a3 = __fma_rn(e3, e3, a3);
    }
    double s = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(-0.0, a0), a1), a2), a3);
    for (int i = sd; i < d; i++) {
      const double e = __dsub_rn(q[i], x[i]);
      s = __fma_rn(e, e, s);
    }
    return s;
  } else {
    const int sd = d & ~7;
    double v[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int i = 0; i < sd; i += 8) {
#pragma unroll
      for (int l = 0; l < 8; l++) {
        const double e = __dsub_rn(q[i + l], x[i + l]);
        v[l] = __dadd_rn(__dmul_rn(e, e), v[l]);
      }
    }
    double s = -0.0;
#pragma unroll
    for (int l = 0; l < 8; l++) s = __dadd_rn(s, v[l]);
    for (int i = sd; i < d; i++) {
      const double e = __dsub_rn(q[i], x[i]);
      s = __dadd_rn(__dmul_rn(e, e), s);
    }
    return s;
  }
}

// Order key of a distance: its bit pattern (-0 counted as +0).
__device__ __forceinline__ uint64_t key64(double v) {
  const uint64_t u = static_cast<uint64_t>(__double_as_longlong(v));
  return u == 0x8000000000000000ull ? 0ull : u;
}

// D[b, i] = distance(query q0 + b, point i) for the batch's rows.
template <int ORDER>
__global__ void __launch_bounds__(kT) dist64_kernel(const double* __restrict__ X, int64_t n, int d,
                                                    const double* __restrict__ Q, int euclid,
                                                    double* __restrict__ D) {
  const int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x;
  if (i >= n) return;
  const int64_t b = blockIdx.y;
  double v = sqdist64<ORDER>(Q + b * d, X + i * d, d);
  if (euclid) v = __dsqrt_rn(v);
  D[b * n + i] = v;
}

// Inclusive prefix sum of one value per thread over the block (blockDim == kT).
__device__ __forceinline__ unsigned block_incl_scan(unsigned v, unsigned* wt) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned t = __shfl_up_sync(kFull, v, o);
    if (lane >= o) v += t;
  }
  if (lane == 31) wt[w] = v;
  __syncthreads();
  unsigned add = 0;
  for (int j = 0; j < w; j++) add += wt[j];
  __syncthreads();
  return v + add;
}

// Block-wide stream compaction of two predicates over one chunk of kT
// elements: each thread's exclusive position among the chunk's set flags
// (thread order = index order) and the chunk's totals.  Every thread of the
// block calls it.
__device__ __forceinline__ void block_compact2(bool a, bool e, unsigned* wa, unsigned* we, unsigned* pa,
                                               unsigned* pe, unsigned* ta, unsigned* te) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned ba = __ballot_sync(kFull, a), be = __ballot_sync(kFull, e);
  if (lane == 0) {
    wa[w] = __popc(ba);
    we[w] = __popc(be);
  }
  __syncthreads();
  unsigned oa = 0, oe = 0, sa = 0, se = 0;
#pragma unroll
  for (int j = 0; j < kT / 32; j++) {
    const unsigned x = wa[j], y = we[j];
    if (j < w) {
      oa += x;
      oe += y;
    }
    sa += x;
    se += y;
  }
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  *pa = oa + __popc(ba & lt);
  *pe = oe + __popc(be & lt);
  *ta = sa;
  *te = se;
}

// Ascending (key, index) bitonic sort of sk/si[0, cnt) in shared memory; the
// arrays hold at least the next power of two >= cnt entries.
__device__ void block_sort_pairs(uint64_t* sk, uint32_t* si, int cnt) {
  int P = 1;
  while (P < cnt) P <<= 1;
  for (int t = cnt + threadIdx.x; t < P; t += kT) {
    sk[t] = ~0ull;
    si[t] = 0xffffffffu;
  }
  __syncthreads();
  for (int size = 2; size <= P; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = threadIdx.x; t < P / 2; t += kT) {
        const int lo = 2 * t - (t & (stride - 1));
        const int hi = lo + stride;
        const uint64_t ka = sk[lo], kb = sk[hi];
        const uint32_t ia = si[lo], ib = si[hi];
        const bool a_gt_b = ka > kb || (ka == kb && ia > ib);
        if (a_gt_b == ((lo & size) == 0)) {
          sk[lo] = kb;
          sk[hi] = ka;
          si[lo] = ib;
          si[hi] = ia;
        }
      }
      __syncthreads();
    }
}

// Per query row (one block): the kk-th smallest key T of the row (1 <= kk <= n),
// the number of keys below T and the number equal to T.
__global__ void __launch_bounds__(kT) select64_kernel(const double* __restrict__ D, int64_t n, int64_t kk,
                                                      uint64_t* __restrict__ thr, int64_t* __restrict__ n_less,
                                                      int64_t* __restrict__ n_eq) {
  __shared__ unsigned hist[256];
  __shared__ unsigned wt[kT / 32];
  __shared__ unsigned s_digit, s_below, s_cnt;
  const double* row = D + (int64_t)blockIdx.x * n;
  uint64_t prefix = 0, mask = 0;
  int64_t need = kk, less = 0;
  unsigned cnt = 0;
  for (int shift = 56; shift >= 0; shift -= 8) {
    hist[threadIdx.x] = 0u;
    __syncthreads();
    for (int64_t i = threadIdx.x; i < n; i += kT) {
      const uint64_t key = key64(row[i]);
      if ((key & mask) == prefix) atomicAdd(&hist[(unsigned)(key >> shift) & 255u], 1u);
    }
    __syncthreads();
    const unsigned c = hist[threadIdx.x];
    const unsigned incl = block_incl_scan(c, wt);
    const unsigned excl = incl - c;
    // exactly one bin holds the need-th key among those matching the prefix
    if ((int64_t)excl < need && need <= (int64_t)incl) {
      s_digit = threadIdx.x;
      s_below = excl;
      s_cnt = c;
    }
    __syncthreads();
    prefix |= (uint64_t)s_digit << shift;
    mask |= 0xffull << shift;
    need -= s_below;
    less += s_below;
    cnt = s_cnt;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    thr[blockIdx.x] = prefix;
    n_less[blockIdx.x] = less;
    n_eq[blockIdx.x] = cnt;
  }
}

// Truncated kNN rows (fuelg_knn_f64).  Row b (query q0 + b): the kk smallest
// (key, index) pairs -- every key below T in index order, then the first
// kk - less keys equal to T -- sorted by (key, index) in shared memory (P
// entries, the next power of two >= kk), then the exclude rule and the
// marshaller's truncation to k with -1 / +inf padding (python/search.rs:
// 485-488, 1163-1170, 1195-1216).  mode: FUELG_EXCLUDE_*; kk = min(k, n) for
// NONE, min(k + 1, n) otherwise.
__global__ void __launch_bounds__(kT) knn64_finish_kernel(const double* __restrict__ D, int64_t n, int kk, int k,
                                                          int mode, int64_t q0, const uint64_t* __restrict__ thr,
                                                          const int64_t* __restrict__ n_less, int P,
                                                          int64_t* __restrict__ out_idx,
                                                          double* __restrict__ out_dist) {
  extern __shared__ __align__(16) unsigned char smem64[];
  uint64_t* sk = reinterpret_cast<uint64_t*>(smem64);
  uint32_t* si = reinterpret_cast<uint32_t*>(sk + P);
  __shared__ unsigned wa[kT / 32], we[kT / 32];
  __shared__ int s_self;
  const int64_t b = blockIdx.x;
  const double* row = D + b * n;
  const uint64_t T = thr[b];
  const int less = (int)n_less[b];  // < kk
  const int take = kk - less;       // >= 1 keys equal to T
  int bl = 0, be = 0;
  for (int64_t c = 0; c < n; c += kT) {
    const int64_t i = c + threadIdx.x;
    const uint64_t key = i < n ? key64(row[i]) : ~0ull;
    const bool isl = i < n && key < T, ise = i < n && key == T;
    unsigned pl, pe, tl, te;
    block_compact2(isl, ise, wa, we, &pl, &pe, &tl, &te);
    if (isl) {
      sk[bl + pl] = key;
      si[bl + pl] = (uint32_t)i;
    }
    if (ise && be + (int)pe < take) {
      sk[less + be + pe] = key;
      si[less + be + pe] = (uint32_t)i;
    }
    bl += (int)tl;
    be = min(be + (int)te, take);
    if (bl >= less && be >= take) break;
  }
  __syncthreads();
  block_sort_pairs(sk, si, kk);
  // the list before truncation: k (or k + 1 for the k+1 rule) entries, and
  // the linear-index rule keeps entry k only when it ties the k-th distance
  int L = kk;
  if (mode == FUELG_EXCLUDE_LINEAR && kk > k) L = sk[k] == sk[k - 1] ? k + 1 : k;
  if (threadIdx.x == 0) s_self = -1;
  __syncthreads();
  const int64_t self = q0 + b;
  if (mode != FUELG_EXCLUDE_NONE)
    for (int j = threadIdx.x; j < L; j += kT)
      if ((int64_t)si[j] == self) s_self = j;
  __syncthreads();
  const int sp = s_self;
  for (int j = threadIdx.x; j < k; j += kT) {
    const int src = j + (sp >= 0 && j >= sp ? 1 : 0);
    const bool have = src < L;
    out_idx[b * k + j] = have ? (int64_t)si[src] : -1;
    out_dist[b * k + j] = have ? __longlong_as_double((long long)sk[src]) : __longlong_as_double(0x7ff0000000000000ll);
  }
}

// Tie-inclusive list length of row b: the keys below and equal to T, less
// the row's own point where the exclude rule drops it (query q0 + b is point
// q0 + b).
__global__ void ties_count64_kernel(const double* __restrict__ D, int64_t n, int B, int64_t q0, int drop_self,
                                    const uint64_t* __restrict__ thr, const int64_t* __restrict__ n_less,
                                    const int64_t* __restrict__ n_eq, int64_t* __restrict__ cnt) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  int64_t c = n_less[b] + n_eq[b];
  const int64_t r = q0 + b;
  if (drop_self && r < n && key64(D[(int64_t)b * n + r]) <= thr[b]) c -= 1;
  cnt[b] = c;
}

// Tie-inclusive rows into CSR at off[b]: the keys below T, sorted by (key,
// index) in shared memory (at most kk - 1 of them; P entries), then every key
// equal to T in index order (written as found).
__global__ void __launch_bounds__(kT) ties64_gather_kernel(const double* __restrict__ D, int64_t n, int64_t q0,
                                                           int drop_self, const uint64_t* __restrict__ thr,
                                                           const int64_t* __restrict__ n_less,
                                                           const int64_t* __restrict__ n_eq,
                                                           const int64_t* __restrict__ off, int P,
                                                           uint64_t* __restrict__ out_key,
                                                           int64_t* __restrict__ out_idx) {
  extern __shared__ __align__(16) unsigned char smem64[];
  uint64_t* sk = reinterpret_cast<uint64_t*>(smem64);
  uint32_t* si = reinterpret_cast<uint32_t*>(sk + P);
  __shared__ unsigned wa[kT / 32], we[kT / 32];
  const int64_t b = blockIdx.x;
  const double* row = D + b * n;
  const uint64_t T = thr[b];
  const int64_t r = q0 + b;
  const bool has_self = drop_self && r < n;
  const uint64_t kself = has_self ? key64(row[r]) : 0ull;
  const int less = (int)(n_less[b] - (has_self && kself < T ? 1 : 0));
  const int64_t eq_total = n_eq[b] - (has_self && kself == T ? 1 : 0);
  const int64_t base = off[b];
  int bl = 0;
  int64_t be = 0;
  for (int64_t c = 0; c < n; c += kT) {
    const int64_t i = c + threadIdx.x;
    const bool keep = i < n && !(has_self && i == r);
    const uint64_t key = i < n ? key64(row[i]) : ~0ull;
    const bool isl = keep && key < T, ise = keep && key == T;
    unsigned pl, pe, tl, te;
    block_compact2(isl, ise, wa, we, &pl, &pe, &tl, &te);
    if (isl) {
      sk[bl + pl] = key;
      si[bl + pl] = (uint32_t)i;
    }
    if (ise) {
      out_key[base + less + be + pe] = key;
      out_idx[base + less + be + pe] = i;
    }
    bl += (int)tl;
    be += te;
    if (bl >= less && be >= eq_total) break;
  }
  __syncthreads();
  block_sort_pairs(sk, si, less);
  for (int j = threadIdx.x; j < less; j += kT) {
    out_key[base + j] = sk[j];
    out_idx[base + j] = si[j];
  }
}

// Range rows: number of points with distance <= radius (the row's own point
// left out when exclude is set).
__global__ void __launch_bounds__(kT) range_count64_kernel(const double* __restrict__ D, int64_t n, int64_t q0,
                                                           int exclude, double radius, int64_t* __restrict__ cnt) {
  __shared__ unsigned long long s_cnt;
  if (threadIdx.x == 0) s_cnt = 0ull;
  __syncthreads();
  const int64_t b = blockIdx.x;
  const double* row = D + b * n;
  const int64_t r = q0 + b;
  unsigned long long c = 0;
  for (int64_t i = threadIdx.x; i < n; i += kT)
    if (row[i] <= radius && !(exclude && i == r)) c++;
  if (c) atomicAdd(&s_cnt, c);
  __syncthreads();
  if (threadIdx.x == 0) cnt[b] = (int64_t)s_cnt;
}

// Range rows into CSR at off[b], in index order (sorted stably by key after).
__global__ void __launch_bounds__(kT) range_gather64_kernel(const double* __restrict__ D, int64_t n, int64_t q0,
                                                            int exclude, double radius,
                                                            const int64_t* __restrict__ off,
                                                            uint64_t* __restrict__ out_key,
                                                            int64_t* __restrict__ out_idx) {
  __shared__ unsigned wa[kT / 32], we[kT / 32];
  const int64_t b = blockIdx.x;
  const double* row = D + b * n;
  const int64_t r = q0 + b;
  const int64_t base = off[b];
  int64_t pos = 0;
  for (int64_t c = 0; c < n; c += kT) {
    const int64_t i = c + threadIdx.x;
    const double v = i < n ? row[i] : 0.0;
    const bool in = i < n && v <= radius && !(exclude && i == r);
    unsigned p, pz, t, tz;
    block_compact2(in, false, wa, we, &p, &pz, &t, &tz);
    if (in) {
      out_key[base + pos + p] = key64(v);
      out_idx[base + pos + p] = i;
    }
    pos += t;
  }
}

template <int ORDER>
__global__ void __launch_bounds__(kT) pairwise64_kernel(const double* __restrict__ X, int64_t n, int d, int euclid,
                                                        int square, int64_t r0, double* __restrict__ out) {
  const int64_t i = r0 + blockIdx.y;
  const int64_t j = (int64_t)blockIdx.x * kT + threadIdx.x;
  if (i >= n || j >= n || (!square && j >= i)) return;
  double v = sqdist64<ORDER>(X + i * d, X + j * d, d);
  if (euclid) v = __dsqrt_rn(v);
  if (square) out[i * n + j] = v;
  else out[i * (i - 1) / 2 + j] = v;
}

__global__ void pad64_kernel(int64_t* __restrict__ idx, double* __restrict__ dist, int64_t count) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) {
    idx[t] = -1;
    dist[t] = __longlong_as_double(0x7ff0000000000000ll);
  }
}

int pow2_at_least(int64_t v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

// Query rows per batch: the batch's distance matrix within kBatchBytes, and
// at most 65535 rows (the grid's y extent).
int64_t batch_rows(int64_t n, int64_t m) {
  int64_t B = (int64_t)(kBatchBytes / (sizeof(double) * (size_t)std::max<int64_t>(n, 1)));
  B = std::max<int64_t>(1, std::min<int64_t>(B, m));
  return std::min<int64_t>(B, 65535);
}

int launch_dist(const F64Scan& x, const double* Q, int64_t B, double* D, cudaStream_t s) {
  const dim3 grid((unsigned)((x.n + kT - 1) / kT), (unsigned)B);
  const int euclid = x.metric == FUELG_METRIC_EUCLIDEAN ? 1 : 0;
  if (x.order == FUELG_ORDER_X86)
    dist64_kernel<FUELG_ORDER_X86><<<grid, kT, 0, s>>>(x.X, x.n, x.d, Q, euclid, D);
  else
    dist64_kernel<FUELG_ORDER_ARM><<<grid, kT, 0, s>>>(x.X, x.n, x.d, Q, euclid, D);
  note_launch();
  FUELG_CUDA(cudaGetLastError());
  return ST_OK;
}

int allow_sort_smem() {
  const int bytes = kMaxSortKeys * (int)(sizeof(uint64_t) + sizeof(uint32_t));
  FUELG_CUDA(cudaFuncSetAttribute(knn64_finish_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  FUELG_CUDA(cudaFuncSetAttribute(ties64_gather_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  return ST_OK;
}

}  // namespace

int f64_knn(const F64Scan& x, const double* Q, int64_t m, int k, int mode, int64_t* out_idx, double* out_dist,
            cudaStream_t s) {
  if (m == 0 || k == 0) return ST_OK;
  const int64_t kq = mode == FUELG_EXCLUDE_NONE ? k : (int64_t)k + 1;
  const int64_t kk = std::min<int64_t>(kq, x.n);
  if (kk == 0) {
    const int64_t cnt = m * k;
    pad64_kernel<<<(unsigned)((cnt + kT - 1) / kT), kT, 0, s>>>(out_idx, out_dist, cnt);
    note_launch();
    FUELG_CUDA(cudaGetLastError());
    return ST_OK;
  }
  FUELG_TRY(allow_sort_smem());
  const int64_t B = batch_rows(x.n, m);
  const int P = pow2_at_least(kk);
  const size_t smem = (size_t)P * (sizeof(uint64_t) + sizeof(uint32_t));
  Scratch D, thr, nl, ne;
  FUELG_TRY(D.alloc(sizeof(double) * (size_t)B * x.n, s));
  FUELG_TRY(thr.alloc(sizeof(uint64_t) * B, s));
  FUELG_TRY(nl.alloc(sizeof(int64_t) * B, s));
  FUELG_TRY(ne.alloc(sizeof(int64_t) * B, s));
  for (int64_t q0 = 0; q0 < m; q0 += B) {
    if (cancel_requested()) {
      set_error("cancelled");
      return ST_ECANCELLED;
    }
    const int64_t Bb = std::min<int64_t>(B, m - q0);
    FUELG_TRY(launch_dist(x, Q + q0 * x.d, Bb, D.as<double>(), s));
    select64_kernel<<<(unsigned)Bb, kT, 0, s>>>(D.as<double>(), x.n, kk, thr.as<uint64_t>(), nl.as<int64_t>(),
                                                ne.as<int64_t>());
    note_launch();
    knn64_finish_kernel<<<(unsigned)Bb, kT, smem, s>>>(D.as<double>(), x.n, (int)kk, k, mode, q0,
                                                       thr.as<uint64_t>(), nl.as<int64_t>(), P,
                                                       out_idx + q0 * k, out_dist + q0 * k);
    note_launch();
    FUELG_CUDA(cudaGetLastError());
  }
  return ST_OK;
}

int f64_lists(const F64Scan& x, const double* Q, int64_t m, bool range, int64_t kq, bool drop_self, double radius,
              std::vector<int64_t>* off, std::vector<int64_t>* idx, std::vector<double>* dist, int64_t* d2h,
              cudaStream_t s) {
  off->assign((size_t)m + 1, 0);
  idx->clear();
  dist->clear();
  if (m == 0 || x.n == 0 || (!range && kq == 0)) return ST_OK;
  const int64_t kk = std::min<int64_t>(kq, x.n);
  const int P = range ? 1 : pow2_at_least(kk);
  const size_t smem = (size_t)P * (sizeof(uint64_t) + sizeof(uint32_t));
  if (!range) FUELG_TRY(allow_sort_smem());
  const int64_t B = batch_rows(x.n, m);
  Scratch D, thr, nl, ne, cnt, boff;
  FUELG_TRY(D.alloc(sizeof(double) * (size_t)B * x.n, s));
  FUELG_TRY(thr.alloc(sizeof(uint64_t) * B, s));
  FUELG_TRY(nl.alloc(sizeof(int64_t) * B, s));
  FUELG_TRY(ne.alloc(sizeof(int64_t) * B, s));
  FUELG_TRY(cnt.alloc(sizeof(int64_t) * B, s));
  FUELG_TRY(boff.alloc(sizeof(int64_t) * (B + 1), s));
  std::vector<int64_t> hc((size_t)B), ho((size_t)B + 1);
  std::vector<uint64_t> hk;
  for (int64_t q0 = 0; q0 < m; q0 += B) {
    if (cancel_requested()) {
      set_error("cancelled");
      return ST_ECANCELLED;
    }
    const int64_t Bb = std::min<int64_t>(B, m - q0);
    FUELG_TRY(launch_dist(x, Q + q0 * x.d, Bb, D.as<double>(), s));
    if (range) {
      range_count64_kernel<<<(unsigned)Bb, kT, 0, s>>>(D.as<double>(), x.n, q0, drop_self ? 1 : 0, radius,
                                                       cnt.as<int64_t>());
      note_launch();
    } else {
      select64_kernel<<<(unsigned)Bb, kT, 0, s>>>(D.as<double>(), x.n, kk, thr.as<uint64_t>(), nl.as<int64_t>(),
                                                  ne.as<int64_t>());
      note_launch();
      ties_count64_kernel<<<(unsigned)((Bb + kT - 1) / kT), kT, 0, s>>>(
          D.as<double>(), x.n, (int)Bb, q0, drop_self ? 1 : 0, thr.as<uint64_t>(), nl.as<int64_t>(),
          ne.as<int64_t>(), cnt.as<int64_t>());
      note_launch();
    }
    FUELG_CUDA(cudaGetLastError());
    FUELG_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, sizeof(int64_t) * Bb, cudaMemcpyDeviceToHost, s));
    FUELG_CUDA(cudaStreamSynchronize(s));
    *d2h += (int64_t)sizeof(int64_t) * Bb;
    ho[0] = 0;
    for (int64_t b = 0; b < Bb; b++) ho[b + 1] = ho[b] + hc[b];
    const int64_t tot = ho[Bb];
    const int64_t base = (*off)[q0];
    for (int64_t b = 0; b < Bb; b++) (*off)[q0 + b + 1] = base + ho[b + 1];
    if (tot == 0) continue;
    FUELG_CUDA(cudaMemcpyAsync(boff.p, ho.data(), sizeof(int64_t) * (Bb + 1), cudaMemcpyHostToDevice, s));
    Scratch ok, oi;
    FUELG_TRY(ok.alloc(sizeof(uint64_t) * tot, s));
    FUELG_TRY(oi.alloc(sizeof(int64_t) * tot, s));
    const uint64_t* keys = ok.as<uint64_t>();
    const int64_t* ids = oi.as<int64_t>();
    Scratch sk, si, tmp;
    if (range) {
      range_gather64_kernel<<<(unsigned)Bb, kT, 0, s>>>(D.as<double>(), x.n, q0, drop_self ? 1 : 0, radius,
                                                        boff.as<int64_t>(), ok.as<uint64_t>(), oi.as<int64_t>());
      note_launch();
      FUELG_CUDA(cudaGetLastError());
      // stable: equal distances keep their index order
      FUELG_TRY(sk.alloc(sizeof(uint64_t) * tot, s));
      FUELG_TRY(si.alloc(sizeof(int64_t) * tot, s));
      size_t tb = 0;
      FUELG_CUDA(cub::DeviceSegmentedSort::StableSortPairs(nullptr, tb, ok.as<uint64_t>(), sk.as<uint64_t>(),
                                                           oi.as<int64_t>(), si.as<int64_t>(), tot, Bb,
                                                           boff.as<int64_t>(), boff.as<int64_t>() + 1, s));
      FUELG_TRY(tmp.alloc(std::max<size_t>(tb, 16), s));
      FUELG_CUDA(cub::DeviceSegmentedSort::StableSortPairs(tmp.p, tb, ok.as<uint64_t>(), sk.as<uint64_t>(),
                                                           oi.as<int64_t>(), si.as<int64_t>(), tot, Bb,
                                                           boff.as<int64_t>(), boff.as<int64_t>() + 1, s));
      keys = sk.as<uint64_t>();
      ids = si.as<int64_t>();
    } else {
      ties64_gather_kernel<<<(unsigned)Bb, kT, smem, s>>>(D.as<double>(), x.n, q0, drop_self ? 1 : 0,
                                                          thr.as<uint64_t>(), nl.as<int64_t>(), ne.as<int64_t>(),
                                                          boff.as<int64_t>(), P, ok.as<uint64_t>(),
                                                          oi.as<int64_t>());
      note_launch();
      FUELG_CUDA(cudaGetLastError());
    }
    const size_t at = idx->size();
    idx->resize(at + (size_t)tot);
    hk.resize((size_t)tot);
    FUELG_CUDA(cudaMemcpyAsync(idx->data() + at, ids, sizeof(int64_t) * tot, cudaMemcpyDeviceToHost, s));
    FUELG_CUDA(cudaMemcpyAsync(hk.data(), keys, sizeof(uint64_t) * tot, cudaMemcpyDeviceToHost, s));
    FUELG_CUDA(cudaStreamSynchronize(s));
    *d2h += (int64_t)(sizeof(int64_t) + sizeof(uint64_t)) * tot;
    dist->resize(at + (size_t)tot);
    memcpy(dist->data() + at, hk.data(), sizeof(double) * (size_t)tot);  // the keys are the distances' bits
  }
  return ST_OK;
}

int f64_pairwise(const double* X, int64_t n, int d, int metric, int order, int form, double* out, cudaStream_t s) {
  const int euclid = metric == FUELG_METRIC_EUCLIDEAN ? 1 : 0;
  const int square = form == FUELG_PAIRWISE_SQUARE ? 1 : 0;
  for (int64_t r0 = 0; r0 < n; r0 += 65535) {
    const dim3 grid((unsigned)((n + kT - 1) / kT), (unsigned)std::min<int64_t>(65535, n - r0));
    if (order == FUELG_ORDER_X86)
      pairwise64_kernel<FUELG_ORDER_X86><<<grid, kT, 0, s>>>(X, n, d, euclid, square, r0, out);
    else
      pairwise64_kernel<FUELG_ORDER_ARM><<<grid, kT, 0, s>>>(X, n, d, euclid, square, r0, out);
    note_launch();
    FUELG_CUDA(cudaGetLastError());
  }
  return ST_OK;
}

}  // namespace fuelg
