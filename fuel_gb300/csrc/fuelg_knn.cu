// fuelg_knn.cu -- exact linear-scan kNN and range search on GB300.
//
// Replaces the per-query heap scan of fuel's linear search
// (src/api/search.rs:154-184, driven by python/search.rs:471-514): every
// (query, point) distance is formed in the reference's own operation order
// (fuelg_common.cuh), keyed as (distance bits, index) so that unsigned order
// equals DistPair order (src/api/search.rs:23-30), and the kk smallest keys
// are kept.  Keeping the kk lexicographically smallest keys is the same set
// KNNHeap returns once knn_results_to_arrays truncates it to k
// (src/api/search.rs:80-151, python/search.rs:1195-1216); the exclude-self
// variants need kk = k+1 (see finalize_knn).
//
// Layout: one thread owns one query row (staged once in shared memory); the
// CTA streams tiles of index rows through shared memory (broadcast reads) and
// every warp of the CTA takes a slice of each tile.  A thread appends a
// candidate to its private shared-memory buffer only when it beats the
// thread's current kk-th key, so the buffer is merged into the thread's
// sorted list (global scratch, L1-resident) only O(kk log(n/kk)) times.
#include <algorithm>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_segmented_sort.cuh>

#include "fuelg_common.cuh"
#include "fuelg_internal.h"

namespace fuelg {

namespace {

constexpr int kThreads = 128;
constexpr int kCB = 16;  // candidate buffer entries per thread, at most (kCbSmallK for small k)
constexpr int kCbSmallK = 8;  // for kk <= 16: a smaller buffer leaves room for more resident CTAs

struct ScanArgs {
  const float* A;
  int64_t m;
  const float* B;
  int64_t n;
  int d;
  int kk;
  int metric;
  int64_t split_len;  // index rows per grid split
  int ws;             // warp splits per CTA (1, 2 or 4)
  int qpb;            // queries per CTA = 32 * 4 / ws
  int pt;             // index rows per shared-memory tile
  int qs, xs;         // row strides (floats) of the query / index tiles
  uint64_t* lists;    // [m][S][2*kk] sorted key lists (kk > 1)
  uint64_t* best;     // [m][S] (kk == 1)
  int a_vec4, b_vec4; // rows may be staged with 16-byte loads (d % 4 == 0 and 16-byte aligned base)
  int* status;
  const volatile int* cancel;
  int kcb;            // candidate buffer entries per thread (<= kCB)
};

__device__ __forceinline__ void stage_rows(float* __restrict__ dst, int dstride, const float* __restrict__ src,
                                           int64_t row0, int rows, int d, bool vec4) {
  if (vec4) {
    const int d4 = d >> 2;
    const float4* s4 = reinterpret_cast<const float4*>(src + row0 * d);
    for (int e = threadIdx.x; e < rows * d4; e += blockDim.x) {
      const int r = e / d4, c = e - r * d4;
      *reinterpret_cast<float4*>(dst + r * dstride + c * 4) = __ldg(s4 + (int64_t)r * d4 + c);
    }
  } else {
    const float* s = src + row0 * d;
    for (int e = threadIdx.x; e < rows * d; e += blockDim.x) {
      const int r = e / d, c = e - r * d;
      dst[r * dstride + c] = __ldg(s + (int64_t)r * d + c);
    }
  }
}

// Merge a thread's unsorted candidate buffer into its sorted kk-list.
__device__ __forceinline__ uint64_t merge_buffer(uint64_t* __restrict__ buf, int cnt, uint64_t* __restrict__ list,
                                                 int& half, int kk) {
  // insertion sort of the (column-major, stride kThreads) buffer
  for (int a = 1; a < cnt; a++) {
    const uint64_t v = buf[a * kThreads];
    int b = a - 1;
    while (b >= 0 && buf[b * kThreads] > v) {
      buf[(b + 1) * kThreads] = buf[b * kThreads];
      b--;
    }
    buf[(b + 1) * kThreads] = v;
  }
  const uint64_t* cur = list + half * kk;
  uint64_t* nxt = list + (half ^ 1) * kk;
  int i = 0, j = 0;
  uint64_t lv = cur[0];
  uint64_t bv = cnt > 0 ? buf[0] : KEY_NONE;
  for (int o = 0; o < kk; o++) {
    if (bv < lv) {
      nxt[o] = bv;
      j++;
      bv = j < cnt ? buf[j * kThreads] : KEY_NONE;
    } else {
      nxt[o] = lv;
      i++;
      lv = i < kk ? cur[i] : KEY_NONE;
    }
  }
  half ^= 1;
  return nxt[kk - 1];
}

// The scan of one CTA: query block qb against index split sy of sgrid.
template <int KIND, int ORDER, int NP, bool KK1>
__device__ __forceinline__ void scan_topk_body(const ScanArgs& a, int64_t qb, int sy, int sgrid) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* qt = reinterpret_cast<float*>(smem_raw);
  float* xt = qt + a.qpb * a.qs;
  uint64_t* buf = reinterpret_cast<uint64_t*>(xt + a.pt * a.xs);
  __shared__ int stop_flag;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int qgroup = warp / a.ws, wsplit = warp % a.ws;
  const int qloc = qgroup * 32 + lane;
  const int64_t q0 = qb * a.qpb;
  const int64_t qi = q0 + qloc;
  const int S = sgrid * a.ws;
  const int s_total = sy * a.ws + wsplit;
  const int64_t p_begin = (int64_t)sy * a.split_len;
  const int64_t p_end = min(a.n, p_begin + a.split_len);
  const bool active = qi < a.m;

  {
    const int qrows = (int)min((int64_t)a.qpb, a.m - q0);
    stage_rows(qt, a.qs, a.A, q0, qrows, a.d, a.a_vec4);
  }
  if (tid == 0) stop_flag = 0;

  uint64_t tau = KEY_NONE;
  uint64_t best = KEY_NONE;
  int cnt = 0, half = 0;
  uint64_t* list = nullptr;
  if (!KK1 && active) {
    list = a.lists + ((uint64_t)qi * S + s_total) * 2ull * a.kk;
    for (int o = 0; o < a.kk; o++) list[o] = KEY_NONE;
  }
  const float* qrow = qt + qloc * a.qs;
  int tile_no = 0;
  for (int64_t t0 = p_begin; t0 < p_end; t0 += a.pt, tile_no++) {
    __syncthreads();
    if (tid == 0 && a.cancel != nullptr && (tile_no & 15) == 15 && *a.cancel) {
      stop_flag = 1;
      atomicOr(a.status, DEV_CANCELLED);
    }
    const int rows = (int)min((int64_t)a.pt, p_end - t0);
    stage_rows(xt, a.xs, a.B, t0, rows, a.d, a.b_vec4);
    __syncthreads();
    if (stop_flag) break;
    if (!active) continue;
    for (int g = wsplit * NP; g < rows; g += a.ws * NP) {
      float dist[NP];
      pair_dists<KIND, ORDER, NP>(qrow, xt + g * a.xs, a.xs, a.d, dist);
#pragma unroll
      for (int p = 0; p < NP; p++) {
        if (g + p < rows) {
          float dv = dist[p];
          if (a.metric == METRIC_EUCLIDEAN) dv = __fsqrt_rn(dv);
          const uint64_t key = make_key(dv, (uint32_t)(t0 + g + p));
          if (KK1) {
            best = key < best ? key : best;
          } else if (key < tau) {
            buf[cnt * kThreads + tid] = key;
            cnt++;
          }
        }
      }
      if (!KK1 && cnt > a.kcb - NP) {
        tau = merge_buffer(buf + tid, cnt, list, half, a.kk);
        cnt = 0;
      }
    }
  }
  if (!active) return;
  if (KK1) {
    a.best[(uint64_t)qi * S + s_total] = best;
  } else {
    if (cnt > 0) tau = merge_buffer(buf + tid, cnt, list, half, a.kk);
    if (half == 1)
      for (int o = 0; o < a.kk; o++) list[o] = list[a.kk + o];
  }
}

template <int KIND, int ORDER, int NP, bool KK1>
__global__ void __launch_bounds__(kThreads) scan_topk_kernel(ScanArgs a) {
  scan_topk_body<KIND, ORDER, NP, KK1>(a, blockIdx.x, blockIdx.y, gridDim.y);
}

// Many independent kNN query sets in one launch: CTA b runs work item b, a
// (set, query block, index split) of its set's own scan arguments -- each set
// with its own data, n, d, k and metric.
struct SetItem {
  int32_t set, sy;
  int64_t qb;
};
template <int ORDER>
__global__ void __launch_bounds__(kThreads) scan_sets_kernel(const ScanArgs* __restrict__ sets,
                                                             const int32_t* __restrict__ sgrid,
                                                             const SetItem* __restrict__ items) {
  const SetItem it = items[blockIdx.x];
  const ScanArgs a = sets[it.set];
  scan_topk_body<KIND_KNN, ORDER, 4, false>(a, it.qb, it.sy, sgrid[it.set]);
}

__device__ __forceinline__ uint64_t warp_min_u64(uint64_t v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const uint64_t o = __shfl_xor_sync(0xffffffffu, v, off);
    v = o < v ? o : v;
  }
  return v;
}

// One warp per query: k-way merge of the S sorted split lists into out[kk].
__global__ void merge_splits_kernel(const uint64_t* __restrict__ lists, int64_t m, int S, int kk,
                                    uint64_t* __restrict__ out) {
  const int64_t qi = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (qi >= m) return;
  const uint64_t* L = lists + ((uint64_t)qi * S + lane) * 2ull * kk;
  int p = 0;
  uint64_t cur = lane < S ? L[0] : KEY_NONE;
  uint64_t* o = out + (uint64_t)qi * kk;
  for (int j = 0; j < kk; j++) {
    const uint64_t mn = warp_min_u64(cur);
    if (lane == 0) o[j] = mn;
    if (mn != KEY_NONE && cur == mn) {
      p++;
      cur = p < kk ? L[p] : KEY_NONE;
    }
  }
}

__global__ void copy_lists_kernel(const uint64_t* __restrict__ lists, int64_t m, int kk, uint64_t* __restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m * kk) return;
  const int64_t qi = e / kk, j = e - qi * kk;
  out[e] = lists[qi * 2 * kk + j];
}

__global__ void min_splits_kernel(const uint64_t* __restrict__ best, int64_t m, int S, uint64_t* __restrict__ out) {
  const int64_t qi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (qi >= m) return;
  uint64_t b = KEY_NONE;
  for (int s = 0; s < S; s++) {
    const uint64_t v = best[qi * S + s];
    b = v < b ? v : b;
  }
  out[qi] = b;
}

// Exclude-self semantics:
//  0 none      first k keys
//  1 linear    python/search.rs:485-488 -- KNNHeap(k) keeps every key tied at
//              the k-th distance; self is then dropped and the row truncated
//              to k.  With the k+1 smallest keys c[0..k]: drop self, and use
//              c[k] only if its distance equals the k-th distance.
//  2 kplus1    python/search.rs:1163-1170 -- search k+1, drop self, take k.
__device__ __forceinline__ void finalize_row(const uint64_t* __restrict__ c, int64_t qi, int kk, int k, int mode,
                                             int64_t* __restrict__ oi, float* __restrict__ od) {
  int w = 0;
  if (mode == 0) {
    for (; w < k && w < kk; w++) {
      const uint64_t key = c[w];
      if (key == KEY_NONE) break;
      oi[w] = key_idx(key);
      od[w] = key_dist(key);
    }
  } else {
    const uint64_t kth = (mode == 1 && k >= 1) ? c[k - 1] : KEY_NONE;
    for (int j = 0; j < kk && w < k; j++) {
      const uint64_t key = c[j];
      if (key == KEY_NONE) break;
      if ((int64_t)key_idx(key) == qi) continue;
      if (mode == 1 && j >= k && !(kth != KEY_NONE && key_dist(key) == key_dist(kth))) break;
      oi[w] = key_idx(key);
      od[w] = key_dist(key);
      w++;
    }
  }
  for (; w < k; w++) {
    oi[w] = -1;
    od[w] = __int_as_float(0x7f800000);
  }
}

__global__ void finalize_kernel(const uint64_t* __restrict__ keys, int64_t m, int kk, int k, int mode,
                                int64_t* __restrict__ out_idx, float* __restrict__ out_dist) {
  const int64_t qi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (qi >= m) return;
  finalize_row(keys + qi * kk, qi, kk, k, mode, out_idx + qi * k, out_dist + qi * k);
}

int vec4_ok(const float* p, int d) { return (d % 4 == 0) && ((reinterpret_cast<uintptr_t>(p) & 15) == 0); }

struct Plan {
  int ws, qpb, pt, qs, xs, np, S_grid;
  int64_t split_len;
  size_t smem;
  int kcb;
};

int make_plan(const ExactScanParams& p, bool kk1, int np, Plan* pl) {
  const int qs = smem_row_stride(p.d);
  const size_t qrow = (size_t)qs * 4;
  int ws;
  if (128 * qrow <= 96 * 1024) ws = 1;
  else if (64 * qrow <= 96 * 1024) ws = 2;
  else if (32 * qrow <= 190 * 1024) ws = 4;
  else {
    set_error("dimension d=%d is too large for the plain FP32 scan (limit ~1500)", p.d);
    return ST_ENOTSUP;
  }
  const int qpb = 32 * 4 / ws;
  const int unit = np * ws;
  int pt = (int)((24 * 1024) / qrow);
  pt = std::max(unit, std::min(128, pt));
  pt = (pt / unit) * unit;
  const int kcb = p.kk <= 16 ? kCbSmallK : kCB;
  size_t smem = (size_t)qpb * qrow + (size_t)pt * qrow + (kk1 ? 0 : (size_t)kThreads * kcb * 8);
  const int64_t qblocks = (p.m + qpb - 1) / qpb;
  int64_t want = (8 * 152 + qblocks - 1) / qblocks;
  int64_t tiles = (p.n + pt - 1) / pt;
  int64_t S_grid = std::max<int64_t>(1, std::min<int64_t>({want, 32 / ws, tiles}));
  int64_t split_len = (p.n + S_grid - 1) / S_grid;
  split_len = ((split_len + pt - 1) / pt) * pt;
  if (split_len == 0) split_len = pt;
  S_grid = std::max<int64_t>(1, (p.n + split_len - 1) / split_len);
  *pl = Plan{ws, qpb, pt, qs, qs, np, (int)S_grid, split_len, smem, kcb};
  return ST_OK;
}

template <int KIND, int ORDER, int NP, bool KK1>
int launch_scan(const ScanArgs& a, const Plan& pl, int64_t qblocks, cudaStream_t stream) {
  auto kern = scan_topk_kernel<KIND, ORDER, NP, KK1>;
  FUELG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem));
  dim3 grid((unsigned)qblocks, (unsigned)pl.S_grid);
  HotTimer* ht = hot_timer();
  if (ht) ht->begin(stream);
  kern<<<grid, kThreads, pl.smem, stream>>>(a); ::fuelg::note_launch();
  if (ht) ht->end(stream);
  FUELG_CUDA(cudaGetLastError());
  return ST_OK;
}

template <int KIND, int ORDER>
int dispatch_np(const ScanArgs& a, const Plan& pl, int64_t qblocks, bool kk1, cudaStream_t s) {
  constexpr int NP = (KIND == KIND_SQDIST && ORDER == ORDER_X86) ? 2 : 4;
  return kk1 ? launch_scan<KIND, ORDER, NP, true>(a, pl, qblocks, s) : launch_scan<KIND, ORDER, NP, false>(a, pl, qblocks, s);
}

int scan_np(int kind, int order) { return (kind == KIND_SQDIST && order == ORDER_X86) ? 2 : 4; }

}  // namespace

int exact_topk(const ExactScanParams& p, uint64_t* out_keys, int* dev_status, cudaStream_t stream) {
  if (p.m == 0 || p.kk == 0) return ST_OK;
  if (p.n == 0) {
    FUELG_CUDA(cudaMemsetAsync(out_keys, 0xff, (size_t)p.m * p.kk * 8, stream));
    return ST_OK;
  }
  if (p.n >= 0xffffffffll) {
    set_error("index too large: n=%lld (limit 2^32-2)", (long long)p.n);
    return ST_ENOTSUP;
  }
  const bool kk1 = p.kk == 1;
  Plan pl;
  FUELG_TRY(make_plan(p, kk1, scan_np(p.kind, p.order), &pl));
  const int S = pl.S_grid * pl.ws;
  // Bound scratch: process queries in batches of at most ~1 GiB of lists.
  const size_t per_query = kk1 ? (size_t)S * 8 : (size_t)S * 2 * p.kk * 8;
  int64_t mb = std::max<int64_t>(pl.qpb, (int64_t)((1ull << 30) / per_query));
  mb = std::min<int64_t>(mb, p.m);
  Scratch lists;
  FUELG_TRY(lists.alloc(per_query * mb, stream));
  for (int64_t b0 = 0; b0 < p.m; b0 += mb) {
    const int64_t mcur = std::min<int64_t>(mb, p.m - b0);
    ScanArgs a{};
    a.A = p.A + b0 * p.d;
    a.m = mcur;
    a.B = p.B;
    a.n = p.n;
    a.d = p.d;
    a.kk = p.kk;
    a.metric = p.metric;
    a.split_len = pl.split_len;
    a.ws = pl.ws;
    a.qpb = pl.qpb;
    a.pt = pl.pt;
    a.kcb = pl.kcb;
    a.qs = pl.qs;
    a.xs = pl.xs;
    a.lists = kk1 ? nullptr : lists.as<uint64_t>();
    a.best = kk1 ? lists.as<uint64_t>() : nullptr;
    a.status = dev_status;
    a.cancel = cancel_word_device();
    a.a_vec4 = vec4_ok(a.A, a.d);
    a.b_vec4 = vec4_ok(a.B, a.d);
    const int64_t qblocks = (mcur + pl.qpb - 1) / pl.qpb;
    int st;
    if (p.kind == KIND_KNN)
      st = p.order == ORDER_X86 ? dispatch_np<KIND_KNN, ORDER_X86>(a, pl, qblocks, kk1, stream)
                                : dispatch_np<KIND_KNN, ORDER_ARM>(a, pl, qblocks, kk1, stream);
    else if (p.kind == KIND_SQDIST)
      st = p.order == ORDER_X86 ? dispatch_np<KIND_SQDIST, ORDER_X86>(a, pl, qblocks, kk1, stream)
                                : dispatch_np<KIND_SQDIST, ORDER_ARM>(a, pl, qblocks, kk1, stream);
    else
      st = p.order == ORDER_X86 ? dispatch_np<KIND_PAIRWISE, ORDER_X86>(a, pl, qblocks, kk1, stream)
                                : dispatch_np<KIND_PAIRWISE, ORDER_ARM>(a, pl, qblocks, kk1, stream);
    if (st != ST_OK) return st;
    uint64_t* ok = out_keys + b0 * p.kk;
    if (kk1) {
      min_splits_kernel<<<(unsigned)((mcur + 255) / 256), 256, 0, stream>>>(lists.as<uint64_t>(), mcur, S, ok); ::fuelg::note_launch();
    } else if (S == 1) {
      const int64_t tot = mcur * p.kk;
      copy_lists_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, stream>>>(lists.as<uint64_t>(), mcur, p.kk, ok); ::fuelg::note_launch();
    } else {
      merge_splits_kernel<<<(unsigned)((mcur * 32 + 255) / 256), 256, 0, stream>>>(lists.as<uint64_t>(), mcur, S,
                                                                                  p.kk, ok); ::fuelg::note_launch();
    }
    FUELG_CUDA(cudaGetLastError());
  }
  return ST_OK;
}

namespace {

// Set of global query q: the last set whose first query is <= q.
__device__ __forceinline__ int set_of(const int64_t* __restrict__ qbegin, int count, int64_t q) {
  int lo = 0, hi = count;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (qbegin[mid] <= q) lo = mid;
    else hi = mid;
  }
  return lo;
}

// One warp per query of every set: k-way merge of its set's S sorted split
// lists (S <= 32), then the set's exclude rule and padding into its outputs.
__global__ void merge_sets_kernel(const ScanArgs* __restrict__ sets, const int32_t* __restrict__ nsplit,
                                  const int64_t* __restrict__ qbegin, int count, const KnnSetOut* __restrict__ outs,
                                  uint64_t* __restrict__ keys, const int64_t* __restrict__ koff) {
  const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (q >= qbegin[count]) return;
  const int st = set_of(qbegin, count, q);
  const int64_t qi = q - qbegin[st];
  const int S = nsplit[st];
  const int kk = sets[st].kk;
  const uint64_t* L = sets[st].lists + ((uint64_t)qi * S + lane) * 2ull * kk;
  uint64_t* o = keys + koff[st] + qi * kk;
  int p = 0;
  uint64_t cur = lane < S ? L[0] : KEY_NONE;
  for (int j = 0; j < kk; j++) {
    const uint64_t mn = warp_min_u64(cur);
    if (lane == 0) o[j] = mn;
    if (mn != KEY_NONE && cur == mn) {
      p++;
      cur = p < kk ? L[p] : KEY_NONE;
    }
  }
  __syncwarp();
  if (lane == 0) {
    const KnnSetOut& so = outs[st];
    finalize_row(o, qi, kk, so.k, so.mode, so.out_idx + qi * so.k, so.out_dist + qi * so.k);
  }
}

}  // namespace

int exact_knn_sets(const KnnSetDev* sets, int count, int order, int* dev_status, cudaStream_t stream) {
  std::vector<ScanArgs> args;
  std::vector<int32_t> nsplit, sgrid;
  std::vector<int64_t> qbegin(1, 0), koff;
  std::vector<KnnSetOut> outs;
  std::vector<SetItem> items;
  size_t smem = 0, list_words = 0, key_words = 0;
  std::vector<size_t> list_off;
  for (int i = 0; i < count; i++) {
    const KnnSetDev& t = sets[i];
    if (t.m == 0 || t.k == 0) continue;
    ExactScanParams p;
    p.A = t.A;
    p.m = t.m;
    p.B = t.B;
    p.n = t.n;
    p.d = t.d;
    p.kind = KIND_KNN;
    p.order = order;
    p.metric = t.metric;
    p.kk = t.mode == 0 ? t.k : t.k + 1;
    if (t.n == 0) {  // no points: every row padded
      Scratch none;
      FUELG_TRY(none.alloc((size_t)t.m * p.kk * 8, stream));
      FUELG_CUDA(cudaMemsetAsync(none.p, 0xff, (size_t)t.m * p.kk * 8, stream));
      FUELG_TRY(finalize_knn(none.as<uint64_t>(), t.m, p.kk, t.k, t.mode, t.out_idx, t.out_dist, stream));
      FUELG_CUDA(cudaStreamSynchronize(stream));
      continue;
    }
    if (t.n >= 0xffffffffll) {
      set_error("set %d: index too large: n=%lld (limit 2^32-2)", i, (long long)t.n);
      return ST_ENOTSUP;
    }
    Plan pl;
    FUELG_TRY(make_plan(p, false, 4, &pl));
    ScanArgs a{};
    a.A = t.A;
    a.m = t.m;
    a.B = t.B;
    a.n = t.n;
    a.d = t.d;
    a.kk = p.kk;
    a.metric = t.metric;
    a.split_len = pl.split_len;
    a.ws = pl.ws;
    a.qpb = pl.qpb;
    a.pt = pl.pt;
    a.kcb = pl.kcb;
    a.qs = pl.qs;
    a.xs = pl.xs;
    a.status = dev_status;
    a.cancel = cancel_word_device();
    a.a_vec4 = vec4_ok(a.A, a.d);
    a.b_vec4 = vec4_ok(a.B, a.d);
    const int S = pl.S_grid * pl.ws;
    list_off.push_back(list_words);
    list_words += (size_t)t.m * S * 2 * p.kk;
    koff.push_back((int64_t)key_words);
    key_words += (size_t)t.m * p.kk;
    const int si = (int)args.size();
    const int64_t qblocks = (t.m + pl.qpb - 1) / pl.qpb;
    for (int64_t qb = 0; qb < qblocks; qb++)
      for (int sy = 0; sy < pl.S_grid; sy++) items.push_back(SetItem{si, sy, qb});
    args.push_back(a);
    nsplit.push_back(S);
    sgrid.push_back(pl.S_grid);
    qbegin.push_back(qbegin.back() + t.m);
    outs.push_back(KnnSetOut{t.out_idx, t.out_dist, t.k, t.mode});
    smem = std::max(smem, pl.smem);
  }
  const int ns = (int)args.size();
  if (ns == 0) return ST_OK;
  if (items.size() >= (1u << 31) || list_words * 8 > (size_t(6) << 30)) {
    set_error("batched kNN: the sets' split lists need %zu bytes (limit 6 GiB); submit fewer or smaller sets",
              list_words * 8);
    return ST_ENOTSUP;
  }
  Scratch dlists, dkeys, dargs, dsplit, dsgrid, dqb, dko, douts, ditems;
  FUELG_TRY(dlists.alloc(list_words * 8, stream));
  FUELG_TRY(dkeys.alloc(key_words * 8, stream));
  for (int i = 0; i < ns; i++) args[i].lists = dlists.as<uint64_t>() + list_off[i];
  FUELG_TRY(dargs.alloc(sizeof(ScanArgs) * ns, stream));
  FUELG_TRY(dsplit.alloc(sizeof(int32_t) * ns, stream));
  FUELG_TRY(dsgrid.alloc(sizeof(int32_t) * ns, stream));
  FUELG_TRY(dqb.alloc(sizeof(int64_t) * (ns + 1), stream));
  FUELG_TRY(dko.alloc(sizeof(int64_t) * ns, stream));
  FUELG_TRY(douts.alloc(sizeof(KnnSetOut) * ns, stream));
  FUELG_TRY(ditems.alloc(sizeof(SetItem) * items.size(), stream));
  FUELG_CUDA(cudaMemcpyAsync(dargs.p, args.data(), sizeof(ScanArgs) * ns, cudaMemcpyHostToDevice, stream));
  FUELG_CUDA(cudaMemcpyAsync(dsplit.p, nsplit.data(), sizeof(int32_t) * ns, cudaMemcpyHostToDevice, stream));
  FUELG_CUDA(cudaMemcpyAsync(dsgrid.p, sgrid.data(), sizeof(int32_t) * ns, cudaMemcpyHostToDevice, stream));
  FUELG_CUDA(cudaMemcpyAsync(dqb.p, qbegin.data(), sizeof(int64_t) * (ns + 1), cudaMemcpyHostToDevice, stream));
  FUELG_CUDA(cudaMemcpyAsync(dko.p, koff.data(), sizeof(int64_t) * ns, cudaMemcpyHostToDevice, stream));
  FUELG_CUDA(cudaMemcpyAsync(douts.p, outs.data(), sizeof(KnnSetOut) * ns, cudaMemcpyHostToDevice, stream));
  FUELG_CUDA(cudaMemcpyAsync(ditems.p, items.data(), sizeof(SetItem) * items.size(), cudaMemcpyHostToDevice, stream));
  auto kern = order == ORDER_X86 ? scan_sets_kernel<ORDER_X86> : scan_sets_kernel<ORDER_ARM>;
  FUELG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  HotTimer* ht = hot_timer();
  if (ht) ht->begin(stream);
  kern<<<(unsigned)items.size(), kThreads, smem, stream>>>(dargs.as<ScanArgs>(), dsgrid.as<int32_t>(),
                                                           ditems.as<SetItem>());
  note_launch();
  if (ht) ht->end(stream);
  FUELG_CUDA(cudaGetLastError());
  const int64_t qtot = qbegin.back();
  merge_sets_kernel<<<(unsigned)((qtot * 32 + 255) / 256), 256, 0, stream>>>(
      dargs.as<ScanArgs>(), dsplit.as<int32_t>(), dqb.as<int64_t>(), ns, douts.as<KnnSetOut>(), dkeys.as<uint64_t>(),
      dko.as<int64_t>());
  note_launch();
  FUELG_CUDA(cudaGetLastError());
  FUELG_CUDA(cudaStreamSynchronize(stream));  // the tables above are freed on return
  return ST_OK;
}

int finalize_knn(const uint64_t* keys, int64_t m, int kk, int k, int exclude_mode, int64_t* out_idx, float* out_dist,
                 cudaStream_t stream) {
  if (m == 0 || k == 0) return ST_OK;
  finalize_kernel<<<(unsigned)((m + 127) / 128), 128, 0, stream>>>(keys, m, kk, k, exclude_mode, out_idx, out_dist); ::fuelg::note_launch();
  FUELG_CUDA(cudaGetLastError());
  return ST_OK;
}

// ---------------------------------------------------------------------------
// The same scan + merge + finalize, driven entirely from a caller-provided
// scratch region (no allocation, no cancel word).  Queries are processed in
// batches sized to the region.  Used by the allocation-free C entry point.
// ---------------------------------------------------------------------------
namespace {

__global__ void finalize_offset_kernel(const uint64_t* __restrict__ keys, int64_t m, int64_t q0, int kk, int k,
                                       int mode, int64_t* __restrict__ out_idx, float* __restrict__ out_dist) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  const int64_t qi = q0 + r;  // query index in the whole call (exclude-self compares against it)
  const uint64_t* c = keys + r * kk;
  int64_t* oi = out_idx + qi * k;
  float* od = out_dist + qi * k;
  int w = 0;
  if (mode == 0) {
    for (; w < k && w < kk; w++) {
      const uint64_t key = c[w];
      if (key == KEY_NONE) break;
      oi[w] = key_idx(key);
      od[w] = key_dist(key);
    }
  } else {
    const uint64_t kth = (mode == 1 && k >= 1) ? c[k - 1] : KEY_NONE;
    for (int j = 0; j < kk && w < k; j++) {
      const uint64_t key = c[j];
      if (key == KEY_NONE) break;
      if ((int64_t)key_idx(key) == qi) continue;
      if (mode == 1 && j >= k && !(kth != KEY_NONE && key_dist(key) == key_dist(kth))) break;
      oi[w] = key_idx(key);
      od[w] = key_dist(key);
      w++;
    }
  }
  for (; w < k; w++) {
    oi[w] = -1;
    od[w] = __int_as_float(0x7f800000);
  }
}

}  // namespace

int exact_knn_in_scratch(const ExactScanParams& p, int k, int exclude_mode, int64_t* out_idx, float* out_dist,
                         void* scratch, size_t scratch_bytes, cudaStream_t stream) {
  if (p.m == 0 || k == 0) return ST_OK;
  const size_t head = 256;  // device status word
  if (scratch_bytes <= head) {
    set_error("scratch region too small");
    return ST_ENOTSUP;
  }
  int* dev_status = static_cast<int*>(scratch);
  uint8_t* base = static_cast<uint8_t*>(scratch) + head;
  const size_t avail = scratch_bytes - head;
  FUELG_CUDA(cudaMemsetAsync(dev_status, 0, sizeof(int), stream));
  if (p.n == 0) {
    const int64_t qb = std::max<int64_t>(1, (int64_t)(avail / ((size_t)p.kk * 8)));
    for (int64_t b0 = 0; b0 < p.m; b0 += qb) {
      const int64_t mcur = std::min<int64_t>(qb, p.m - b0);
      FUELG_CUDA(cudaMemsetAsync(base, 0xff, (size_t)mcur * p.kk * 8, stream));
      finalize_offset_kernel<<<(unsigned)((mcur + 127) / 128), 128, 0, stream>>>(
          reinterpret_cast<uint64_t*>(base), mcur, b0, p.kk, k, exclude_mode, out_idx, out_dist); ::fuelg::note_launch();
    }
    FUELG_CUDA(cudaGetLastError());
    return ST_OK;
  }
  if (p.n >= 0xffffffffll) {
    set_error("index too large: n=%lld (limit 2^32-2)", (long long)p.n);
    return ST_ENOTSUP;
  }
  const bool kk1 = p.kk == 1;
  Plan pl;
  FUELG_TRY(make_plan(p, kk1, scan_np(p.kind, p.order), &pl));
  // per query: split lists (or best keys) + the merged keys
  auto per_query = [&](int S) { return (kk1 ? (size_t)S * 8 : (size_t)S * 2 * p.kk * 8) + (size_t)p.kk * 8; };
  while (pl.S_grid > 1 && per_query(pl.S_grid * pl.ws) * pl.qpb > avail) {
    pl.S_grid = std::max(1, pl.S_grid / 2);
    int64_t split_len = (p.n + pl.S_grid - 1) / pl.S_grid;
    split_len = ((split_len + pl.pt - 1) / pl.pt) * pl.pt;
    pl.split_len = split_len;
    pl.S_grid = (int)std::max<int64_t>(1, (p.n + split_len - 1) / split_len);
  }
  const int S = pl.S_grid * pl.ws;
  const size_t pq = per_query(S);
  if (pq * pl.qpb > avail) {
    set_error("k=%d needs %zu bytes of scratch per %d queries; the static region holds %zu", k, pq * pl.qpb,
              pl.qpb, avail);
    return ST_ENOTSUP;
  }
  int64_t mb = (int64_t)(avail / pq);
  mb = std::max<int64_t>(pl.qpb, (mb / pl.qpb) * pl.qpb);
  mb = std::min<int64_t>(mb, p.m);
  uint64_t* lists = reinterpret_cast<uint64_t*>(base);
  uint64_t* keys = lists + (pq / 8 - p.kk) * (size_t)mb;
  for (int64_t b0 = 0; b0 < p.m; b0 += mb) {
    const int64_t mcur = std::min<int64_t>(mb, p.m - b0);
    ScanArgs a{};
    a.A = p.A + b0 * p.d;
    a.m = mcur;
    a.B = p.B;
    a.n = p.n;
    a.d = p.d;
    a.kk = p.kk;
    a.metric = p.metric;
    a.split_len = pl.split_len;
    a.ws = pl.ws;
    a.qpb = pl.qpb;
    a.pt = pl.pt;
    a.kcb = pl.kcb;
    a.qs = pl.qs;
    a.xs = pl.xs;
    a.lists = kk1 ? nullptr : lists;
    a.best = kk1 ? lists : nullptr;
    a.status = dev_status;
    a.cancel = nullptr;
    a.a_vec4 = vec4_ok(a.A, a.d);
    a.b_vec4 = vec4_ok(a.B, a.d);
    const int64_t qblocks = (mcur + pl.qpb - 1) / pl.qpb;
    int st;
    if (p.order == ORDER_X86) st = dispatch_np<KIND_KNN, ORDER_X86>(a, pl, qblocks, kk1, stream);
    else st = dispatch_np<KIND_KNN, ORDER_ARM>(a, pl, qblocks, kk1, stream);
    if (st != ST_OK) return st;
    if (kk1) {
      min_splits_kernel<<<(unsigned)((mcur + 255) / 256), 256, 0, stream>>>(lists, mcur, S, keys); ::fuelg::note_launch();
    } else if (S == 1) {
      const int64_t tot = mcur * p.kk;
      copy_lists_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, stream>>>(lists, mcur, p.kk, keys); ::fuelg::note_launch();
    } else {
      merge_splits_kernel<<<(unsigned)((mcur * 32 + 255) / 256), 256, 0, stream>>>(lists, mcur, S, p.kk, keys); ::fuelg::note_launch();
    }
    finalize_offset_kernel<<<(unsigned)((mcur + 127) / 128), 128, 0, stream>>>(keys, mcur, b0, p.kk, k, exclude_mode,
                                                                             out_idx, out_dist); ::fuelg::note_launch();
    FUELG_CUDA(cudaGetLastError());
  }
  return ST_OK;
}

// ---------------------------------------------------------------------------
// Range search (linear_scan_range, src/api/search.rs:154-166): two passes of
// the same scan -- count, then fill at scanned offsets -- then a segmented
// sort of the (distance, index) keys of every query.
// ---------------------------------------------------------------------------
namespace {

template <int KIND, int ORDER, bool FILL>
__global__ void __launch_bounds__(kThreads) range_kernel(ScanArgs a, float radius, const float* __restrict__ radii,
                                                         int exclude_self, int64_t* __restrict__ counts,
                                                         const int64_t* __restrict__ offs, uint64_t* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* qt = reinterpret_cast<float*>(smem_raw);
  float* xt = qt + a.qpb * a.qs;
  constexpr int NP = (KIND == KIND_SQDIST && ORDER == ORDER_X86) ? 2 : 4;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int qgroup = warp / a.ws, wsplit = warp % a.ws;
  const int qloc = qgroup * 32 + lane;
  const int64_t q0 = (int64_t)blockIdx.x * a.qpb;
  const int64_t qi = q0 + qloc;
  const int S = gridDim.y * a.ws;
  const int s_total = blockIdx.y * a.ws + wsplit;
  const int64_t p_begin = (int64_t)blockIdx.y * a.split_len;
  const int64_t p_end = min(a.n, p_begin + a.split_len);
  const bool active = qi < a.m;
  stage_rows(qt, a.qs, a.A, q0, (int)min((int64_t)a.qpb, a.m - q0), a.d, a.a_vec4);
  int64_t c = 0;
  int64_t pos = (FILL && active) ? offs[qi * S + s_total] : 0;
  if (radii && active) radius = radii[qi];  // per-row radius (tie-inclusive kNN rows)
  const float* qrow = qt + qloc * a.qs;
  for (int64_t t0 = p_begin; t0 < p_end; t0 += a.pt) {
    __syncthreads();
    const int rows = (int)min((int64_t)a.pt, p_end - t0);
    stage_rows(xt, a.xs, a.B, t0, rows, a.d, a.b_vec4);
    __syncthreads();
    if (!active) continue;
    for (int g = wsplit * NP; g < rows; g += a.ws * NP) {
      float dist[NP];
      pair_dists<KIND, ORDER, NP>(qrow, xt + g * a.xs, a.xs, a.d, dist);
#pragma unroll
      for (int p = 0; p < NP; p++) {
        if (g + p < rows) {
          float dv = dist[p];
          if (a.metric == METRIC_EUCLIDEAN) dv = __fsqrt_rn(dv);
          const int64_t idx = t0 + g + p;
          if (dv <= radius && !(exclude_self && idx == qi)) {
            if (FILL) out[pos++] = make_key(dv, (uint32_t)idx);
            else c++;
          }
        }
      }
    }
  }
  if (!FILL && active) counts[qi * S + s_total] = c;
}

__global__ void csr_offsets_kernel(const int64_t* __restrict__ scanned, int64_t m, int S, int64_t* __restrict__ off) {
  const int64_t qi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (qi > m) return;
  off[qi] = scanned[qi * S];  // scanned has m*S+1 entries (exclusive scan + total)
}

__global__ void split_keys_kernel(const uint64_t* __restrict__ keys, int64_t total, int64_t* __restrict__ idx,
                                  float* __restrict__ dist) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= total) return;
  idx[e] = key_idx(keys[e]);
  dist[e] = key_dist(keys[e]);
}

template <int KIND, int ORDER>
int launch_range(const ScanArgs& a, const Plan& pl, int64_t qblocks, float radius, const float* radii, int ex,
                 int64_t* counts, const int64_t* offs, uint64_t* out, bool fill, cudaStream_t s) {
  dim3 grid((unsigned)qblocks, (unsigned)pl.S_grid);
  if (fill) {
    auto kern = range_kernel<KIND, ORDER, true>;
    FUELG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem));
    kern<<<grid, kThreads, pl.smem, s>>>(a, radius, radii, ex, counts, offs, out); ::fuelg::note_launch();
  } else {
    auto kern = range_kernel<KIND, ORDER, false>;
    FUELG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem));
    kern<<<grid, kThreads, pl.smem, s>>>(a, radius, radii, ex, counts, offs, out); ::fuelg::note_launch();
  }
  FUELG_CUDA(cudaGetLastError());
  return ST_OK;
}

}  // namespace

int exact_range(const ExactScanParams& p, float radius, int exclude_self, int64_t** d_off, int64_t** d_idx,
                float** d_dist, int64_t* total, int* dev_status, cudaStream_t stream, const float* radii) {
  (void)dev_status;
  *d_off = nullptr;
  *d_idx = nullptr;
  *d_dist = nullptr;
  *total = 0;
  FUELG_CUDA(cudaMalloc(d_off, sizeof(int64_t) * (p.m + 1)));
  if (p.m == 0 || p.n == 0) {
    FUELG_CUDA(cudaMemsetAsync(*d_off, 0, sizeof(int64_t) * (p.m + 1), stream));
    return ST_OK;
  }
  Plan pl;
  FUELG_TRY(make_plan(p, true, scan_np(p.kind, p.order), &pl));
  const int S = pl.S_grid * pl.ws;
  const int64_t mS = p.m * S;
  Scratch counts, scanned, tmp, keys, keys_sorted;
  FUELG_TRY(counts.alloc(sizeof(int64_t) * (mS + 1), stream));
  FUELG_TRY(scanned.alloc(sizeof(int64_t) * (mS + 1), stream));
  FUELG_CUDA(cudaMemsetAsync(counts.p, 0, sizeof(int64_t) * (mS + 1), stream));
  ScanArgs a{};
  a.A = p.A;
  a.m = p.m;
  a.B = p.B;
  a.n = p.n;
  a.d = p.d;
  a.kk = 0;
  a.metric = p.metric;
  a.split_len = pl.split_len;
  a.ws = pl.ws;
  a.qpb = pl.qpb;
  a.pt = pl.pt;
  a.kcb = pl.kcb;
  a.qs = pl.qs;
  a.xs = pl.xs;
  a.a_vec4 = vec4_ok(a.A, a.d);
  a.b_vec4 = vec4_ok(a.B, a.d);
  const int64_t qblocks = (p.m + pl.qpb - 1) / pl.qpb;
  auto run = [&](bool fill, const int64_t* offs, uint64_t* out) -> int {
    if (p.kind != KIND_KNN) {
      set_error("range search uses the linear-scan distance kernel");
      return ST_EINVAL;
    }
    return p.order == ORDER_X86
               ? launch_range<KIND_KNN, ORDER_X86>(a, pl, qblocks, radius, radii, exclude_self, counts.as<int64_t>(),
                                                   offs, out, fill, stream)
               : launch_range<KIND_KNN, ORDER_ARM>(a, pl, qblocks, radius, radii, exclude_self, counts.as<int64_t>(),
                                                   offs, out, fill, stream);
  };
  FUELG_TRY(run(false, nullptr, nullptr));
  size_t tb = 0;
  FUELG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, counts.as<int64_t>(), scanned.as<int64_t>(), mS + 1, stream));
  FUELG_TRY(tmp.alloc(tb, stream));
  FUELG_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tb, counts.as<int64_t>(), scanned.as<int64_t>(), mS + 1, stream));
  int64_t tot = 0;
  FUELG_CUDA(cudaMemcpyAsync(&tot, scanned.as<int64_t>() + mS, sizeof(int64_t), cudaMemcpyDeviceToHost, stream));
  FUELG_CUDA(cudaStreamSynchronize(stream));
  csr_offsets_kernel<<<(unsigned)((p.m + 1 + 255) / 256), 256, 0, stream>>>(scanned.as<int64_t>(), p.m, S, *d_off); ::fuelg::note_launch();
  FUELG_CUDA(cudaGetLastError());
  *total = tot;
  if (tot == 0) return ST_OK;
  FUELG_TRY(keys.alloc(sizeof(uint64_t) * tot, stream));
  FUELG_TRY(keys_sorted.alloc(sizeof(uint64_t) * tot, stream));
  FUELG_TRY(run(true, scanned.as<int64_t>(), keys.as<uint64_t>()));
  size_t sb = 0;
  FUELG_CUDA(cub::DeviceSegmentedSort::SortKeys(nullptr, sb, keys.as<uint64_t>(), keys_sorted.as<uint64_t>(), tot,
                                                p.m, *d_off, *d_off + 1, stream));
  Scratch sort_tmp;
  FUELG_TRY(sort_tmp.alloc(sb, stream));
  FUELG_CUDA(cub::DeviceSegmentedSort::SortKeys(sort_tmp.p, sb, keys.as<uint64_t>(), keys_sorted.as<uint64_t>(), tot,
                                                p.m, *d_off, *d_off + 1, stream));
  FUELG_CUDA(cudaMalloc(d_idx, sizeof(int64_t) * tot));
  FUELG_CUDA(cudaMalloc(d_dist, sizeof(float) * tot));
  split_keys_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, stream>>>(keys_sorted.as<uint64_t>(), tot, *d_idx,
                                                                       *d_dist); ::fuelg::note_launch();
  FUELG_CUDA(cudaGetLastError());
  return ST_OK;
}

}  // namespace fuelg
