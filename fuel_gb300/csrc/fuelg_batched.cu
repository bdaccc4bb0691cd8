// fuelg_batched.cu -- many independent Lloyd k-means problems in one pass
// per iteration.
//
// Every problem keeps fuel's Lloyd semantics exactly as fuelg_kmeans_lloyd
// does (src/cluster/kmeans/lloyd.rs:12-202 with fixed initial centres): the
// initial assignment in the vec_pairwise_sqdist order, later passes in the
// math::sqdist order, strict < over centres (first index wins), empty
// clusters keep their centre, centres = correctly rounded f32 of the exact
// mean (integer sums at the problem's scale 2^e_lo, 32-bit slices in 64-bit
// counters, order independent), iteration counting with the initial pass as
// iteration 1 and the changed == 0 stop.  Results are bit-identical to one
// fuelg_kmeans_lloyd call per problem.
//
// Layout: all problems' points are packed row-major one after another; work
// items are 256-row slices of one problem, handed to persistent CTAs in
// contiguous ranges so a CTA reloads a problem's centres into shared memory
// only when its range crosses into the next problem.  One kernel per
// iteration assigns every point of every problem and, for points whose label
// changed, adds +x / -x to the cluster sums: per CTA in shared memory when a
// problem's k*d*L counters fit (many points per counter: few global atomics),
// straight to global counters otherwise.  A second kernel turns the sums into
// centres.  The middle iterations are one CUDA graph replayed.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/fuelg.h"
#include "fuelg_common.cuh"
#include "fuelg_exact.cuh"
#include "fuelg_internal.h"
#include "fuelg_tc_common.cuh"

namespace fuelg {
namespace {

constexpr int kItemRows = 256;       // rows per work item = threads per CTA
constexpr int kCentreCap = 16384;    // centre floats staged in shared memory (64 KB)
constexpr int kAggCap = 2048;        // per-CTA sum counters in shared memory (16 KB)

struct BProb {
  int64_t x_off;     // float offset of the problem's rows
  int64_t n;
  int64_t lab_off;   // label offset
  int64_t c_off;     // centre float offset (k * d)
  int64_t limb_off;  // counter offset (k * d * L)
  int32_t cnt_off;   // count offset (k)
  int32_t d, k, L, e_lo;
  int32_t item_begin;  // first work item
  int32_t active;      // 0: skipped (bad data)
  int64_t cost_begin;  // cumulative work before this problem's first item
  int64_t item_cost;   // work of one item (~ k * d)
  int32_t all_item_begin;  // first 256-row item over all problems (inertia)
  int32_t tc;              // assigned by the tensor-core screen (no CUDA-core items)
};

// First work item whose work offset is >= c (work offsets: the problem's
// cost_begin + j * item_cost for its item j), so CTAs can take contiguous item
// ranges of equal work instead of equal item counts.
__device__ __forceinline__ int64_t item_at_cost(const BProb* __restrict__ probs, int P, int items_total, int64_t c) {
  int lo = 0, hi = P;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (probs[mid].cost_begin <= c) lo = mid;
    else hi = mid;
  }
  const BProb& pr = probs[lo];
  const int64_t items = (lo + 1 < P ? probs[lo + 1].item_begin : items_total) - pr.item_begin;
  const int64_t j = (c - pr.cost_begin + pr.item_cost - 1) / pr.item_cost;
  return j >= items ? pr.item_begin + items : pr.item_begin + j;
}

template <int D>
struct Dim {
  static constexpr int value = D;
};

// Exponent range of one problem's data: items of 64K values.
__global__ void batched_range_kernel(const float* __restrict__ X, const int64_t* __restrict__ off,
                                     const int32_t* __restrict__ blk_begin, int P, int* __restrict__ out) {
  int lo_b = 0, hi_b = P;  // problem of this block
  while (hi_b - lo_b > 1) {
    const int mid = (lo_b + hi_b) >> 1;
    if (blk_begin[mid] <= (int)blockIdx.x) lo_b = mid;
    else hi_b = mid;
  }
  const int p = lo_b;
  const int64_t b0 = off[p], b1 = off[p + 1];
  const int64_t s0 = b0 + (int64_t)(blockIdx.x - blk_begin[p]) * 65536;
  const int64_t s1 = min(s0 + 65536, b1);
  int lo = 1 << 30, hi = -(1 << 30), bad = 0;
  for (int64_t e = s0 + threadIdx.x; e < s1; e += blockDim.x) {
    uint32_t mant;
    int l, h;
    bool z, b;
    f32_parts(X[e], mant, l, h, z, b);
    if (b) bad = 1;
    if (!z && !b) {
      lo = min(lo, l);
      hi = max(hi, h);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&out[3 * p], lo);
    atomicMax(&out[3 * p + 1], hi);
    if (bad) atomicOr(&out[3 * p + 2], 1);
  }
}

// Adds the exact slices of +-x (coordinate `dim` of a point) to cluster c.
__device__ __forceinline__ void add_coord(unsigned long long* __restrict__ dst, float x, int e_lo, int L, bool neg) {
  const unsigned __int128 v = fixed_of(x, e_lo, neg);
  for (int l = 0; l < L; l++) {
    const unsigned long long sl = (unsigned long long)((v >> (32 * l)) & 0xffffffffu);
    if (sl) atomicAdd(dst + l, sl);
  }
}

// One iteration over all problems: assignment + sum updates of changed points.
template <int KIND, int ORDER>
__global__ void __launch_bounds__(kItemRows) batched_assign_kernel(
    const BProb* __restrict__ probs, int P, int items_total, const float* __restrict__ X,
    const float* __restrict__ C, int32_t* __restrict__ labels, unsigned long long* __restrict__ limbs,
    int32_t* __restrict__ counts, int32_t* __restrict__ pchg, int first, int64_t work_total, int ccap) {
  extern __shared__ __align__(16) unsigned char smem_b[];
  float* cs = reinterpret_cast<float*>(smem_b);                                           // [ccap]
  unsigned long long* agg = reinterpret_cast<unsigned long long*>(cs + ccap);            // [kAggCap]
  int* aggc = reinterpret_cast<int*>(agg + kAggCap);                                      // [256]
  __shared__ int s_chg;
  const int64_t it0 = item_at_cost(probs, P, items_total, (int64_t)((__int128)work_total * blockIdx.x / gridDim.x));
  const int64_t it1 =
      blockIdx.x + 1 == gridDim.x ? items_total
                                  : item_at_cost(probs, P, items_total,
                                                 (int64_t)((__int128)work_total * (blockIdx.x + 1) / gridDim.x));
  int p = -1;
  BProb pr{};
  bool staged = false, use_agg = false;
  // flush this CTA's partial sums / counts / change count of problem p
  auto flush = [&]() {
    __syncthreads();
    if (p < 0 || !pr.active) return;
    if (threadIdx.x == 0 && s_chg) atomicAdd(&pchg[p], s_chg);
    if (use_agg) {
      for (int e = threadIdx.x; e < pr.k * pr.d * pr.L; e += blockDim.x)
        if (agg[e]) atomicAdd(limbs + pr.limb_off + e, agg[e]);
      for (int e = threadIdx.x; e < pr.k; e += blockDim.x)
        if (aggc[e]) atomicAdd(&counts[pr.cnt_off + e], aggc[e]);
    }
  };
  for (int64_t item = it0; item < it1; item++) {
    if (p < 0 || (p + 1 < P && item >= probs[p + 1].item_begin)) {
      // next problem: flush the previous one, stage this one's centres
      flush();
      int lo = 0, hi = P;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (probs[mid].item_begin <= item) lo = mid;
        else hi = mid;
      }
      __syncthreads();
      p = lo;
      pr = probs[p];
      staged = pr.k * pr.d <= ccap;
      use_agg = pr.k * pr.d * pr.L <= kAggCap && pr.k <= 256;
      if (pr.active) {
        if (staged)
          for (int e = threadIdx.x; e < pr.k * pr.d; e += blockDim.x) cs[e] = C[pr.c_off + e];
        if (use_agg) {
          for (int e = threadIdx.x; e < pr.k * pr.d * pr.L; e += blockDim.x) agg[e] = 0;
          for (int e = threadIdx.x; e < pr.k; e += blockDim.x) aggc[e] = 0;
        }
      }
      if (threadIdx.x == 0) s_chg = 0;
      __syncthreads();
    }
    if (!pr.active) continue;
    const int64_t i = (item - pr.item_begin) * kItemRows + threadIdx.x;
    const bool live = i < pr.n;
    int best = -1;
    const float* xr = X + pr.x_off + (live ? i : 0) * pr.d;
    const float* cbase = staged ? cs : C + pr.c_off;
    if (live) {
      float bd = 0.0f;
      auto scan = [&](auto dimc) {
        constexpr int DD = decltype(dimc)::value;
        float xv[DD];
#pragma unroll
        for (int t = 0; t < DD; t++) xv[t] = __ldg(xr + t);
        for (int c = 0; c < pr.k; c++) {
          const float* cc = cbase + c * DD;
          // centre values by 16-byte (8-byte for d = 2) loads, one per 4 (2) values
          auto cv = [&](int t) -> float {
            if constexpr (DD % 4 == 0) {
              const float4 v = reinterpret_cast<const float4*>(cc)[t >> 2];
              return (t & 3) == 0 ? v.x : (t & 3) == 1 ? v.y : (t & 3) == 2 ? v.z : v.w;
            } else if constexpr (DD % 2 == 0) {
              const float2 v = reinterpret_cast<const float2*>(cc)[t >> 1];
              return (t & 1) == 0 ? v.x : v.y;
            } else {
              return cc[t];
            }
          };
          const float dv = exact_dist_fn<KIND, ORDER, DD>([&](int t) { return xv[t]; }, cv);
          if (best < 0 || dv < bd) {
            bd = dv;
            best = c;
          }
        }
      };
      switch (pr.d) {
        case 2: scan(Dim<2>{}); break;
        case 8: scan(Dim<8>{}); break;
        case 32: scan(Dim<32>{}); break;
        case 64: scan(Dim<64>{}); break;
        default:
          for (int c = 0; c < pr.k; c++) {
            const float dv = exact_dist_scalar<KIND, ORDER>(xr, C + pr.c_off + (int64_t)c * pr.d, pr.d);
            if (best < 0 || dv < bd) {
              bd = dv;
              best = c;
            }
          }
      }
    }
    const int old = live ? (first ? -1 : labels[pr.lab_off + i]) : -1;
    if (live && best != old) {
      labels[pr.lab_off + i] = best;
      if (!first) atomicAdd(&s_chg, 1);
      unsigned long long* base = use_agg ? agg : limbs + pr.limb_off;
      if (use_agg) {
        atomicAdd(&aggc[best], 1);
        if (old >= 0) atomicAdd(&aggc[old], -1);
      } else {
        atomicAdd(&counts[pr.cnt_off + best], 1);
        if (old >= 0) atomicAdd(&counts[pr.cnt_off + old], -1);
      }
      for (int t = 0; t < pr.d; t++) {
        const float xv = __ldg(xr + t);
        add_coord(base + ((int64_t)best * pr.d + t) * pr.L, xv, pr.e_lo, pr.L, false);
        if (old >= 0) add_coord(base + ((int64_t)old * pr.d + t) * pr.L, xv, pr.e_lo, pr.L, true);
      }
    }
  }
  flush();
}

// Centres from the sums: canonicalise each coordinate's counters (carry
// propagation modulo 2^(32L)) and round the exact mean; empty clusters keep
// their centre.  Also records per-problem convergence: conv[p] = the first
// iteration (counting the initial pass as 1) with no changed label.
__global__ void batched_mean_kernel(const BProb* __restrict__ probs, int P, const int64_t* __restrict__ kd_begin,
                                    int64_t kd_total, unsigned long long* __restrict__ limbs,
                                    const int32_t* __restrict__ counts, float* __restrict__ C, int write_centers) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < kd_total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = P;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (kd_begin[mid] <= e) lo = mid;
      else hi = mid;
    }
    while (lo + 1 < P && kd_begin[lo + 1] <= e) lo++;
    const BProb& pr = probs[lo];
    if (!pr.active) continue;
    const int64_t local = e - kd_begin[lo];
    const int L = pr.L;
    unsigned long long* lp = limbs + pr.limb_off + local * L;
    unsigned __int128 tot = 0;
    for (int l = 0; l < L; l++) tot += (unsigned __int128)lp[l] << (32 * l);
    if (L < 4) tot &= (((unsigned __int128)1) << (32 * (L & 3))) - 1;
    for (int l = 0; l < L; l++) lp[l] = (unsigned long long)((tot >> (32 * l)) & 0xffffffffu);
    const int j = (int)(local / pr.d);
    const int cnt = counts[pr.cnt_off + j];
    if (cnt <= 0 || !write_centers) continue;
    const bool neg = (tot >> (32 * L - 1)) & 1;
    unsigned __int128 mag = tot;
    if (neg) {
      if (L < 4) {
        mag = (((unsigned __int128)1) << (32 * (L & 3))) - tot;
        mag &= (((unsigned __int128)1) << (32 * (L & 3))) - 1;
      } else {
        mag = (unsigned __int128)0 - tot;
      }
    }
    const float v = mag == 0 ? 0.0f : rn_ratio_f32(mag, (unsigned long long)cnt, pr.e_lo);
    C[pr.c_off + local] = neg ? -v : v;
  }
}

// After each pass: record the iteration and convergence, reset the change
// counters.  iter[0] counts passes (the initial one is 1).
__global__ void batched_step_kernel(int P, int32_t* __restrict__ pchg, int32_t* __restrict__ conv,
                                    int32_t* __restrict__ last_chg, int32_t* __restrict__ iter,
                                    int* __restrict__ und_n) {
  const int it = iter[0] + 1;
  for (int p = threadIdx.x; p < P; p += blockDim.x) {
    const int c = pchg[p];
    last_chg[p] = c;
    if (it > 1 && c == 0 && conv[p] == 0) conv[p] = it;
    pchg[p] = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    iter[0] = it;
    *und_n = 0;
  }
}

// Sum of squared distances to the final centres, per problem (near-FP64:
// SqDiffAcc per row, FP64 across rows).
__global__ void batched_inertia_kernel(const BProb* __restrict__ probs, int P, int items_total,
                                       const float* __restrict__ X, const float* __restrict__ C,
                                       const int32_t* __restrict__ labels, double* __restrict__ inertia) {
  for (int64_t item = blockIdx.x; item < items_total; item += gridDim.x) {
    int lo = 0, hi = P;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (probs[mid].all_item_begin <= item) lo = mid;
      else hi = mid;
    }
    const BProb& pr = probs[lo];
    const int64_t i = (item - pr.all_item_begin) * kItemRows + threadIdx.x;
    double s = 0.0;
    if (pr.active && i < pr.n) {
      const float* x = X + pr.x_off + i * pr.d;
      const float* c = C + pr.c_off + (int64_t)labels[pr.lab_off + i] * pr.d;
      SqDiffAcc sa;
      for (int t = 0; t < pr.d; t++) {
        sa.add(x[t], c[t]);
        if ((t & 31) == 31) sa.renorm();
      }
      s = sa.value();
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s != 0.0) atomicAdd(&inertia[lo], s);
  }
}

// ---------------------------------------------------------------------------
// Tensor-core tier for problems with 32 <= d <= 64 and k <= 256: each
// 128-row item of a problem is screened with split-BF16 products (x_hi c_hi +
// x_hi c_lo + x_lo c_hi, one 64-wide K chunk, FP32 accumulators in TMEM)
// against the problem's centres staged in shared memory; a row is decided
// when every other centre's lower bound exceeds the best centre's upper bound
// (the error bound of the single-problem screen), otherwise its candidate
// centres are re-scored with fuel's exact f32 arithmetic.  Labels are
// therefore identical to the CUDA-core tier.
// ---------------------------------------------------------------------------
constexpr int kTcRows = 128;

struct BTcArgs {
  const int32_t* tcp;         // problem ids served here
  const int32_t* item_begin;  // [ntc + 1] first 128-row item of each
  const int64_t* cta_begin;   // [grid + 1] first item of each CTA (ranges of equal estimated cost)
  int ntc, items;
  float alpha;                // operand + accumulation error per |x||c|
  int* status;
  unsigned long long* undecided;  // rows re-scored exactly (count over the call)
  int32_t* und_p;                 // this pass's undecided rows: problem, row
  int32_t* und_i;
  uint32_t* und_m;                // and their candidate centres: und_w bit words per row
  int und_w;
  int* und_n;
  // passes after the first: changed rows (row, new and old global cluster)
  // listed for the bucketed sums while the list has room, and the per-key
  // counts (key 2 gc: rows entering cluster gc, 2 gc + 1: rows leaving it)
  int32_t *chg_row, *chg_new, *chg_old, *hist;
  int* chg_n;
  int chg_cap;
};


// |v|^2 in FP32 as 8 interleaved chains + a 3-level tree (error <= (ceil(d/8) + 3) u |v|^2).
template <class F>
__device__ __forceinline__ float norm2_blocked(F v, int d) {
  float p[8];
#pragma unroll
  for (int l = 0; l < 8; l++) p[l] = 0.0f;
  for (int e = 0; e < d; e += 8) {
#pragma unroll
    for (int l = 0; l < 8; l++)
      if (e + l < d) {
        const float x = v(e + l);
        p[l] = fmaf(x, x, p[l]);
      }
  }
  return ((p[0] + p[1]) + (p[2] + p[3])) + ((p[4] + p[5]) + (p[6] + p[7]));
}

// Warp-specialised persistent screen over a list of 128-row items:
//   warps 0-3  loaders: thread 0 copies the NEXT item's rows (contiguous in
//              memory) into one of two staging buffers with one bulk copy; all
//              128 convert the current item's rows from staging into BF16 hi /
//              lo (SW128) and |x|^2, one row per thread, into one of two A
//              buffers; on a problem change they stage the problem's centres
//              (hi / lo, SW128), norms and parameters
//   warp 4     TMEM owner; lane 0 issues the three products per K step
//              (x_hi c_hi + x_hi c_lo + x_lo c_hi) into one of two 256-column
//              accumulators and commits
//   warps 5-8  epilogue: screen, labels, sums of changed rows
// so the row copy of item t+1, its conversion, the MMAs and the epilogue of
// item t overlap.  Barriers: stage_full[s] (bulk copy bytes), a_full[b] (128
// loader arrivals), acc_full[b] (the MMA commit), item_done[b] (128 epilogue
// arrivals: A[b], TMEM[b] and the item's parameters are free again).  On a
// problem change the loaders first wait for the previous item to retire, so
// the single centre buffer is never replaced under a reader.  Every wait is
// bounded.
constexpr int kTcThreads = 288;
constexpr uint32_t kTcA = 32768;   // one A buffer: hi 16 KB + lo 16 KB
constexpr uint32_t kTcB = 65536;   // the centre buffer: hi 32 KB + lo 32 KB (256 centres)
constexpr uint32_t kTcS = 32768;   // one staging buffer: 128 rows x 64 f32
constexpr uint32_t kTcOffB = 2 * kTcA, kTcOffS = kTcOffB + kTcB, kTcSmall = kTcOffS + 2 * kTcS;

struct ItemMeta {  // one item's problem parameters, written by the loaders
  int64_t n, lab_off, limb_off, x_off;
  int32_t p, i0, kp, d, k, L, e_lo, cnt_off;
};

// + norms (2 x 256 floats), maxima (4), row norms (2 x 128), metadata (2), 9 mbarriers,
// TMEM address and abort word, 1 KB alignment
constexpr size_t kTcSmem =
    1024 + kTcSmall + 4 * 2 * 256 + 4 * 4 + 4 * 2 * 128 + sizeof(ItemMeta) * 2 + 8 * 9 + 8 + 64;

// Every loader thread (warps 0-3, named barrier 1) learns whether all of
// them passed `v`.
__device__ __forceinline__ bool loaders_all(bool v) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n bar.red.and.pred p, 1, 128, q;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(r)
      : "r"((uint32_t)v)
      : "memory");
  return r != 0;
}

template <int KIND, int ORDER>
__global__ void __launch_bounds__(kTcThreads, 1) batched_tc_assign_kernel(
    const BProb* __restrict__ probs, BTcArgs ta, const float* __restrict__ X, const float* __restrict__ C,
    int32_t* __restrict__ labels, unsigned long long* __restrict__ limbs, int32_t* __restrict__ counts,
    int32_t* __restrict__ pchg, int first) {
  extern __shared__ __align__(1024) unsigned char smem_t[];
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_t) + 1023) & ~(uintptr_t)1023);
  unsigned char* sBh = base + kTcOffB;
  unsigned char* sBl = sBh + kTcB / 2;
  float* cn2s = reinterpret_cast<float*>(base + kTcSmall);  // [256] |c|^2 of the staged problem
  float* cns = cn2s + 256;                                   // [256] |c|
  float* cmaxs = cns + 256;                                  // [0] max |c|^2 (bits), spare
  float* xn2s = cmaxs + 4;                                   // [2 buffers][128] |x|^2
  ItemMeta* meta = reinterpret_cast<ItemMeta*>(xn2s + 2 * 128);
  uint64_t* stage_full = reinterpret_cast<uint64_t*>(meta + 2);
  uint64_t* a_full = stage_full + 2;
  uint64_t* acc_full = a_full + 2;
  uint64_t* item_done = acc_full + 2;
  uint64_t* fin = item_done + 2;
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(fin + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_holder + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int b = 0; b < 2; b++) {
      tcx::mbar_init(&stage_full[b], 1);
      tcx::mbar_init(&a_full[b], kTcRows);
      tcx::mbar_init(&acc_full[b], 1);
      tcx::mbar_init(&item_done[b], kTcRows);
    }
    tcx::mbar_init(fin, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 4) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tcx::smem_u32(tmem_holder)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tcx::tc_fence_before();
  __syncthreads();
  tcx::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  // this CTA's items: a contiguous range of equal estimated cost
  const int64_t it0 = ta.cta_begin[blockIdx.x], it1 = ta.cta_begin[blockIdx.x + 1];
  const int64_t nlt = it1 - it0;
  auto problem_of = [&](int64_t item, int q0) {
    int q = q0 < 0 ? 0 : q0;
    if (q0 < 0 || item >= ta.item_begin[q + 1]) {
      int lo = 0, hi = ta.ntc;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (ta.item_begin[mid] <= item) lo = mid;
        else hi = mid;
      }
      q = lo;
    }
    return q;
  };
  // bytes of an item's rows that one bulk copy brings in (0: the direct-load path)
  auto bulk_bytes = [&](const BProb& pr, int64_t i0) -> uint32_t {
    if (!pr.active || (pr.d & 3) != 0 || (pr.x_off & 3) != 0 || pr.d > 64) return 0u;
    const int64_t rows = min((int64_t)kTcRows, pr.n - i0);
    return (uint32_t)(rows * pr.d * 4);
  };

  if (warp < 4) {
    // ---- loaders ----------------------------------------------------------
    int q = -1, cur_p = -1, qn = -1;
    int issued[2] = {0, 0};  // copies (or plain arrivals) armed per staging buffer, thread 0
    // the first item's rows
    if (tid == 0 && nlt > 0) {
      issued[0] = 1;
      qn = problem_of(it0, -1);
      const BProb pn = probs[ta.tcp[qn]];
      const int64_t i0n = (it0 - ta.item_begin[qn]) * kTcRows;
      const uint32_t by = bulk_bytes(pn, i0n);
      if (by) {
        tcx::mbar_expect_tx(&stage_full[0], by);
        tcx::bulk_load(base + kTcOffS, X + pn.x_off + i0n * pn.d, by, &stage_full[0]);
      } else {
        tcx::mbar_arrive(&stage_full[0]);
      }
    }
    for (int64_t lt = 0; lt < nlt; lt++) {
      const int b = (int)(lt & 1);
      const uint32_t ph = (uint32_t)((lt >> 1) & 1);
      // item lt-2 retired: its A buffer, accumulator and parameters are free.
      // The loaders leave together (a vote on their named barrier), so the
      // barriers below never wait for a loader that left.
      bool ok = !*abort_flag && tcx::mbar_wait(&item_done[b], ph ^ 1u, abort_flag);
      if (!ok && !*abort_flag) atomicOr(ta.status, DEV_TIMEOUT);
      if (!loaders_all(ok)) {
        *abort_flag = 1;
        break;
      }
      const int64_t item = it0 + lt;
      q = problem_of(item, q);
      const int p = ta.tcp[q];
      const BProb pr = probs[p];
      const int kp = (pr.k + 15) & ~15;
      const int64_t i0 = (item - ta.item_begin[q]) * kTcRows;
      if (p != cur_p) {
        // a new problem: the previous item must retire before its centres go
        if (lt > 0) {
          const int pb = (int)((lt - 1) & 1);
          ok = !*abort_flag && tcx::mbar_wait(&item_done[pb], (uint32_t)(((lt - 1) >> 1) & 1), abort_flag);
          if (!ok && !*abort_flag) atomicOr(ta.status, DEV_TIMEOUT);
          if (!loaders_all(ok)) {
            *abort_flag = 1;
            break;
          }
        }
        cur_p = p;
        for (int e = tid; e < kp * 8; e += kTcRows) {
          const int j = e >> 3, ch = e & 7;
          uint32_t hw[4], lw[4];
#pragma unroll
          for (int l = 0; l < 8; l += 2) {
            const int t0 = 8 * ch + l;
            const float c0 = (j < pr.k && t0 < pr.d) ? C[pr.c_off + (int64_t)j * pr.d + t0] : 0.0f;
            const float c1 = (j < pr.k && t0 + 1 < pr.d) ? C[pr.c_off + (int64_t)j * pr.d + t0 + 1] : 0.0f;
            const __nv_bfloat162 h = __floats2bfloat162_rn(c0, c1);
            const float2 hf = __bfloat1622float2(h);
            const __nv_bfloat162 lo = __floats2bfloat162_rn(c0 - hf.x, c1 - hf.y);
            hw[l / 2] = *reinterpret_cast<const uint32_t*>(&h);
            lw[l / 2] = *reinterpret_cast<const uint32_t*>(&lo);
          }
          const uint32_t off = (uint32_t)j * 128u + ((uint32_t)(ch ^ (j & 7)) << 4);
          *reinterpret_cast<uint4*>(sBh + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
          *reinterpret_cast<uint4*>(sBl + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        }
        if (tid == 0) cmaxs[0] = 0.0f;
        asm volatile("bar.sync 1, %0;" ::"n"(kTcRows) : "memory");  // loaders only
        float m2 = 0.0f;
        for (int j = tid; j < 256; j += kTcRows) {
          float v = 0.0f;
          if (j < pr.k) {
            const float* cj = C + pr.c_off + (int64_t)j * pr.d;
            v = norm2_blocked([&](int t) { return cj[t]; }, pr.d);
          }
          // +inf past k: the epilogue reads them four at a time, and a padding
          // column's screen value is then +inf (never the minimum)
          cn2s[j] = j < pr.k ? v : __int_as_float(0x7f800000);
          cns[j] = sqrtf(v);
          m2 = fmaxf(m2, v);
        }
        // non-negative floats order like their bit patterns
        atomicMax(reinterpret_cast<int*>(cmaxs), __float_as_int(m2));
      }
      // the next item's rows into the other staging buffer: its previous
      // contents (item lt-1) were converted before every loader passed the
      // vote above
      if (tid == 0 && lt + 1 < nlt) {
        const int s = (int)((lt + 1) & 1);
        issued[s]++;
        qn = problem_of(item + 1, qn);
        const BProb pn = probs[ta.tcp[qn]];
        const int64_t i0n = (item + 1 - ta.item_begin[qn]) * kTcRows;
        const uint32_t by = bulk_bytes(pn, i0n);
        if (by) {
          tcx::mbar_expect_tx(&stage_full[s], by);
          tcx::bulk_load(base + kTcOffS + (uint32_t)s * kTcS, X + pn.x_off + i0n * pn.d, by, &stage_full[s]);
        } else {
          tcx::mbar_arrive(&stage_full[s]);
        }
      }
      // this item's rows -> BF16 hi / lo (zero padded), FP32 norms; thread = row
      unsigned char* sAh = base + (uint32_t)b * kTcA;
      unsigned char* sAl = sAh + kTcA / 2;
      const int64_t i = i0 + tid;
      const bool live = pr.active && i < pr.n;
      ok = !*abort_flag && tcx::mbar_wait(&stage_full[b], ph, abort_flag);
      if (!ok && !*abort_flag) atomicOr(ta.status, DEV_TIMEOUT);
      if (!loaders_all(ok)) {
        *abort_flag = 1;
        break;
      }
      const bool bulk = bulk_bytes(pr, i0) != 0;
      const float* srow = reinterpret_cast<const float*>(base + kTcOffS + (uint32_t)b * kTcS) + tid * pr.d;
      const float* xr = X + pr.x_off + (live ? i : 0) * pr.d;
      float pn[8];
#pragma unroll
      for (int l = 0; l < 8; l++) pn[l] = 0.0f;
      // chunks of 8 values in a per-row rotated order (row t starts at chunk
      // t & 7), so the staging reads of a warp spread over the banks; the
      // norm keeps its 8 interleaved chains of ceil(d/8) terms and 3-level tree
#pragma unroll 2
      for (int jj = 0; jj < 8; jj++) {
        const int j = (jj + tid) & 7;
        float x[8];
        if (live && bulk && 8 * j + 7 < pr.d) {
          const float4 a4 = *reinterpret_cast<const float4*>(srow + 8 * j);
          const float4 b4 = *reinterpret_cast<const float4*>(srow + 8 * j + 4);
          x[0] = a4.x, x[1] = a4.y, x[2] = a4.z, x[3] = a4.w, x[4] = b4.x, x[5] = b4.y, x[6] = b4.z, x[7] = b4.w;
        } else if (live && bulk) {
#pragma unroll
          for (int l = 0; l < 8; l++) x[l] = 8 * j + l < pr.d ? srow[8 * j + l] : 0.0f;
        } else {
#pragma unroll
          for (int l = 0; l < 8; l++) x[l] = (live && 8 * j + l < pr.d) ? __ldg(xr + 8 * j + l) : 0.0f;
        }
        uint32_t hw[4], lw[4];
#pragma unroll
        for (int l = 0; l < 8; l += 2) {
          const __nv_bfloat162 h = __floats2bfloat162_rn(x[l], x[l + 1]);
          const float2 hf = __bfloat1622float2(h);
          const __nv_bfloat162 lo = __floats2bfloat162_rn(x[l] - hf.x, x[l + 1] - hf.y);
          hw[l / 2] = *reinterpret_cast<const uint32_t*>(&h);
          lw[l / 2] = *reinterpret_cast<const uint32_t*>(&lo);
          pn[l] = fmaf(x[l], x[l], pn[l]);
          pn[l + 1] = fmaf(x[l + 1], x[l + 1], pn[l + 1]);
        }
        const uint32_t off = (uint32_t)tid * 128u + ((uint32_t)(j ^ (tid & 7)) << 4);
        *reinterpret_cast<uint4*>(sAh + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        *reinterpret_cast<uint4*>(sAl + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
      }
      xn2s[b * 128 + tid] = ((pn[0] + pn[1]) + (pn[2] + pn[3])) + ((pn[4] + pn[5]) + (pn[6] + pn[7]));
      if (tid == 0) {
        ItemMeta m;
        m.n = pr.n;
        m.lab_off = pr.lab_off;
        m.limb_off = pr.limb_off;
        m.x_off = pr.x_off;
        m.p = p;
        m.i0 = (int32_t)i0;
        m.kp = pr.active ? kp : 0;
        m.d = pr.d;
        m.k = pr.k;
        m.L = pr.L;
        m.e_lo = pr.e_lo;
        m.cnt_off = pr.cnt_off;
        meta[b] = m;
      }
      // generic-proxy smem writes -> visible to the tensor core's async proxy
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tcx::mbar_arrive(&a_full[b]);
    }
    // a copy still in flight must not outlive the CTA: the last one armed on
    // each staging buffer lands before the exit (also after an abort)
    if (tid == 0) {
      volatile int never = 0;
      for (int s = 0; s < 2; s++)
        if (issued[s] > 0 && !tcx::mbar_wait(&stage_full[s], (uint32_t)((issued[s] - 1) & 1), &never))
          atomicOr(ta.status, DEV_TIMEOUT);
    }
  } else if (warp == 4) {
    // ---- MMA issuer ---------------------------------------------------------
    if (lane == 0) {
      for (int64_t lt = 0; lt < nlt && !*abort_flag; lt++) {
        const int b = (int)(lt & 1);
        const uint32_t ph = (uint32_t)((lt >> 1) & 1);
        if (!tcx::mbar_wait(&a_full[b], ph, abort_flag)) {
          if (!*abort_flag) atomicOr(ta.status, DEV_TIMEOUT);
          *abort_flag = 1;
          break;
        }
        tcx::tc_fence_after();
        const int kp = meta[b].kp;
        if (kp > 0) {
          unsigned char* sAh = base + (uint32_t)b * kTcA;
          const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kp >> 3) << 17) |
                                 ((uint32_t)(kTcRows >> 4) << 24);
          const uint64_t ah = tcx::smem_desc_sw128(tcx::smem_u32(sAh));
          const uint64_t al = tcx::smem_desc_sw128(tcx::smem_u32(sAh + kTcA / 2));
          const uint64_t bh = tcx::smem_desc_sw128(tcx::smem_u32(sBh));
          const uint64_t bl = tcx::smem_desc_sw128(tcx::smem_u32(sBl));
          const uint32_t d_tmem = tmem + (uint32_t)b * 256u;
          // K steps of 16 that hold data (the zero columns past d add nothing)
          const int nks = (meta[b].d + 15) >> 4;
#pragma unroll
          for (int kk = 0; kk < 4; kk++)
            if (kk < nks) tcx::umma_bf16(d_tmem, ah + 2 * kk, bh + 2 * kk, idesc, kk ? 1u : 0u);
#pragma unroll
          for (int kk = 0; kk < 4; kk++)
            if (kk < nks) tcx::umma_bf16(d_tmem, ah + 2 * kk, bl + 2 * kk, idesc, 1u);
#pragma unroll
          for (int kk = 0; kk < 4; kk++)
            if (kk < nks) tcx::umma_bf16(d_tmem, al + 2 * kk, bh + 2 * kk, idesc, 1u);
        }
        tcx::umma_commit(&acc_full[b]);
      }
      // every MMA issued here has completed before TMEM is freed
      tcx::umma_commit(fin);
      volatile int never = 0;
      if (!tcx::mbar_wait(fin, 0, &never)) atomicOr(ta.status, DEV_TIMEOUT);
    }
  } else {
    // ---- epilogue: warp w reads TMEM lanes 32 * (w % 4) .. +32 ---------------
    const int g = warp & 3;
    const int row = g * 32 + lane;
    const double u24 = 5.9604644775390625e-08;
    for (int64_t lt = 0; lt < nlt; lt++) {
      const int b = (int)(lt & 1);
      const uint32_t ph = (uint32_t)((lt >> 1) & 1);
      bool ok = !*abort_flag && tcx::mbar_wait(&acc_full[b], ph, abort_flag);
      if (!ok) {
        if (!*abort_flag) atomicOr(ta.status, DEV_TIMEOUT);
        *abort_flag = 1;
      }
      if (!__all_sync(0xffffffffu, ok)) break;  // warp-uniform exit
      tcx::tc_fence_after();
      const ItemMeta mt = meta[b];
      const int kp = mt.kp;
      const int64_t i = (int64_t)mt.i0 + row;
      const bool live = kp > 0 && i < mt.n;
      // the row's current label, fetched while the screen runs
      const int old = live ? (first ? -1 : labels[mt.lab_off + i]) : -1;
      const float cmax0 = cmaxs[0];
      const float nx = xn2s[b * 128 + row];
      const float beta = (float)(((mt.d + 7) / 8 + 3 + 9) * u24 * 1.01);
      const float gamma = (float)((mt.d + 4) * u24 * 1.01);
      const uint32_t taddr = tmem + ((uint32_t)(g * 32) << 16) + (uint32_t)b * 256u;
      const float xl = sqrtf(nx);
      float best = __int_as_float(0x7f800000);
      int bj = 0;
      bool undecided = false;
      // candidate centres of an undecided row: 32-column words (bit w of
      // cm_set: word w holds candidates)
      uint32_t cmask[8];
      uint32_t cm_set = 0;
      if (kp > 0) {
        // screen, two passes over the TMEM columns (32 per wait).  Pass 1: the
        // smallest screen value (four independent running minima over the
        // columns of each residue mod 4; the padding columns past k read +inf
        // norms).  The best centre's upper bound is taken with the problem's
        // norm maxima (at least its own error term), so it needs no column
        // index.  Pass 2: the first column holding the smallest value is the
        // best centre (first index wins ties, as in a scan), and every other
        // column whose lower bound reaches the bound is a candidate; columns
        // above T cannot reach it with the largest error of the problem.
        float b4[4] = {best, best, best, best};
        for (int c0 = 0; c0 < kp; c0 += 32) {
          uint32_t r[2][16];
#pragma unroll
          for (int h = 0; h < 2; h++)
            if (c0 + 16 * h < kp) tcx::tmem_ld16_nowait(taddr + c0 + 16 * h, r[h]);
          tcx::tmem_ld_wait();
#pragma unroll
          for (int h = 0; h < 2; h++) tcx::tmem_regs_ready(r[h]);
#pragma unroll
          for (int h = 0; h < 2; h++) {
            if (c0 + 16 * h >= kp) break;
#pragma unroll
            for (int v = 0; v < 4; v++) {
              const float4 c4 = *reinterpret_cast<const float4*>(cn2s + c0 + 16 * h + 4 * v);
              const float cc[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
              for (int u = 0; u < 4; u++)
                b4[u] = fminf(b4[u], fmaf(-2.0f, __uint_as_float(r[h][4 * v + u]), nx + cc[u]));
            }
          }
        }
        best = fminf(fminf(b4[0], b4[1]), fminf(b4[2], b4[3]));
        const float amax = (ta.alpha * xl * sqrtf(cmax0) + beta * (nx + cmax0)) * (1.0f + gamma);
        const float hi_b = best + amax + gamma * fabsf(best);
        const float T = (hi_b + amax) * (1.0f + 2.0f * gamma) * (1.0f + 9.5367431640625e-07f);
        bool found = false;
        for (int c0 = 0; c0 < kp; c0 += 32) {
          uint32_t bits = 0;
          uint32_t r[2][16];
#pragma unroll
          for (int h = 0; h < 2; h++)
            if (c0 + 16 * h < kp) tcx::tmem_ld16_nowait(taddr + c0 + 16 * h, r[h]);
          tcx::tmem_ld_wait();
#pragma unroll
          for (int h = 0; h < 2; h++) tcx::tmem_regs_ready(r[h]);
#pragma unroll
          for (int h = 0; h < 2; h++) {
            if (c0 + 16 * h >= kp) break;
#pragma unroll
            for (int v = 0; v < 4; v++) {
              const float4 c4 = *reinterpret_cast<const float4*>(cn2s + c0 + 16 * h + 4 * v);
              const float cc[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
              for (int u = 0; u < 4; u++) {
                const int col = c0 + 16 * h + 4 * v + u;
                const float dt = fmaf(-2.0f, __uint_as_float(r[h][4 * v + u]), nx + cc[u]);
                if (!found && dt == best) {
                  found = true;
                  bj = col;
                } else if (!(T > 0.0f) || !(dt > T)) {  // padding columns (+inf) only when T <= 0
                  const float e =
                      (ta.alpha * xl * cns[col] + beta * (nx + cc[u])) * (1.0f + gamma) + gamma * fabsf(dt);
                  if (!(dt - e > hi_b)) bits |= 1u << (16 * h + 4 * v + u);
                }
              }
            }
          }
          if (bits) {
            undecided = true;
            cmask[c0 >> 5] = bits;
            cm_set |= 1u << (c0 >> 5);
          }
        }
        // no column equal to the minimum (a NaN screen value): the re-score
        // decides among every centre
        if (!found) {
          undecided = true;
          for (int w = 0; w < (kp + 31) / 32; w++) cmask[w] = 0xffffffffu;
          cm_set = (1u << ((kp + 31) / 32)) - 1u;
        }
      }
      // the item's accumulator, tile and parameters are no longer read
      tcx::tc_fence_before();
      tcx::mbar_arrive(&item_done[b]);
      if (kp == 0) continue;
      const int p = mt.p;
      const int lab = bj;
      {
        const unsigned um = __ballot_sync(0xffffffffu, live && undecided);
        if (lane == 0 && um) atomicAdd(ta.undecided, (unsigned long long)__popc(um));
      }
      if (live && undecided) {
        // the exact re-score kernel decides this row among its candidates
        // and the screen's best
        const int u = atomicAdd(ta.und_n, 1);
        ta.und_p[u] = p;
        ta.und_i[u] = (int32_t)i;
        uint32_t* um = ta.und_m + (int64_t)u * ta.und_w;
        for (int w = 0; w < ta.und_w; w++) {
          uint32_t m = ((cm_set >> w) & 1u) ? cmask[w] : 0u;
          if (w == (bj >> 5)) m |= 1u << (bj & 31);
          um[w] = m;
        }
      }
      const bool chg = live && !undecided && lab != old;
      const unsigned cm = __ballot_sync(0xffffffffu, chg);
      if (!first && lane == 0 && cm) atomicAdd(&pchg[p], __popc(cm));
      if (chg) {
        labels[mt.lab_off + i] = lab;
        atomicAdd(&counts[mt.cnt_off + lab], 1);
        if (old >= 0) atomicAdd(&counts[mt.cnt_off + old], -1);
      }
      // the first pass's sums (every row enters) are made after the pass by
      // the bucketed kernels below
      if (first) continue;
      // later passes: the changed rows go to the change list (bucketed and
      // summed after the pass) while it has room
      bool listed = false;
      {
        const unsigned cmw = __ballot_sync(0xffffffffu, chg);
        if (cmw) {
          int at = 0;
          if (lane == 0) at = atomicAdd(ta.chg_n, __popc(cmw));
          at = __shfl_sync(0xffffffffu, at, 0) + __popc(cmw & ((1u << lane) - 1u));
          if (chg && at < ta.chg_cap) {
            listed = true;
            ta.chg_row[at] = (int32_t)i;
            ta.chg_new[at] = mt.cnt_off + lab;
            ta.chg_old[at] = mt.cnt_off + old;
            atomicAdd(&ta.hist[2 * (mt.cnt_off + lab)], 1);
            atomicAdd(&ta.hist[2 * (mt.cnt_off + old) + 1], 1);
          }
        }
      }
      // the others' coordinates into the exact sums: the warp takes the
      // rows that enter one cluster (or leave one) together -- lanes over
      // consecutive coordinates, the group's 32-bit slices summed in 64-bit
      // registers (at most 32 slices: no overflow), one atomic per counter --
      // which gives the counters the same values as one add per row, since the
      // counters add modulo 2^64
      for (int dir = 0; dir < 2; dir++) {
        const bool mine = chg && !listed && (dir == 0 || old >= 0);
        const int key = dir == 0 ? lab : old;
        unsigned pend = __ballot_sync(0xffffffffu, mine);
        while (pend) {
          const int src = __ffs(pend) - 1;
          const int ks = __shfl_sync(0xffffffffu, key, src);
          const unsigned grp = __ballot_sync(0xffffffffu, mine && key == ks);
          pend &= ~grp;
          unsigned long long* dst = limbs + mt.limb_off + (int64_t)ks * mt.d * mt.L;
          for (int tb = 0; tb < mt.d; tb += 32) {
            const int t = tb + lane;
            const bool tv = t < mt.d;
            unsigned long long acc[4] = {0ull, 0ull, 0ull, 0ull};
            unsigned gm = grp;
            while (gm) {
              const int r = __ffs(gm) - 1;
              gm &= gm - 1;
              const int64_t is = __shfl_sync(0xffffffffu, i, r);
              if (tv) {
                const unsigned __int128 v = fixed_of(__ldg(X + mt.x_off + is * mt.d + t), mt.e_lo, dir == 1);
#pragma unroll
                for (int l = 0; l < 4; l++)
                  if (l < mt.L) acc[l] += (unsigned long long)((v >> (32 * l)) & 0xffffffffu);
              }
            }
            if (tv) {
#pragma unroll
              for (int l = 0; l < 4; l++)
                if (l < mt.L && acc[l]) atomicAdd(dst + (int64_t)t * mt.L + l, acc[l]);
            }
          }
        }
      }
    }
  }
  tcx::tc_fence_before();
  __syncthreads();
  if (warp == 4) {
    tcx::tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
  }
}

// Exact assignment of the rows the tensor-core screen left undecided: one
// warp per row, lanes over the centres (fuel's f32 operation order), the
// smallest (distance, index) key wins -- the first minimum, as in the
// CUDA-core pass -- then the row's sums move if its label changed.
template <int KIND, int ORDER>
__global__ void __launch_bounds__(256) batched_rescore_kernel(
    const BProb* __restrict__ probs, const int32_t* __restrict__ und_p, const int32_t* __restrict__ und_i,
    const uint32_t* __restrict__ und_m, int und_w, const int* __restrict__ und_n, const float* __restrict__ X,
    const float* __restrict__ C,
    int32_t* __restrict__ labels, unsigned long long* __restrict__ limbs, int32_t* __restrict__ counts,
    int32_t* __restrict__ pchg, int first) {
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const int cnt = *und_n;
  for (int u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < cnt; u += nw) {
    const int p = und_p[u];
    const int64_t i = und_i[u];
    const BProb& pr = probs[p];
    const float* xr = X + pr.x_off + i * pr.d;
    uint64_t best = ~0ull;
    // the candidates (every centre whose lower bound reached the screen
    // best's upper bound, and that best): lane t scores the t-th of each 32
    const uint32_t* um = und_m + (int64_t)u * und_w;
    int w = 0;
    uint32_t m = um[0];
    for (;;) {
      int c = -1, got = 0;
      while (got < 32) {
        while (m == 0 && w + 1 < und_w) m = um[++w];
        if (m == 0) break;
        const int b = __ffs(m) - 1;
        m &= m - 1;
        if (got == lane) c = w * 32 + b;
        got++;
      }
      if (c >= 0 && c < pr.k) {
        const float dv = exact_dist_scalar<KIND, ORDER>(xr, C + pr.c_off + (int64_t)c * pr.d, pr.d);
        const uint64_t key = ((uint64_t)__float_as_uint(dv) << 32) | (uint32_t)c;
        best = key < best ? key : best;
      }
      if (got < 32) break;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const uint64_t v = ((uint64_t)__shfl_xor_sync(0xffffffffu, (uint32_t)(best >> 32), o) << 32) |
                         __shfl_xor_sync(0xffffffffu, (uint32_t)best, o);
      best = v < best ? v : best;
    }
    const int lab = (int)(uint32_t)best;
    const int old = first ? -1 : labels[pr.lab_off + i];
    if (lab == old) continue;
    if (lane == 0) {
      labels[pr.lab_off + i] = lab;
      if (!first) atomicAdd(&pchg[p], 1);
      atomicAdd(&counts[pr.cnt_off + lab], 1);
      if (old >= 0) atomicAdd(&counts[pr.cnt_off + old], -1);
    }
    if (first) continue;  // the first pass's sums: tc_first_sum_kernel
    for (int t = lane; t < pr.d; t += 32) {
      const float xv = __ldg(xr + t);
      add_coord(limbs + pr.limb_off + ((int64_t)lab * pr.d + t) * pr.L, xv, pr.e_lo, pr.L, false);
      if (old >= 0) add_coord(limbs + pr.limb_off + ((int64_t)old * pr.d + t) * pr.L, xv, pr.e_lo, pr.L, true);
    }
  }
}

// The first pass's exact sums of the tensor-core problems, after every row
// has its label (so a warp sums runs of rows of one cluster in registers
// instead of one atomic per row and counter): bucket offsets per cluster (one
// warp per problem: exclusive prefix of its final counts, from the problem's
// first row of the bucket array), the rows scattered into their clusters'
// buckets, then one warp per 32 bucket entries.
__global__ void tc_first_offsets_kernel(const BProb* __restrict__ probs, const int32_t* __restrict__ tcp, int ntc,
                                        const int64_t* __restrict__ row_base, const int32_t* __restrict__ counts,
                                        int64_t* __restrict__ boff, int32_t* __restrict__ cursor) {
  const int lane = threadIdx.x & 31;
  const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= ntc) return;
  const BProb pr = probs[tcp[q]];
  int64_t carry = row_base[q];
  for (int j0 = 0; j0 < pr.k; j0 += 32) {
    const int j = j0 + lane;
    const int c = j < pr.k ? counts[pr.cnt_off + j] : 0;
    int a = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, a, o);
      if (lane >= o) a += u;
    }
    if (j < pr.k) {
      boff[pr.cnt_off + j] = carry + a - c;
      cursor[pr.cnt_off + j] = 0;
    }
    carry += __shfl_sync(0xffffffffu, a, 31);
  }
}

__global__ void __launch_bounds__(kTcRows) tc_first_scatter_kernel(
    const BProb* __restrict__ probs, const int32_t* __restrict__ tcp, const int32_t* __restrict__ item_begin,
    int ntc, const int32_t* __restrict__ labels, const int64_t* __restrict__ boff, int32_t* __restrict__ cursor,
    int32_t* __restrict__ b_row, int32_t* __restrict__ b_gc) {
  const int item = blockIdx.x;
  int lo = 0, hi = ntc;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (item_begin[mid] <= item) lo = mid;
    else hi = mid;
  }
  const BProb pr = probs[tcp[lo]];
  const int64_t i = (int64_t)(item - item_begin[lo]) * kTcRows + threadIdx.x;
  const bool live = pr.active && i < pr.n;
  const int gc = live ? pr.cnt_off + labels[pr.lab_off + i] : -1;
  // one reservation per cluster among the warp's rows
  const unsigned grp = __match_any_sync(0xffffffffu, gc);
  const int lead = __ffs(grp) - 1;
  int at = 0;
  if (live && (int)(threadIdx.x & 31) == lead) at = atomicAdd(&cursor[gc], __popc(grp));
  at = __shfl_sync(0xffffffffu, at, lead) + __popc(grp & ((1u << (threadIdx.x & 31)) - 1u));
  if (live) {
    const int64_t e = boff[gc] + at;
    b_row[e] = (int32_t)i;
    b_gc[e] = gc;
  }
}

__global__ void __launch_bounds__(256) tc_first_sum_kernel(const BProb* __restrict__ probs,
                                                           const int32_t* __restrict__ gc_prob, int64_t entries,
                                                           const int32_t* __restrict__ b_row,
                                                           const int32_t* __restrict__ b_gc,
                                                           const float* __restrict__ X,
                                                           unsigned long long* __restrict__ limbs) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32;
  if (w0 >= entries) return;
  const int64_t e = w0 + lane;
  const int myrow = e < entries ? b_row[e] : 0;
  const int mygc = e < entries ? b_gc[e] : -1;
  int cur = -1;
  BProb pr{};
  unsigned long long a0[4] = {0ull, 0ull, 0ull, 0ull}, a1[4] = {0ull, 0ull, 0ull, 0ull};
  auto flush = [&]() {
    if (cur < 0) return;
    unsigned long long* dst = limbs + pr.limb_off + (int64_t)(cur - pr.cnt_off) * pr.d * pr.L;
    for (int l = 0; l < pr.L; l++) {
      if (lane < pr.d && a0[l]) atomicAdd(dst + (int64_t)lane * pr.L + l, a0[l]);
      if (lane + 32 < pr.d && a1[l]) atomicAdd(dst + (int64_t)(lane + 32) * pr.L + l, a1[l]);
      a0[l] = 0ull;
      a1[l] = 0ull;
    }
  };
#pragma unroll 4
  for (int t = 0; t < 32; t++) {
    const int gc = __shfl_sync(0xffffffffu, mygc, t);
    if (gc < 0) break;
    const int row = __shfl_sync(0xffffffffu, myrow, t);
    if (gc != cur) {
      flush();
      cur = gc;
      pr = probs[gc_prob[gc]];
    }
    const float* xr = X + pr.x_off + (int64_t)row * pr.d;
    const float x0 = lane < pr.d ? __ldg(xr + lane) : 0.0f;
    const float x1 = lane + 32 < pr.d ? __ldg(xr + lane + 32) : 0.0f;
    const unsigned __int128 v0 = fixed_of(x0, pr.e_lo, false), v1 = fixed_of(x1, pr.e_lo, false);
#pragma unroll
    for (int l = 0; l < 4; l++) {
      if (l < pr.L) {
        a0[l] += (unsigned long long)((v0 >> (32 * l)) & 0xffffffffu);
        a1[l] += (unsigned long long)((v1 >> (32 * l)) & 0xffffffffu);
      }
    }
  }
  flush();
}

// Passes after the first: the listed changes' exact sums.  Bucket offsets per
// key (one warp per problem: its keys' exclusive prefix, the problem's region
// taken from a global counter; the counts and cursors are cleared for the next
// pass), the listed rows scattered under their keys (one reservation per key
// among a warp's rows), then one warp per 32 bucket entries sums runs of one
// key in registers (rows leaving a cluster negated).  ctl: [0] listed rows,
// [1] region counter, [2] bucket entries of the pass.
__global__ void chg_offsets_kernel(const BProb* __restrict__ probs, const int32_t* __restrict__ tcp, int ntc,
                                   int32_t* __restrict__ hist, int64_t* __restrict__ boff,
                                   int32_t* __restrict__ cursor, int* __restrict__ ctl) {
  const int lane = threadIdx.x & 31;
  const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= ntc) return;
  const BProb pr = probs[tcp[q]];
  const int nk = 2 * pr.k, k0 = 2 * pr.cnt_off;
  int tot = 0;
  for (int j0 = 0; j0 < nk; j0 += 32) tot += (j0 + lane < nk) ? hist[k0 + j0 + lane] : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
  if (tot == 0) return;
  int base = 0;
  if (lane == 0) base = atomicAdd(&ctl[1], tot);
  int64_t carry = __shfl_sync(0xffffffffu, base, 0);
  for (int j0 = 0; j0 < nk; j0 += 32) {
    const int j = j0 + lane;
    const int c = j < nk ? hist[k0 + j] : 0;
    int a = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, a, o);
      if (lane >= o) a += u;
    }
    if (j < nk) {
      boff[k0 + j] = carry + a - c;
      cursor[k0 + j] = 0;
      hist[k0 + j] = 0;
    }
    carry += __shfl_sync(0xffffffffu, a, 31);
  }
}

__global__ void __launch_bounds__(256) chg_scatter_kernel(const int32_t* __restrict__ chg_row,
                                                          const int32_t* __restrict__ chg_new,
                                                          const int32_t* __restrict__ chg_old, int cap,
                                                          const int64_t* __restrict__ boff,
                                                          int32_t* __restrict__ cursor, int32_t* __restrict__ b_row,
                                                          int32_t* __restrict__ b_key, int* __restrict__ ctl) {
  const int lane = threadIdx.x & 31;
  const int n = min(ctl[0], cap);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl[2] = ctl[1];  // this pass's bucket entries
    ctl[1] = 0;
  }
  const int stride = gridDim.x * blockDim.x;
  for (int e0 = blockIdx.x * blockDim.x; e0 < n; e0 += stride) {
    const int e = e0 + threadIdx.x;
    const bool v = e < n;
    const int row = v ? chg_row[e] : 0;
#pragma unroll
    for (int dir = 0; dir < 2; dir++) {
      const int key = v ? 2 * (dir ? chg_old[e] : chg_new[e]) + dir : -1;
      const unsigned grp = __match_any_sync(0xffffffffu, key);
      const int lead = __ffs(grp) - 1;
      int at = 0;
      if (v && lane == lead) at = atomicAdd(&cursor[key], __popc(grp));
      at = __shfl_sync(0xffffffffu, at, lead) + __popc(grp & ((1u << lane) - 1u));
      if (v) {
        const int64_t b = boff[key] + at;
        b_row[b] = row;
        b_key[b] = key;
      }
    }
  }
}

__global__ void __launch_bounds__(256) chg_sum_kernel(const BProb* __restrict__ probs,
                                                      const int32_t* __restrict__ gc_prob,
                                                      const int32_t* __restrict__ b_row,
                                                      const int32_t* __restrict__ b_key, const float* __restrict__ X,
                                                      unsigned long long* __restrict__ limbs, int* __restrict__ ctl) {
  const int lane = threadIdx.x & 31;
  const int64_t entries = ctl[2];
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl[0] = 0;  // the list, for the next pass
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; w0 < entries; w0 += nw * 32) {
    const int64_t e = w0 + lane;
    const int myrow = e < entries ? b_row[e] : 0;
    const int mykey = e < entries ? b_key[e] : -1;
    int cur = -1;
    BProb pr{};
    unsigned long long a0[4] = {0ull, 0ull, 0ull, 0ull}, a1[4] = {0ull, 0ull, 0ull, 0ull};
    auto flush = [&]() {
      if (cur < 0) return;
      unsigned long long* dst = limbs + pr.limb_off + (int64_t)((cur >> 1) - pr.cnt_off) * pr.d * pr.L;
#pragma unroll
      for (int l = 0; l < 4; l++) {
        if (l < pr.L) {
          if (lane < pr.d && a0[l]) atomicAdd(dst + (int64_t)lane * pr.L + l, a0[l]);
          if (lane + 32 < pr.d && a1[l]) atomicAdd(dst + (int64_t)(lane + 32) * pr.L + l, a1[l]);
        }
        a0[l] = 0ull;
        a1[l] = 0ull;
      }
    };
#pragma unroll 4
    for (int t = 0; t < 32; t++) {
      const int key = __shfl_sync(0xffffffffu, mykey, t);
      if (key < 0) break;
      const int row = __shfl_sync(0xffffffffu, myrow, t);
      if (key != cur) {
        flush();
        cur = key;
        pr = probs[gc_prob[key >> 1]];
      }
      const float* xr = X + pr.x_off + (int64_t)row * pr.d;
      const bool neg = (key & 1) != 0;
      const float x0 = lane < pr.d ? __ldg(xr + lane) : 0.0f;
      const float x1 = lane + 32 < pr.d ? __ldg(xr + lane + 32) : 0.0f;
      const unsigned __int128 v0 = fixed_of(x0, pr.e_lo, neg), v1 = fixed_of(x1, pr.e_lo, neg);
#pragma unroll
      for (int l = 0; l < 4; l++) {
        if (l < pr.L) {
          a0[l] += (unsigned long long)((v0 >> (32 * l)) & 0xffffffffu);
          a1[l] += (unsigned long long)((v1 >> (32 * l)) & 0xffffffffu);
        }
      }
    }
    flush();
  }
}

struct DevBuf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  ~DevBuf() {
    if (p) cudaFreeAsync(p, s);
  }
  int alloc(size_t b, cudaStream_t st) {
    s = st;
    if (cudaMallocFromPoolAsync(&p, b ? b : 16, lib_pool(), st) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      set_error("device allocation of %zu bytes failed", b);
      return ST_ENOMEM;
    }
    return ST_OK;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

// Launch shapes chosen per problem mix by timing the candidates once (the
// first middle iteration of the first call with that mix), cached per
// process.  Key: the sorted multiset of (d, k bucket) of the problems.
struct Tuned {
  int blocks_per_sm = 0;
};
std::mutex g_tune_mu;
std::map<std::vector<int>, Tuned> g_tuned;

}  // namespace
}  // namespace fuelg

using namespace fuelg;

extern "C" int fuelg_kmeans_batched(fuelg_kmeans_problem* probs, int32_t count, int32_t max_iter, int32_t order,
                                    int32_t precision, int32_t flags, fuelg_stats* stats) {
  if (count < 0 || (count > 0 && !probs) || max_iter < 1) {
    set_error("invalid batched kmeans arguments count=%d max_iter=%d", count, max_iter);
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
  if (precision == FUELG_PREC_AUTO) precision = FUELG_PREC_SPLIT_BF16;  // the screen takes the problems it serves
  for (int p = 0; p < count; p++) {
    const fuelg_kmeans_problem& q = probs[p];
    if (q.n < 1 || q.d < 1 || q.k < 1 || !q.data || !q.init || !q.out_centers || !q.out_labels) {
      set_error("invalid problem %d (n=%lld d=%d k=%d)", p, (long long)q.n, q.d, q.k);
      return ST_EINVAL;
    }
    if (q.n >= (1ll << 31) || (int64_t)q.k * q.d > (1ll << 28)) {
      set_error("problem %d too large for the batched engine", p);
      return ST_ENOTSUP;
    }
  }
  if (stats) memset(stats, 0, sizeof(*stats));
  if (count == 0) return ST_OK;
  cudaStream_t s;
  FUELG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct SG {
    cudaStream_t s;
    ~SG() { cudaStreamDestroy(s); }
  } sg{s};
  // the CUDA-core kernel's stream (forked from s and joined back every pass)
  cudaStream_t s2;
  FUELG_CUDA(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
  SG sg2{s2};
  cudaEvent_t ev_fork, ev_join;
  FUELG_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
  FUELG_CUDA(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
  struct EG2 {
    cudaEvent_t a, b;
    ~EG2() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } eg2{ev_fork, ev_join};
  const int64_t launches0 = launch_count();
  cudaEvent_t ev0, ev1, evh0, evh1;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  cudaEventCreate(&evh0);
  cudaEventCreate(&evh1);
  struct EG {
    cudaEvent_t a, b, c, d;
    ~EG() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      cudaEventDestroy(c);
      cudaEventDestroy(d);
    }
  } eg{ev0, ev1, evh0, evh1};
  cudaEventRecord(ev0, s);

  // layout
  const int P = count;
  std::vector<BProb> hp(P);
  std::vector<int64_t> xoff(P + 1, 0), kdb(P + 1, 0);
  std::vector<int32_t> rblk(P + 1, 0);
  int64_t xs = 0, cs = 0, ls = 0, ks = 0, kd = 0;
  int64_t items = 0;      // CUDA-core 256-row items
  int64_t all_items = 0;  // 256-row items of every problem (inertia)
  int64_t work = 0;
  std::vector<int32_t> tcp, tc_begin;  // tensor-core problems and their 128-row item starts
  int64_t tc_items = 0, tc_rows = 0;
  int tc_kmax = 1;
  int64_t rb = 0;
  for (int p = 0; p < P; p++) {
    const fuelg_kmeans_problem& q = probs[p];
    hp[p].x_off = xs;
    hp[p].n = q.n;
    hp[p].lab_off = ls;
    hp[p].c_off = cs;
    hp[p].cnt_off = (int32_t)ks;
    hp[p].d = q.d;
    hp[p].k = q.k;
    // tensor-core tier: split-BF16 screen for 32 <= d <= 64, k <= 256
    hp[p].tc = (precision != FUELG_PREC_FP32 && q.d >= 32 && q.d <= 64 && q.k <= 256) ? 1 : 0;
    hp[p].item_begin = (int32_t)items;
    hp[p].all_item_begin = (int32_t)all_items;
    hp[p].cost_begin = work;
    hp[p].item_cost = (int64_t)q.k * q.d + 64;  // distance work + per-row overhead
    const int64_t its = hp[p].tc ? 0 : (q.n + kItemRows - 1) / kItemRows;
    work += hp[p].item_cost * its;
    all_items += (q.n + kItemRows - 1) / kItemRows;
    if (hp[p].tc) {
      tcp.push_back(p);
      tc_begin.push_back((int32_t)tc_items);
      tc_items += (q.n + kTcRows - 1) / kTcRows;
      tc_rows += q.n;
      tc_kmax = std::max(tc_kmax, q.k);
    }
    xoff[p] = xs;
    kdb[p] = kd;
    rblk[p] = (int32_t)rb;
    xs += (q.n * q.d + 3) & ~3ll;  // 16-byte aligned rows for d % 4 == 0
    cs += (int64_t)q.k * q.d;
    ls += q.n;
    ks += q.k;
    kd += (int64_t)q.k * q.d;
    items += its;
    rb += (q.n * q.d + 65535) / 65536;
  }
  xoff[P] = xs;
  kdb[P] = kd;
  rblk[P] = (int32_t)rb;
  tc_begin.push_back((int32_t)tc_items);
  // 32-bit item starts; centre keys 2 gc + 1 (gc < ks) of the change list are 32-bit
  if (all_items >= (1ll << 31) || tc_items >= (1ll << 31) || ks >= (1ll << 30)) {
    set_error("batch too large");
    return ST_ENOTSUP;
  }
  DevBuf dX, dC, dLab, dCnt, dOff, dRb, dRange, dProbs, dKdb, dPchg, dConv, dLast, dIter, dInert, dLimbs, dTcp,
      dTcb, dSt, dUnd, dCtaB;
  FUELG_TRY(dX.alloc(sizeof(float) * xs, s));
  FUELG_TRY(dC.alloc(sizeof(float) * cs, s));
  FUELG_TRY(dLab.alloc(sizeof(int32_t) * ls, s));
  FUELG_TRY(dCnt.alloc(sizeof(int32_t) * ks, s));
  FUELG_TRY(dOff.alloc(sizeof(int64_t) * (P + 1), s));
  FUELG_TRY(dRb.alloc(sizeof(int32_t) * (P + 1), s));
  FUELG_TRY(dRange.alloc(sizeof(int) * 3 * P, s));
  FUELG_CUDA(cudaMemsetAsync(dX.p, 0, sizeof(float) * xs, s));  // alignment padding between problems reads as 0
  for (int p = 0; p < P; p++) {
    FUELG_CUDA(cudaMemcpyAsync(dX.as<float>() + hp[p].x_off, probs[p].data, sizeof(float) * probs[p].n * probs[p].d,
                               cudaMemcpyDefault, s));
    FUELG_CUDA(cudaMemcpyAsync(dC.as<float>() + hp[p].c_off, probs[p].init, sizeof(float) * probs[p].k * probs[p].d,
                               cudaMemcpyDefault, s));
  }
  FUELG_CUDA(cudaMemcpyAsync(dOff.p, xoff.data(), sizeof(int64_t) * (P + 1), cudaMemcpyHostToDevice, s));
  FUELG_CUDA(cudaMemcpyAsync(dRb.p, rblk.data(), sizeof(int32_t) * (P + 1), cudaMemcpyHostToDevice, s));
  {
    std::vector<int> init(3 * P);
    for (int p = 0; p < P; p++) {
      init[3 * p] = 1 << 30;
      init[3 * p + 1] = -(1 << 30);
      init[3 * p + 2] = 0;
    }
    FUELG_CUDA(cudaMemcpyAsync(dRange.p, init.data(), sizeof(int) * 3 * P, cudaMemcpyHostToDevice, s));
    FUELG_CUDA(cudaStreamSynchronize(s));  // `init` leaves scope
  }
  if (rb > 0) {
    batched_range_kernel<<<(unsigned)rb, 256, 0, s>>>(dX.as<float>(), dOff.as<int64_t>(), dRb.as<int32_t>(), P,
                                                      dRange.as<int>());
    note_launch();
    FUELG_CUDA(cudaGetLastError());
  }
  std::vector<int> hr(3 * P);
  FUELG_CUDA(cudaMemcpyAsync(hr.data(), dRange.p, sizeof(int) * 3 * P, cudaMemcpyDeviceToHost, s));
  FUELG_CUDA(cudaStreamSynchronize(s));
  int64_t limbs_total = 0;
  for (int p = 0; p < P; p++) {
    int e_lo = hr[3 * p], e_hi = hr[3 * p + 1];
    if (e_lo > e_hi) e_lo = e_hi = 0;  // all zeros
    int logn = 0;
    while ((1ll << logn) <= hp[p].n) logn++;
    const int bits = (e_hi - e_lo + 1) + logn + 1;
    const int L = (bits + 31) / 32;
    hp[p].active = (hr[3 * p + 2] == 0 && L <= 4) ? 1 : 0;
    hp[p].L = std::max(1, std::min(4, L));
    hp[p].e_lo = e_lo;
    hp[p].limb_off = limbs_total;
    limbs_total += (int64_t)hp[p].k * hp[p].d * hp[p].L;
  }
  FUELG_TRY(dLimbs.alloc(sizeof(unsigned long long) * limbs_total, s));
  FUELG_TRY(dProbs.alloc(sizeof(BProb) * P, s));
  FUELG_TRY(dKdb.alloc(sizeof(int64_t) * (P + 1), s));
  FUELG_TRY(dPchg.alloc(sizeof(int32_t) * P, s));
  FUELG_TRY(dConv.alloc(sizeof(int32_t) * P, s));
  FUELG_TRY(dLast.alloc(sizeof(int32_t) * P, s));
  FUELG_TRY(dIter.alloc(sizeof(int32_t), s));
  FUELG_TRY(dInert.alloc(sizeof(double) * P, s));
  FUELG_CUDA(cudaMemcpyAsync(dProbs.p, hp.data(), sizeof(BProb) * P, cudaMemcpyHostToDevice, s));
  const int ntc = (int)tcp.size();
  FUELG_TRY(dTcp.alloc(sizeof(int32_t) * std::max(1, ntc), s));
  FUELG_TRY(dTcb.alloc(sizeof(int32_t) * (ntc + 1), s));
  FUELG_TRY(dSt.alloc(sizeof(int) * 4, s));
  if (ntc) FUELG_CUDA(cudaMemcpyAsync(dTcp.p, tcp.data(), sizeof(int32_t) * ntc, cudaMemcpyHostToDevice, s));
  FUELG_CUDA(cudaMemcpyAsync(dTcb.p, tc_begin.data(), sizeof(int32_t) * (ntc + 1), cudaMemcpyHostToDevice, s));
  FUELG_CUDA(cudaMemsetAsync(dSt.p, 0, sizeof(int) * 4, s));
  FUELG_CUDA(cudaMemcpyAsync(dKdb.p, kdb.data(), sizeof(int64_t) * (P + 1), cudaMemcpyHostToDevice, s));
  FUELG_CUDA(cudaMemsetAsync(dLimbs.p, 0, sizeof(unsigned long long) * limbs_total, s));
  FUELG_CUDA(cudaMemsetAsync(dCnt.p, 0, sizeof(int32_t) * ks, s));
  FUELG_CUDA(cudaMemsetAsync(dPchg.p, 0, sizeof(int32_t) * P, s));
  FUELG_CUDA(cudaMemsetAsync(dConv.p, 0, sizeof(int32_t) * P, s));
  FUELG_CUDA(cudaMemsetAsync(dIter.p, 0, sizeof(int32_t), s));
  FUELG_CUDA(cudaMemsetAsync(dInert.p, 0, sizeof(double) * P, s));

  // centre staging sized for the problems this kernel serves (those without
  // the tensor-core screen): more resident CTAs when their centres are small
  int ccap = 4;
  for (int p = 0; p < P; p++)
    if (!hp[p].tc) ccap = std::max<int64_t>(ccap, std::min<int64_t>(kCentreCap, (int64_t)hp[p].k * hp[p].d));
  ccap = (ccap + 3) & ~3;
  // With tensor-core problems in the batch the CUDA-core kernel runs beside the
  // screen (its own stream, joined before the centre update): with the centres
  // of the problems it serves (d < 32) one of its CTAs fits beside the
  // screen's on every SM, and its warps use the issue slots the screen's
  // epilogue leaves.
  const bool concurrent = items > 0 && tc_items > 0;
  const size_t smem = sizeof(float) * ccap + sizeof(unsigned long long) * kAggCap + sizeof(int) * 256;
  auto k_init = order == FUELG_ORDER_X86 ? batched_assign_kernel<KIND_PAIRWISE, ORDER_X86>
                                         : batched_assign_kernel<KIND_PAIRWISE, ORDER_ARM>;
  auto k_iter = order == FUELG_ORDER_X86 ? batched_assign_kernel<KIND_SQDIST, ORDER_X86>
                                         : batched_assign_kernel<KIND_SQDIST, ORDER_ARM>;
  FUELG_CUDA(cudaFuncSetAttribute(k_init, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  FUELG_CUDA(cudaFuncSetAttribute(k_iter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  auto t_init = order == FUELG_ORDER_X86 ? batched_tc_assign_kernel<KIND_PAIRWISE, ORDER_X86>
                                         : batched_tc_assign_kernel<KIND_PAIRWISE, ORDER_ARM>;
  auto t_iter = order == FUELG_ORDER_X86 ? batched_tc_assign_kernel<KIND_SQDIST, ORDER_X86>
                                         : batched_tc_assign_kernel<KIND_SQDIST, ORDER_ARM>;
  const size_t tsmem = kTcSmem;
  FUELG_CUDA(cudaFuncSetAttribute(t_init, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsmem));
  FUELG_CUDA(cudaFuncSetAttribute(t_iter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsmem));
  BTcArgs ta{};
  ta.tcp = dTcp.as<int32_t>();
  ta.item_begin = dTcb.as<int32_t>();
  ta.ntc = ntc;
  ta.items = (int)tc_items;
  {
    // operand rounding of hi + lo (3.01 * 2^-16) + FP32 accumulation of 3 x 64 products
    const double rel = 3.01 * std::ldexp(1.0, -16) + 3.0 * 64 * std::ldexp(1.0, -23) * (1.0 + std::ldexp(1.0, -7));
    ta.alpha = (float)(2.0 * rel * 1.01);
  }
  ta.status = dSt.as<int>();
  ta.undecided = reinterpret_cast<unsigned long long*>(dSt.as<int>() + 2);
  ta.und_n = dSt.as<int>() + 1;
  ta.und_w = (tc_kmax + 31) / 32;
  FUELG_TRY(dUnd.alloc(sizeof(int32_t) * (2 + ta.und_w) * std::max<int64_t>(1, tc_rows), s));
  ta.und_p = dUnd.as<int32_t>();
  ta.und_i = dUnd.as<int32_t>() + std::max<int64_t>(1, tc_rows);
  ta.und_m = reinterpret_cast<uint32_t*>(dUnd.as<int32_t>() + 2 * std::max<int64_t>(1, tc_rows));
  // the first pass's bucketed sums of the tensor-core problems: the bucket
  // array (row, cluster) reuses the undecided list's memory once the first
  // re-score is done; rows of each active problem from row_base[q]
  DevBuf dBoff, dCur, dGcp, dRowB;
  int64_t tc_entries = 0;
  if (tc_items > 0) {
    std::vector<int64_t> rowb(ntc + 1);
    for (int q = 0; q < ntc; q++) {
      rowb[q] = tc_entries;
      if (hp[tcp[q]].active) tc_entries += hp[tcp[q]].n;
    }
    rowb[ntc] = tc_entries;
    std::vector<int32_t> gcp(std::max<int64_t>(1, ks));
    for (int p = 0; p < P; p++)
      for (int j = 0; j < hp[p].k; j++) gcp[hp[p].cnt_off + j] = p;
    FUELG_TRY(dBoff.alloc(sizeof(int64_t) * std::max<int64_t>(1, ks), s));
    FUELG_TRY(dCur.alloc(sizeof(int32_t) * std::max<int64_t>(1, ks), s));
    FUELG_TRY(dGcp.alloc(sizeof(int32_t) * std::max<int64_t>(1, ks), s));
    FUELG_TRY(dRowB.alloc(sizeof(int64_t) * (ntc + 1), s));
    FUELG_CUDA(cudaMemcpyAsync(dGcp.p, gcp.data(), sizeof(int32_t) * gcp.size(), cudaMemcpyHostToDevice, s));
    FUELG_CUDA(cudaMemcpyAsync(dRowB.p, rowb.data(), sizeof(int64_t) * (ntc + 1), cudaMemcpyHostToDevice, s));
  }
  // later passes: the change list (room for half the tensor-core rows; the
  // rest of a pass's changes take the epilogue's direct sums), its per-key
  // counts, offsets and cursors, the buckets and three control words
  DevBuf dChg, dHist, dKoff, dKcur, dBk, dCtl;
  // (bucket positions and the region counter are 32-bit: at most 2^29 listed rows)
  const int chg_cap = (int)std::max<int64_t>(1, std::min<int64_t>(tc_rows / 2, 1ll << 29));
  if (tc_items > 0) {
    FUELG_TRY(dChg.alloc(sizeof(int32_t) * 3 * (size_t)chg_cap, s));
    FUELG_TRY(dHist.alloc(sizeof(int32_t) * 2 * std::max<int64_t>(1, ks), s));
    FUELG_TRY(dKoff.alloc(sizeof(int64_t) * 2 * std::max<int64_t>(1, ks), s));
    FUELG_TRY(dKcur.alloc(sizeof(int32_t) * 2 * std::max<int64_t>(1, ks), s));
    FUELG_TRY(dBk.alloc(sizeof(int32_t) * 4 * (size_t)chg_cap, s));
    FUELG_TRY(dCtl.alloc(sizeof(int) * 4, s));
    FUELG_CUDA(cudaMemsetAsync(dHist.p, 0, sizeof(int32_t) * 2 * std::max<int64_t>(1, ks), s));
    FUELG_CUDA(cudaMemsetAsync(dCtl.p, 0, sizeof(int) * 4, s));
    ta.chg_row = dChg.as<int32_t>();
    ta.chg_new = ta.chg_row + chg_cap;
    ta.chg_old = ta.chg_new + chg_cap;
    ta.hist = dHist.as<int32_t>();
    ta.chg_n = dCtl.as<int>();
    ta.chg_cap = chg_cap;
  }
  auto r_init = order == FUELG_ORDER_X86 ? batched_rescore_kernel<KIND_PAIRWISE, ORDER_X86>
                                         : batched_rescore_kernel<KIND_PAIRWISE, ORDER_ARM>;
  auto r_iter = order == FUELG_ORDER_X86 ? batched_rescore_kernel<KIND_SQDIST, ORDER_X86>
                                         : batched_rescore_kernel<KIND_SQDIST, ORDER_ARM>;
  int sms = 152;
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  // tuned launch shape for this mix of (d, k) buckets
  std::vector<int> key;
  for (int p = 0; p < P; p++) key.push_back(hp[p].d * 16 + std::min(15, (int)std::log2((double)hp[p].k)));
  std::sort(key.begin(), key.end());
  int bps = 0;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) bps = it->second.blocks_per_sm;
  }
  auto grid_for = [&](int b) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(items, (int64_t)sms * b)); };
  // one persistent screen CTA per SM, each over a contiguous range of items of
  // equal estimated cost (row loads + an epilogue that grows with the centres)
  const unsigned tc_grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(tc_items, (int64_t)sms));
  {
    std::vector<double> icost(ntc);
    double total = 0.0;
    for (int q = 0; q < ntc; q++) {
      const int kp = (hp[tcp[q]].k + 15) & ~15;
      icost[q] = 64.0 + 2.0 * kp;
      total += icost[q] * (tc_begin[q + 1] - tc_begin[q]);
    }
    std::vector<int64_t> cb(tc_grid + 1, 0);
    cb[tc_grid] = tc_items;
    double acc = 0.0;
    int q = 0;
    for (unsigned c = 1; c < tc_grid; c++) {
      const double target = total * c / tc_grid;
      while (q < ntc && acc + icost[q] * (tc_begin[q + 1] - tc_begin[q]) < target) {
        acc += icost[q] * (tc_begin[q + 1] - tc_begin[q]);
        q++;
      }
      int64_t at = tc_items;
      if (q < ntc) at = std::min<int64_t>(tc_begin[q + 1], tc_begin[q] + (int64_t)std::ceil((target - acc) / icost[q]));
      cb[c] = std::max(cb[c - 1], at);
    }
    FUELG_TRY(dCtaB.alloc(sizeof(int64_t) * (tc_grid + 1), s));
    FUELG_CUDA(cudaMemcpyAsync(dCtaB.p, cb.data(), sizeof(int64_t) * (tc_grid + 1), cudaMemcpyHostToDevice, s));
    ta.cta_begin = dCtaB.as<int64_t>();
  }
  const unsigned mean_grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((kd + 255) / 256, (int64_t)sms * 8));
  const int fixed = (flags & FUELG_LLOYD_FIXED_ITERS) ? 1 : 0;
  (void)fixed;  // every pass runs; the reported count follows the changed == 0 stop unless fixed

  auto pass = [&](bool first, bool write, unsigned grid) -> int {
    cudaStream_t sc = s;
    if (concurrent) {
      FUELG_CUDA(cudaEventRecord(ev_fork, s));
      FUELG_CUDA(cudaStreamWaitEvent(s2, ev_fork, 0));
      sc = s2;
    }
    if (items > 0) {
      if (first)
        k_init<<<grid, kItemRows, smem, sc>>>(dProbs.as<BProb>(), P, (int)items, dX.as<float>(), dC.as<float>(),
                                             dLab.as<int32_t>(), dLimbs.as<unsigned long long>(), dCnt.as<int32_t>(),
                                             dPchg.as<int32_t>(), 1, work, ccap);
      else
        k_iter<<<grid, kItemRows, smem, sc>>>(dProbs.as<BProb>(), P, (int)items, dX.as<float>(), dC.as<float>(),
                                             dLab.as<int32_t>(), dLimbs.as<unsigned long long>(), dCnt.as<int32_t>(),
                                             dPchg.as<int32_t>(), 0, work, ccap);
      note_launch();
    }
    if (tc_items > 0) {
      (first ? t_init : t_iter)<<<tc_grid, kTcThreads, tsmem, s>>>(dProbs.as<BProb>(), ta, dX.as<float>(),
                                                                 dC.as<float>(), dLab.as<int32_t>(),
                                                                 dLimbs.as<unsigned long long>(),
                                                                 dCnt.as<int32_t>(), dPchg.as<int32_t>(),
                                                                 first ? 1 : 0);
      note_launch();
      (first ? r_init : r_iter)<<<sms * 8, 256, 0, s>>>(dProbs.as<BProb>(), ta.und_p, ta.und_i, ta.und_m, ta.und_w,
                                                        ta.und_n,
                                                        dX.as<float>(), dC.as<float>(), dLab.as<int32_t>(),
                                                        dLimbs.as<unsigned long long>(), dCnt.as<int32_t>(),
                                                        dPchg.as<int32_t>(), first ? 1 : 0);
      note_launch();
      if (first) {
        int32_t* b_row = dUnd.as<int32_t>();
        int32_t* b_gc = b_row + std::max<int64_t>(1, tc_rows);
        tc_first_offsets_kernel<<<(unsigned)((ntc * 32 + 255) / 256), 256, 0, s>>>(
            dProbs.as<BProb>(), ta.tcp, ntc, dRowB.as<int64_t>(), dCnt.as<int32_t>(), dBoff.as<int64_t>(),
            dCur.as<int32_t>());
        note_launch();
        tc_first_scatter_kernel<<<(unsigned)tc_items, kTcRows, 0, s>>>(dProbs.as<BProb>(), ta.tcp, ta.item_begin, ntc,
                                                                       dLab.as<int32_t>(), dBoff.as<int64_t>(),
                                                                       dCur.as<int32_t>(), b_row, b_gc);
        note_launch();
        if (tc_entries > 0) {
          tc_first_sum_kernel<<<(unsigned)((tc_entries + 255) / 256), 256, 0, s>>>(
              dProbs.as<BProb>(), dGcp.as<int32_t>(), tc_entries, b_row, b_gc, dX.as<float>(),
              dLimbs.as<unsigned long long>());
          note_launch();
        }
      } else {
        int32_t* b_row = dBk.as<int32_t>();
        int32_t* b_key = b_row + 2 * (size_t)chg_cap;
        chg_offsets_kernel<<<(unsigned)((ntc * 32 + 255) / 256), 256, 0, s>>>(
            dProbs.as<BProb>(), ta.tcp, ntc, dHist.as<int32_t>(), dKoff.as<int64_t>(), dKcur.as<int32_t>(),
            dCtl.as<int>());
        note_launch();
        chg_scatter_kernel<<<(unsigned)(sms * 4), 256, 0, s>>>(ta.chg_row, ta.chg_new, ta.chg_old, chg_cap,
                                                               dKoff.as<int64_t>(), dKcur.as<int32_t>(), b_row, b_key,
                                                               dCtl.as<int>());
        note_launch();
        chg_sum_kernel<<<(unsigned)(sms * 8), 256, 0, s>>>(dProbs.as<BProb>(), dGcp.as<int32_t>(), b_row, b_key,
                                                           dX.as<float>(), dLimbs.as<unsigned long long>(),
                                                           dCtl.as<int>());
        note_launch();
      }
    }
    if (concurrent) {
      FUELG_CUDA(cudaEventRecord(ev_join, s2));
      FUELG_CUDA(cudaStreamWaitEvent(s, ev_join, 0));
    }
    // canonical counters every pass; new centres only when another pass follows
    batched_mean_kernel<<<mean_grid, 256, 0, s>>>(dProbs.as<BProb>(), P, dKdb.as<int64_t>(), kd,
                                                  dLimbs.as<unsigned long long>(), dCnt.as<int32_t>(), dC.as<float>(),
                                                  write ? 1 : 0);
    note_launch();
    batched_step_kernel<<<1, 512, 0, s>>>(P, dPchg.as<int32_t>(), dConv.as<int32_t>(), dLast.as<int32_t>(),
                                          dIter.as<int32_t>(), dSt.as<int>() + 1);
    note_launch();
    FUELG_CUDA(cudaGetLastError());
    return ST_OK;
  };
  cudaEventRecord(evh0, s);
  // iteration 1: initial assignment (pairwise order), every point enters
  FUELG_TRY(pass(true, max_iter > 1, grid_for(bps ? bps : 3)));
  int done = 1;
  // autotune: time the candidate shapes on the first middle iterations
  if (!bps && max_iter > 2) {
    float best_ms = 1e30f;
    int best_b = 3;
    for (int b : {2, 4, 8}) {
      if (done >= max_iter - 1) break;
      cudaEvent_t t0, t1;
      cudaEventCreate(&t0);
      cudaEventCreate(&t1);
      cudaEventRecord(t0, s);
      FUELG_TRY(pass(false, true, grid_for(b)));
      cudaEventRecord(t1, s);
      FUELG_CUDA(cudaEventSynchronize(t1));
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, t0, t1);
      cudaEventDestroy(t0);
      cudaEventDestroy(t1);
      done++;
      if (ms < best_ms) {
        best_ms = ms;
        best_b = b;
      }
    }
    bps = best_b;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[key].blocks_per_sm = bps;
  }
  if (!bps) bps = 3;
  // middle iterations: one captured graph, replayed
  const int middle = std::max(0, max_iter - 1 - done);
  if (middle > 0) {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    FUELG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const int64_t l0 = launch_count();
    const int rc = pass(false, true, grid_for(bps));
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (rc != ST_OK) return rc;
    if (ce != cudaSuccess) {
      set_error("graph capture failed: %s", cudaGetErrorString(ce));
      return ST_ECUDA;
    }
    const int64_t per_pass = launch_count() - l0;
    note_launch((int)(-per_pass));  // counted per replay below
    ce = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
      set_error("graph instantiate failed: %s", cudaGetErrorString(ce));
      return ST_ECUDA;
    }
    for (int i = 0; i < middle; i++) {
      ce = cudaGraphLaunch(exec, s);
      if (ce != cudaSuccess) break;
      note_launch((int)per_pass);
    }
    cudaGraphExecDestroy(exec);
    FUELG_CUDA(ce);
    done += middle;
  }
  // last iteration: assignment, no centre update
  if (done < max_iter) {
    FUELG_TRY(pass(false, false, grid_for(bps)));
    done++;
  }
  cudaEventRecord(evh1, s);
  {
    const unsigned ig = (unsigned)std::max<int64_t>(1, std::min<int64_t>(all_items, (int64_t)sms * 8));
    batched_inertia_kernel<<<ig, kItemRows, 0, s>>>(dProbs.as<BProb>(), P, (int)all_items, dX.as<float>(),
                                                    dC.as<float>(), dLab.as<int32_t>(), dInert.as<double>());
    note_launch();
    FUELG_CUDA(cudaGetLastError());
  }
  // results
  std::vector<int32_t> conv(P), lab32;
  std::vector<double> inert(P);
  FUELG_CUDA(cudaMemcpyAsync(conv.data(), dConv.p, sizeof(int32_t) * P, cudaMemcpyDeviceToHost, s));
  FUELG_CUDA(cudaMemcpyAsync(inert.data(), dInert.p, sizeof(double) * P, cudaMemcpyDeviceToHost, s));
  lab32.resize(ls);
  FUELG_CUDA(cudaMemcpyAsync(lab32.data(), dLab.p, sizeof(int32_t) * ls, cudaMemcpyDeviceToHost, s));
  for (int p = 0; p < P; p++)
    FUELG_CUDA(cudaMemcpyAsync(probs[p].out_centers, dC.as<float>() + hp[p].c_off,
                               sizeof(float) * probs[p].k * probs[p].d, cudaMemcpyDefault, s));
  int hst4[4] = {0, 0, 0, 0};
  FUELG_CUDA(cudaMemcpyAsync(hst4, dSt.p, sizeof(hst4), cudaMemcpyDeviceToHost, s));
  cudaEventRecord(ev1, s);
  FUELG_CUDA(cudaStreamSynchronize(s));
  const int hst = hst4[0];
  unsigned long long undecided_rows = 0;
  memcpy(&undecided_rows, hst4 + 2, sizeof(undecided_rows));
  if (hst & DEV_TIMEOUT) {
    set_error("a device wait timed out");
    return ST_ETIMEOUT;
  }
  int64_t d2h = (int64_t)sizeof(int32_t) * ls + (int64_t)sizeof(float) * cs;
  for (int p = 0; p < P; p++) {
    fuelg_kmeans_problem& q = probs[p];
    if (!hp[p].active) {
      q.status = ST_ENOTSUP;
      q.out_iters = 0;
      q.out_inertia = 0.0;
      continue;
    }
    for (int64_t i = 0; i < q.n; i++) q.out_labels[i] = lab32[hp[p].lab_off + i];
    const int it = (!(flags & FUELG_LLOYD_FIXED_ITERS) && conv[p] > 0) ? conv[p] : max_iter;
    q.out_iters = it;
    q.out_inertia = inert[p];
    q.status = ST_OK;
  }
  if (stats) {
    float ms = 0.0f, hms = 0.0f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    cudaEventElapsedTime(&hms, evh0, evh1);
    stats->device_ms = ms;
    stats->hot_kernel_ms = hms;
    stats->hot_kernel_launches = max_iter;
    stats->h2d_bytes = (int64_t)sizeof(float) * (xs + cs);
    stats->d2h_bytes = d2h;
    int64_t evals = 0;
    for (int p = 0; p < P; p++) evals += hp[p].n * hp[p].k;
    stats->distance_evals = evals * max_iter;
    stats->iterations = max_iter;
    stats->rescored = (int64_t)undecided_rows;
    stats->precision_used = tc_items > 0 ? precision : 0;
    stats->kernel_launches = (int32_t)(launch_count() - launches0);
  }
  return ST_OK;
}
