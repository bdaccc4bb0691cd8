// fuelg_knn_tc.cu -- tensor-core (tcgen05 / TMEM / TMA) linear-scan kNN.
//
// Each CTA owns 128 query rows: their BF16 copy stays resident in shared
// memory while the index streams through in 256-row tiles.  One thread issues
// tcgen05.mma (M=128, N=256, K=16, BF16 operands, FP32 accumulators in TMEM,
// two accumulators alternating); four epilogue warps read their query's 256
// dot products with tcgen05.ld, form D~ = |q|^2 + |x|^2 - 2 q.x and keep the
// query's kk2 best (D~, index) keys with the same threshold-filter + sorted
// list scheme as the exact scan.
//
// Exact mode: when every value of the index and the queries is an integer of
// magnitude <= 256 and 2 d V^2 < 2^24, every BF16 product, every FP32 partial
// sum and D~ itself are exact integers below 2^24 -- D~ then IS fuel's f32
// distance (src/distance/squared_euclidean.rs sums the same exact integers),
// whatever the summation order, and the screen keys are final.
// Otherwise the kk2 = kk + margin best screened keys are re-scored with the
// reference's f32 operation order and kept only when a rigorous bound proves
// every unscreened point is strictly worse than the kk-th re-scored key; the
// queries that fail the proof are re-run through the exact scan.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include <cuda_fp16.h>

#include "fuelg_common.cuh"
#include "fuelg_internal.h"
#include "fuelg_tc_common.cuh"

namespace fuelg {

using namespace tcx;

namespace {

constexpr int QM = 128;        // queries per CTA (UMMA M)
constexpr int XN = 128;        // index rows per tile (UMMA N)
constexpr int kEpiWarps = 4;   // epilogue warps: one per TMEM lane quarter
constexpr int kEpi = 32 * kEpiWarps;
constexpr int kThreadsKT = 64 + kEpi;
constexpr int kCtasPerSm = 2;  // 2 x (2 TMEM buffers of XN columns) = all 512 columns
constexpr int kSmemPerCta = 112 * 1024;
constexpr int kApp = 256;      // appended candidates per query between compactions

struct KnnTcArgs {
  int64_t m, n;
  int kc;        // K chunks of 64
  int ks_last;   // K steps of 16 with data in the last chunk (1..4)
  int kk2;       // keys kept per query (the list stride)
  const int32_t* row_k;  // per query row k (rows keep kk2_of(row_k[q]) <= kk2 keys), or nullptr
  int margin_mode;  // kk2_of mode of this launch
  int exact;     // D~ is exact (integer data)
  int split;     // hi + lo BF16 operands (three products)
  int stages;
  const float* qn2;  // |q|^2 per query row
  const float* xn2;  // |x|^2 per index row (padded rows: 0)
  float xmax_n2;     // max |x|^2 over the index (filter slack)
  uint64_t* lists;     // [CTA][QM][kk2 + kApp]: kept keys + append log of the rows a CTA works on
  uint64_t* out_keys;  // [piece][QM][kk2]: each piece's kept keys
  // Work decomposition: CTA c works through pieces [cta_pb[c], cta_pb[c+1]);
  // piece p = query block piece_qb[p] against index tiles [piece_t0[p], piece_t1[p]).
  const int32_t* piece_qb;
  const int32_t* piece_t0;
  const int32_t* piece_t1;
  const int32_t* cta_pb;
  uint32_t idesc;
  int* status;
  const volatile int* cancel;
  uint64_t wait_ns;  // limit of the pipeline waits (pipeline_wait_ns)
};


constexpr int kSel = 8;  // keys per lane in a selection (appended or prefix): 256 per warp
constexpr float kF16Max = 65504.0f;  // largest finite FP16 value

// Screened keys kept for a query of k neighbours: k plus the margin the
// error-bound proof needs.  Margin modes: 0 exact screened squared distances
// (none), 1 BF16 / split BF16 (max(8, k/8)), 2 FP16 (max(8, k/4): its larger
// screen error needs more ranks between the k-th and the last kept key).
__host__ __device__ __forceinline__ int kk2_of(int k, int mode) {
  const int m = mode == 0 ? 0 : (mode == 1 ? k / 8 : k / 4);
  return mode == 0 ? k : k + (m > 8 ? m : 8);
}

// Number of held keys below t over the warp.
__device__ __forceinline__ int warp_count_hi_below(const uint32_t (&hi)[2 * kSel], uint32_t t) {
  int c = 0;
#pragma unroll
  for (int i = 0; i < 2 * kSel; i++) c += hi[i] < t ? 1 : 0;
  return __reduce_add_sync(0xffffffffu, c);
}

// Warp-cooperative selection for one query: the union of its
// na (<= 256) appended keys and its plen (<= kk <= 256) kept keys is reduced
// to its kk smallest, written unsorted back over cur[0, min(kk, na + plen)).
// The kk-th smallest key is found by a bitwise binary search over the
// distance word (counting with a warp reduction) and, only when several keys
// share that distance, over the index word; keys are unique.  Each search
// starts below the bits that the smallest and largest candidate word share.
// In place: every lane has read its keys before the first warp-wide
// exchange, and every store comes after the last.  No shared memory, no sort.
// Returns the kk-th smallest key, or KEY_NONE while fewer than kk are held,
// on every lane.
__device__ __noinline__ uint64_t warp_select(const uint64_t* __restrict__ app, int na, uint64_t* cur, int plen,
                                             int kk, int lane) {
  uint64_t key[2 * kSel];
#pragma unroll
  for (int i = 0; i < kSel; i++) {
    const int e = lane + 32 * i;
    key[i] = e < na ? app[e] : KEY_NONE;
    key[kSel + i] = e < plen ? cur[e] : KEY_NONE;
  }
  uint32_t hi[2 * kSel];
  uint32_t hmin = 0xffffffffu, hmax = 0;
#pragma unroll
  for (int i = 0; i < 2 * kSel; i++) {
    hi[i] = (uint32_t)(key[i] >> 32);
    if (key[i] != KEY_NONE) {
      hmin = min(hmin, hi[i]);
      hmax = max(hmax, hi[i]);
    }
  }
  const int total = na + plen;
  uint64_t kth = KEY_NONE;
  if (total >= kk) {
    // the kk-th distance word lies in [hmin, hmax]: search the bits below
    // their common prefix only
    hmin = __reduce_min_sync(0xffffffffu, hmin);
    hmax = __reduce_max_sync(0xffffffffu, hmax);
    int top = hmin == hmax ? -1 : 31 - __clz(hmin ^ hmax);
    uint32_t H = top >= 0 ? hmin & ~((2u << top) - 1u) : hmin;
    for (int b = top; b >= 0; b--) {
      const uint32_t t = H | (1u << b);
      if (warp_count_hi_below(hi, t) < kk) H = t;
    }
    // keys below H: fewer than kk; keys with hi == H: the rest is taken from them
    const int below = warp_count_hi_below(hi, H);
    int eq = 0;
    uint32_t lmin = 0xffffffffu, lmax = 0;
#pragma unroll
    for (int i = 0; i < 2 * kSel; i++)
      if (hi[i] == H) {
        eq++;
        lmin = min(lmin, (uint32_t)key[i]);
        lmax = max(lmax, (uint32_t)key[i]);
      }
    eq = __reduce_add_sync(0xffffffffu, eq);
    lmax = __reduce_max_sync(0xffffffffu, lmax);
    const int need = kk - below;
    uint32_t Lo = lmax;
    if (eq != need) {
      lmin = __reduce_min_sync(0xffffffffu, lmin);
      top = lmin == lmax ? -1 : 31 - __clz(lmin ^ lmax);
      Lo = top >= 0 ? lmin & ~((2u << top) - 1u) : lmin;
      for (int b = top; b >= 0; b--) {
        const uint32_t t = Lo | (1u << b);
        int c = 0;
#pragma unroll
        for (int i = 0; i < 2 * kSel; i++) c += (hi[i] == H && (uint32_t)key[i] < t) ? 1 : 0;
        if (__reduce_add_sync(0xffffffffu, c) < need) Lo = t;
      }
    }
    kth = ((uint64_t)H << 32) | Lo;
  }
  // compact the kept keys: lane offsets by a warp scan of per-lane counts
  int mine = 0;
#pragma unroll
  for (int i = 0; i < 2 * kSel; i++) mine += (key[i] != KEY_NONE && key[i] <= kth) ? 1 : 0;
  int incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  int pos = incl - mine;
#pragma unroll
  for (int i = 0; i < 2 * kSel; i++)
    if (key[i] != KEY_NONE && key[i] <= kth) cur[pos++] = key[i];
  __syncwarp();
  return total >= kk ? kth : KEY_NONE;
}

// 16-way register select without local memory: v[j] for a runtime j.
__device__ __forceinline__ float sel16(const float (&v)[16], int j) {
  float l1[8], l2[4], l3[2];
#pragma unroll
  for (int i = 0; i < 8; i++) l1[i] = (j & 1) ? v[2 * i + 1] : v[2 * i];
#pragma unroll
  for (int i = 0; i < 4; i++) l2[i] = (j & 2) ? l1[2 * i + 1] : l1[2 * i];
#pragma unroll
  for (int i = 0; i < 2; i++) l3[i] = (j & 4) ? l2[2 * i + 1] : l2[2 * i];
  return (j & 8) ? l3[1] : l3[0];
}

// Sort each row of kk2 (<= 256) keys ascending: one warp per row, 8 keys
// per lane (element e = lane * 8 + r), bitonic network in registers.
__global__ void __launch_bounds__(256) sort_rows_kernel(uint64_t* __restrict__ keys, int64_t rows, int kk2) {
  const int lane = threadIdx.x & 31;
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (row >= rows) return;
  uint64_t* kr = keys + row * kk2;
  uint64_t v[8];
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int e = lane * 8 + r;
    v[r] = e < kk2 ? kr[e] : KEY_NONE;
  }
#pragma unroll
  for (int k2 = 2; k2 <= 256; k2 <<= 1) {
#pragma unroll
    for (int j = k2 >> 1; j > 0; j >>= 1) {
      if (j >= 8) {
#pragma unroll
        for (int r = 0; r < 8; r++) {
          const uint64_t o = ((uint64_t)__shfl_xor_sync(0xffffffffu, (uint32_t)(v[r] >> 32), j >> 3) << 32) |
                             __shfl_xor_sync(0xffffffffu, (uint32_t)v[r], j >> 3);
          const int e = lane * 8 + r;
          const bool up = (e & k2) == 0;
          const bool lower = (e & j) == 0;
          v[r] = (lower == up) ? (o < v[r] ? o : v[r]) : (o > v[r] ? o : v[r]);
        }
      } else {
#pragma unroll
        for (int r = 0; r < 8; r++) {
          if (r & j) continue;
          const int e = lane * 8 + r;
          const bool up = (e & k2) == 0;
          const uint64_t x = v[r], y = v[r ^ j];
          const bool sw = up ? (x > y) : (x < y);
          v[r] = sw ? y : x;
          v[r ^ j] = sw ? x : y;
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int e = lane * 8 + r;
    if (e < kk2) kr[e] = v[r];
  }
}

constexpr int kMaxSplits = 128;

// One warp per query: k-way merge of the sorted lists its query block's
// pieces kept -- piece p holds rows in[p][0, QM)[0, kk2); the block's pieces are
// [qb_pb[qb], qb_pb[qb + 1]), at most kMaxSplits -- into out[q][0, kk2); lane l
// owns pieces l, l+32, ...
__global__ void __launch_bounds__(256) merge_tc_splits_kernel(const uint64_t* __restrict__ in, int64_t m,
                                                              const int32_t* __restrict__ qb_pb, int kk2,
                                                              uint64_t* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= m) return;
  const int64_t qb = q / QM, row = q - qb * QM;
  const int p0 = qb_pb[qb], S = qb_pb[qb + 1] - p0;
  int pos[kMaxSplits / 32];
  uint64_t head[kMaxSplits / 32];
#pragma unroll
  for (int t = 0; t < kMaxSplits / 32; t++) {
    const int sp = lane + 32 * t;
    pos[t] = 0;
    head[t] = sp < S ? in[((size_t)(p0 + sp) * QM + row) * kk2] : KEY_NONE;
  }
  for (int j = 0; j < kk2; j++) {
    uint64_t mn = head[0];
#pragma unroll
    for (int t = 1; t < kMaxSplits / 32; t++) mn = head[t] < mn ? head[t] : mn;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const uint64_t v = ((uint64_t)__shfl_xor_sync(0xffffffffu, (uint32_t)(mn >> 32), o) << 32) |
                         __shfl_xor_sync(0xffffffffu, (uint32_t)mn, o);
      mn = v < mn ? v : mn;
    }
    if (lane == 0) out[(size_t)q * kk2 + j] = mn;
    if (mn == KEY_NONE) continue;
#pragma unroll
    for (int t = 0; t < kMaxSplits / 32; t++)
      if (head[t] == mn) {  // keys are unique: one list advances
        const int sp = lane + 32 * t;
        pos[t]++;
        head[t] = pos[t] < kk2 ? in[((size_t)(p0 + sp) * QM + row) * kk2 + pos[t]] : KEY_NONE;
      }
  }
}

__global__ void __launch_bounds__(kThreadsKT, kCtasPerSm)
    knn_tc_kernel(const __grid_constant__ CUtensorMap tmQ, const __grid_constant__ CUtensorMap tmX,
                  const __grid_constant__ CUtensorMap tmQlo, const __grid_constant__ CUtensorMap tmXlo, KnnTcArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const uint32_t a_chunk = QM * BK * 2;  // 16 KB
  const uint32_t b_bytes = XN * BK * 2;  // 16 KB per stage
  const int NS = a.stages;
  uint8_t* sA = base;
  // A: the query tile (hi chunks, then lo chunks in split mode), resident
  uint8_t* sB = base + (size_t)(a.split ? 2 : 1) * a.kc * a_chunk;
  const int nb = a.split ? 2 * a.kc : a.kc;  // B chunks per tile: x_hi (then x_lo)
  uint64_t* full = reinterpret_cast<uint64_t*>(sB + (size_t)NS * b_bytes);
  uint64_t* empty = full + NS;
  uint64_t* accf = empty + NS;
  uint64_t* acce = accf + 2;
  uint64_t* afull = acce + 2;
  uint64_t* aempty = afull + 1;  // the MMAs reading a piece's query tile are done
  uint64_t* fin = aempty + 1;
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(fin + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_holder + 1);
  // [kEpiWarps][2][XN] index norms, read as float4: 16-byte aligned
  float* xnsm = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(tmem_holder + 2) + 15) & ~(uintptr_t)15);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // this CTA's pieces: (query block, index tile range), worked through in order
  const int pb = a.cta_pb[blockIdx.x], pe = a.cta_pb[blockIdx.x + 1];
  const size_t qstride = (size_t)a.kk2 + kApp;
  uint64_t* const lists_cta = a.lists + (size_t)blockIdx.x * QM * qstride;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], kEpiWarps);
    }
    mbar_init(afull, 1);
    mbar_init(aempty, 1);
    mbar_init(fin, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                 "r"(2 * XN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_holder;

  if (warp == 0) {
    if (lane == 0) {
      prefetch_tmap(&tmQ);
      prefetch_tmap(&tmX);
      const uint64_t pol_q = policy_evict_first(), pol_x = policy_evict_last();
      uint32_t stage = 0, phase = 0, armed = 0, last_ph = 0;
      int loaded = 0;  // query tiles loaded (afull phases)
      for (int p = pb; p < pe && !*abort_flag; p++) {
        const int li = p - pb;
        const int q0 = a.piece_qb[p] * QM;
        if (li > 0 && !mbar_wait(aempty, (uint32_t)((li - 1) & 1), abort_flag, a.wait_ns)) {
          if (!*abort_flag) atomicOr(a.status, DEV_TIMEOUT);
          *abort_flag = 1;
          break;
        }
        // the piece's query tile (hi chunks, then lo chunks in split mode)
        mbar_expect_tx(afull, (uint32_t)(a.split ? 2 : 1) * a.kc * a_chunk);
        for (int kc = 0; kc < a.kc; kc++) tma_load_2d_hint(sA + (size_t)kc * a_chunk, &tmQ, kc * BK, q0, afull, pol_q);
        if (a.split)
          for (int kc = 0; kc < a.kc; kc++)
            tma_load_2d_hint(sA + (size_t)(a.kc + kc) * a_chunk, &tmQlo, kc * BK, q0, afull, pol_q);
        loaded++;
        for (int64_t t = a.piece_t0[p]; t < a.piece_t1[p] && !*abort_flag; t++) {
          if ((t & 63) == 63 && a.cancel != nullptr && *a.cancel) {
            atomicOr(a.status, DEV_CANCELLED);
            *abort_flag = 1;
            break;
          }
          for (int j = 0; j < nb; j++) {
            if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag, a.wait_ns)) {
              if (!*abort_flag) atomicOr(a.status, DEV_TIMEOUT);
              *abort_flag = 1;
              break;
            }
            mbar_expect_tx(&full[stage], b_bytes);
            armed |= 1u << stage;
            last_ph = (last_ph & ~(1u << stage)) | (phase << stage);
            tma_load_2d_hint(sB + (size_t)stage * b_bytes, j < a.kc ? &tmX : &tmXlo, (j % a.kc) * BK,
                             (int)(t * XN), &full[stage], pol_x);
            if (++stage == (uint32_t)NS) {
              stage = 0;
              phase ^= 1;
            }
          }
        }
      }
      // never leave a TMA copy writing shared memory: wait (bounded) for the
      // last query tile and the last load armed on every stage
      volatile int never = 0;
      if (loaded > 0 && !mbar_wait(afull, (uint32_t)((loaded - 1) & 1), &never)) atomicOr(a.status, DEV_TIMEOUT);
      for (int s2 = 0; s2 < NS; s2++)
        if (armed & (1u << s2))
          if (!mbar_wait(&full[s2], (last_ph >> s2) & 1u, &never)) atomicOr(a.status, DEV_TIMEOUT);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      uint32_t stage = 0, phase = 0;
      int64_t gt = 0;  // tiles so far over all pieces: accumulator buffer and parity
      bool ok = true;
      for (int p = pb; ok && p < pe && !*abort_flag; p++) {
        const int li = p - pb;
        if (!mbar_wait(afull, (uint32_t)(li & 1), abort_flag, a.wait_ns)) {
          if (!*abort_flag) atomicOr(a.status, DEV_TIMEOUT);
          *abort_flag = 1;
          break;
        }
        tc_fence_after();
        for (int64_t t = a.piece_t0[p]; ok && t < a.piece_t1[p] && !*abort_flag; t++, gt++) {
          const uint32_t buf = (uint32_t)(gt & 1), accph = (uint32_t)((gt >> 1) & 1);
          if (!mbar_wait(&acce[buf], accph ^ 1, abort_flag, a.wait_ns)) {
            if (!*abort_flag) atomicOr(a.status, DEV_TIMEOUT);
            *abort_flag = 1;
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t d_tmem = tmem_base + buf * XN;
          for (int j = 0; j < nb; j++) {
            if (!mbar_wait(&full[stage], phase, abort_flag, a.wait_ns)) {
              if (!*abort_flag) atomicOr(a.status, DEV_TIMEOUT);
              *abort_flag = 1;
              ok = false;
              break;
            }
            tc_fence_after();
            // B = x_hi[kc]: q_hi . x_hi (+ q_lo . x_hi); B = x_lo[kc]: q_hi . x_lo
            const int kc = j % a.kc;
            const uint64_t ad = smem_desc_sw128(smem_u32(sA + (size_t)kc * a_chunk));
            const uint64_t bd = smem_desc_sw128(smem_u32(sB + (size_t)stage * b_bytes));
            // K steps of 16 that hold data: the zero columns past d add nothing
            const int nks = kc == a.kc - 1 ? a.ks_last : BK / 16;
#pragma unroll
            for (int kk = 0; kk < BK / 16; kk++)
              if (kk < nks) umma_bf16(d_tmem, ad + 2 * kk, bd + 2 * kk, a.idesc, (j | kk) != 0 ? 1u : 0u);
            if (a.split && j < a.kc) {
              const uint64_t al = smem_desc_sw128(smem_u32(sA + (size_t)(a.kc + kc) * a_chunk));
#pragma unroll
              for (int kk = 0; kk < BK / 16; kk++)
                if (kk < nks) umma_bf16(d_tmem, al + 2 * kk, bd + 2 * kk, a.idesc, 1u);
            }
            umma_commit(&empty[stage]);
            if (++stage == (uint32_t)NS) {
              stage = 0;
              phase ^= 1;
            }
          }
          if (!ok) break;
          umma_commit(&accf[buf]);
        }
        // the query tile may be replaced once these MMAs are done
        umma_commit(aempty);
      }
      umma_commit(fin);
      volatile int never = 0;
      if (!mbar_wait(fin, 0, &never)) atomicOr(a.status, DEV_TIMEOUT);
    }
  } else {
    // Epilogue: warp w handles query rows 32*(w%4).. (its TMEM lane quarter)
    // over every column; each query keeps its kk2 smallest keys (unsorted)
    // plus an append log of candidates below its running kk2-th key.
    const int g = warp & 3;
    const int ew = warp - 2;
    const int row = g * 32 + lane;  // TMEM lane = query row of the tile
    float* nsm_w = xnsm + ew * 2 * XN;
    uint64_t* const app = lists_cta + row * qstride + a.kk2;  // this row's append log
    int64_t gt = 0;  // tiles so far over all pieces (accumulator buffer and parity)
    bool alive = true;
    for (int p = pb; alive && p < pe; p++) {
      const int64_t q0 = (int64_t)a.piece_qb[p] * QM;
      const int64_t qi = q0 + row;
      const bool valid = qi < a.m;
      const float nq = valid ? a.qn2[qi] : 0.0f;
      const int kkr = (a.row_k != nullptr && valid) ? kk2_of(a.row_k[qi], a.margin_mode) : a.kk2;  // this row's keys
      uint64_t tau = KEY_NONE;  // kk2-th key held
      float tau_d = __int_as_float(0x7f800000);
      int na = 0, plen = 0;
      // Screen filter in the shifted domain: a column can enter only if
      // |x|^2 - 2 q.x <= tau - |q|^2 (+ slack covering the rounding of both
      // forms when the data are not exact integers); the screened distance is
      // formed only for the rare columns that pass.
      auto threshold = [&]() -> float {
        if (!valid) return -__int_as_float(0x7f800000);
        if (tau == KEY_NONE) return __int_as_float(0x7f800000);
        const float th = tau_d - nq;
        return a.exact ? th : th + (nq + a.xmax_n2 + tau_d) * 3.814697265625e-06f;  // 2^-18
      };
      // Lanes whose append log passed `lim` entries are reduced to their kk2
      // smallest keys, one query at a time, by the whole warp.
      auto flush_rows = [&](unsigned need) {
        __syncwarp();
        while (need) {
          const int src = __ffs(need) - 1;
          need &= need - 1;
          const int sna = __shfl_sync(0xffffffffu, na, src);
          const int splen = __shfl_sync(0xffffffffu, plen, src);
          const int skk = __shfl_sync(0xffffffffu, kkr, src);
          uint64_t* lb = lists_cta + (g * 32 + src) * qstride;
          const uint64_t nt = warp_select(lb + a.kk2, sna, lb, splen, skk, lane);
          if (lane == src) {
            tau = nt;
            tau_d = nt == KEY_NONE ? __int_as_float(0x7f800000) : key_dist(nt);
            plen = min(kkr, plen + na);
            na = 0;
          }
        }
      };
      float thr = threshold();
      const int64_t t0 = a.piece_t0[p], t1 = a.piece_t1[p];
      // norms of the tile's XN columns: 4 per lane, fetched one tile ahead
      float4 pn = __ldg(reinterpret_cast<const float4*>(a.xn2 + t0 * XN) + lane);
      for (int64_t t = t0; t < t1; t++, gt++) {
        const uint32_t b = (uint32_t)(gt & 1), accph = (uint32_t)((gt >> 1) & 1);
        const int64_t p0 = t * XN;
        float* nsm = nsm_w + b * XN;
        reinterpret_cast<float4*>(nsm)[lane] = pn;
        if (t + 1 < t1) pn = __ldg(reinterpret_cast<const float4*>(a.xn2 + p0 + XN) + lane);
        bool ok = !*abort_flag && mbar_wait(&accf[b], accph, abort_flag, a.wait_ns);
        if (!ok) {
          if (!*abort_flag) atomicOr(a.status, DEV_TIMEOUT);
          *abort_flag = 1;
        }
        if (!__all_sync(0xffffffffu, ok)) {  // warp-uniform exit
          alive = false;
          break;
        }
        __syncwarp();
        tc_fence_after();
        const uint32_t taddr = tmem_base + ((uint32_t)(g * 32) << 16) + b * XN;
#pragma unroll 1
        for (int c0 = 0; c0 < XN; c0 += 64) {
          uint32_t r[4][16];
#pragma unroll
          for (int h = 0; h < 4; h++) tmem_ld16_nowait(taddr + c0 + 16 * h, r[h]);
          tmem_ld_wait();
#pragma unroll
          for (int h = 0; h < 4; h++) tmem_regs_ready(r[h]);
          // shifted screen values f = |x|^2 - 2 q.x (in place) and each group's
          // minimum (short dependency chains, four groups interleaved)
          float mnh[4];
#pragma unroll
          for (int h = 0; h < 4; h++) {
            const float4* n4 = reinterpret_cast<const float4*>(nsm + c0 + 16 * h);
#pragma unroll
            for (int v = 0; v < 4; v++) {
              const float4 q4 = n4[v];
              // f = fma(-2, q.x, |x|^2), two columns per paired instruction
              fma2_rn(r[h][4 * v], r[h][4 * v + 1], -2.0f, q4.x, q4.y);
              fma2_rn(r[h][4 * v + 2], r[h][4 * v + 3], -2.0f, q4.z, q4.w);
            }
            // minimum of the 16 columns with three-input minima (16 -> 6 -> 2 -> 1)
            float m6[6];
#pragma unroll
            for (int j = 0; j < 5; j++)
              m6[j] = min3_f32(__uint_as_float(r[h][3 * j]), __uint_as_float(r[h][3 * j + 1]),
                               __uint_as_float(r[h][3 * j + 2]));
            m6[5] = __uint_as_float(r[h][15]);
            mnh[h] = fminf(min3_f32(m6[0], m6[1], m6[2]), min3_f32(m6[3], m6[4], m6[5]));
          }
#pragma unroll
          for (int h = 0; h < 4; h++) {
            if (mnh[h] <= thr) {
              // the few passing columns, one loop trip each; the screened
              // distance is D~ = |q|^2 + (|x|^2 - 2 q.x) in f32
              float f[16];
#pragma unroll
              for (int j = 0; j < 16; j++) f[j] = __uint_as_float(r[h][j]);
              unsigned b8[8];
#pragma unroll
              for (int j = 0; j < 8; j++)
                b8[j] = (f[2 * j] <= thr ? 1u : 0u) | (f[2 * j + 1] <= thr ? 2u : 0u);
#pragma unroll
              for (int j = 0; j < 4; j++) b8[j] = b8[2 * j] | (b8[2 * j + 1] << 2);
              unsigned mask = (b8[0] | (b8[1] << 4)) | ((b8[2] | (b8[3] << 4)) << 8);
              while (mask) {
                const int j = __ffs(mask) - 1;
                mask &= mask - 1;
                const int64_t pt = p0 + c0 + 16 * h + j;
                float dt = nq + sel16(f, j);
                if (!a.exact) dt = fmaxf(dt, 0.0f);
                if (dt <= tau_d && pt < a.n) {
                  const uint64_t key = make_key(dt, (uint32_t)pt);
                  if (key < tau) app[na++] = key;
                }
              }
            }
          }
          // at most 64 appends per lane per chunk: compact before the log can overflow
          const unsigned full = __ballot_sync(0xffffffffu, na > kApp - 64);
          if (full) {
            flush_rows(full);
            thr = threshold();
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&acce[b]);
      }
      if (!alive) break;
      {
        const unsigned need = __ballot_sync(0xffffffffu, na > 0);
        if (need) flush_rows(need);
      }
      // kept keys out (unsorted; sorted afterwards), one query at a time per
      // warp (coalesced); slots past the held count are KEY_NONE.  Piece p's
      // lists sit at rows [p*QM, p*QM + QM) of the output.
      __syncwarp();
      for (int src = 0; src < 32; src++) {
        if (q0 + g * 32 + src >= a.m) break;
        const int splen = __shfl_sync(0xffffffffu, plen, src);
        const uint64_t* from = lists_cta + (g * 32 + src) * qstride;
        uint64_t* to = a.out_keys + ((size_t)p * QM + g * 32 + src) * a.kk2;
        for (int o = lane; o < a.kk2; o += 32) to[o] = o < splen ? from[o] : KEY_NONE;
      }
      __syncwarp();
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(2 * XN) : "memory");
  }
}

// Rows -> BF16 copy padded to dp columns and rows_pad rows (zeros), |row|^2 in
// FP32, plus an integer-data census: flags[0] |= non-integer or |v| > 256,
// flags[1] = max |v| (as float bits; non-negative so integer order works).
template <bool F16>
__global__ void knn_prep_kernel(const float* __restrict__ X, int64_t rows, int64_t rows_pad, int d, int dp,
                                void* __restrict__ out, __nv_bfloat16* __restrict__ out_lo,
                                float* __restrict__ n2, int* __restrict__ flags) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  int bad = 0;
  float vmax = 0.0f;
  for (int64_t r = (int64_t)blockIdx.x * nw + warp; r < rows_pad; r += (int64_t)gridDim.x * nw) {
    float acc = 0.0f;
    for (int c = lane; c < dp; c += 32) {
      const float x = (r < rows && c < d) ? __ldg(X + r * d + c) : 0.0f;
      if (F16) {
        static_cast<__half*>(out)[r * dp + c] = __float2half_rn(x);
      } else {
        const __nv_bfloat16 hi = __float2bfloat16_rn(x);
        static_cast<__nv_bfloat16*>(out)[r * dp + c] = hi;
        if (out_lo) out_lo[r * dp + c] = __float2bfloat16_rn(x - __bfloat162float(hi));
      }
      acc = fmaf(x, x, acc);
      if (x != rintf(x) || fabsf(x) > 256.0f) bad = 1;
      vmax = fmaxf(vmax, fabsf(x));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (lane == 0) n2[r] = acc;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    bad |= __shfl_xor_sync(0xffffffffu, bad, off);
    vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, off));
  }
  if (lane == 0) {
    if (bad) atomicOr(&flags[0], 1);
    atomicMax(&flags[1], __float_as_int(vmax));
  }
}

// Re-score the kk2 screened candidates of every query with the reference's
// own f32 order (8-lane groups = fuel's SIMD lanes, 4 candidates per warp
// step), sort them by (distance, index) in the metric's domain, and prove that
// no unscreened point can displace the kk-th: every unscreened point has
// D~ >= D~_last, so its reference distance is >= D~_last - E_max.  Queries that
// fail the proof are flagged for the exact scan.
template <int ORDER>
__global__ void knn_rescore_kernel(const float* __restrict__ Q, const float* __restrict__ X, int64_t n, int d,
                                   int64_t m, int kk, int kk2, const int32_t* __restrict__ row_k, int margin_mode,
                                   int metric, const uint64_t* __restrict__ keys_in,
                                   uint64_t* __restrict__ keys_out, const float* __restrict__ qn2, float xmax_norm,
                                   float xmax_n2, float alpha, float beta, float gamma, float abs_a,
                                   int32_t* __restrict__ redo, int32_t* __restrict__ nredo) {
  extern __shared__ __align__(16) float qsm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t qi = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (qi >= m) return;
  float* qs = qsm + (size_t)wib * (d + 4);
  for (int e = lane; e < d; e += 32) qs[e] = __ldg(Q + qi * d + e);
  __syncwarp();
  const uint64_t* kin = keys_in + qi * kk2;
  uint64_t* kout = keys_out + qi * kk2;
  // this row's k and kept keys (the list stride stays kk2)
  const int kq = row_k != nullptr ? row_k[qi] : kk;
  const int kk2q = row_k != nullptr ? kk2_of(kq, margin_mode) : kk2;
  for (int c = kk2q + lane; c < kk2; c += 32) kout[c] = KEY_NONE;
  // exact keys of the candidates, written in place of the screened ones
  const int l = lane & 7, grp = lane >> 3;
  float last_screen = 0.0f;
  for (int c0 = 0; c0 < kk2q; c0 += 4) {
    const int c = c0 + grp;
    const uint64_t sk = c < kk2q ? kin[c] : KEY_NONE;
    // a key that names no index row (never produced by a completed screen)
    // is treated as empty, so no read leaves X
    const bool real = sk != KEY_NONE && (int64_t)key_idx(sk) < n;
    const uint32_t idx = real ? key_idx(sk) : 0u;
    const float* x = X + (int64_t)idx * d;
    const int sd = d & ~7;
    float acc = 0.0f;
    for (int i = l; i < sd; i += 8) {
      const float df = __fsub_rn(qs[i], __ldg(x + i));
      acc = ORDER == ORDER_X86 ? __fmaf_rn(df, df, acc) : __fadd_rn(sq_rn(df), acc);
    }
    float s = __shfl_sync(0xffffffffu, acc, lane & ~7);
#pragma unroll
    for (int t = 1; t < 8; t++) s = __fadd_rn(s, __shfl_sync(0xffffffffu, acc, (lane & ~7) + t));
    for (int i = sd; i < d; i++) {
      const float df = __fsub_rn(qs[i], __ldg(x + i));
      s = ORDER == ORDER_X86 ? __fmaf_rn(df, df, s) : __fadd_rn(s, sq_rn(df));
    }
    if (metric == METRIC_EUCLIDEAN) s = __fsqrt_rn(s);
    if (l == 0 && c < kk2q) kout[c] = real ? make_key(s, idx) : KEY_NONE;
    if (real) last_screen = fmaxf(last_screen, key_dist(sk));
  }
  // the largest screened distance kept (candidates are sorted by screened key)
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) last_screen = fmaxf(last_screen, __shfl_xor_sync(0xffffffffu, last_screen, off));
  __syncwarp();
  // sort the kk2 exact keys (small: insertion sort by lane 0)
  if (lane == 0) {
    for (int a1 = 1; a1 < kk2q; a1++) {
      const uint64_t v = kout[a1];
      int b = a1 - 1;
      while (b >= 0 && kout[b] > v) {
        kout[b + 1] = kout[b];
        b--;
      }
      kout[b + 1] = v;
    }
    // proof: only needed when every slot was filled (otherwise every point was kept)
    const bool full_list = kin[kk2q - 1] != KEY_NONE;
    if (full_list) {
      const float nq = qn2[qi];
      const float qn = sqrtf(nq);
      const float e = (alpha * qn * xmax_norm + beta * (nq + xmax_n2)) * (1.0f + gamma) + gamma * last_screen +
                      abs_a * (qn + xmax_norm);
      const float lower = last_screen - e;  // every unscreened point's reference squared distance is >= this
      const uint64_t kth = kout[kq - 1];
      bool ok;
      if (metric == METRIC_EUCLIDEAN) ok = kth != KEY_NONE && lower > 0.0f && key_dist(kth) < __fsqrt_rd(lower);
      else ok = kth != KEY_NONE && key_dist(kth) < lower;
      if (!ok) redo[atomicAdd(nredo, 1)] = (int32_t)qi;
    }
  }
}

__global__ void gather_rows_kernel(const float* __restrict__ Q, int d, const int32_t* __restrict__ rows,
                                   const int32_t* __restrict__ nrows, float* __restrict__ out) {
  const int cnt = *nrows;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < (int64_t)cnt * d;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / d, c = e - r * d;
    out[e] = Q[(int64_t)rows[r] * d + c];
  }
}

__global__ void scatter_keys_kernel(const uint64_t* __restrict__ src, int kk, int kk2,
                                    const int32_t* __restrict__ rows, int cnt, uint64_t* __restrict__ dst) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)cnt * kk2) return;
  const int64_t r = e / kk2, j = e - r * kk2;
  dst[(int64_t)rows[r] * kk2 + j] = j < kk ? src[r * kk + j] : KEY_NONE;
}

}  // namespace

namespace {
// Shared memory of knn_tc_kernel without the B stages.
size_t knn_tc_fixed_smem(int d, int split) {
  const int dp = ((d + BK - 1) / BK) * BK;
  const size_t a_bytes = (size_t)(split ? 2 : 1) * (dp / BK) * QM * BK * 2;
  return 1024 + a_bytes + 8 * 32 + 16 + (size_t)kEpiWarps * 2 * XN * sizeof(float);
}
int margin_mode_of(int tier) { return tier == TC_F16 ? 2 : 1; }
}  // namespace

bool knn_tc_supported(int64_t n, int d, int kk, int tier) {
  if (d < 32 || d > 256 || kk < 1) return false;
  // TMA row coordinates are signed 32-bit: the padded index must stay below 2^31 rows
  if (n >= (1ll << 31) - 4096) return false;
  // kept keys per query are selected 8 per lane by one warp
  if (kk2_of(kk, margin_mode_of(tier)) > 32 * kSel) return false;
  return knn_tc_fixed_smem(d, tier == TC_SPLIT) + 2 * (size_t)XN * BK * 2 <= kSmemPerCta;
}

// Top-kk keys of every query via the tensor-core screen.  out_keys: [m, kk]
// (device).  X32/Q32: the f32 rows (for the exact re-score).
struct TcIndex {
  int64_t n = 0, npad = 0;
  int d = 0, dp = 0;
  __nv_bfloat16* xb = nullptr;  // [npad, dp] BF16, zero padded
  __nv_bfloat16* xlo = nullptr; // [npad, dp] BF16 of x - xb (split tier; built on first use)
  __half* xh = nullptr;         // [npad, dp] FP16 (FP16 tier; built on first use)
  float* xn2 = nullptr;         // [npad] FP32 |x|^2 (padded rows 0)
  bool integer = false;         // every value an integer with |v| <= 256
  float vmax = 0.0f;            // max |v|
  float xmax_n2 = 0.0f;         // max |x|^2
  CUtensorMap tmX, tmXlo, tmXh;
};

int knn_tc_index_class(const TcIndex* t) {
  if (t->integer) return TC_CLASS_INTEGER;
  return t->vmax <= kF16Max ? TC_CLASS_F16_RANGE : TC_CLASS_WIDE;
}

void knn_tc_index_free(TcIndex* t) {
  if (!t) return;
  if (t->xb) cudaFree(t->xb);
  if (t->xn2) cudaFree(t->xn2);
  if (t->xlo) cudaFree(t->xlo);
  if (t->xh) cudaFree(t->xh);
  delete t;
}

int knn_tc_index_build(const float* X32, int64_t n, int d, cudaStream_t stream, TcIndex** out) {
  *out = nullptr;
  TcIndex* t = new TcIndex();
  struct Guard {
    TcIndex*& t;
    ~Guard() { knn_tc_index_free(t); }
  } guard{t};
  t->n = n;
  t->d = d;
  t->dp = ((d + BK - 1) / BK) * BK;
  t->npad = ((n + XN - 1) / XN) * XN;
  FUELG_CUDA(cudaMalloc(&t->xb, (size_t)t->npad * t->dp * 2));
  FUELG_CUDA(cudaMalloc(&t->xn2, sizeof(float) * t->npad));
  Scratch flags;
  FUELG_TRY(flags.alloc(sizeof(int) * 2, stream));
  FUELG_CUDA(cudaMemsetAsync(flags.p, 0, sizeof(int) * 2, stream));
  knn_prep_kernel<false><<<8 * 152, 256, 0, stream>>>(X32, n, t->npad, d, t->dp, t->xb, nullptr, t->xn2,
                                                      flags.as<int>());
  ::fuelg::note_launch();
  FUELG_CUDA(cudaGetLastError());
  int hf[2];
  FUELG_CUDA(cudaMemcpyAsync(hf, flags.p, sizeof(hf), cudaMemcpyDeviceToHost, stream));
  std::vector<float> h((size_t)t->npad);
  FUELG_CUDA(cudaMemcpyAsync(h.data(), t->xn2, sizeof(float) * t->npad, cudaMemcpyDeviceToHost, stream));
  FUELG_CUDA(cudaStreamSynchronize(stream));
  t->integer = hf[0] == 0;
  memcpy(&t->vmax, &hf[1], sizeof(float));
  for (float v : h) t->xmax_n2 = std::max(t->xmax_n2, v);
  FUELG_TRY(make_map_bf16(&t->tmX, t->xb, t->npad, t->dp, XN));
  *out = t;
  t = nullptr;  // owned by the caller now
  return ST_OK;
}

// Adds the BF16 residual copy x - BF16(x) of the index (split tier), once.
int knn_tc_index_add_lo(TcIndex* t, const float* X32, cudaStream_t stream) {
  if (t->xlo) return ST_OK;
  FUELG_CUDA(cudaMalloc(&t->xlo, (size_t)t->npad * t->dp * 2));
  Scratch hi, n2, flags;
  FUELG_TRY(hi.alloc((size_t)t->npad * t->dp * 2, stream));
  FUELG_TRY(n2.alloc(sizeof(float) * t->npad, stream));
  FUELG_TRY(flags.alloc(sizeof(int) * 2, stream));
  knn_prep_kernel<false><<<8 * 152, 256, 0, stream>>>(X32, t->n, t->npad, t->d, t->dp, hi.as<__nv_bfloat16>(),
                                                      t->xlo, n2.as<float>(), flags.as<int>());
  ::fuelg::note_launch();
  FUELG_CUDA(cudaGetLastError());
  FUELG_TRY(make_map_bf16(&t->tmXlo, t->xlo, t->npad, t->dp, XN));
  FUELG_CUDA(cudaStreamSynchronize(stream));
  return ST_OK;
}

int knn_tc_index_add_f16(TcIndex* t, const float* X32, cudaStream_t stream) {
  if (t->xh) return ST_OK;
  if (!(t->vmax <= kF16Max)) {
    set_error("index values exceed the FP16 range (max |v| = %g)", (double)t->vmax);
    return ST_ENOTSUP;
  }
  FUELG_CUDA(cudaMalloc(&t->xh, (size_t)t->npad * t->dp * 2));
  Scratch n2, flags;
  FUELG_TRY(n2.alloc(sizeof(float) * t->npad, stream));
  FUELG_TRY(flags.alloc(sizeof(int) * 2, stream));
  knn_prep_kernel<true><<<8 * 152, 256, 0, stream>>>(X32, t->n, t->npad, t->d, t->dp, t->xh, nullptr,
                                                     n2.as<float>(), flags.as<int>());
  ::fuelg::note_launch();
  FUELG_CUDA(cudaGetLastError());
  FUELG_TRY(make_map_bf16(&t->tmXh, t->xh, t->npad, t->dp, XN));  // 2-byte elements: same box geometry
  FUELG_CUDA(cudaStreamSynchronize(stream));
  return ST_OK;
}

int knn_tc_topk(const TcIndex* ti, const float* Q32, int64_t m, const float* X32, int kk, int order, int metric,
                int tier, uint64_t* out_keys, int* dev_status, cudaStream_t stream, int64_t* rescored,
                int* exact_out, const int32_t* row_k) {
  const int64_t n = ti->n;
  const int d = ti->d;
  const int dp = ti->dp;
  const int kc = dp / BK;
  const int64_t mpad = ((m + QM - 1) / QM) * QM;
  const bool f16 = tier == TC_F16;
  int split = tier == TC_SPLIT ? 1 : 0;
  if (split && !ti->xlo) {
    set_error("split-BF16 kNN needs the index residual copy");
    return ST_ENOTSUP;
  }
  if (f16 && !ti->xh) {
    set_error("FP16 kNN needs the index FP16 copy");
    return ST_ENOTSUP;
  }
  Scratch qb, qlo, qn2, flags;
  FUELG_TRY(qb.alloc((size_t)mpad * dp * 2, stream));
  if (split) FUELG_TRY(qlo.alloc((size_t)mpad * dp * 2, stream));
  FUELG_TRY(qn2.alloc(sizeof(float) * mpad, stream));
  FUELG_TRY(flags.alloc(sizeof(int) * 2, stream));
  FUELG_CUDA(cudaMemsetAsync(flags.p, 0, sizeof(int) * 2, stream));
  if (f16)
    knn_prep_kernel<true><<<8 * 152, 256, 0, stream>>>(Q32, m, mpad, d, dp, qb.p, nullptr, qn2.as<float>(),
                                                       flags.as<int>());
  else
    knn_prep_kernel<false><<<8 * 152, 256, 0, stream>>>(Q32, m, mpad, d, dp, qb.p,
                                                        split ? qlo.as<__nv_bfloat16>() : nullptr, qn2.as<float>(),
                                                        flags.as<int>());
  ::fuelg::note_launch();
  FUELG_CUDA(cudaGetLastError());
  int hf[2];
  FUELG_CUDA(cudaMemcpyAsync(hf, flags.p, sizeof(hf), cudaMemcpyDeviceToHost, stream));
  FUELG_CUDA(cudaStreamSynchronize(stream));
  float qmax;
  memcpy(&qmax, &hf[1], sizeof(float));
  if (f16 && !(qmax <= kF16Max)) {
    set_error("query values exceed the FP16 range (max |q| = %g)", (double)qmax);
    return ST_ENOTSUP;
  }
  const float vmax = std::max(qmax, ti->vmax);
  const bool integer = hf[0] == 0 && ti->integer;
  const bool exact = integer && 2.0 * dp * (double)vmax * vmax < 16777216.0;
  *exact_out = exact ? 1 : 0;
  if (exact) split = 0;  // integer data: the one-product screen (BF16 or FP16) is already exact
  // screened keys kept per query: exact sqeuclidean needs none extra
  const int mmode = (exact && metric == METRIC_SQEUCLIDEAN) ? 0 : margin_mode_of(tier);
  const int margin = kk2_of(kk, mmode) - kk;
  const int kk2 = kk + margin;

  const size_t b_bytes = (size_t)XN * BK * 2;
  const size_t fixed = knn_tc_fixed_smem(d, split);
  int stages = (int)((kSmemPerCta - fixed) / b_bytes);
  stages = std::max(2, std::min(6, stages));
  const size_t smem = fixed + stages * b_bytes;
  if (smem > kSmemPerCta) {
    set_error("tensor-core kNN tile does not fit shared memory (d=%d)", d);
    return ST_ENOTSUP;
  }
  // Work decomposition.  The queries run in batches.  A batch of whole waves
  // (a multiple of the GPU's CTA slots in query blocks) has one CTA per
  // block: the hardware hands blocks to free slots as they come, which
  // evens out blocks of unequal cost.  A batch of less than a wave (a small
  // query count, or the last part of a large one) would leave slots idle, so
  // there each block's index scan is cut into s equal tile ranges (quanta);
  // the quanta, block-major, are dealt out L at a time to consecutive CTAs,
  // L = ceil(quanta / slots).  s is the count (quanta of >= 16 tiles, at most
  // kMaxSplits - 2 pieces per block) that minimises the longest CTA's work,
  // L (ntiles / s + 4) tiles with 4 tiles' worth charged per piece for its
  // pipeline refill and its list's start.  A CTA's quanta fall into pieces at
  // query-block boundaries; a block cut into several pieces gets one kept
  // list per piece, merged afterwards.
  const int64_t ntiles_all = (n + XN - 1) / XN;
  const int64_t slots = 152 * kCtasPerSm;
  const int64_t wave_q = slots * QM;
  constexpr int kMaxQuanta = kMaxSplits - 2;
  auto quanta_of = [&](int64_t qbl) -> int {
    int best = 1;
    double best_cost = 0.0;
    for (int sq = 1; sq <= kMaxQuanta; sq++) {
      if (sq > 1 && ntiles_all / sq < 16) break;
      const int64_t L = (qbl * sq + slots - 1) / slots;
      const double cost = (double)L * ((double)ntiles_all / sq + 4.0);
      if (sq == 1 || cost < best_cost) best = sq, best_cost = cost;
    }
    // tunable: FUELG_KNN_QUANTA fixes s
    if (const char* e = getenv("FUELG_KNN_QUANTA"))
      best = (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)atoi(e), (int64_t)kMaxQuanta, ntiles_all}));
    return best;
  };
  struct Batch {
    int64_t b0, mcur, G, P;
    bool merge;
    std::vector<int32_t> tab;  // piece_qb[P] piece_t0[P] piece_t1[P] cta_pb[G+1] qb_pb[blocks+1]
  };
  // Bound scratch: whole-wave batches whose lists take at most ~1 GiB.
  const int64_t mb_waves =
      std::max<int64_t>(1, (int64_t)((1ull << 30) / ((size_t)(3 * kk2 + kApp) * 8)) / wave_q) * wave_q;
  std::vector<Batch> batches;
  size_t lists_rows = 0, kept_rows = 0, merge_rows = 0, tab_max = 0;
  int64_t mb = 0;  // largest batch
  for (int64_t b0 = 0; b0 < m;) {
    const int64_t rem = m - b0;
    Batch bt;
    bt.b0 = b0;
    bt.mcur = rem >= wave_q ? std::min<int64_t>(mb_waves, rem / wave_q * wave_q) : rem;
    const int64_t qbl = (bt.mcur + QM - 1) / QM;
    const int sq = bt.mcur >= wave_q ? 1 : quanta_of(qbl);
    const int64_t nq_all = qbl * sq;
    const int64_t L = bt.mcur >= wave_q ? 1 : (nq_all + slots - 1) / slots;
    bt.G = (nq_all + L - 1) / L;
    std::vector<int32_t> pq, pt0, pt1, cpb(1, 0), qpb(1, 0);
    for (int64_t c = 0; c < bt.G; c++) {
      const int64_t qe = std::min<int64_t>(nq_all, (c + 1) * L);
      for (int64_t qu = c * L; qu < qe;) {
        // a run of this CTA's quanta inside one block is one piece
        const int64_t blk = qu / sq, j0 = qu - blk * sq;
        const int64_t j1 = std::min<int64_t>(sq, j0 + (qe - qu));
        pq.push_back((int32_t)blk);
        pt0.push_back((int32_t)(ntiles_all * j0 / sq));
        pt1.push_back((int32_t)(ntiles_all * j1 / sq));
        qu += j1 - j0;
      }
      cpb.push_back((int32_t)pq.size());
    }
    bt.P = (int64_t)pq.size();
    bt.merge = false;
    for (int64_t p = 0, blk = 0; p < bt.P; p++) {
      if (pt0[p] != 0 || pt1[p] != ntiles_all) bt.merge = true;
      while (blk < pq[p]) qpb.push_back((int32_t)p), blk++;
      if (p + 1 == bt.P) qpb.push_back((int32_t)bt.P);
    }
    for (int64_t blk = 0; blk < qbl; blk++)
      if (qpb[blk + 1] - qpb[blk] > kMaxSplits) {
        set_error("kNN work decomposition cuts a query block into more than %d pieces", kMaxSplits);
        return ST_EINVAL;
      }
    bt.tab.reserve(3 * bt.P + bt.G + 1 + qbl + 1);
    bt.tab.insert(bt.tab.end(), pq.begin(), pq.end());
    bt.tab.insert(bt.tab.end(), pt0.begin(), pt0.end());
    bt.tab.insert(bt.tab.end(), pt1.begin(), pt1.end());
    bt.tab.insert(bt.tab.end(), cpb.begin(), cpb.end());
    bt.tab.insert(bt.tab.end(), qpb.begin(), qpb.end());
    lists_rows = std::max(lists_rows, (size_t)bt.G * QM);
    kept_rows = std::max(kept_rows, (size_t)bt.P * QM);
    if (bt.merge) merge_rows = std::max(merge_rows, (size_t)bt.mcur);
    tab_max = std::max(tab_max, bt.tab.size());
    mb = std::max(mb, bt.mcur);
    b0 += bt.mcur;
    batches.push_back(std::move(bt));
  }
  Scratch lists, kept_sp, kept_m, kept2, redo, nredo, plan;
  FUELG_TRY(lists.alloc(lists_rows * (kk2 + kApp) * 8, stream));
  FUELG_TRY(kept_sp.alloc(kept_rows * kk2 * 8, stream));
  if (merge_rows) FUELG_TRY(kept_m.alloc(merge_rows * kk2 * 8, stream));
  FUELG_TRY(plan.alloc(sizeof(int32_t) * tab_max, stream));
  if (margin) {
    FUELG_TRY(kept2.alloc((size_t)mb * kk2 * 8, stream));
    FUELG_TRY(redo.alloc(sizeof(int32_t) * mb, stream));
    FUELG_TRY(nredo.alloc(sizeof(int32_t), stream));
  }
  auto kern = knn_tc_kernel;
  FUELG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  // integer data aside, keep the error-bound constants of the Lloyd screen
  const double u8 = std::ldexp(1.0, -8), u23 = std::ldexp(1.0, -23), u24 = std::ldexp(1.0, -24);
  // operand rounding (2u + u^2 per BF16 product with u = 2^-8; 3.01 * 2^-16
  // with hi + lo; u = 2^-11 per FP16 value in the normal range) plus FP32
  // accumulation in the tensor core over dp (3 dp) products.  FP16 values below
  // 2^-14 round with an absolute error of at most 2^-25 instead: the distance
  // (2 q.x) takes 2^-24 (|q|_1 + |x|_1) <= 2^-24 sqrt(dp) (|q| + |x|) more.
  const double u11 = std::ldexp(1.0, -11);
  const double rel = split ? 3.01 * std::ldexp(1.0, -16) + 3.0 * dp * u23 * (1.0 + 2 * u8)
                     : f16 ? (2 * u11 + u11 * u11) + dp * u23 * (1.0 + 2 * u11)
                           : (2 * u8 + u8 * u8) + dp * u23 * (1.0 + 2 * u8);
  const float abs_a = (f16 && !exact) ? (float)(u24 * std::sqrt((double)dp) * 1.01) : 0.0f;
  // exact integer data: the screen and fuel's own f32 sum are both exact
  const float alpha = exact ? 0.0f : (float)(2.0 * rel * 1.01);
  // (+3 u: the screened value is rounded as fl(|q|^2 + fl(|x|^2 - 2 q.x)))
  const float beta = exact ? 0.0f : (float)(((d + 31) / 32 + 9) * u24 * 1.01 + 4 * u24);
  const float gamma = exact ? 0.0f : (float)((d + 4) * u24 * 1.01);
  // max |x|^2 over the index, for the proof
  const float xmax_n2 = ti->xmax_n2;
  const float xmax_norm = sqrtf(xmax_n2) * (1.0f + 1e-6f);
  int64_t total_redo = 0;
  HotTimer* ht = hot_timer();
  for (const Batch& bt : batches) {
    const int64_t b0 = bt.b0, mcur = bt.mcur, G = bt.G, P = bt.P;
    const bool merge = bt.merge;
    KnnTcArgs a{};
    a.m = mcur;
    a.n = n;
    a.kc = kc;
    a.ks_last = ((d + 15) / 16) - (kc - 1) * (BK / 16);
    a.kk2 = kk2;
    a.row_k = row_k != nullptr ? row_k + b0 : nullptr;
    a.margin_mode = mmode;
    a.exact = exact ? 1 : 0;
    a.split = split;
    a.stages = stages;
    a.qn2 = qn2.as<float>() + b0;
    a.xn2 = ti->xn2;
    a.xmax_n2 = xmax_n2;
    a.lists = lists.as<uint64_t>();
    a.out_keys = kept_sp.as<uint64_t>();
    // this batch's pieces
    FUELG_CUDA(cudaMemcpyAsync(plan.p, bt.tab.data(), bt.tab.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                               stream));
    const int32_t* dtab = plan.as<int32_t>();
    a.piece_qb = dtab;
    a.piece_t0 = dtab + P;
    a.piece_t1 = dtab + 2 * P;
    a.cta_pb = dtab + 3 * P;
    const int32_t* qb_pb = dtab + 3 * P + G + 1;
    // instruction descriptor: D=F32, A=B=BF16 (format 1) or FP16 (format 0), K-major, N=XN, M=QM
    a.idesc = (1u << 4) | (f16 ? 0u : (1u << 7) | (1u << 10)) | ((uint32_t)(XN >> 3) << 17) |
              ((uint32_t)(QM >> 4) << 24);
    a.status = dev_status;
    a.cancel = cancel_word_device();
    a.wait_ns = pipeline_wait_ns();
    // the query map addresses rows b0.. through the y coordinate
    CUtensorMap tmQb, tmQl;
    FUELG_TRY(make_map_bf16(&tmQb, qb.as<__nv_bfloat16>() + b0 * dp, mpad - b0, dp, QM));
    if (split) FUELG_TRY(make_map_bf16(&tmQl, qlo.as<__nv_bfloat16>() + b0 * dp, mpad - b0, dp, QM));
    else tmQl = tmQb;
    const dim3 grid((unsigned)G);
    if (ht) ht->begin(stream);
    const CUtensorMap& tmXs = f16 ? ti->tmXh : ti->tmX;
    kern<<<grid, kThreadsKT, smem, stream>>>(tmQb, tmXs, tmQl, split ? ti->tmXlo : tmXs, a);
    ::fuelg::note_launch();
    if (ht) ht->end(stream);
    FUELG_CUDA(cudaGetLastError());
    uint64_t* dst = out_keys + b0 * kk;
    // each piece's kept keys in (distance, index) order; with one piece per
    // block the pieces' rows are the queries' rows
    const int64_t srows = merge ? P * QM : mcur;
    sort_rows_kernel<<<(unsigned)((srows * 32 + 255) / 256), 256, 0, stream>>>(kept_sp.as<uint64_t>(), srows, kk2);
    ::fuelg::note_launch();
    uint64_t* kept = kept_sp.as<uint64_t>();
    if (merge) {
      merge_tc_splits_kernel<<<(unsigned)((mcur * 32 + 255) / 256), 256, 0, stream>>>(kept_sp.as<uint64_t>(), mcur,
                                                                                      qb_pb, kk2, kept_m.as<uint64_t>());
      ::fuelg::note_launch();
      kept = kept_m.as<uint64_t>();
    }
    FUELG_CUDA(cudaGetLastError());
    if (margin == 0) {
      FUELG_CUDA(cudaMemcpyAsync(dst, kept, (size_t)mcur * kk * 8, cudaMemcpyDeviceToDevice, stream));
      continue;
    }
    FUELG_CUDA(cudaMemsetAsync(nredo.p, 0, sizeof(int32_t), stream));
    const size_t rsm = (size_t)8 * (d + 4) * sizeof(float);
    const unsigned rg = (unsigned)((mcur * 32 + 255) / 256);
    if (order == ORDER_X86)
      knn_rescore_kernel<ORDER_X86><<<rg, 256, rsm, stream>>>(Q32 + b0 * d, X32, n, d, mcur, kk, kk2,
                                                              row_k != nullptr ? row_k + b0 : nullptr, mmode, metric,
                                                              kept, kept2.as<uint64_t>(),
                                                              qn2.as<float>() + b0, xmax_norm, xmax_n2, alpha, beta,
                                                              gamma, abs_a, redo.as<int32_t>(), nredo.as<int32_t>());
    else
      knn_rescore_kernel<ORDER_ARM><<<rg, 256, rsm, stream>>>(Q32 + b0 * d, X32, n, d, mcur, kk, kk2,
                                                              row_k != nullptr ? row_k + b0 : nullptr, mmode, metric,
                                                              kept, kept2.as<uint64_t>(),
                                                              qn2.as<float>() + b0, xmax_norm, xmax_n2, alpha, beta,
                                                              gamma, abs_a, redo.as<int32_t>(), nredo.as<int32_t>());
    ::fuelg::note_launch();
    FUELG_CUDA(cudaGetLastError());
    // first kk exact keys of every query
    FUELG_CUDA(cudaMemcpy2DAsync(dst, (size_t)kk * 8, kept2.p, (size_t)kk2 * 8, (size_t)kk * 8, (size_t)mcur,
                                 cudaMemcpyDeviceToDevice, stream));
    int h_redo = 0;
    FUELG_CUDA(cudaMemcpyAsync(&h_redo, nredo.p, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
    FUELG_CUDA(cudaStreamSynchronize(stream));
    if (h_redo > 0) {
      // queries the proof could not certify: exact scan
      Scratch qre, kre;
      FUELG_TRY(qre.alloc(sizeof(float) * (size_t)h_redo * d, stream));
      FUELG_TRY(kre.alloc(sizeof(uint64_t) * (size_t)h_redo * kk, stream));
      gather_rows_kernel<<<4 * 152, 256, 0, stream>>>(Q32 + b0 * d, d, redo.as<int32_t>(), nredo.as<int32_t>(),
                                                      qre.as<float>()); ::fuelg::note_launch();
      ExactScanParams sp;
      sp.A = qre.as<float>();
      sp.m = h_redo;
      sp.B = X32;
      sp.n = n;
      sp.d = d;
      sp.kind = KIND_KNN;
      sp.order = order;
      sp.metric = metric;
      sp.kk = kk;
      FUELG_TRY(exact_topk(sp, kre.as<uint64_t>(), dev_status, stream));
      scatter_keys_kernel<<<(unsigned)(((int64_t)h_redo * kk + 255) / 256), 256, 0, stream>>>(
          kre.as<uint64_t>(), kk, kk, redo.as<int32_t>(), h_redo, dst); ::fuelg::note_launch();
      FUELG_CUDA(cudaGetLastError());
      total_redo += h_redo;
    }
  }
  if (rescored) *rescored = margin ? m * (int64_t)kk2 + total_redo * n : 0;
  return ST_OK;
}

}  // namespace fuelg
