// fuelg_tc.cu -- tensor-core (tcgen05 / TMEM / TMA) screen for the Lloyd
// assignment, with exact re-scoring of every point the screen cannot decide.
//
// Per 128-point tile the CTA computes the 128 x kp block of dot products
// X_tile . C^T on the 5th-generation tensor cores (kind::f16, BF16 operands,
// FP32 accumulators in TMEM), then each epilogue thread forms the screened
// squared distances D~_j = ||x||^2 + ||c_j||^2 - 2 x.c_j for its point and a
// rigorous per-pair error bound E_j that covers the BF16 (or split hi+lo BF16)
// rounding of the operands, the FP32 accumulation inside the tensor core, the
// epilogue arithmetic and the rounding of fuel's own FP32 distance.  The point
// is decided on the spot when the best centre j* satisfies
//     D~_j - E_j > D~_j* + E_j*   for every j != j*,
// because then fuel's own f32 distance to j* is strictly smaller than to any
// other centre (src/cluster/kmeans/lloyd.rs:165-172, strict '<').  Otherwise
// the candidate set {j : D~_j - E_j <= D~_j* + E_j*} is re-scored with the
// reference's exact f32 operation order (fuelg_common.cuh) and the first
// minimum wins -- so the assignment is identical to the plain exact path.
//
// Kernel structure (one CTA per SM, persistent over point tiles):
//   warp 0      TMA producer: 128x64 BF16 point chunk + kp x 64 centre chunk
//               per pipeline stage (128-byte swizzle), mbarrier complete_tx
//   warp 1      TMEM owner and single-thread tcgen05.mma issuer (M=128,
//               N=kp, K=16 per instruction), tcgen05.commit to free stages
//   warps 2-5   epilogue: tcgen05.ld of the accumulator rows, screen, write
// Two TMEM accumulators alternate so the epilogue of tile t overlaps the MMAs
// of tile t+1.  Every mbarrier wait is bounded (globaltimer); on expiry the
// kernel records DEV_TIMEOUT, stops all roles and still frees its TMEM.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "fuelg_common.cuh"
#include "fuelg_internal.h"
#include "fuelg_prep.cuh"
#include "fuelg_sums.cuh"
#include "fuelg_tc_common.cuh"

namespace fuelg {

using namespace tcx;

namespace {

constexpr int BM = 128;  // points per tile (UMMA M)
constexpr int kTcThreads = 192;

// Exact re-score of the undecided points: each candidate centre is scored
// with the reference's own f32 operation order, first minimum wins.  One warp
// per undecided point; the lanes mirror the reference's SIMD lanes:
//   8-lane kinds (math::sqdist on non-x86, the linear-scan distance): 8 lanes
//     per candidate, lane l owns accumulator l, 4 candidates at a time;
//   avx2::sqdist_f32: 32 lanes per candidate, lane 8u+l owns accumulator u,l;
//   pairwise chains (initial pass): one lane per candidate.
template <int KIND, int ORDER>
__device__ __forceinline__ float warp_candidate_dist(const float* __restrict__ x, const float* __restrict__ c, int d,
                                                     int lane) {
  constexpr bool LANE8 = (KIND == KIND_KNN) || (KIND == KIND_SQDIST && ORDER == ORDER_ARM);
  constexpr bool FMA8 = (KIND == KIND_KNN && ORDER == ORDER_X86);
  if constexpr (LANE8) {
    const int l = lane & 7, g0 = lane & ~7;
    const int sd = d & ~7;
    float acc = 0.0f;
#pragma unroll 8
    for (int i = l; i < sd; i += 8) {
      const float df = __fsub_rn(x[i], c[i]);
      acc = FMA8 ? __fmaf_rn(df, df, acc) : __fadd_rn(sq_rn(df), acc);
    }
    float s = __shfl_sync(0xffffffffu, acc, g0);
#pragma unroll
    for (int t = 1; t < 8; t++) s = __fadd_rn(s, __shfl_sync(0xffffffffu, acc, g0 + t));
    for (int i = sd; i < d; i++) {
      const float df = __fsub_rn(x[i], c[i]);
      s = FMA8 ? __fmaf_rn(df, df, s) : __fadd_rn(s, sq_rn(df));
    }
    return s;  // valid on every lane of the group
  } else if constexpr (KIND == KIND_SQDIST) {  // x86 avx2::sqdist_f32, d >= 4
    const int nb = d / 32;
    float a = 0.0f;
#pragma unroll 8
    for (int b = 0; b < nb; b++) {
      const float df = __fsub_rn(x[b * 32 + lane], c[b * 32 + lane]);
      a = __fmaf_rn(df, df, a);
    }
    const int l = lane & 7;
    const float a0 = __shfl_sync(0xffffffffu, a, l), a1 = __shfl_sync(0xffffffffu, a, l + 8);
    const float a2 = __shfl_sync(0xffffffffu, a, l + 16), a3 = __shfl_sync(0xffffffffu, a, l + 24);
    float cl = __fadd_rn(__fadd_rn(a0, a1), __fadd_rn(a2, a3));
    int i = nb * 32;
    for (; i + 8 <= d; i += 8) {
      const float df = __fsub_rn(x[i + l], c[i + l]);
      cl = __fmaf_rn(df, df, cl);
    }
    float v[8];
#pragma unroll
    for (int t = 0; t < 8; t++) v[t] = __shfl_sync(0xffffffffu, cl, t);
    float s = __fadd_rn(__fadd_rn(__fadd_rn(v[0], v[4]), __fadd_rn(v[1], v[5])),
                        __fadd_rn(__fadd_rn(v[2], v[6]), __fadd_rn(v[3], v[7])));
    for (; i < d; i++) {
      const float df = __fsub_rn(x[i], c[i]);
      s = __fmaf_rn(df, df, s);
    }
    return s;
  } else {
    return exact_dist_scalar<KIND, ORDER>(x, c, d);  // one lane, one chain
  }
}

// One warp re-scores one undecided point x against its candidate centres
// (bit j of um[0..mw) set: centre j), PER at a time (this lane's slot is
// lane / G); returns the first centre with the smallest exact distance, on
// every lane.
template <int KIND, int ORDER>
__device__ __forceinline__ int rescore_point(const float* __restrict__ x, const float* __restrict__ C, int d, int mw,
                                             const uint64_t* __restrict__ um, int lane) {
  constexpr bool LANE8 = (KIND == KIND_KNN) || (KIND == KIND_SQDIST && ORDER == ORDER_ARM);
  constexpr int G = LANE8 ? 8 : (KIND == KIND_SQDIST ? 32 : 1);  // lanes per candidate
  constexpr int PER = 32 / G;                                      // candidates per warp step
  uint64_t best = KEY_NONE;
  int w = 0;
  uint64_t m = um[0];
  const int slot = lane / G;
  for (;;) {
    int got = 0, j = 0;
    while (got < PER) {
      while (m == 0 && w + 1 < mw) m = um[++w];
      if (m == 0) break;
      const int b = __ffsll((long long)m) - 1;
      m &= m - 1;
      if (got == slot) j = w * 64 + b;
      got++;
    }
    if (got == 0) break;
    const bool mine = slot < got;
    if (!mine) j = 0;  // idle slots score centre 0 and discard it
    // lloyd.rs:166-168 calls sqdist(centre, point); the initial pairwise
    // kernel takes (point, centre).  The squares are identical either way.
    const float dist = warp_candidate_dist<KIND, ORDER>(x, C + (int64_t)j * d, d, lane);
    if (mine && (lane % G) == 0) {
      const uint64_t key = make_key(dist, (uint32_t)j);
      best = key < best ? key : best;
    }
    if (got < PER) break;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const uint64_t o = __shfl_xor_sync(0xffffffffu, best, off);
    best = o < best ? o : best;
  }
  return (int)key_idx(best);
}

struct TcArgs {
  int64_t n;
  int d, k, kp, kc, stages;
  const float* nx;  // ||x||^2 per point (f32 of an FP64 sum)
  const float* xn;  // ||x||
  const float* nc;  // ||c||^2 per (padded) centre, as two halves: nc[j] + nc[kp + j]
  int32_t* lab_new;
  int32_t* ulist;
  uint64_t* umask;
  int32_t* ucount;
  int mw;
  float alpha, beta, gamma;
  uint32_t idesc;
  uint32_t tmem_cols;
  int a_tiled;  // A copies are tile-major (see prep_offset)
  float s_scale;              // nonneg data: sum|x_i c_i| <= dot * s_scale
  int sep_lo;                 // hi+lo: the hi.lo + lo.hi terms have their own accumulator
  const int* neg_flag;        // != 0 when X holds a negative value
  int* status;
  const volatile int* cancel;
  // Fused pass (every pass after the first of a k-means call): the labels of
  // decided points are committed here (change list, histograms); the
  // undecided ones go to ulist for the re-score kernel, which commits them
  // and plans the buckets -- no lab_new and no commit kernel.
  int fused;
  int32_t* labels;
  SumsCommit sc;
};

// MODE: kBf16 (A, B single BF16), kSplit (A and B hi + lo: three products),
// kScaledA (A exact in BF16 -- integers of a scaled copy -- and B hi + lo: two
// products; the A lo term of the split form is identically zero).
constexpr int kBf16 = 0, kSplit = 1, kScaledA = 2;

template <int MODE>
__global__ void __launch_bounds__(kTcThreads, 2)
    lloyd_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmAlo,
                    const __grid_constant__ CUtensorMap tmB, const __grid_constant__ CUtensorMap tmBlo, TcArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const uint32_t a_bytes = BM * BK * 2;
  const uint32_t b_bytes = (uint32_t)a.kp * BK * 2;
  constexpr bool ALO = MODE == kSplit, BLO = MODE != kBf16;
  const uint32_t stage_bytes = (ALO ? 2u : 1u) * a_bytes + (BLO ? 2u : 1u) * b_bytes;
  // stage layout: A | B | A lo (kSplit) | B lo (kSplit, kScaledA)
  const uint32_t off_alo = a_bytes + b_bytes, off_blo = (ALO ? 2u : 1u) * a_bytes + b_bytes;
  const int NS = a.stages;
  uint64_t* full = reinterpret_cast<uint64_t*>(base + (size_t)NS * stage_bytes);
  uint64_t* empty = full + NS;
  uint64_t* accf = empty + NS;
  uint64_t* acce = accf + 2;
  uint64_t* fin = acce + 2;
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(fin + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_holder + 1);
  // centre norms (16-byte aligned: pass 2 reads them four at a time)
  float* snc = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(tmem_holder + 4) + 15) & ~(uintptr_t)15);
  float* scn = snc + a.kp;
  int32_t* h_in = reinterpret_cast<int32_t*>(scn + a.kp);  // fused: per-CTA in/out histograms
  int32_t* h_out = h_in + a.kp;
  // the centre norms again, 16-byte aligned, +inf past k up to a multiple of 64
  float* sncd = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(h_out + a.kp) + 15) & ~(uintptr_t)15);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ntiles = (a.n + BM - 1) / BM;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], BM / 32);  // one arrive per epilogue warp
    }
    mbar_init(fin, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                 "r"(a.tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_holder;
  // X does not depend on the predecessor kernel: the producer issues the A
  // (point) tiles of the first NS stages before waiting for it; the centre
  // tiles (B) and norms come from the predecessor.
  int pre = 0;
  if (warp == 0 && lane == 0) {
    prefetch_tmap(&tmA);
    if (ALO) prefetch_tmap(&tmAlo);
    const uint64_t pol_a = policy_evict_first();
    int64_t t = blockIdx.x;
    int kc = 0;
    for (int st = 0; st < NS && t < ntiles; st++) {
      uint8_t* sA = base + (size_t)st * stage_bytes;
      mbar_expect_tx(&full[st], stage_bytes);
      const int ax = a.a_tiled ? 0 : kc * BK;
      const int ay = a.a_tiled ? (int)((t * a.kc + kc) * BM) : (int)(t * BM);
      tma_load_2d_hint(sA, &tmA, ax, ay, &full[st], pol_a);
      if (ALO) tma_load_2d_hint(sA + off_alo, &tmAlo, ax, ay, &full[st], pol_a);
      pre++;
      if (++kc == a.kc) {
        kc = 0;
        t += gridDim.x;
      }
    }
  }
  griddep_wait();
  griddep_launch();
  // The centre norms and the per-CTA histograms belong to the epilogue: its
  // warps stage them behind their own barrier, so the producer's first
  // centre chunk goes out without waiting for these loads.
  // Per CTA, for the epilogue's uniform bound: the largest centre norms and
  // whether every norm is finite and below 2^124.
  float sncmax = 0.0f, scnmax = 0.0f;
  bool cta_finite = true;
  if (warp >= 2) {
    const int kp64 = (a.kp + 63) & ~63;
    for (int j = threadIdx.x - 64; j < kp64; j += BM) {
      // squared norms: the sum of the two halves the centre update wrote
      const float nc2 = j < a.kp ? a.nc[j] + a.nc[a.kp + j] : 0.0f;
      if (j < a.kp) {
        snc[j] = nc2;
        scn[j] = sqrtf(nc2);
        h_in[j] = 0;
        h_out[j] = 0;
      }
      sncd[j] = j < a.k ? nc2 : __int_as_float(0x7f800000);
    }
    named_bar_sync(1, BM);
    for (int j = 0; j < a.k; j++) {
      const float s2 = snc[j], c1 = scn[j];
      cta_finite = cta_finite && s2 < 0x1p124f && c1 < 0x1p62f;
      sncmax = fmaxf(sncmax, s2);
      scnmax = fmaxf(scnmax, c1);
    }
  }

  if (warp == 0) {
    if (lane == 0) {
      prefetch_tmap(&tmB);
      if (BLO) prefetch_tmap(&tmBlo);
      const uint64_t pol_a = policy_evict_first(), pol_b = policy_evict_last();
      uint32_t stage = 0, phase = 0;
      uint32_t armed = 0, last_ph = 0;  // per-stage bit: armed at least once / parity of the last arm
      int tile_no = 0;
      for (int64_t t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x, tile_no++) {
        if (a.cancel != nullptr && *a.cancel) {
          atomicOr(a.status, DEV_CANCELLED);
          *abort_flag = 1;
          break;
        }
        for (int kc = 0; kc < a.kc; kc++) {
          uint8_t* sA = base + (size_t)stage * stage_bytes;
          uint8_t* sB = sA + a_bytes;
          armed |= 1u << stage;
          last_ph = (last_ph & ~(1u << stage)) | (phase << stage);
          if (pre > 0) {
            // A already in flight (issued before the dependency wait)
            pre--;
          } else {
            if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag)) {
              if (!*abort_flag) atomicOr(a.status, DEV_TIMEOUT);
              *abort_flag = 1;
              break;
            }
            mbar_expect_tx(&full[stage], stage_bytes);
            const int ax = a.a_tiled ? 0 : kc * BK;
            const int ay = a.a_tiled ? (int)((t * a.kc + kc) * BM) : (int)(t * BM);
            tma_load_2d_hint(sA, &tmA, ax, ay, &full[stage], pol_a);
            if (ALO) tma_load_2d_hint(sA + off_alo, &tmAlo, ax, ay, &full[stage], pol_a);
          }
          tma_load_2d_hint(sB, &tmB, kc * BK, 0, &full[stage], pol_b);
          if (BLO) tma_load_2d_hint(sA + off_blo, &tmBlo, kc * BK, 0, &full[stage], pol_b);
          if (++stage == (uint32_t)NS) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
      // Never leave the CTA with a TMA copy still writing shared memory: wait
      // (bounded) for the last load armed on every stage.
      for (int s2 = 0; s2 < NS; s2++)
        if (armed & (1u << s2)) {
          volatile int never = 0;
          if (!mbar_wait(&full[s2], (last_ph >> s2) & 1u, &never)) atomicOr(a.status, DEV_TIMEOUT);
        }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      uint32_t stage = 0, phase = 0;
      int64_t lt = 0;
      for (int64_t t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x, lt++) {
        const uint32_t buf = (uint32_t)(lt & 1), accph = (uint32_t)((lt >> 1) & 1);
        if (!mbar_wait(&acce[buf], accph ^ 1, abort_flag)) {
          if (!*abort_flag) atomicOr(a.status, DEV_TIMEOUT);
          *abort_flag = 1;
          break;
        }
        tc_fence_after();
        // split: hi.hi accumulates at [0, kp), the hi.lo + lo.hi terms at [kp, 2kp)
        const uint32_t acc_cols = (BLO && a.sep_lo ? 2u : 1u) * (uint32_t)a.kp;
        const uint32_t d_tmem = tmem_base + buf * acc_cols;
        const uint32_t d_lo = d_tmem + (a.sep_lo ? (uint32_t)a.kp : 0u);
        bool ok = true;
        for (int kc = 0; kc < a.kc; kc++) {
          if (!mbar_wait(&full[stage], phase, abort_flag)) {
            if (!*abort_flag) atomicOr(a.status, DEV_TIMEOUT);
            *abort_flag = 1;
            ok = false;
            break;
          }
          tc_fence_after();
          uint8_t* sA = base + (size_t)stage * stage_bytes;
          uint8_t* sB = sA + a_bytes;
          const uint64_t ad = smem_desc_sw128(smem_u32(sA));
          const uint64_t bd = smem_desc_sw128(smem_u32(sB));
#pragma unroll
          for (int kk = 0; kk < BK / 16; kk++) {
            // advance 16 BF16 (32 bytes) along K inside the swizzled row
            umma_bf16(d_tmem, ad + 2 * kk, bd + 2 * kk, a.idesc, (kc | kk) != 0 ? 1u : 0u);
            if (BLO) {
              const uint64_t bdlo = smem_desc_sw128(smem_u32(sA + off_blo));
              umma_bf16(d_lo, ad + 2 * kk, bdlo + 2 * kk, a.idesc, (a.sep_lo && (kc | kk) == 0) ? 0u : 1u);
            }
            if (ALO) {
              const uint64_t adlo = smem_desc_sw128(smem_u32(sA + off_alo));
              umma_bf16(d_lo, adlo + 2 * kk, bd + 2 * kk, a.idesc, 1u);
            }
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
      // every MMA this thread issued has completed before TMEM is freed
      umma_commit(fin);
      volatile int never = 0;
      if (!mbar_wait(fin, 0, &never)) atomicOr(a.status, DEV_TIMEOUT);
    }
  } else {
    // epilogue: warps 2..5 -> TMEM lane groups 2,3,0,1
    const int g = warp & 3;
    const int row = g * 32 + lane;
    // fused: commit a label (warp-collective; act: this lane has one) --
    // change list by one reservation per warp, histograms in shared memory
    auto commit = [&](bool act, int64_t i, int lb, int old) {
      bool ch = false;
      if (act) {
        ch = lb != old;
        if (ch) a.labels[i] = lb;
      }
      const unsigned chm = __ballot_sync(0xffffffffu, ch);
      if (chm) {
        int base = 0;
        if (lane == 0) base = atomicAdd(a.sc.nchg, __popc(chm));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (ch) {
          const int pos = base + __popc(chm & ((1u << lane) - 1u));
          a.sc.chg_i[pos] = (int32_t)i;
          a.sc.chg_old[pos] = old;
          a.sc.chg_new[pos] = lb;
          atomicAdd(&h_in[lb], 1);
          atomicAdd(&h_out[old], 1);
        }
      }
    };
    int64_t lt = 0;
    const bool nonneg = *a.neg_flag == 0;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, lt++) {
      const uint32_t buf = (uint32_t)(lt & 1), accph = (uint32_t)((lt >> 1) & 1);
      // this point's norms and current label, loaded while the tile's MMAs run
      const int64_t i = t * BM + row;
      const bool valid = i < a.n;
      const float nxi = valid ? a.nx[i] : 0.0f;
      const float xni = valid ? a.xn[i] : 0.0f;
      const int32_t old_lab = (a.fused && valid) ? a.labels[i] : -1;
      const bool ok = !*abort_flag && mbar_wait(&accf[buf], accph, abort_flag);
      if (!ok) {
        if (!*abort_flag) atomicOr(a.status, DEV_TIMEOUT);
        *abort_flag = 1;
      }
      if (!__all_sync(0xffffffffu, ok)) break;  // warp-uniform exit
      tc_fence_after();
      const uint32_t acc_cols = (BLO && a.sep_lo ? 2u : 1u) * (uint32_t)a.kp;
      const uint32_t taddr = tmem_base + ((uint32_t)(g * 32) << 16) + buf * acc_cols;
      float best = __int_as_float(0x7f800000), best_dot = 0.0f;
      int bj = 0;
      uint64_t m0 = 0, m1 = 0, m2 = 0, m3 = 0;
      if (a.kp <= 64) {
        // Pass 1 without branches, per 32 columns (TMEM -> registers): the
        // screen values dt_c = fma(-2, v_c, nxi + snc_c) (padding columns: +inf
        // through sncd) reduced by a tree that keeps the smallest value, its
        // first index and dot product, and the second smallest value (the left
        // operand wins ties, so the first index wins, as in a scan).
        float second = __int_as_float(0x7f800000), vmax = 0.0f;
#pragma unroll
        for (int r = 0; r < 2; r++) {
          if (32 * r >= a.kp) break;
          uint32_t rh[2][16], rl[2][16];
#pragma unroll
          for (int h = 0; h < 2; h++)
            if (32 * r + 16 * h < a.kp) {
              tmem_ld16_nowait(taddr + 32 * r + 16 * h, rh[h]);
              if (BLO && a.sep_lo) tmem_ld16_nowait(taddr + a.kp + 32 * r + 16 * h, rl[h]);
            }
          tmem_ld_wait();
#pragma unroll
          for (int h = 0; h < 2; h++) {
            tmem_regs_ready(rh[h]);
            if (BLO && a.sep_lo) tmem_regs_ready(rl[h]);
          }
          float v[32], m[32], dv[32], s2[16];
          int id[32];
#pragma unroll
          for (int h = 0; h < 2; h++) {
            const bool ld = 32 * r + 16 * h < a.kp;
#pragma unroll
            for (int j = 0; j < 16; j++) {
              float x = ld ? __uint_as_float(rh[h][j]) : 0.0f;
              if (BLO && a.sep_lo && ld) x += __uint_as_float(rl[h][j]);
              v[16 * h + j] = x;
            }
          }
          const float4* sd4 = reinterpret_cast<const float4*>(sncd + 32 * r);
#pragma unroll
          for (int q = 0; q < 8; q++) {
            const float4 s4 = sd4[q];
            m[4 * q + 0] = fmaf(-2.0f, v[4 * q + 0], nxi + s4.x);
            m[4 * q + 1] = fmaf(-2.0f, v[4 * q + 1], nxi + s4.y);
            m[4 * q + 2] = fmaf(-2.0f, v[4 * q + 2], nxi + s4.z);
            m[4 * q + 3] = fmaf(-2.0f, v[4 * q + 3], nxi + s4.w);
          }
#pragma unroll
          for (int c = 0; c < 32; c++) {
            dv[c] = v[c];
            id[c] = 32 * r + c;
          }
#pragma unroll
          for (int c = 0; c < 32; c += 2) {
            const bool rt = m[c + 1] < m[c];
            s2[c >> 1] = rt ? m[c] : m[c + 1];
            m[c] = rt ? m[c + 1] : m[c];
            id[c] = rt ? id[c + 1] : id[c];
            dv[c] = rt ? dv[c + 1] : dv[c];
          }
#pragma unroll
          for (int w = 2; w < 32; w <<= 1)
#pragma unroll
            for (int c = 0; c < 32; c += 2 * w) {
              const bool rt = m[c + w] < m[c];
              const float lose = rt ? m[c] : m[c + w];
              s2[c >> 1] = min3_f32(lose, s2[c >> 1], s2[(c + w) >> 1]);
              m[c] = rt ? m[c + w] : m[c];
              id[c] = rt ? id[c + w] : id[c];
              dv[c] = rt ? dv[c + w] : dv[c];
            }
          if (r == 0) {
            best = m[0];
            bj = id[0];
            best_dot = dv[0];
            second = s2[0];
          } else {
            const bool rt = m[0] < best;
            second = min3_f32(rt ? best : m[0], second, s2[0]);
            best = rt ? m[0] : best;
            bj = rt ? id[0] : bj;
            best_dot = rt ? dv[0] : best_dot;
          }
          if (nonneg) {
            float mx = vmax;
#pragma unroll
            for (int c = 0; c < 32; c += 2) mx = max3_f32(mx, v[c], v[c + 1]);
            vmax = mx;
          }
        }
        const float sb = nonneg ? fmaxf(best_dot, 0.0f) * a.s_scale : xni * scn[bj];
        const float eb = (a.alpha * sb + a.beta * (nxi + snc[bj])) * (1.0f + a.gamma) + a.gamma * fabsf(best);
        const float hi = best + eb;
        // Every other column j has dt_j >= second, and its rounded bound e_j
        // (at most five roundings of non-negative terms) stays below
        // (C + gamma |dt_j|)(1 + 2^-24)^5, C = the bound's other terms at the
        // largest S_j and snc_j; t - gamma' |t| grows with t, so with
        // tb >= (C + gamma |second|)(1 + 2^-18) a value second - tb two ulps
        // above hi makes the per-column test below pass for every j.  Finite
        // norms below 2^124 keep every dt finite.
        constexpr float kInfl = 1.0f + 0x1p-18f;
        const float smax = nonneg ? fmaxf(vmax, 0.0f) * a.s_scale : xni * scnmax;
        const float cmax = (a.alpha * smax + a.beta * (nxi + sncmax)) * (1.0f + a.gamma) * kInfl;
        const float tb = fmaf(a.gamma * kInfl, fabsf(second), cmax);
        const float hu = __fadd_ru(__fmaf_ru(fabsf(hi), 0x1p-22f, hi), 0x1p-125f);
        const bool easy = cta_finite && nxi < 0x1p124f && (second - tb) >= hu;
        if (__any_sync(0xffffffffu, !easy)) {
          // pass 2: every other centre whose lower bound reaches the best's
          // upper bound (the columns re-read from TMEM, 32 per wait)
          uint32_t blo = 0, bhi = 0;
#pragma unroll
          for (int r = 0; r < 2; r++) {
            if (32 * r >= a.kp) break;
            uint32_t rh[2][16], rl[2][16];
#pragma unroll
            for (int h = 0; h < 2; h++)
              if (32 * r + 16 * h < a.kp) {
                tmem_ld16_nowait(taddr + 32 * r + 16 * h, rh[h]);
                if (BLO && a.sep_lo) tmem_ld16_nowait(taddr + a.kp + 32 * r + 16 * h, rl[h]);
              }
            tmem_ld_wait();
#pragma unroll
            for (int h = 0; h < 2; h++) {
              tmem_regs_ready(rh[h]);
              if (BLO && a.sep_lo) tmem_regs_ready(rl[h]);
            }
            uint32_t bits = 0;
#pragma unroll
            for (int h = 0; h < 2; h++) {
              if (32 * r + 16 * h >= a.kp) break;
#pragma unroll
              for (int q = 0; q < 4; q++) {
                const int c4 = 32 * r + 16 * h + 4 * q;
                const float4 n4 = *reinterpret_cast<const float4*>(snc + c4);
                const float4 s4 = *reinterpret_cast<const float4*>(scn + c4);
                const float nn[4] = {n4.x, n4.y, n4.z, n4.w}, ss[4] = {s4.x, s4.y, s4.z, s4.w};
#pragma unroll
                for (int u = 0; u < 4; u++) {
                  float x = __uint_as_float(rh[h][4 * q + u]);
                  if (BLO && a.sep_lo) x += __uint_as_float(rl[h][4 * q + u]);
                  const float dt = fmaf(-2.0f, x, nxi + nn[u]);
                  const float sj = nonneg ? fmaxf(x, 0.0f) * a.s_scale : xni * ss[u];
                  const float e = (a.alpha * sj + a.beta * (nxi + nn[u])) * (1.0f + a.gamma) + a.gamma * fabsf(dt);
                  bits |= (!(dt - e > hi) ? 1u : 0u) << (16 * h + 4 * q + u);
                }
              }
            }
            if (r == 0) blo = bits;
            else bhi = bits;
          }
          const uint64_t kmask = a.k >= 64 ? ~0ull : ((1ull << a.k) - 1ull);
          m0 = ((((uint64_t)bhi) << 32) | blo) & kmask & ~(1ull << bj);
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&acce[buf]);
      } else {
      // pass 1: screened argmin (first index wins ties)
      for (int c0 = 0; c0 < a.kp; c0 += 16) {
        float v[16];
        tmem_ld16(taddr + c0, v);
        if (BLO && a.sep_lo) {
          float w[16];
          tmem_ld16(taddr + a.kp + c0, w);
#pragma unroll
          for (int j = 0; j < 16; j++) v[j] += w[j];
        }
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const int col = c0 + j;
          if (col < a.k) {
            const float dt = fmaf(-2.0f, v[j], nxi + snc[col]);
            if (dt < best) {
              best = dt;
              bj = col;
              best_dot = v[j];
            }
          }
        }
      }
      // S_j bounds sum_i |x_i c_ij|: |x||c_j| in general, the (inflated) dot product for nonnegative data
      const float sb = nonneg ? fmaxf(best_dot, 0.0f) * a.s_scale : xni * scn[bj];
      const float eb = (a.alpha * sb + a.beta * (nxi + snc[bj])) * (1.0f + a.gamma) + a.gamma * fabsf(best);
      const float hi = best + eb;
      // pass 2: every other centre whose lower bound reaches the best's upper bound
      for (int c0 = 0; c0 < a.kp; c0 += 16) {
        float v[16];
        tmem_ld16(taddr + c0, v);
        if (BLO && a.sep_lo) {
          float w[16];
          tmem_ld16(taddr + a.kp + c0, w);
#pragma unroll
          for (int j = 0; j < 16; j++) v[j] += w[j];
        }
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const int col = c0 + j;
          if (col < a.k && col != bj) {
            const float dt = fmaf(-2.0f, v[j], nxi + snc[col]);
            const float sj = nonneg ? fmaxf(v[j], 0.0f) * a.s_scale : xni * scn[col];
            const float e = (a.alpha * sj + a.beta * (nxi + snc[col])) * (1.0f + a.gamma) + a.gamma * fabsf(dt);
            if (!(dt - e > hi)) {
              const uint64_t bit = 1ull << (col & 63);
              const int w = col >> 6;
              if (w == 0) m0 |= bit;
              else if (w == 1) m1 |= bit;
              else if (w == 2) m2 |= bit;
              else m3 |= bit;
            }
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[buf]);
      }
      const bool und = (m0 | m1 | m2 | m3) != 0;
      if (a.fused) commit(valid && !und, i, bj, old_lab);  // undecided points: committed by the re-score kernel
      if (valid) {
        if (!und) {
          if (!a.fused) a.lab_new[i] = bj;
        } else {
          const uint64_t bit = 1ull << (bj & 63);
          const int w = bj >> 6;
          if (w == 0) m0 |= bit;
          else if (w == 1) m1 |= bit;
          else if (w == 2) m2 |= bit;
          else m3 |= bit;
          if (!a.fused) a.lab_new[i] = -1;
          const int u = atomicAdd(a.ucount, 1);
          a.ulist[u] = (int32_t)i;
          uint64_t* um = a.umask + (int64_t)u * a.mw;
          um[0] = m0;
          if (a.mw > 1) um[1] = m1;
          if (a.mw > 2) um[2] = m2;
          if (a.mw > 3) um[3] = m3;
        }
      }
    }
    if (a.fused) {
      // this CTA's histograms into the global ones
      named_bar_sync(1, BM);
      for (int j = threadIdx.x - 64; j < a.k; j += BM) {
        if (h_in[j]) atomicAdd(&a.sc.cin[j], h_in[j]);
        if (h_out[j]) atomicAdd(&a.sc.cout[j], h_out[j]);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(a.tmem_cols)
                 : "memory");
  }
}

// X (f32) -> BF16 hi (and lo) copies, norms: one warp per row (prep_row in
// fuelg_prep.cuh).
template <bool SPLIT>
__global__ void prep_rows_kernel(const float* __restrict__ X, int64_t rows, int64_t valid_rows, int d, int dp,
                                 int tile_kc, __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                                 float* __restrict__ nrm2, float* __restrict__ nrm, int* __restrict__ neg_flag,
                                 int32_t* __restrict__ zero_word, float scale) {
  griddep_wait();
  griddep_launch();
  if (zero_word != nullptr && blockIdx.x == 0 && threadIdx.x == 0) *zero_word = 0;
  bool anyneg = false;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const bool vec = ((d & 3) == 0) && ((reinterpret_cast<uintptr_t>(X) & 15) == 0);
  for (int64_t r = (int64_t)blockIdx.x * nw + warp; r < rows; r += (int64_t)gridDim.x * nw)
    anyneg |= prep_row<SPLIT>(X + r * d, r, r < valid_rows, vec, d, dp, tile_kc, hi, lo, nrm2, nrm, lane, scale);
  if (neg_flag != nullptr && __any_sync(0xffffffffu, anyneg) && (threadIdx.x & 31) == 0) atomicOr(neg_flag, 1);
}

// Smallest non-zero and largest |x| over X (as ordered float bits): out[0]
// (start 0x7f800000) and out[1] (start 0).
__global__ void abs_range_kernel(const float* __restrict__ X, int64_t count, unsigned* __restrict__ out) {
  unsigned lo = 0x7f800000u, hi = 0u;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = tid; e < count; e += nth) {
    const unsigned b = __float_as_uint(X[e]) & 0x7fffffffu;
    if (b != 0u) lo = min(lo, b);
    hi = max(hi, b);
  }
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&out[0], lo);
    atomicMax(&out[1], hi);
  }
}

// Scaled-integer copy of X for the kScaledA screen: every value x must be
// s * I (|I| <= 256, I = rint(x / s)) to within |x - I s| <= 2^-21 |x|; the
// copy holds I (exact in BF16), tile-major like prep_rows_kernel, with the
// norms of x itself.  Any value outside the form sets *fail.
__global__ void prep_scaled_kernel(const float* __restrict__ X, int64_t rows, int64_t valid_rows, int d, int dp,
                                   int tile_kc, float s, __nv_bfloat16* __restrict__ q, float* __restrict__ nrm2,
                                   float* __restrict__ nrm, int* __restrict__ neg_flag, int* __restrict__ fail) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  bool anyneg = false, bad = false;
  const bool vec = (d & 3) == 0 && (reinterpret_cast<uintptr_t>(X) & 15) == 0;
  // I = rint(x * fl(1/s)): for x within 2^-21 relative of I s with |I| <= 256
  // the product is within 2^-12 of I, so this is rint(x / s); any other x
  // fails the check below whichever integer it rounds to.
  const float inv_s = __frcp_rn(s);
  for (int64_t r = (int64_t)blockIdx.x * nw + warp; r < rows; r += (int64_t)gridDim.x * nw) {
    const bool v = r < valid_rows;
    const float* xr = X + r * d;
    float acc = 0.0f;
    // up to 8 chunks of 4 values per lane are loaded before any is used
    for (int cb = 4 * lane; cb < dp; cb += 128 * 8) {
      float x8[8][4];
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const int c0 = cb + 128 * u;
        if (v && vec && c0 + 3 < d) {
          const float4 t4 = __ldg(reinterpret_cast<const float4*>(xr + c0));
          x8[u][0] = t4.x, x8[u][1] = t4.y, x8[u][2] = t4.z, x8[u][3] = t4.w;
        } else {
#pragma unroll
          for (int t = 0; t < 4; t++) x8[u][t] = (v && c0 + t < d) ? __ldg(xr + c0 + t) : 0.0f;
        }
      }
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const int c0 = cb + 128 * u;
        if (c0 >= dp) break;
        const float* x4 = x8[u];
        float i4[4];
#pragma unroll
        for (int t = 0; t < 4; t++) {
          i4[t] = rintf(__fmul_rn(x4[t], inv_s));
          bad |= !(fabsf(i4[t]) <= 256.0f) || !(fabsf(fmaf(-i4[t], s, x4[t])) <= 4.76837158203125e-07f * fabsf(x4[t]));
          acc = fmaf(x4[t], x4[t], acc);
          anyneg |= x4[t] < 0.0f;
        }
        __nv_bfloat162 h01 = __floats2bfloat162_rn(i4[0], i4[1]);
        __nv_bfloat162 h23 = __floats2bfloat162_rn(i4[2], i4[3]);
        uint2 pk;
        pk.x = *reinterpret_cast<uint32_t*>(&h01);
        pk.y = *reinterpret_cast<uint32_t*>(&h23);
        *reinterpret_cast<uint2*>(q + prep_offset(r, c0, dp, tile_kc)) = pk;
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (lane == 0) {
      nrm2[r] = acc;
      nrm[r] = sqrtf(acc);
    }
  }
  if (__any_sync(0xffffffffu, anyneg) && lane == 0) atomicOr(neg_flag, 1);
  if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(fail, 1);
}

template <int KIND, int ORDER>
__global__ void rescore_kernel(const float* __restrict__ X, const float* __restrict__ C, int d, int mw,
                               const int32_t* __restrict__ ulist, const uint64_t* __restrict__ umask,
                               const int32_t* __restrict__ ucount, int32_t* __restrict__ lab_new,
                               unsigned long long* __restrict__ tally) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int cnt = *ucount;
  if (blockIdx.x == 0 && threadIdx.x == 0) *tally += (unsigned long long)cnt;
  for (int64_t u = gw; u < cnt; u += nwarps) {
    const int64_t i = ulist[u];
    const int lb = rescore_point<KIND, ORDER>(X + i * d, C, d, mw, umask + u * mw, lane);
    if (lane == 0) lab_new[i] = lb;
  }
}

// Same re-score with the point row and the current candidate rows staged in
// shared memory by all 32 lanes (coalesced 16-byte loads, one round trip),
// then the sequential per-lane accumulations read shared memory.  4 warps per
// block; used for d <= 1024.
template <int KIND, int ORDER>
__global__ void __launch_bounds__(128) rescore_smem_kernel(const float* __restrict__ X, const float* __restrict__ C,
                                                           int d, int ds, int mw, const int32_t* __restrict__ ulist,
                                                           const uint64_t* __restrict__ umask,
                                                           const int32_t* __restrict__ ucount,
                                                           int32_t* __restrict__ lab_new,
                                                           unsigned long long* __restrict__ tally,
                                                           int32_t* __restrict__ labels, SumsCommit sc, int commit,
                                                           int64_t cap) {
  constexpr bool LANE8 = (KIND == KIND_KNN) || (KIND == KIND_SQDIST && ORDER == ORDER_ARM);
  constexpr int G = LANE8 ? 8 : 32;
  constexpr int PER = 32 / G;
  extern __shared__ __align__(16) float rs_smem[];
  griddep_wait();
  griddep_launch();
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  float* xs = rs_smem + (size_t)wib * (PER + 1) * ds;
  float* cs = xs + ds;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  // the warp's first list entry and candidate word are read with the count
  // (cap: entries the list and mask buffers hold)
  const int64_t g0 = gw < cap ? gw : 0;
  const int64_t i_next = ulist[g0];
  const uint64_t m_next = umask[g0 * mw];
  const int cnt = *ucount;
  if (blockIdx.x == 0 && threadIdx.x == 0) *tally += (unsigned long long)cnt;
  const bool v4 = (d & 3) == 0;
  for (int64_t u = gw; u < cnt; u += nwarps) {
    const int64_t i = u == gw ? i_next : ulist[u];
    // the committed label, read now: off the path after the distances
    const int32_t old = (commit && lane == 0) ? labels[i] : 0;
    const float* x = X + i * d;
    __syncwarp();
    // 16-byte rows by asynchronous copies: the point row and the first group
    // of candidate rows below arrive in one round trip
    if (v4)
      for (int e = lane; e < d / 4; e += 32) cp_async16(xs + 4 * e, x + 4 * e);
    else
      for (int e = lane; e < d; e += 32) xs[e] = __ldg(x + e);
    uint64_t best = KEY_NONE;
    int w = 0;
    uint64_t m = u == gw ? m_next : umask[u * mw];
    const int slot = lane / G;
    for (;;) {
      int got = 0, j = 0;
      int js[PER];
      while (got < PER) {
        while (m == 0 && w + 1 < mw) m = umask[u * mw + (++w)];
        if (m == 0) break;
        const int b = __ffsll((long long)m) - 1;
        m &= m - 1;
        js[got] = w * 64 + b;
        if (got == slot) j = js[got];
        got++;
      }
      if (got == 0) break;
      __syncwarp();
      for (int t = 0; t < got; t++) {
        const float* c = C + (int64_t)js[t] * d;
        float* dst = cs + (size_t)t * ds;
        if (v4)
          for (int e = lane; e < d / 4; e += 32) cp_async16(dst + 4 * e, c + 4 * e);
        else
          for (int e = lane; e < d; e += 32) dst[e] = __ldg(c + e);
      }
      cp_async_wait_all();
      __syncwarp();
      const bool mine = slot < got;
      if (!mine) j = 0;
      const float dist = warp_candidate_dist<KIND, ORDER>(xs, cs + (size_t)(mine ? slot : 0) * ds, d, lane);
      if (mine && (lane % G) == 0) {
        const uint64_t key = make_key(dist, (uint32_t)j);
        best = key < best ? key : best;
      }
      if (got < PER) break;
    }
    cp_async_wait_all();  // (every row has a candidate: nothing is left in flight)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const uint64_t o = __shfl_xor_sync(0xffffffffu, best, off);
      best = o < best ? o : best;
    }
    if (lane == 0) {
      const int32_t lb = (int32_t)key_idx(best);
      if (!commit) {
        lab_new[i] = lb;
      } else {
        // fused pass: commit this point's label (few points: global atomics)
        if (lb != old) {
          labels[i] = lb;
          const int pos = atomicAdd(sc.nchg, 1);
          sc.chg_i[pos] = (int32_t)i;
          sc.chg_old[pos] = old;
          sc.chg_new[pos] = lb;
          atomicAdd(&sc.cin[lb], 1);
          atomicAdd(&sc.cout[old], 1);
        }
      }
    }
  }
}

}  // namespace

// Per-call state of the tensor-core Lloyd tier: the BF16 copy of X is made
// once per k-means call; the centre copy every iteration.
struct TcLloydState {
  bool split = false;
  int mode = kBf16;    // kBf16, kSplit or kScaledA (split tier on scaled-integer data)
  float scale = 1.0f;  // kScaledA: X = scale * (integer copy); centre copies hold fl(scale * c)
  int dp = 0, kp = 0, kc = 0, mw = 0, stages = 0;
  int64_t arows = 0;  // rows of the tile-major A copies (whole tiles)
  int ctas_per_sm = 1;
  bool sep_lo = false;
  size_t smem = 0;
  Scratch xhi, xlo, xnrm2, xnrm, chi, clo, cnrm2, cnrm, ulist, umask, ucount, rescored_total, negf;
  CUtensorMap tmA, tmAlo, tmB, tmBlo;
};

bool lloyd_tc_supported(int d, int k) { return d >= 32 && k >= 1 && k <= 256; }

int lloyd_tc_prepare(const LloydParams& p, TcLloydState* st, cudaStream_t stream) {
  const int64_t n = p.n;
  st->split = p.precision == 2;
  st->dp = (p.d + 7) & ~7;
  st->kp = (p.k + 15) & ~15;
  st->kc = (st->dp + BK - 1) / BK;
  st->mw = (st->kp + 63) / 64;
  st->arows = ((n + BM - 1) / BM) * BM;
  const size_t xb = (size_t)st->arows * st->kc * BK * 2;
  FUELG_TRY(st->xhi.alloc(xb, stream));
  FUELG_TRY(st->xnrm2.alloc(sizeof(float) * st->arows, stream));
  FUELG_TRY(st->xnrm.alloc(sizeof(float) * st->arows, stream));
  FUELG_TRY(st->negf.alloc(sizeof(int), stream));
  FUELG_CUDA(cudaMemsetAsync(st->negf.p, 0, sizeof(int), stream));
  // Split tier on data that are integers |I| <= 256 times one scale s (to
  // within 2^-21 relative; quantised data such as 8-bit pixel values / 255):
  // the scaled copy I is exact in BF16, so the A lo term of the split form is
  // zero and A is one BF16 copy (half the bytes) -- kScaledA.  s = the smallest
  // non-zero |x|; the conversion kernel verifies every value.
  st->mode = st->split ? kSplit : kBf16;
  st->scale = 1.0f;
  if (st->split && getenv("FUELG_TC_NO_SCALED") == nullptr) {
    Scratch rng, fail;
    FUELG_TRY(rng.alloc(sizeof(unsigned) * 2, stream));
    FUELG_TRY(fail.alloc(sizeof(int), stream));
    const unsigned init[2] = {0x7f800000u, 0u};
    FUELG_CUDA(cudaMemcpyAsync(rng.p, init, sizeof(init), cudaMemcpyHostToDevice, stream));
    FUELG_CUDA(cudaMemsetAsync(fail.p, 0, sizeof(int), stream));
    abs_range_kernel<<<8 * 152, 256, 0, stream>>>(p.X, n * (int64_t)p.d, rng.as<unsigned>());
    ::fuelg::note_launch();
    unsigned hr[2];
    FUELG_CUDA(cudaMemcpyAsync(hr, rng.p, sizeof(hr), cudaMemcpyDeviceToHost, stream));
    FUELG_CUDA(cudaStreamSynchronize(stream));
    float lo, hi;
    memcpy(&lo, &hr[0], sizeof(float));
    memcpy(&hi, &hr[1], sizeof(float));
    if (hr[0] < 0x7f800000u && hr[1] < 0x7f800000u && (double)hi <= 256.0 * (double)lo * (1.0 + 1e-6)) {
      prep_scaled_kernel<<<8 * 152, 256, 0, stream>>>(p.X, st->arows, n, p.d, st->kc * BK, st->kc, lo,
                                                      st->xhi.as<__nv_bfloat16>(), st->xnrm2.as<float>(),
                                                      st->xnrm.as<float>(), st->negf.as<int>(), fail.as<int>());
      ::fuelg::note_launch();
      FUELG_CUDA(cudaGetLastError());
      int hf = 1;
      FUELG_CUDA(cudaMemcpyAsync(&hf, fail.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
      FUELG_CUDA(cudaStreamSynchronize(stream));
      if (hf == 0) {
        st->mode = kScaledA;
        st->scale = lo;
      } else {
        FUELG_CUDA(cudaMemsetAsync(st->negf.p, 0, sizeof(int), stream));
      }
    }
  }
  const bool alo = st->mode == kSplit, blo = st->mode != kBf16;
  const size_t a_bytes = BM * BK * 2, b_bytes = (size_t)st->kp * BK * 2;
  const size_t stage_bytes = (alo ? 2 : 1) * a_bytes + (blo ? 2 : 1) * b_bytes;
  // Tunables (defaults measured on GB300): FUELG_TC_STAGES pipeline depth,
  // FUELG_TC_CTAS_PER_SM resident CTAs per SM (shared memory is divided).
  int per_sm = 2;
  if (const char* e = getenv("FUELG_TC_CTAS_PER_SM")) per_sm = std::max(1, std::min(2, atoi(e)));
  const size_t budget = per_sm == 1 ? 200 * 1024 : 100 * 1024;
  int stages = (int)(budget / stage_bytes);
  if (const char* e = getenv("FUELG_TC_STAGES")) stages = atoi(e);
  stages = std::max(2, std::min(8, stages));
  {
    uint32_t cols = 32;
    st->sep_lo = blo && st->kp <= 128;
    while (cols < (uint32_t)((st->sep_lo ? 4 : 2) * st->kp)) cols <<= 1;
    if (cols * per_sm > 512) per_sm = 1;
    if (per_sm == 1 && getenv("FUELG_TC_STAGES") == nullptr) stages = std::max(2, std::min(8, (int)((200 * 1024) / stage_bytes)));
  }
  st->ctas_per_sm = per_sm;
  st->stages = stages;
  st->smem = 1024 + stages * stage_bytes + 8 * (2 * stages + 5) + 16 + 16 + 16 * st->kp + 16 +
              4 * ((st->kp + 63) / 64 * 64) + 16;
  if (st->smem > 227 * 1024) {
    set_error("tensor-core Lloyd tile does not fit shared memory (k=%d)", p.k);
    return ST_ENOTSUP;
  }
  if (alo) FUELG_TRY(st->xlo.alloc(xb, stream));
  const size_t cb = (size_t)st->kp * st->dp * 2;
  FUELG_TRY(st->chi.alloc(cb, stream));
  if (blo) FUELG_TRY(st->clo.alloc(cb, stream));
  // [2][kp]: the centre update writes the squared norm in two halves (the
  // first-pass preparation writes the first, the second stays zero)
  FUELG_TRY(st->cnrm2.alloc(sizeof(float) * 2 * st->kp, stream));
  FUELG_CUDA(cudaMemsetAsync(st->cnrm2.p, 0, sizeof(float) * 2 * st->kp, stream));
  FUELG_TRY(st->cnrm.alloc(sizeof(float) * st->kp, stream));
  FUELG_TRY(st->ulist.alloc(sizeof(int32_t) * n, stream));
  FUELG_TRY(st->umask.alloc(sizeof(uint64_t) * n * st->mw, stream));
  FUELG_TRY(st->ucount.alloc(sizeof(int32_t), stream));
  FUELG_TRY(st->rescored_total.alloc(sizeof(unsigned long long), stream));
  FUELG_CUDA(cudaMemsetAsync(st->rescored_total.p, 0, sizeof(unsigned long long), stream));
  if (st->mode != kScaledA) {
    auto pk = alo ? prep_rows_kernel<true> : prep_rows_kernel<false>;
    pk<<<8 * 152, 256, 0, stream>>>(p.X, st->arows, n, p.d, st->kc * BK, st->kc, st->xhi.as<__nv_bfloat16>(),
                                    alo ? st->xlo.as<__nv_bfloat16>() : (__nv_bfloat16*)nullptr,
                                    st->xnrm2.as<float>(), st->xnrm.as<float>(), st->negf.as<int>(), nullptr, 1.0f);
    ::fuelg::note_launch();
    FUELG_CUDA(cudaGetLastError());
  }
  // A: tile-major [arows * kc, 64] -- each box is one contiguous 16 KB block
  FUELG_TRY(tcx::make_map_bf16(&st->tmA, st->xhi.p, st->arows * st->kc, BK, BM));
  FUELG_TRY(tcx::make_map_bf16(&st->tmB, st->chi.p, st->kp, st->dp, st->kp));
  st->tmAlo = st->tmA;
  st->tmBlo = st->tmB;
  if (alo) FUELG_TRY(tcx::make_map_bf16(&st->tmAlo, st->xlo.p, st->arows * st->kc, BK, BM));
  if (blo) FUELG_TRY(tcx::make_map_bf16(&st->tmBlo, st->clo.p, st->kp, st->dp, st->kp));
  auto kern = st->mode == kScaledA ? lloyd_tc_kernel<kScaledA>
              : st->mode == kSplit ? lloyd_tc_kernel<kSplit> : lloyd_tc_kernel<kBf16>;
  FUELG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)st->smem));
  return ST_OK;
}

namespace {
// One screen launch.  fused == nullptr: lab_new receives every label (the
// undecided ones from the re-score kernel launched after it); otherwise the
// pass commits into fused->labels itself (TcArgs).  prep: convert the centres
// first (else the previous centre update wrote their BF16 copies).
int tc_pass(const LloydParams& p, TcLloydState* st, const float* centers, bool first, int32_t* lab_new,
            int32_t* labels, const SumsCommit* fused, bool prep, int* dev_status, cudaStream_t stream) {
  const int64_t n = p.n;
  // centre copies and norms for this iteration (padded rows are zero); block 0
  // also clears the undecided-point counter for this pass
  if (prep) {
    auto pk = st->split ? prep_rows_kernel<true> : prep_rows_kernel<false>;
    FUELG_TRY(launch_pdl(pk, dim3((st->kp + 7) / 8), dim3(256), 0, stream, centers, (int64_t)st->kp, (int64_t)p.k,
                         p.d, st->dp, 0, st->chi.as<__nv_bfloat16>(),
                         st->split ? st->clo.as<__nv_bfloat16>() : (__nv_bfloat16*)nullptr, st->cnrm2.as<float>(),
                         st->cnrm.as<float>(), (int*)nullptr, st->ucount.as<int32_t>(), st->scale));
  }
  TcArgs a{};
  a.n = n;
  a.d = p.d;
  a.k = p.k;
  a.kp = st->kp;
  a.kc = st->kc;
  a.stages = st->stages;
  a.nx = st->xnrm2.as<float>();
  a.xn = st->xnrm.as<float>();
  a.nc = st->cnrm2.as<float>();
  a.lab_new = lab_new;
  a.ulist = st->ulist.as<int32_t>();
  a.umask = st->umask.as<uint64_t>();
  a.ucount = st->ucount.as<int32_t>();
  a.mw = st->mw;
  // Error-bound constants.  Operand rounding: u = 2^-8 per BF16 value, so a
  // BF16 product is within (2u + u^2)|x_i c_i|; hi+lo leaves x_lo c_lo and the
  // residuals, within 3.01 * 2^-16 |x_i c_i|.  FP32 accumulation of KP terms in
  // the tensor core: within KP * 2^-23 of their absolute sum (allowing
  // truncation); with hi+lo the hi.hi terms and the (2^-8 smaller) hi.lo +
  // lo.hi terms use separate accumulators.  Both scale with
  // S = sum_i |x_i c_i| <= |x||c| (for nonnegative data S = x.c itself).  The
  // distance takes 2 x.c.  Norms and epilogue roundings stay within beta
  // (|x|^2 + |c|^2); fuel's own f32 sum of d squares within (d + 4) 2^-24 of
  // the distance (gamma).  kScaledA: x = s I + e with |e| <= 2^-21 |x| and I
  // exact; B = hi + lo of fl(s c) is within (2^-16 + 2^-24)|s c| of s c, so the
  // operand error is (2^-16 + 2 2^-24)(1 + d) + d with d = 2^-21 (taken as
  // 2^-20), and the two accumulators add KP 2^-23 (1 + 2u) + KP 2^-23 2.01 u.
  const double KP = (double)st->kc * BK;
  const double u8 = std::ldexp(1.0, -8), u23 = std::ldexp(1.0, -23), u24 = std::ldexp(1.0, -24);
  double rel;
  if (st->mode == kScaledA) {
    const double dl = std::ldexp(1.0, -20);
    rel = (std::ldexp(1.0, -16) + 2 * u24) * (1.0 + dl) + dl +
          (KP * u23 * (1.0 + 2 * u8) + (st->sep_lo ? 1.0 : 2.0) * KP * u23 * 2.01 * u8) * (1.0 + dl) + u24;
  } else if (st->split && st->sep_lo)
    rel = 3.01 * std::ldexp(1.0, -16) + KP * u23 * (1.0 + 2 * u8) + 2.0 * KP * u23 * 2.01 * u8 + u24;
  else if (st->split)
    rel = 3.01 * std::ldexp(1.0, -16) + 3.0 * KP * u23 * (1.0 + 2 * u8);
  else
    rel = (2 * u8 + u8 * u8) + KP * u23 * (1.0 + 2 * u8);
  a.alpha = (float)(2.0 * rel * 1.01);
  a.s_scale = (float)(1.0 / (1.0 - 1.01 * rel) * (1.0 + std::ldexp(1.0, -20)));
  a.neg_flag = st->negf.as<int>();
  a.beta = (float)(((p.d + 31) / 32 + 9) * std::ldexp(1.0, -24) * 1.01);
  a.gamma = (float)((p.d + 4) * std::ldexp(1.0, -24) * 1.01);
  // instruction descriptor: D=F32, A=B=BF16, K-major both, N=kp, M=128
  a.a_tiled = 1;
  a.idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(st->kp >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
  uint32_t cols = 32;
  while (cols < (uint32_t)((st->sep_lo ? 4 : 2) * st->kp)) cols <<= 1;
  a.tmem_cols = cols;
  a.sep_lo = st->sep_lo ? 1 : 0;
  a.status = dev_status;
  a.cancel = cancel_word_device();
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t ntiles = (n + BM - 1) / BM;
  const int grid = (int)std::min<int64_t>(ntiles, (int64_t)sms * st->ctas_per_sm);
  if (fused) {
    a.fused = 1;
    a.labels = labels;
    a.sc = *fused;
  }
  HotTimer* ht = hot_timer();
  if (ht) ht->begin(stream);
  {
    auto kern = st->mode == kScaledA ? lloyd_tc_kernel<kScaledA>
                : st->mode == kSplit ? lloyd_tc_kernel<kSplit> : lloyd_tc_kernel<kBf16>;
    FUELG_TRY(launch_pdl(kern, dim3(grid), dim3(kTcThreads), st->smem, stream, st->tmA, st->tmAlo, st->tmB,
                         st->tmBlo, a));
  }
  if (ht) ht->end(stream);
  FUELG_CUDA(cudaGetLastError());
  const int rgrid = 8 * sms;
  const int kind = first ? KIND_PAIRWISE : KIND_SQDIST;
  if (kind == KIND_PAIRWISE) {
    if (p.order == ORDER_X86)
      rescore_kernel<KIND_PAIRWISE, ORDER_X86><<<rgrid, 256, 0, stream>>>(p.X, centers, p.d, st->mw, a.ulist, a.umask,
                                                                         a.ucount, a.lab_new, st->rescored_total.as<unsigned long long>());
    else
      rescore_kernel<KIND_PAIRWISE, ORDER_ARM><<<rgrid, 256, 0, stream>>>(p.X, centers, p.d, st->mw, a.ulist, a.umask,
                                                                         a.ucount, a.lab_new, st->rescored_total.as<unsigned long long>()); ::fuelg::note_launch();
  } else {
    // staged row stride: 16-byte aligned and == 8 (mod 32) floats, so the four
    // 8-lane groups of a warp read four different bank groups
    int ds = (p.d + 3) & ~3;
    while (ds % 32 != 8) ds += 4;
    if (p.d <= 1024) {
      const int per = p.order == ORDER_X86 ? 1 : 4;
      const size_t sm = (size_t)4 * (per + 1) * ds * sizeof(float);
      const int g2 = 2 * sms;  // one wave: a few hundred points per pass after the first
      if (p.order == ORDER_X86) {
        auto kfn = rescore_smem_kernel<KIND_SQDIST, ORDER_X86>;
        FUELG_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        FUELG_TRY(launch_pdl(kfn, dim3(g2), dim3(128), sm, stream, p.X, centers, p.d, ds, st->mw,
                             (const int32_t*)a.ulist, (const uint64_t*)a.umask, (const int32_t*)a.ucount, a.lab_new,
                             st->rescored_total.as<unsigned long long>(), labels, a.sc, fused ? 1 : 0,
                             (int64_t)p.n));
      } else {
        auto kfn = rescore_smem_kernel<KIND_SQDIST, ORDER_ARM>;
        FUELG_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        FUELG_TRY(launch_pdl(kfn, dim3(g2), dim3(128), sm, stream, p.X, centers, p.d, ds, st->mw,
                             (const int32_t*)a.ulist, (const uint64_t*)a.umask, (const int32_t*)a.ucount, a.lab_new,
                             st->rescored_total.as<unsigned long long>(), labels, a.sc, fused ? 1 : 0,
                             (int64_t)p.n));
      }
    } else if (fused) {
      set_error("the fused Lloyd pass needs d <= 1024");
      return ST_EINVAL;
    } else if (p.order == ORDER_X86) {
      rescore_kernel<KIND_SQDIST, ORDER_X86><<<rgrid, 256, 0, stream>>>(p.X, centers, p.d, st->mw, a.ulist, a.umask,
                                                                       a.ucount, a.lab_new, st->rescored_total.as<unsigned long long>()); ::fuelg::note_launch();
    } else {
      rescore_kernel<KIND_SQDIST, ORDER_ARM><<<rgrid, 256, 0, stream>>>(p.X, centers, p.d, st->mw, a.ulist, a.umask,
                                                                       a.ucount, a.lab_new, st->rescored_total.as<unsigned long long>()); ::fuelg::note_launch();
    }
  }
FUELG_CUDA(cudaGetLastError());
  return ST_OK;
}

}  // namespace

int lloyd_assign_tc(const LloydParams& p, TcLloydState* st, const float* centers, bool first, int32_t* lab_new,
                    int* dev_status, cudaStream_t stream) {
  return tc_pass(p, st, centers, first, lab_new, nullptr, nullptr, true, dev_status, stream);
}

// A later pass: the screen commits the decided labels, the re-score kernel
// the undecided ones and plans the buckets (d <= 1024).  The centre copies
// were written by the previous centre update (lloyd_tc_centre_prep), which
// also cleared the undecided-point counter.
int lloyd_tc_pass_fused(const LloydParams& p, TcLloydState* st, const float* centers, int32_t* labels,
                        const SumsCommit& sc, int* dev_status, cudaStream_t stream) {
  return tc_pass(p, st, centers, false, nullptr, labels, &sc, false, dev_status, stream);
}

bool lloyd_tc_scaled(const TcLloydState* st) { return st->mode == kScaledA; }

CentrePrep lloyd_tc_centre_prep(TcLloydState* st) {
  CentrePrep cp;
  cp.hi = st->chi.as<__nv_bfloat16>();
  cp.lo = st->split ? st->clo.as<__nv_bfloat16>() : nullptr;
  cp.nrm2 = st->cnrm2.as<float>();
  cp.dp = st->dp;
  cp.kp = st->kp;
  cp.zero_word = st->ucount.as<int32_t>();
  cp.scale = st->scale;
  return cp;
}

int lloyd_tc_rescored_total(TcLloydState* st, cudaStream_t stream, int64_t* out) {
  unsigned long long h = 0;
  FUELG_CUDA(cudaMemcpyAsync(&h, st->rescored_total.p, sizeof(h), cudaMemcpyDeviceToHost, stream));
  FUELG_CUDA(cudaStreamSynchronize(stream));
  *out = (int64_t)h;
  return ST_OK;
}

TcLloydState* lloyd_tc_new() { return new TcLloydState(); }
void lloyd_tc_delete(TcLloydState* s) { delete s; }

}  // namespace fuelg
