// fuelg_sums.cuh -- device pieces of the exact centroid-sum update shared by
// the update kernels (fuelg_sums.cu) and the fused tensor-core Lloyd pass
// (fuelg_tc.cu), which commits its labels and plans the buckets itself.
#pragma once

#include <cstdint>

namespace fuelg {

constexpr int kRows = 32;     // rows per accumulation chunk
constexpr int kSmemK = 4096;  // clusters whose histograms fit shared memory

// Device state a fused assignment pass writes instead of the commit kernel:
// the change list (point, old, new label) with its length and the
// per-cluster in/out histograms; the bucket plan is made by the scatter
// kernel that follows.
struct SumsCommit {
  int32_t *chg_i, *chg_old, *chg_new, *nchg;
  int32_t *cin, *cout;  // histograms (zeroed by the previous centre update)
  int32_t *off_in, *off_out, *chunk_off, *counts, *chunk_info;
  int k;
};

// One full warp (lane = its lane index): bucket offsets and the chunk table
// (in-chunks of cluster 0..k-1, then out-chunks), member counts, and
// chunk_info[c] = cluster of chunk c (bit 31: an out-chunk), from the
// complete in/out histograms.  Warp-shuffle scans over 32-entry tiles.  The
// histograms and counts of the first kPlanPre tiles (k <= 128) are loaded
// up front, so a small k costs one round trip to memory, not one per tile.
constexpr int kPlanPre = 4;
__device__ __forceinline__ void plan_body(int lane, int k, const int32_t* __restrict__ cin,
                                          const int32_t* __restrict__ cout, int32_t* __restrict__ off_in,
                                          int32_t* __restrict__ off_out, int32_t* __restrict__ chunk_off,
                                          int32_t* __restrict__ counts, int32_t* __restrict__ chunk_info) {
  int32_t pin[kPlanPre], pout[kPlanPre], pcnt[kPlanPre];
#pragma unroll
  for (int t = 0; t < kPlanPre; t++) {
    const int j = 32 * t + lane;
    const bool v = j < k;
    pin[t] = v ? cin[j] : 0;
    pout[t] = v ? cout[j] : 0;
    pcnt[t] = v ? counts[j] : 0;
  }
  int32_t carry_c = 0;
  // one 32-cluster tile of one pass, given this lane's histogram entry c
  auto tile = [&](int pass, int t0, int32_t c, int32_t& carry_m) {
    const int j = t0 + lane;
    int32_t* off = pass == 0 ? off_in : off_out;
    const int32_t nc = (c + kRows - 1) / kRows;
    int32_t a = c, b = nc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t ua = __shfl_up_sync(0xffffffffu, a, o), ub = __shfl_up_sync(0xffffffffu, b, o);
      if (lane >= o) {
        a += ua;
        b += ub;
      }
    }
    if (j < k) {
      off[j] = carry_m + a - c;
      const int32_t c0 = carry_c + b - nc;
      chunk_off[pass * k + j] = c0;
      for (int q = 0; q < nc; q++) chunk_info[c0 + q] = j | (pass << 31);
    }
    carry_m += __shfl_sync(0xffffffffu, a, 31);
    carry_c += __shfl_sync(0xffffffffu, b, 31);
  };
  for (int pass = 0; pass < 2; pass++) {
    int32_t carry_m = 0;
#pragma unroll
    for (int t = 0; t < kPlanPre; t++)
      if (32 * t < k) tile(pass, 32 * t, pass == 0 ? pin[t] : pout[t], carry_m);
    for (int t0 = 32 * kPlanPre; t0 < k; t0 += 32) {
      const int j = t0 + lane;
      tile(pass, t0, j < k ? (pass == 0 ? cin[j] : cout[j]) : 0, carry_m);
    }
  }
#pragma unroll
  for (int t = 0; t < kPlanPre; t++) {
    const int j = 32 * t + lane;
    if (j < k) counts[j] = pcnt[t] + pin[t] - pout[t];
  }
  for (int j = 32 * kPlanPre + lane; j < k; j += 32) counts[j] += cin[j] - cout[j];
  if (lane == 0) chunk_off[2 * k] = carry_c;
}

// Clusters a scatter kernel plans for itself (the fused tensor-core pass
// has k <= 256).
constexpr int kPlanMaxK = 256;

// One full warp: the bucket offsets alone (exclusive prefix sums of the in
// and out histograms) into oin / oout -- shared memory of the calling block.
// All histogram entries are loaded before the scans (one round trip).
__device__ __forceinline__ void plan_offsets(int lane, int k, const int32_t* __restrict__ cin,
                                             const int32_t* __restrict__ cout, int32_t* oin, int32_t* oout) {
  int32_t vi[kPlanMaxK / 32], vo[kPlanMaxK / 32];
#pragma unroll
  for (int t = 0; t < kPlanMaxK / 32; t++) {
    const int j = 32 * t + lane;
    vi[t] = j < k ? cin[j] : 0;
    vo[t] = j < k ? cout[j] : 0;
  }
  int32_t ci = 0, co = 0;
#pragma unroll
  for (int t = 0; t < kPlanMaxK / 32; t++) {
    if (32 * t >= k) break;
    int32_t a = vi[t], b = vo[t];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t ua = __shfl_up_sync(0xffffffffu, a, o), ub = __shfl_up_sync(0xffffffffu, b, o);
      if (lane >= o) {
        a += ua;
        b += ub;
      }
    }
    const int j = 32 * t + lane;
    if (j < k) {
      oin[j] = ci + a - vi[t];
      oout[j] = co + b - vo[t];
    }
    ci += __shfl_sync(0xffffffffu, a, 31);
    co += __shfl_sync(0xffffffffu, b, 31);
  }
}

}  // namespace fuelg
