// fuelg_sums.cu -- exact, order-independent centroid sums for Lloyd.
//
// fuel keeps f32 running sums updated by per-chunk f32 deltas
// (src/cluster/kmeans/lloyd.rs:154-199), so its centres depend on the rayon
// chunking.  Here every coordinate sum is kept EXACTLY as an integer: each f32
// value x is an integer multiple of 2^e_lo, where e_lo is the weight of the
// lowest set mantissa bit over all of X, so x = I(x) * 2^e_lo with |I(x)| <
// 2^(e_hi - e_lo + 1).  A running sum is stored modulo 2^(32L) as L
// uint64 limbs of 32-bit slices (two's complement), updated only for the
// points whose label changed (+x into the new cluster, -x out of the old).
// Integer addition is associative, so the slices may be accumulated with
// atomics in any order and the result is bit-for-bit deterministic.  The
// centre is then the correctly rounded (round-to-nearest-even) f32 of the
// exact mean sum/count -- the value an exact-arithmetic Lloyd would produce.
// Empty clusters keep their centre (lloyd.rs:138-146).
#include <algorithm>
#include <cmath>

#include "fuelg_common.cuh"
#include "fuelg_exact.cuh"
#include "fuelg_internal.h"
#include "fuelg_prep.cuh"
#include "fuelg_sums.cuh"

namespace fuelg {

namespace {

__device__ __forceinline__ void range_acc(float x, int& lo, int& hi, int& bad) {
  uint32_t mant;
  int l, h;
  bool z, b;
  f32_parts(x, mant, l, h, z, b);
  if (b) bad = 1;
  if (!z && !b) {
    lo = min(lo, l);
    hi = max(hi, h);
  }
}

__global__ void exp_range_kernel(const float* __restrict__ X, int64_t count, int* __restrict__ out) {
  int lo = 1 << 30, hi = -(1 << 30), bad = 0;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
  if ((reinterpret_cast<uintptr_t>(X) & 15) == 0) {
    const int64_t c4 = count / 4;
    const float4* X4 = reinterpret_cast<const float4*>(X);
    for (int64_t e = tid; e < c4; e += nth) {
      const float4 v = __ldg(X4 + e);
      range_acc(v.x, lo, hi, bad);
      range_acc(v.y, lo, hi, bad);
      range_acc(v.z, lo, hi, bad);
      range_acc(v.w, lo, hi, bad);
    }
    for (int64_t e = c4 * 4 + tid; e < count; e += nth) range_acc(X[e], lo, hi, bad);
  } else {
    for (int64_t e = tid; e < count; e += nth) range_acc(X[e], lo, hi, bad);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, off));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, off));
    bad |= __shfl_xor_sync(0xffffffffu, bad, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&out[0], lo);
    atomicMax(&out[1], hi);
    if (bad) atomicOr(&out[2], 1);
  }
}

// Changed labels -> change list + per-cluster in/out histograms.  `first`: no
// previous label (the initial assignment puts every point in).  Histograms are
// aggregated in shared memory per block when k fits (integer counts: exact).

__device__ __forceinline__ void commit_body(int bid, int nblk, int32_t* h_in, int32_t* h_out,
                                            const int32_t* __restrict__ lab_new, int64_t n, int first, int k,
                                            int32_t* __restrict__ labels, int32_t* __restrict__ chg_i,
                                            int32_t* __restrict__ chg_old, int32_t* __restrict__ chg_new,
                                            int32_t* __restrict__ nchg, int32_t* __restrict__ cin,
                                            int32_t* __restrict__ cout) {
  const bool local = k <= kSmemK;
  if (local)
    for (int j = threadIdx.x; j < k; j += blockDim.x) h_in[j] = h_out[j] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (int64_t base0 = (int64_t)bid * blockDim.x; base0 < n; base0 += (int64_t)nblk * blockDim.x) {
    const int64_t i = base0 + threadIdx.x;
    bool ch = false;
    int32_t nw = 0, old = -1;
    if (i < n) {
      nw = lab_new[i];
      old = first ? -1 : labels[i];
      ch = nw != old;
      if (ch) labels[i] = nw;
    }
    const unsigned mask = __ballot_sync(0xffffffffu, ch);
    if (mask) {
      int base = 0;
      if (lane == 0) base = atomicAdd(nchg, __popc(mask));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (ch) {
        const int pos = base + __popc(mask & ((1u << lane) - 1));
        chg_i[pos] = (int32_t)i;
        chg_old[pos] = old;
        chg_new[pos] = nw;
        if (local) {
          atomicAdd(&h_in[nw], 1);
          if (old >= 0) atomicAdd(&h_out[old], 1);
        } else {
          atomicAdd(&cin[nw], 1);
          if (old >= 0) atomicAdd(&cout[old], 1);
        }
      }
    }
  }
  __syncthreads();
  if (local)
    for (int j = threadIdx.x; j < k; j += blockDim.x) {
      if (h_in[j]) atomicAdd(&cin[j], h_in[j]);
      if (h_out[j]) atomicAdd(&cout[j], h_out[j]);
    }
}

// Commit, then the last block to finish (a ticket after a fence: no
// waiting) plans the buckets from the complete histograms.
__global__ void commit_changes_kernel(const int32_t* __restrict__ lab_new, int64_t n, int first, int k,
                                      int32_t* __restrict__ labels, int32_t* __restrict__ chg_i,
                                      int32_t* __restrict__ chg_old, int32_t* __restrict__ chg_new,
                                      int32_t* __restrict__ nchg, int32_t* __restrict__ cin,
                                      int32_t* __restrict__ cout, unsigned* __restrict__ done,
                                      int32_t* __restrict__ off_in, int32_t* __restrict__ off_out,
                                      int32_t* __restrict__ chunk_off, int32_t* __restrict__ counts,
                                      int32_t* __restrict__ chunk_info) {
  __shared__ int32_t h_in[kSmemK], h_out[kSmemK];
  __shared__ unsigned s_last;
  griddep_wait();
  griddep_launch();
  commit_body(blockIdx.x, gridDim.x, h_in, h_out, lab_new, n, first, k, labels, chg_i, chg_old, chg_new, nchg, cin,
              cout);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(done, 1u) == gridDim.x - 1 ? 1u : 0u;
  __syncthreads();
  if (s_last) {
    __threadfence();
    if (threadIdx.x < 32) plan_body(threadIdx.x, k, cin, cout, off_in, off_out, chunk_off, counts, chunk_info);
    if (threadIdx.x == 0) *done = 0;
  }
}

__device__ __forceinline__ void scatter_body(int bid, int nblk, int32_t* c_in, int32_t* c_out,
                                             const int32_t* __restrict__ chg_i, const int32_t* __restrict__ chg_old,
                                             const int32_t* __restrict__ chg_new, const int32_t* __restrict__ nchg,
                                             int k, const int32_t* __restrict__ off_in,
                                             const int32_t* __restrict__ off_out, int32_t* __restrict__ cur_in,
                                             int32_t* __restrict__ cur_out, int32_t* __restrict__ bucket_in,
                                             int32_t* __restrict__ bucket_out) {
  const int cnt = *nchg;
  const bool local = k <= kSmemK;
  for (int e0 = bid * blockDim.x; e0 < cnt; e0 += nblk * blockDim.x) {
    const int e = e0 + threadIdx.x;
    const bool v = e < cnt;
    int32_t i = 0, o = -1, w = 0;
    if (v) {
      i = chg_i[e];
      o = chg_old[e];
      w = chg_new[e];
    }
    if (!local) {
      if (v) {
        bucket_in[off_in[w] + atomicAdd(&cur_in[w], 1)] = i;
        if (o >= 0) bucket_out[off_out[o] + atomicAdd(&cur_out[o], 1)] = i;
      }
      continue;
    }
    // block-local ranks, one global reservation per (block, cluster)
    __syncthreads();
    for (int j = threadIdx.x; j < k; j += blockDim.x) c_in[j] = c_out[j] = 0;
    __syncthreads();
    int r_in = 0, r_out = 0;
    if (v) {
      r_in = atomicAdd(&c_in[w], 1);
      if (o >= 0) r_out = atomicAdd(&c_out[o], 1);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < k; j += blockDim.x) {
      c_in[j] = c_in[j] ? atomicAdd(&cur_in[j], c_in[j]) : 0;
      c_out[j] = c_out[j] ? atomicAdd(&cur_out[j], c_out[j]) : 0;
    }
    __syncthreads();
    if (v) {
      bucket_in[off_in[w] + c_in[w] + r_in] = i;
      if (o >= 0) bucket_out[off_out[o] + c_out[o] + r_out] = i;
    }
  }
}

// plan != 0 (the fused pass, k <= kPlanMaxK): the histograms are complete
// but unplanned -- every block derives the bucket offsets it needs in shared
// memory, and block 0's second warp writes the full plan (offsets, chunk
// table, counts) for the accumulation kernel.
__global__ void bucket_scatter_kernel(const int32_t* __restrict__ chg_i, const int32_t* __restrict__ chg_old,
                                      const int32_t* __restrict__ chg_new, const int32_t* __restrict__ nchg, int k,
                                      int32_t* __restrict__ off_in, int32_t* __restrict__ off_out,
                                      int32_t* __restrict__ cur_in, int32_t* __restrict__ cur_out,
                                      int32_t* __restrict__ bucket_in, int32_t* __restrict__ bucket_out, int plan,
                                      const int32_t* __restrict__ cin, const int32_t* __restrict__ cout,
                                      int32_t* __restrict__ chunk_off, int32_t* __restrict__ counts,
                                      int32_t* __restrict__ chunk_info) {
  __shared__ int32_t c_in[kSmemK], c_out[kSmemK];
  __shared__ int32_t s_off[2 * kPlanMaxK];
  griddep_wait();
  griddep_launch();
  const int32_t* oin = off_in;
  const int32_t* oout = off_out;
  if (plan) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) plan_offsets(lane, k, cin, cout, s_off, s_off + kPlanMaxK);
    if (warp == 1 && blockIdx.x == 0) plan_body(lane, k, cin, cout, off_in, off_out, chunk_off, counts, chunk_info);
    __syncthreads();
    oin = s_off;
    oout = s_off + kPlanMaxK;
  }
  scatter_body(blockIdx.x, gridDim.x, c_in, c_out, chg_i, chg_old, chg_new, nchg, k, oin, oout, cur_in, cur_out,
               bucket_in, bucket_out);
}

// 64-bit form of fixed_of for L <= 2 (|I(x)| < 2^63 by construction).
__device__ __forceinline__ unsigned long long fixed_of64(float x, int e_lo, bool negate) {
  const uint32_t bits = __float_as_uint(x);
  const uint32_t eb = (bits >> 23) & 0xffu;
  const uint32_t m = bits & 0x7fffffu;
  if ((bits & 0x7fffffffu) == 0) return 0;
  const uint32_t mant = eb ? (m | 0x800000u) : m;
  const int sh = (eb == 0 ? -149 : (int)eb - 150) - e_lo;
  const unsigned long long v = sh >= 0 ? ((unsigned long long)mant << sh) : (unsigned long long)(mant >> (-sh));
  const bool neg = ((bits >> 31) != 0) != negate;
  return neg ? 0ull - v : v;
}

// One chunk of <= 32 rows of one cluster, signed; thread per coordinate.
// Work item w = chunk * ty + slab (slab: 256 coordinates).
template <int L>
__device__ __forceinline__ void accumulate_body(int bid, int nblk, int ty, int32_t* rid, const float* __restrict__ X,
                                                int d, int k, int e_lo, const int32_t* __restrict__ chunk_off,
                                                const int32_t* __restrict__ chunk_info,
                                                const int32_t* __restrict__ cin, const int32_t* __restrict__ cout,
                                                const int32_t* __restrict__ off_in,
                                                const int32_t* __restrict__ off_out,
                                                const int32_t* __restrict__ bucket_in,
                                                const int32_t* __restrict__ bucket_out,
                                                unsigned long long* __restrict__ limbs) {
  const int total = chunk_off[2 * k];
  for (int w = bid; w < total * ty; w += nblk) {
    const int c = w / ty, slab = w - c * ty;
    const int32_t info = chunk_info[c];
    const bool out = info < 0;
    const int j = info & 0x7fffffff;
    const int r0 = (c - chunk_off[(out ? k : 0) + j]) * kRows;
    const int cnt = out ? cout[j] : cin[j];
    const int rows = min(kRows, cnt - r0);
    const int32_t* src = (out ? bucket_out + off_out[j] : bucket_in + off_in[j]) + r0;
    __syncthreads();
    if (threadIdx.x < kRows) rid[threadIdx.x] = threadIdx.x < rows ? src[threadIdx.x] : -1;
    __syncthreads();
    for (int t = slab * blockDim.x + threadIdx.x; t < d; t += ty * blockDim.x) {
      float xv[kRows];
#pragma unroll
      for (int q = 0; q < kRows; q++) xv[q] = rid[q] >= 0 ? __ldg(X + (int64_t)rid[q] * d + t) : 0.0f;
      unsigned long long acc[L];
#pragma unroll
      for (int l = 0; l < L; l++) acc[l] = 0;
#pragma unroll
      for (int q = 0; q < kRows; q++) {
        if (L <= 2) {
          const unsigned long long v = fixed_of64(xv[q], e_lo, out);
          acc[0] += v & 0xffffffffull;
          if (L == 2) acc[L == 2 ? 1 : 0] += v >> 32;
        } else {
          const unsigned __int128 v = fixed_of(xv[q], e_lo, out);
#pragma unroll
          for (int l = 0; l < L; l++) acc[l] += (unsigned long long)((v >> (32 * l)) & 0xffffffffu);
        }
      }
      unsigned long long* dst = limbs + ((int64_t)j * d + t) * L;
#pragma unroll
      for (int l = 0; l < L; l++)
        if (acc[l]) atomicAdd(dst + l, acc[l]);  // integer: exact in any order
    }
  }
}

template <int L>
__global__ void __launch_bounds__(256) accumulate_kernel(const float* __restrict__ X, int d, int k, int e_lo, int ty,
                                                         const int32_t* __restrict__ chunk_off,
                                                         const int32_t* __restrict__ chunk_info,
                                                         const int32_t* __restrict__ cin,
                                                         const int32_t* __restrict__ cout,
                                                         const int32_t* __restrict__ off_in,
                                                         const int32_t* __restrict__ off_out,
                                                         const int32_t* __restrict__ bucket_in,
                                                         const int32_t* __restrict__ bucket_out,
                                                         unsigned long long* __restrict__ limbs) {
  __shared__ int32_t rid[kRows];
  griddep_wait();
  griddep_launch();
  accumulate_body<L>(blockIdx.x, gridDim.x, ty, rid, X, d, k, e_lo, chunk_off, chunk_info, cin, cout, off_in, off_out,
                     bucket_in, bucket_out, limbs);
}

// Canonicalise one coordinate's limbs (lv: their values, lp: where they
// live) and, for a non-empty cluster (cnt > 0) when write_centers, write its
// exact mean as the correctly rounded f32 centre coordinate to *cptr.
// Returns the coordinate's centre value after the update (oldc: before it).
template <int L>
__device__ __forceinline__ float mean_of(unsigned long long* __restrict__ lp, const unsigned long long* lv, int cnt,
                                         int e_lo, float* __restrict__ cptr, float oldc, int write_centers) {
  unsigned __int128 tot = 0;
#pragma unroll
  for (int l = 0; l < L; l++) tot += (unsigned __int128)lv[l] << (32 * l);
  if constexpr (L < 4) tot &= (((unsigned __int128)1) << (32 * (L % 4))) - 1;
#pragma unroll
  for (int l = 0; l < L; l++) lp[l] = (unsigned long long)((tot >> (32 * l)) & 0xffffffffu);
  if (cnt <= 0 || !write_centers) return oldc;
  const bool neg = (tot >> (32 * L - 1)) & 1;
  unsigned __int128 mag = tot;
  if (neg) {
    if constexpr (L < 4) {
      mag = (((unsigned __int128)1) << (32 * (L % 4))) - tot;
      mag &= (((unsigned __int128)1) << (32 * (L % 4))) - 1;
    } else {
      mag = (unsigned __int128)0 - tot;
    }
  }
  float v = mag == 0 ? 0.0f : rn_ratio_f32(mag, (unsigned long long)cnt, e_lo);
  v = neg ? -v : v;
  *cptr = v;
  return v;
}

// mean_of for coordinate e of the [k][d] sums.
template <int L>
__device__ __forceinline__ float mean_elem(unsigned long long* __restrict__ limbs, int64_t e, int d, int e_lo,
                                           const int32_t* __restrict__ counts, float* __restrict__ centers,
                                           int write_centers) {
  unsigned long long* lp = limbs + e * L;
  unsigned long long lv[L];
#pragma unroll
  for (int l = 0; l < L; l++) lv[l] = lp[l];
  return mean_of<L>(lp, lv, counts[(int)(e / d)], e_lo, centers + e, centers[e], write_centers);
}

// Hand the change count to the host and reset the per-pass counters.
__device__ __forceinline__ void mean_handoff(int bid, int nblk, int32_t* __restrict__ nchg,
                                             int32_t* __restrict__ changed, int32_t* __restrict__ zero4k, int nzero) {
  if (bid == 0 && threadIdx.x == 0) {
    *changed = *nchg;
    *nchg = 0;
  }
  for (int64_t e = (int64_t)bid * blockDim.x + threadIdx.x; e < nzero; e += (int64_t)nblk * blockDim.x)
    zero4k[e] = 0;
}

template <int L>
__global__ void mean_kernel(unsigned long long* __restrict__ limbs, int64_t kd, int d, int e_lo,
                            const int32_t* __restrict__ counts, float* __restrict__ centers, int write_centers,
                            int32_t* __restrict__ nchg, int32_t* __restrict__ changed, int32_t* __restrict__ zero4k,
                            int nzero) {
  griddep_wait();
  griddep_launch();
  mean_handoff(blockIdx.x, gridDim.x, nchg, changed, zero4k, nzero);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < kd; e += (int64_t)gridDim.x * blockDim.x)
    mean_elem<L>(limbs, e, d, e_lo, counts, centers, write_centers);
}

// The same update, two blocks per centre row (each one half of its columns),
// which also writes the row's BF16 copies (of fl(scale * c)) and squared-norm
// halves for the next pass's tensor-core screen (rows j >= k: zero padding
// rows of the copies).  Every thread converts the coordinates it computed;
// each half's squared norm is a per-thread FP32 sum of at most ceil(dp/512)
// terms and an 8-level tree, stored at nrm2[h * kp + j]; the screen adds the
// two halves: within (ceil(d/32) + 9) 2^-24 relative -- the beta term of the
// screen's bound.
template <int L, bool SPLIT>
__global__ void __launch_bounds__(256) mean_prep_kernel(unsigned long long* __restrict__ limbs, int k, int d,
                                                        int e_lo, const int32_t* __restrict__ counts,
                                                        float* __restrict__ centers, int32_t* __restrict__ nchg,
                                                        int32_t* __restrict__ changed, int32_t* __restrict__ zero4k,
                                                        int nzero, CentrePrep cp) {
  __shared__ float part[8];
  griddep_wait();
  griddep_launch();
  mean_handoff(blockIdx.x, gridDim.x, nchg, changed, zero4k, nzero);
  if (cp.zero_word != nullptr && blockIdx.x == 0 && threadIdx.x == 0) *cp.zero_word = 0;
  const int j = blockIdx.x >> 1, half = blockIdx.x & 1;
  const int cpb = ((cp.dp + 1) / 2 + 255) & ~255;  // columns of the first half
  const int c_lo = half * cpb, c_hi = min(cp.dp, c_lo + cpb);
  float acc = 0.0f;
  // the limbs, old centre values and count this thread needs, loaded before
  // any is used (one memory round trip for rows of up to kPer * 256 columns)
  constexpr int kPer = 4;
  unsigned long long lv[kPer][L];
  float oldc[kPer];
  const int cnt = j < k ? counts[j] : 0;
#pragma unroll
  for (int u = 0; u < kPer; u++) {
    const int c = c_lo + threadIdx.x + u * 256;
    const bool v = j < k && c < d && c < c_hi;
    const int64_t e = (int64_t)j * d + c;
#pragma unroll
    for (int l = 0; l < L; l++) lv[u][l] = v ? limbs[e * L + l] : 0ull;
    oldc[u] = v ? centers[e] : 0.0f;
  }
  auto emit = [&](int c, float v) {
    const float t = __fmul_rn(cp.scale, v);
    const __nv_bfloat16 h = __float2bfloat16_rn(t);
    cp.hi[(int64_t)j * cp.dp + c] = h;
    if (SPLIT) cp.lo[(int64_t)j * cp.dp + c] = __float2bfloat16_rn(t - __bfloat162float(h));
    acc = fmaf(v, v, acc);
  };
#pragma unroll
  for (int u = 0; u < kPer; u++) {
    const int c = c_lo + threadIdx.x + u * 256;
    if (c >= c_hi) break;
    const int64_t e = (int64_t)j * d + c;
    const float v = (j < k && c < d) ? mean_of<L>(limbs + e * L, lv[u], cnt, e_lo, centers + e, oldc[u], 1) : 0.0f;
    emit(c, v);
  }
  for (int c = c_lo + threadIdx.x + kPer * 256; c < c_hi; c += blockDim.x) {
    const float v = (j < k && c < d) ? mean_elem<L>(limbs, (int64_t)j * d + c, d, e_lo, counts, centers, 1) : 0.0f;
    emit(c, v);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    const float a01 = part[0] + part[1], a23 = part[2] + part[3], a45 = part[4] + part[5], a67 = part[6] + part[7];
    const float nn = (a01 + a23) + (a45 + a67);
    cp.nrm2[half * cp.kp + j] = nn;
  }
}

}  // namespace

struct ExactSums {
  int L = 0, e_lo = 0, k = 0, d = 0;
  int64_t n = 0;
  Scratch limbs, counts, chg_i, chg_old, chg_new, nchg, cin, cout, off_in, off_out, cur, chunk_off, chunk_info,
      bucket_in, bucket_out, range, done;
  int64_t max_chunks = 0;
};

ExactSums* exact_sums_new() { return new ExactSums(); }
void exact_sums_delete(ExactSums* s) { delete s; }

// Scan X for its exponent range; returns ST_ENOTSUP when the exact integer
// form would need more than 128 bits (or X holds inf/NaN): callers fall back.
int exact_sums_init(ExactSums* s, const float* X, int64_t n, int d, int k, cudaStream_t stream) {
  s->n = n;
  s->d = d;
  s->k = k;
  FUELG_TRY(s->range.alloc(sizeof(int) * 3, stream));
  int init[3] = {1 << 30, -(1 << 30), 0};
  FUELG_CUDA(cudaMemcpyAsync(s->range.p, init, sizeof(init), cudaMemcpyHostToDevice, stream));
  exp_range_kernel<<<8 * 152, 256, 0, stream>>>(X, n * (int64_t)d, s->range.as<int>()); ::fuelg::note_launch();
  FUELG_CUDA(cudaGetLastError());
  int h[3];
  FUELG_CUDA(cudaMemcpyAsync(h, s->range.p, sizeof(h), cudaMemcpyDeviceToHost, stream));
  FUELG_CUDA(cudaStreamSynchronize(stream));
  if (h[2]) {
    set_error("data holds inf or NaN");
    return ST_ENOTSUP;
  }
  int e_lo = h[0], e_hi = h[1];
  if (e_lo > e_hi) e_lo = e_hi = 0;  // all zeros
  int logn = 0;
  while ((1ll << logn) < n + 1) logn++;
  const int bits = (e_hi - e_lo + 1) + logn + 1;
  const int L = (bits + 31) / 32;
  if (L > 4) {
    set_error("exponent range of the data (%d bits) exceeds the exact 128-bit centroid sums", e_hi - e_lo + 1);
    return ST_ENOTSUP;
  }
  s->L = L;
  s->e_lo = e_lo;
  FUELG_TRY(s->limbs.alloc(sizeof(unsigned long long) * (size_t)k * d * L, stream));
  FUELG_CUDA(cudaMemsetAsync(s->limbs.p, 0, sizeof(unsigned long long) * (size_t)k * d * L, stream));
  FUELG_TRY(s->counts.alloc(sizeof(int32_t) * k, stream));
  FUELG_CUDA(cudaMemsetAsync(s->counts.p, 0, sizeof(int32_t) * k, stream));
  FUELG_TRY(s->chg_i.alloc(sizeof(int32_t) * n, stream));
  FUELG_TRY(s->chg_old.alloc(sizeof(int32_t) * n, stream));
  FUELG_TRY(s->chg_new.alloc(sizeof(int32_t) * n, stream));
  FUELG_TRY(s->nchg.alloc(sizeof(int32_t), stream));
  FUELG_CUDA(cudaMemsetAsync(s->nchg.p, 0, sizeof(int32_t), stream));
  FUELG_TRY(s->cin.alloc(sizeof(int32_t) * 4 * (size_t)k, stream));  // cin, cout, cur_in, cur_out
  FUELG_CUDA(cudaMemsetAsync(s->cin.p, 0, sizeof(int32_t) * 4 * (size_t)k, stream));
  FUELG_TRY(s->off_in.alloc(sizeof(int32_t) * 2 * (size_t)k, stream));
  FUELG_TRY(s->chunk_off.alloc(sizeof(int32_t) * (2 * (size_t)k + 1), stream));
  FUELG_TRY(s->bucket_in.alloc(sizeof(int32_t) * n, stream));
  FUELG_TRY(s->bucket_out.alloc(sizeof(int32_t) * n, stream));
  s->max_chunks = 2 * (n / kRows) + 2 * (int64_t)k + 2;
  FUELG_TRY(s->chunk_info.alloc(sizeof(int32_t) * s->max_chunks, stream));
  FUELG_TRY(s->done.alloc(sizeof(unsigned), stream));
  FUELG_CUDA(cudaMemsetAsync(s->done.p, 0, sizeof(unsigned), stream));
  return ST_OK;
}

int exact_sums_L(const ExactSums* s) { return s->L; }

// Device pointers for a fused pass that commits its labels itself.
void exact_sums_commit_view(ExactSums* s, SumsCommit* v) {
  const int k = s->k;
  v->chg_i = s->chg_i.as<int32_t>();
  v->chg_old = s->chg_old.as<int32_t>();
  v->chg_new = s->chg_new.as<int32_t>();
  v->nchg = s->nchg.as<int32_t>();
  v->cin = s->cin.as<int32_t>();
  v->cout = v->cin + k;
  v->off_in = s->off_in.as<int32_t>();
  v->off_out = v->off_in + k;
  v->chunk_off = s->chunk_off.as<int32_t>();
  v->counts = s->counts.as<int32_t>();
  v->chunk_info = s->chunk_info.as<int32_t>();
  v->k = k;
}

// Update after a committed pass (labels, change list and histograms in
// place; the bucket plan too unless plan_in_scatter): scatter the changed
// points into per-cluster buckets, add their exact fixed-point rows into the
// sums, and write the new centres -- with cp, also the BF16 centre copies the
// next tensor-core screen reads.  *changed (device) receives the number of
// changed labels.  plan_in_scatter needs k <= kPlanMaxK.
int exact_sums_update(ExactSums* s, const float* X, bool write_centers, float* centers, int32_t* changed,
                      const CentrePrep* cp, cudaStream_t stream, bool plan_in_scatter) {
  if (plan_in_scatter && s->k > kPlanMaxK) {
    set_error("the scatter-side bucket plan needs k <= %d", kPlanMaxK);
    return ST_EINVAL;
  }
  const int k = s->k, d = s->d;
  int32_t* cin = s->cin.as<int32_t>();
  int32_t* cur_in = cin + 2 * k;
  int32_t* cur_out = cin + 3 * k;
  int32_t* off_in = s->off_in.as<int32_t>();
  int32_t* off_out = off_in + k;
  const int ty = (d + 255) / 256;
  FUELG_TRY(launch_pdl(bucket_scatter_kernel, dim3(2 * 152), dim3(256), 0, stream,
                       (const int32_t*)s->chg_i.as<int32_t>(), (const int32_t*)s->chg_old.as<int32_t>(),
                       (const int32_t*)s->chg_new.as<int32_t>(), (const int32_t*)s->nchg.as<int32_t>(), k, off_in,
                       off_out, cur_in, cur_out, s->bucket_in.as<int32_t>(), s->bucket_out.as<int32_t>(),
                       plan_in_scatter ? 1 : 0, (const int32_t*)cin, (const int32_t*)(cin + k),
                       s->chunk_off.as<int32_t>(), s->counts.as<int32_t>(), s->chunk_info.as<int32_t>()));
  const dim3 g((unsigned)std::min<int64_t>(s->max_chunks * ty, 8 * 152));
  const int64_t kd = (int64_t)k * d;
  const unsigned mg = (unsigned)std::min<int64_t>((kd + 255) / 256, 8 * 152);
  const bool prep = cp != nullptr && cp->hi != nullptr && write_centers;
  auto run = [&](auto Lc) -> int {
    constexpr int LL = decltype(Lc)::value;
    FUELG_TRY(launch_pdl(accumulate_kernel<LL>, g, dim3(256), 0, stream, X, d, k, s->e_lo, ty,
                         (const int32_t*)s->chunk_off.as<int32_t>(), (const int32_t*)s->chunk_info.as<int32_t>(),
                         (const int32_t*)cin, (const int32_t*)(cin + k), (const int32_t*)off_in,
                         (const int32_t*)off_out, (const int32_t*)s->bucket_in.as<int32_t>(),
                         (const int32_t*)s->bucket_out.as<int32_t>(), s->limbs.as<unsigned long long>()));
    if (prep) {
      auto mk = cp->lo != nullptr ? mean_prep_kernel<LL, true> : mean_prep_kernel<LL, false>;
      FUELG_TRY(launch_pdl(mk, dim3((unsigned)(2 * cp->kp)), dim3(256), 0, stream, s->limbs.as<unsigned long long>(), k, d,
                           s->e_lo, (const int32_t*)s->counts.as<int32_t>(), centers, s->nchg.as<int32_t>(), changed,
                           cin, 4 * k, *cp));
    } else {
      FUELG_TRY(launch_pdl(mean_kernel<LL>, dim3(mg), dim3(256), 0, stream, s->limbs.as<unsigned long long>(), kd, d,
                           s->e_lo, (const int32_t*)s->counts.as<int32_t>(), centers, write_centers ? 1 : 0,
                           s->nchg.as<int32_t>(), changed, cin, 4 * k));
    }
    return ST_OK;
  };
  switch (s->L) {
    case 1: FUELG_TRY(run(std::integral_constant<int, 1>())); break;
    case 2: FUELG_TRY(run(std::integral_constant<int, 2>())); break;
    case 3: FUELG_TRY(run(std::integral_constant<int, 3>())); break;
    default: FUELG_TRY(run(std::integral_constant<int, 4>())); break;
  }
  return ST_OK;
}

// Apply one assignment pass: commit lab_new into labels, record the changes,
// update the exact sums and counts, and write the new centres (and, with cp,
// their BF16 copies).  *changed (device) receives the number of changed labels.
int exact_sums_step(ExactSums* s, const float* X, const int32_t* lab_new, int32_t* labels, bool first,
                    bool write_centers, float* centers, int32_t* changed, int* dev_status, cudaStream_t stream,
                    const CentrePrep* cp) {
  (void)dev_status;
  const int64_t n = s->n;
  const int k = s->k;
  int32_t* cin = s->cin.as<int32_t>();
  int32_t* cout = cin + k;
  int32_t* off_in = s->off_in.as<int32_t>();
  int32_t* off_out = off_in + k;
  // counters were zeroed at init and are reset by the centre update after every pass
  FUELG_TRY(launch_pdl(commit_changes_kernel, dim3((unsigned)std::min<int64_t>((n + 255) / 256, 2 * 152)), dim3(256),
                       0, stream, lab_new, n, first ? 1 : 0, k, labels, s->chg_i.as<int32_t>(),
                       s->chg_old.as<int32_t>(), s->chg_new.as<int32_t>(), s->nchg.as<int32_t>(), cin, cout,
                       s->done.as<unsigned>(), off_in, off_out, s->chunk_off.as<int32_t>(), s->counts.as<int32_t>(),
                       s->chunk_info.as<int32_t>()));
  return exact_sums_update(s, X, write_centers, centers, changed, cp, stream, false);
}

}  // namespace fuelg
