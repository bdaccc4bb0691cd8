// fuelg_common.cuh -- shared device helpers for the GB300 linear-scan / Lloyd engine.
//
// Distance arithmetic here reproduces, operation for operation, the f32
// kernels kno10/fuel compiles for its host ISA (summation "profiles"):
//   ORDER_ARM : src/math/unroll.rs, src/math/scalar.rs and the portable
//               fallback of src/distance/squared_euclidean.rs:99-133
//   ORDER_X86 : src/math/avx2.rs and src/distance/squared_euclidean.rs:16-39
// Every add/mul below is an explicit round-to-nearest intrinsic so nvcc can
// never contract it into an FMA; every FMA the reference performs is an
// explicit __fmaf_rn.  The result is bit-identical to fuel on that ISA.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace fuelg {

enum Order : int { ORDER_ARM = 0, ORDER_X86 = 1 };
// Which reference kernel a distance must match:
//   KIND_KNN      DistanceFunction<SquaredEuclidean>::distance (linear scan)
//   KIND_SQDIST   math::sqdist -> VecOps::vec_sqdist (Lloyd iterations >= 2)
//   KIND_PAIRWISE VecOps::vec_pairwise_sqdist per-pair order (Lloyd iteration 1)
enum Kind : int { KIND_KNN = 0, KIND_SQDIST = 1, KIND_PAIRWISE = 2 };
enum Metric : int { METRIC_SQEUCLIDEAN = 0, METRIC_EUCLIDEAN = 1 };

// Device-side error bits reported back through a status word.
enum DevErr : int { DEV_OK = 0, DEV_CANCELLED = 1, DEV_TIMEOUT = 2, DEV_BADARG = 4 };

constexpr uint64_t KEY_NONE = ~0ull;

// (distance, index) packed so that unsigned order == DistPair order
// (src/api/search.rs:23-30) for non-negative distances.
__device__ __forceinline__ uint64_t make_key(float dist, uint32_t idx) {
  return (static_cast<uint64_t>(__float_as_uint(dist)) << 32) | idx;
}
__device__ __forceinline__ float key_dist(uint64_t k) { return __uint_as_float(static_cast<uint32_t>(k >> 32)); }
__device__ __forceinline__ uint32_t key_idx(uint64_t k) { return static_cast<uint32_t>(k & 0xffffffffu); }

__device__ __forceinline__ float sq_rn(float x) { return __fmul_rn(x, x); }

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialisation may start while its predecessor drains; it must call
// griddep_wait() before touching any memory the predecessor (or an earlier
// kernel) reads or writes.  Without the launch attribute this is a no-op.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// Lets the next kernel of the stream (launched with the same attribute) be
// scheduled once every CTA of this grid has passed here or exited; its CTAs
// then run up to their own griddep_wait(), which still waits for this whole
// grid to complete.  Called right after griddep_wait(): the successor is
// scheduled only once this kernel's own predecessors have completed.
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
// 16-byte asynchronous global -> shared copy (both addresses 16-byte
// aligned); cp_async_wait_all() waits for the calling thread's copies.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// ---------------------------------------------------------------------------
// Per-pair distances, NP point rows against one query row, all in shared
// memory.  q: query row; xb: first of NP rows with stride xs (floats).  The
// 8-blocks use 16-byte loads, so rows must be 16-byte aligned.
// ---------------------------------------------------------------------------

// 8 lane accumulators.  FMA lanes + FMA tail (x86 squared_euclidean.rs:16-39)
// or mul-then-add lanes + tail (fallback :99-133 == unroll::sqdist :16-38).
template <bool FMA, int NP>
__device__ __forceinline__ void dist_lane8(const float* __restrict__ q, const float* __restrict__ xb, int xs, int d,
                                           float (&out)[NP]) {
  float acc[NP][8];
#pragma unroll
  for (int p = 0; p < NP; p++)
#pragma unroll
    for (int l = 0; l < 8; l++) acc[p][l] = 0.0f;
  const int sd = d & ~7;
  for (int i = 0; i < sd; i += 8) {
    const float4 qa = *reinterpret_cast<const float4*>(q + i);
    const float4 qb = *reinterpret_cast<const float4*>(q + i + 4);
    const float qv[8] = {qa.x, qa.y, qa.z, qa.w, qb.x, qb.y, qb.z, qb.w};
#pragma unroll
    for (int p = 0; p < NP; p++) {
      const float4 xa = *reinterpret_cast<const float4*>(xb + p * xs + i);
      const float4 xc = *reinterpret_cast<const float4*>(xb + p * xs + i + 4);
      const float xv[8] = {xa.x, xa.y, xa.z, xa.w, xc.x, xc.y, xc.z, xc.w};
#pragma unroll
      for (int l = 0; l < 8; l++) {
        const float df = __fsub_rn(qv[l], xv[l]);
        if (FMA) acc[p][l] = __fmaf_rn(df, df, acc[p][l]);
        else acc[p][l] = __fadd_rn(sq_rn(df), acc[p][l]);
      }
    }
  }
#pragma unroll
  for (int p = 0; p < NP; p++) {
    float s = acc[p][0];  // (-0.0 + a0) == a0 for a0 >= +0
#pragma unroll
    for (int l = 1; l < 8; l++) s = __fadd_rn(s, acc[p][l]);
    for (int i = sd; i < d; i++) {
      const float df = __fsub_rn(q[i], xb[p * xs + i]);
      if (FMA) s = __fmaf_rn(df, df, s);
      else s = __fadd_rn(s, sq_rn(df));
    }
    out[p] = s;
  }
}

// One sequential chain per pair.  FMA chain (avx2 micro_sqdist_f32,
// avx2.rs:903-975) or mul-then-add chain (unroll pairwise :227-303 and
// scalar.rs:10-16).
template <bool FMA, int NP>
__device__ __forceinline__ void dist_chain(const float* __restrict__ q, const float* __restrict__ xb, int xs, int d,
                                           float (&out)[NP]) {
  float acc[NP];
#pragma unroll
  for (int p = 0; p < NP; p++) acc[p] = 0.0f;
  const int d4 = d & ~3;
  for (int i = 0; i < d4; i += 4) {
    const float4 qa = *reinterpret_cast<const float4*>(q + i);
#pragma unroll
    for (int p = 0; p < NP; p++) {
      const float4 xa = *reinterpret_cast<const float4*>(xb + p * xs + i);
      float df;
      df = __fsub_rn(qa.x, xa.x);
      acc[p] = FMA ? __fmaf_rn(df, df, acc[p]) : __fadd_rn(acc[p], sq_rn(df));
      df = __fsub_rn(qa.y, xa.y);
      acc[p] = FMA ? __fmaf_rn(df, df, acc[p]) : __fadd_rn(acc[p], sq_rn(df));
      df = __fsub_rn(qa.z, xa.z);
      acc[p] = FMA ? __fmaf_rn(df, df, acc[p]) : __fadd_rn(acc[p], sq_rn(df));
      df = __fsub_rn(qa.w, xa.w);
      acc[p] = FMA ? __fmaf_rn(df, df, acc[p]) : __fadd_rn(acc[p], sq_rn(df));
    }
  }
  for (int i = d4; i < d; i++) {
#pragma unroll
    for (int p = 0; p < NP; p++) {
      const float df = __fsub_rn(q[i], xb[p * xs + i]);
      acc[p] = FMA ? __fmaf_rn(df, df, acc[p]) : __fadd_rn(acc[p], sq_rn(df));
    }
  }
#pragma unroll
  for (int p = 0; p < NP; p++) out[p] = acc[p];
}

// avx2::sqdist_f32 (avx2.rs:103-151): four 8-lane FMA accumulators over
// 32-blocks, combined (acc0+acc1)+(acc2+acc3), FMA over remaining 8-blocks,
// horizontal_sum_f32 (avx2.rs:69-81) = ((v0+v4)+(v1+v5))+((v2+v6)+(v3+v7)),
// FMA tail.  d < 4 goes to scalar.rs (mul-then-add chain), math/mod.rs:53-63.
template <int NP>
__device__ __forceinline__ void dist_sqdist_x86(const float* __restrict__ q, const float* __restrict__ xb, int xs,
                                                int d, float (&out)[NP]) {
  if (d < 4) {
    dist_chain<false, NP>(q, xb, xs, d, out);
    return;
  }
#pragma unroll
  for (int p = 0; p < NP; p++) {
    const float* x = xb + p * xs;
    float a[4][8];
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
      for (int l = 0; l < 8; l++) a[u][l] = 0.0f;
    int i = 0;
    for (; i + 32 <= d; i += 32) {
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const float4 qa = *reinterpret_cast<const float4*>(q + i + u * 8);
        const float4 qb = *reinterpret_cast<const float4*>(q + i + u * 8 + 4);
        const float4 xa = *reinterpret_cast<const float4*>(x + i + u * 8);
        const float4 xc = *reinterpret_cast<const float4*>(x + i + u * 8 + 4);
        const float qv[8] = {qa.x, qa.y, qa.z, qa.w, qb.x, qb.y, qb.z, qb.w};
        const float xv[8] = {xa.x, xa.y, xa.z, xa.w, xc.x, xc.y, xc.z, xc.w};
#pragma unroll
        for (int l = 0; l < 8; l++) {
          const float df = __fsub_rn(qv[l], xv[l]);
          a[u][l] = __fmaf_rn(df, df, a[u][l]);
        }
      }
    }
    float c[8];
#pragma unroll
    for (int l = 0; l < 8; l++) c[l] = __fadd_rn(__fadd_rn(a[0][l], a[1][l]), __fadd_rn(a[2][l], a[3][l]));
    for (; i + 8 <= d; i += 8) {
#pragma unroll
      for (int l = 0; l < 8; l++) {
        const float df = __fsub_rn(q[i + l], x[i + l]);
        c[l] = __fmaf_rn(df, df, c[l]);
      }
    }
    float s = __fadd_rn(__fadd_rn(__fadd_rn(c[0], c[4]), __fadd_rn(c[1], c[5])),
                        __fadd_rn(__fadd_rn(c[2], c[6]), __fadd_rn(c[3], c[7])));
    for (; i < d; i++) {
      const float df = __fsub_rn(q[i], x[i]);
      s = __fmaf_rn(df, df, s);
    }
    out[p] = s;
  }
}

// Dispatch: the reference kernel for (KIND, ORDER), math/mod.rs:51-63.
template <int KIND, int ORDER, int NP>
__device__ __forceinline__ void pair_dists(const float* __restrict__ q, const float* __restrict__ xb, int xs, int d,
                                           float (&out)[NP]) {
  if constexpr (KIND == KIND_KNN) {
    dist_lane8<ORDER == ORDER_X86, NP>(q, xb, xs, d, out);
  } else if constexpr (KIND == KIND_SQDIST) {
    if constexpr (ORDER == ORDER_X86) dist_sqdist_x86<NP>(q, xb, xs, d, out);
    else dist_lane8<false, NP>(q, xb, xs, d, out);  // unroll::sqdist; d<4 scalar is the same arithmetic
  } else {
    if constexpr (ORDER == ORDER_X86) {
      if (d < 4) dist_chain<false, NP>(q, xb, xs, d, out);
      else dist_chain<true, NP>(q, xb, xs, d, out);
    } else {
      dist_chain<false, NP>(q, xb, xs, d, out);
    }
  }
}

// Same arithmetic as pair_dists<KIND, ORDER, 1>, reading both rows with scalar
// loads from any address (global memory, no alignment requirement).  Used to
// re-score the few candidates a tensor-core screen cannot decide.
template <int KIND, int ORDER>
__device__ __forceinline__ float exact_dist_scalar(const float* __restrict__ q, const float* __restrict__ x, int d) {
  const bool lane8 = (KIND == KIND_KNN) || (KIND == KIND_SQDIST && ORDER == ORDER_ARM);
  const bool fma8 = (KIND == KIND_KNN && ORDER == ORDER_X86);
  if (lane8) {
    float acc[8];
#pragma unroll
    for (int l = 0; l < 8; l++) acc[l] = 0.0f;
    const int sd = d & ~7;
    for (int i = 0; i < sd; i += 8) {
#pragma unroll
      for (int l = 0; l < 8; l++) {
        const float df = __fsub_rn(__ldg(q + i + l), __ldg(x + i + l));
        acc[l] = fma8 ? __fmaf_rn(df, df, acc[l]) : __fadd_rn(sq_rn(df), acc[l]);
      }
    }
    float s = acc[0];
#pragma unroll
    for (int l = 1; l < 8; l++) s = __fadd_rn(s, acc[l]);
    for (int i = sd; i < d; i++) {
      const float df = __fsub_rn(__ldg(q + i), __ldg(x + i));
      s = fma8 ? __fmaf_rn(df, df, s) : __fadd_rn(s, sq_rn(df));
    }
    return s;
  }
  if (KIND == KIND_SQDIST) {  // x86 avx2::sqdist_f32
    if (d < 4) {
      float s = 0.0f;
      for (int i = 0; i < d; i++) {
        const float df = __fsub_rn(__ldg(q + i), __ldg(x + i));
        s = __fadd_rn(s, sq_rn(df));
      }
      return s;
    }
    float a[4][8];
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
      for (int l = 0; l < 8; l++) a[u][l] = 0.0f;
    int i = 0;
    for (; i + 32 <= d; i += 32) {
#pragma unroll
      for (int u = 0; u < 4; u++)
#pragma unroll
        for (int l = 0; l < 8; l++) {
          const float df = __fsub_rn(__ldg(q + i + u * 8 + l), __ldg(x + i + u * 8 + l));
          a[u][l] = __fmaf_rn(df, df, a[u][l]);
        }
    }
    float c[8];
#pragma unroll
    for (int l = 0; l < 8; l++) c[l] = __fadd_rn(__fadd_rn(a[0][l], a[1][l]), __fadd_rn(a[2][l], a[3][l]));
    for (; i + 8 <= d; i += 8) {
#pragma unroll
      for (int l = 0; l < 8; l++) {
        const float df = __fsub_rn(__ldg(q + i + l), __ldg(x + i + l));
        c[l] = __fmaf_rn(df, df, c[l]);
      }
    }
    float s = __fadd_rn(__fadd_rn(__fadd_rn(c[0], c[4]), __fadd_rn(c[1], c[5])),
                        __fadd_rn(__fadd_rn(c[2], c[6]), __fadd_rn(c[3], c[7])));
    for (; i < d; i++) {
      const float df = __fsub_rn(__ldg(q + i), __ldg(x + i));
      s = __fmaf_rn(df, df, s);
    }
    return s;
  }
  // KIND_PAIRWISE: one chain; FMA chain for x86 with d >= 4
  const bool fma_chain = (ORDER == ORDER_X86) && d >= 4;
  float s = 0.0f;
  for (int i = 0; i < d; i++) {
    const float df = __fsub_rn(__ldg(q + i), __ldg(x + i));
    s = fma_chain ? __fmaf_rn(df, df, s) : __fadd_rn(s, sq_rn(df));
  }
  return s;
}

// exact_dist_scalar's arithmetic for a compile-time d, with the two operands
// given as element accessors q(i) / x(i) (registers, shared or global memory).
// The operation sequence is the same, so the result is bit-identical.
template <int KIND, int ORDER, int D, class QF, class XF>
__device__ __forceinline__ float exact_dist_fn(QF q, XF x) {
  constexpr bool lane8 = (KIND == KIND_KNN) || (KIND == KIND_SQDIST && ORDER == ORDER_ARM);
  constexpr bool fma8 = (KIND == KIND_KNN && ORDER == ORDER_X86);
  if constexpr (lane8) {
    // A lane's first term is added to +0: the sum is the square itself
    // (x*x >= +0, NaN stays the canonical NaN), so it is taken as is.
    float acc[8];
    constexpr int sd = D & ~7;
    if constexpr (sd >= 8) {
#pragma unroll
      for (int l = 0; l < 8; l++) acc[l] = sq_rn(__fsub_rn(q(l), x(l)));
    } else {
#pragma unroll
      for (int l = 0; l < 8; l++) acc[l] = 0.0f;
    }
#pragma unroll
    for (int i = 8; i < sd; i += 8) {
#pragma unroll
      for (int l = 0; l < 8; l++) {
        const float df = __fsub_rn(q(i + l), x(i + l));
        acc[l] = fma8 ? __fmaf_rn(df, df, acc[l]) : __fadd_rn(sq_rn(df), acc[l]);
      }
    }
    float s = acc[0];
#pragma unroll
    for (int l = 1; l < 8; l++) s = __fadd_rn(s, acc[l]);
#pragma unroll
    for (int i = sd; i < D; i++) {
      const float df = __fsub_rn(q(i), x(i));
      s = (sd == 0 && i == 0) ? sq_rn(df) : (fma8 ? __fmaf_rn(df, df, s) : __fadd_rn(s, sq_rn(df)));
    }
    return s;
  } else if constexpr (KIND == KIND_SQDIST) {  // x86 avx2::sqdist_f32
    if constexpr (D < 4) {
      float s = 0.0f;
#pragma unroll
      for (int i = 0; i < D; i++) {
        const float df = __fsub_rn(q(i), x(i));
        s = __fadd_rn(s, sq_rn(df));
      }
      return s;
    } else {
      float a[4][8];
#pragma unroll
      for (int u = 0; u < 4; u++)
#pragma unroll
        for (int l = 0; l < 8; l++) a[u][l] = 0.0f;
      constexpr int d32 = D & ~31;
#pragma unroll
      for (int i = 0; i < d32; i += 32) {
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
          for (int l = 0; l < 8; l++) {
            const float df = __fsub_rn(q(i + u * 8 + l), x(i + u * 8 + l));
            a[u][l] = __fmaf_rn(df, df, a[u][l]);
          }
      }
      float c[8];
#pragma unroll
      for (int l = 0; l < 8; l++) c[l] = __fadd_rn(__fadd_rn(a[0][l], a[1][l]), __fadd_rn(a[2][l], a[3][l]));
      constexpr int d8 = d32 + ((D - d32) & ~7);
#pragma unroll
      for (int i = d32; i < d8; i += 8) {
#pragma unroll
        for (int l = 0; l < 8; l++) {
          const float df = __fsub_rn(q(i + l), x(i + l));
          c[l] = __fmaf_rn(df, df, c[l]);
        }
      }
      float s = __fadd_rn(__fadd_rn(__fadd_rn(c[0], c[4]), __fadd_rn(c[1], c[5])),
                          __fadd_rn(__fadd_rn(c[2], c[6]), __fadd_rn(c[3], c[7])));
#pragma unroll
      for (int i = d8; i < D; i++) {
        const float df = __fsub_rn(q(i), x(i));
        s = __fmaf_rn(df, df, s);
      }
      return s;
    }
  } else {  // KIND_PAIRWISE: one chain; FMA chain for x86 with d >= 4
    constexpr bool fma_chain = (ORDER == ORDER_X86) && D >= 4;
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < D; i++) {
      const float df = __fsub_rn(q(i), x(i));
      s = fma_chain ? __fmaf_rn(df, df, s) : __fadd_rn(s, sq_rn(df));
    }
    return s;
  }
}

// Row stride (floats) for shared-memory tiles: 16-byte aligned rows whose
// stride is an odd number of float4s, so eight lanes reading eight different
// rows with 16-byte loads hit 32 distinct banks.
__host__ __device__ inline int smem_row_stride(int d) {
  int s = (d + 3) & ~3;
  if (((s >> 2) & 1) == 0) s += 4;
  return s;
}

// Sum of squared differences (x - c)^2 to near-FP64 accuracy on FP32
// arithmetic (the FP64 pipe runs at a small fraction of the FP32 rate):
// x - c = dh + dl exactly (Knuth's two-sum), dh^2 = p + pe exactly (FMA), so
// (x - c)^2 = p + (pe + dl (2 dh + dl)), the second part within 2^-46 of p
// relative; the p terms go into a float-float accumulator (two-sum, the
// rounding errors collected in a second float).  pe is exact for |dh| >=
// 2^-50 (its bits are multiples of 2^-146, above the subnormal step); an
// element with 0 < |dh| < 2^-50 or |dh| >= 2^60 (or a non-finite difference)
// is added in FP64 instead.  renorm() folds the low float back into the
// high one (a fast two-sum); calling it every few dozen terms keeps the low
// part within a few ulps of the high one, so the relative error stays near
// 2^-40 per renormalised run of terms.
__device__ __forceinline__ void two_sum_f32(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

struct SqDiffAcc {
  float sh = 0.0f, sl = 0.0f;
  double slow = 0.0;
  __device__ __forceinline__ void add(float xv, float cv) {
    float dh, dl;
    two_sum_f32(xv, -cv, dh, dl);
    const float ad = fabsf(dh);
    if (!(ad < 0x1p60f && (ad >= 0x1p-50f || ad == 0.0f))) {  // rare: FP64
      const double df = (double)xv - (double)cv;
      slow = fma(df, df, slow);
      dh = 0.0f;
      dl = 0.0f;
    }
    const float p = __fmul_rn(dh, dh);
    const float q = __fmaf_rn(dl, __fadd_rn(__fadd_rn(dh, dh), dl), __fmaf_rn(dh, dh, -p));
    float e;
    two_sum_f32(sh, p, sh, e);
    sl = __fadd_rn(sl, __fadd_rn(e, q));
  }
  __device__ __forceinline__ void renorm() {
    const float s = __fadd_rn(sh, sl);
    sl = __fsub_rn(sl, __fsub_rn(s, sh));
    sh = s;
  }
  __device__ __forceinline__ double value() const { return ((double)sh + (double)sl) + slow; }
};

}  // namespace fuelg
