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

#include "fuelg_common.cuh"
#include "fuelg_internal.h"

namespace fuelg {

namespace {

constexpr int BM = 128;  // points per tile (UMMA M)
constexpr int BK = 64;   // BF16 elements per K chunk = one 128-byte swizzle row
constexpr int kTcThreads = 192;
constexpr uint64_t kWaitNs = 4000000000ull;  // 4 s: far beyond any legitimate wait

struct TcArgs {
  int64_t n;
  int d, k, kp, kc, stages;
  const float* nx;  // ||x||^2 per point (f32 of an FP64 sum)
  const float* xn;  // ||x||
  const float* nc;  // ||c||^2 per (padded) centre
  const float* cn;  // ||c||
  int32_t* lab_new;
  int32_t* ulist;
  uint64_t* umask;
  int32_t* ucount;
  int mw;
  float alpha, beta, gamma;
  uint32_t idesc;
  uint32_t tmem_cols;
  int* status;
  const volatile int* cancel;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false when the barrier did not complete within kWaitNs or the
// CTA is aborting.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255) == 0) {
      if (*abort_flag) return false;
      if (globaltimer() - t0 > kWaitNs) return false;
    }
  }
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row
// groups 1024 bytes apart (SBO), descriptor version 1, base 1024-aligned.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  uint64_t desc = 0;
  desc |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  desc |= (uint64_t)1 << 16;             // leading byte offset (unused for swizzled K-major)
  desc |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
  desc |= (uint64_t)1 << 46;             // version
  desc |= (uint64_t)2 << 61;             // SWIZZLE_128B
  return desc;
}
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
          d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

template <bool SPLIT>
__global__ void __launch_bounds__(kTcThreads, 1)
    lloyd_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmAlo,
                    const __grid_constant__ CUtensorMap tmB, const __grid_constant__ CUtensorMap tmBlo, TcArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const uint32_t a_bytes = BM * BK * 2;
  const uint32_t b_bytes = (uint32_t)a.kp * BK * 2;
  const uint32_t stage_bytes = (SPLIT ? 2u : 1u) * (a_bytes + b_bytes);
  const int NS = a.stages;
  uint64_t* full = reinterpret_cast<uint64_t*>(base + (size_t)NS * stage_bytes);
  uint64_t* empty = full + NS;
  uint64_t* accf = empty + NS;
  uint64_t* acce = accf + 2;
  uint64_t* fin = acce + 2;
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(fin + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_holder + 1);
  float* snc = reinterpret_cast<float*>(tmem_holder + 4);
  float* scn = snc + a.kp;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ntiles = (a.n + BM - 1) / BM;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], BM);
    }
    mbar_init(fin, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int j = threadIdx.x; j < a.kp; j += blockDim.x) {
    snc[j] = a.nc[j];
    scn[j] = a.cn[j];
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

  if (warp == 0) {
    if (lane == 0) {
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
          if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag)) {
            if (!*abort_flag) atomicOr(a.status, DEV_TIMEOUT);
            *abort_flag = 1;
            break;
          }
          uint8_t* sA = base + (size_t)stage * stage_bytes;
          uint8_t* sB = sA + a_bytes;
          mbar_expect_tx(&full[stage], stage_bytes);
          armed |= 1u << stage;
          last_ph = (last_ph & ~(1u << stage)) | (phase << stage);
          tma_load_2d(sA, &tmA, kc * BK, (int)(t * BM), &full[stage]);
          tma_load_2d(sB, &tmB, kc * BK, 0, &full[stage]);
          if (SPLIT) {
            tma_load_2d(sB + b_bytes, &tmAlo, kc * BK, (int)(t * BM), &full[stage]);
            tma_load_2d(sB + b_bytes + a_bytes, &tmBlo, kc * BK, 0, &full[stage]);
          }
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
        const uint32_t d_tmem = tmem_base + buf * (uint32_t)a.kp;
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
            if (SPLIT) {
              const uint64_t adlo = smem_desc_sw128(smem_u32(sB + b_bytes));
              const uint64_t bdlo = smem_desc_sw128(smem_u32(sB + b_bytes + a_bytes));
              umma_bf16(d_tmem, ad + 2 * kk, bdlo + 2 * kk, a.idesc, 1u);
              umma_bf16(d_tmem, adlo + 2 * kk, bd + 2 * kk, a.idesc, 1u);
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
    int64_t lt = 0;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, lt++) {
      const uint32_t buf = (uint32_t)(lt & 1), accph = (uint32_t)((lt >> 1) & 1);
      if (*abort_flag || !mbar_wait(&accf[buf], accph, abort_flag)) {
        if (!*abort_flag) atomicOr(a.status, DEV_TIMEOUT);
        *abort_flag = 1;
        break;
      }
      tc_fence_after();
      const int64_t i = t * BM + row;
      const bool valid = i < a.n;
      const float nxi = valid ? a.nx[i] : 0.0f;
      const float xni = valid ? a.xn[i] : 0.0f;
      const uint32_t taddr = tmem_base + ((uint32_t)(g * 32) << 16) + buf * (uint32_t)a.kp;
      // pass 1: screened argmin (first index wins ties)
      float best = __int_as_float(0x7f800000);
      int bj = 0;
      for (int c0 = 0; c0 < a.kp; c0 += 16) {
        float v[16];
        tmem_ld16(taddr + c0, v);
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const int col = c0 + j;
          if (col < a.k) {
            const float dt = fmaf(-2.0f, v[j], nxi + snc[col]);
            if (dt < best) {
              best = dt;
              bj = col;
            }
          }
        }
      }
      const float eb = (a.alpha * xni * scn[bj] + a.beta * (nxi + snc[bj])) * (1.0f + a.gamma) + a.gamma * fabsf(best);
      const float hi = best + eb;
      // pass 2: every other centre whose lower bound reaches the best's upper bound
      uint64_t m0 = 0, m1 = 0, m2 = 0, m3 = 0;
      for (int c0 = 0; c0 < a.kp; c0 += 16) {
        float v[16];
        tmem_ld16(taddr + c0, v);
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const int col = c0 + j;
          if (col < a.k && col != bj) {
            const float dt = fmaf(-2.0f, v[j], nxi + snc[col]);
            const float e = (a.alpha * xni * scn[col] + a.beta * (nxi + snc[col])) * (1.0f + a.gamma) +
                            a.gamma * fabsf(dt);
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
      mbar_arrive(&acce[buf]);
      if (valid) {
        if ((m0 | m1 | m2 | m3) == 0) {
          a.lab_new[i] = bj;
        } else {
          const uint64_t bit = 1ull << (bj & 63);
          const int w = bj >> 6;
          if (w == 0) m0 |= bit;
          else if (w == 1) m1 |= bit;
          else if (w == 2) m2 |= bit;
          else m3 |= bit;
          a.lab_new[i] = -1;
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
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(a.tmem_cols)
                 : "memory");
  }
}

// X (f32) -> BF16 hi (and lo = BF16(x - hi)) copies with rows padded to dp
// (a multiple of 8, zero filled), plus ||x||^2 (FP64 sum rounded) and ||x||.
template <bool SPLIT>
__global__ void prep_rows_kernel(const float* __restrict__ X, int64_t rows, int64_t valid_rows, int d, int dp,
                                 __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                                 float* __restrict__ nrm2, float* __restrict__ nrm) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int64_t r = (int64_t)blockIdx.x * nw + warp; r < rows; r += (int64_t)gridDim.x * nw) {
    double s = 0.0;
    const bool v = r < valid_rows;
    for (int c = lane; c < dp; c += 32) {
      const float x = (v && c < d) ? X[r * d + c] : 0.0f;
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      hi[r * dp + c] = h;
      if (SPLIT) lo[r * dp + c] = __float2bfloat16_rn(x - __bfloat162float(h));
      s = fma((double)x, (double)x, s);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) {
      const float f = __double2float_rn(s);
      nrm2[r] = f;
      nrm[r] = __double2float_rn(sqrt(s));
    }
  }
}

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
    for (int i = l; i < sd; i += 8) {
      const float df = __fsub_rn(__ldg(x + i), __ldg(c + i));
      acc = FMA8 ? __fmaf_rn(df, df, acc) : __fadd_rn(sq_rn(df), acc);
    }
    float s = __shfl_sync(0xffffffffu, acc, g0);
#pragma unroll
    for (int t = 1; t < 8; t++) s = __fadd_rn(s, __shfl_sync(0xffffffffu, acc, g0 + t));
    for (int i = sd; i < d; i++) {
      const float df = __fsub_rn(__ldg(x + i), __ldg(c + i));
      s = FMA8 ? __fmaf_rn(df, df, s) : __fadd_rn(s, sq_rn(df));
    }
    return s;  // valid on every lane of the group
  } else if constexpr (KIND == KIND_SQDIST) {  // x86 avx2::sqdist_f32, d >= 4
    const int nb = d / 32;
    float a = 0.0f;
    for (int b = 0; b < nb; b++) {
      const float df = __fsub_rn(__ldg(x + b * 32 + lane), __ldg(c + b * 32 + lane));
      a = __fmaf_rn(df, df, a);
    }
    const int l = lane & 7;
    const float a0 = __shfl_sync(0xffffffffu, a, l), a1 = __shfl_sync(0xffffffffu, a, l + 8);
    const float a2 = __shfl_sync(0xffffffffu, a, l + 16), a3 = __shfl_sync(0xffffffffu, a, l + 24);
    float cl = __fadd_rn(__fadd_rn(a0, a1), __fadd_rn(a2, a3));
    int i = nb * 32;
    for (; i + 8 <= d; i += 8) {
      const float df = __fsub_rn(__ldg(x + i + l), __ldg(c + i + l));
      cl = __fmaf_rn(df, df, cl);
    }
    float v[8];
#pragma unroll
    for (int t = 0; t < 8; t++) v[t] = __shfl_sync(0xffffffffu, cl, t);
    float s = __fadd_rn(__fadd_rn(__fadd_rn(v[0], v[4]), __fadd_rn(v[1], v[5])),
                        __fadd_rn(__fadd_rn(v[2], v[6]), __fadd_rn(v[3], v[7])));
    for (; i < d; i++) {
      const float df = __fsub_rn(__ldg(x + i), __ldg(c + i));
      s = __fmaf_rn(df, df, s);
    }
    return s;
  } else {
    return exact_dist_scalar<KIND, ORDER>(x, c, d);  // one lane, one chain
  }
}

template <int KIND, int ORDER>
__global__ void rescore_kernel(const float* __restrict__ X, const float* __restrict__ C, int d, int mw,
                               const int32_t* __restrict__ ulist, const uint64_t* __restrict__ umask,
                               const int32_t* __restrict__ ucount, int32_t* __restrict__ lab_new,
                               unsigned long long* __restrict__ tally) {
  constexpr bool LANE8 = (KIND == KIND_KNN) || (KIND == KIND_SQDIST && ORDER == ORDER_ARM);
  constexpr int G = LANE8 ? 8 : (KIND == KIND_SQDIST ? 32 : 1);  // lanes per candidate
  constexpr int PER = 32 / G;                                      // candidates per warp step
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int cnt = *ucount;
  if (blockIdx.x == 0 && threadIdx.x == 0) *tally += (unsigned long long)cnt;
  for (int64_t u = gw; u < cnt; u += nwarps) {
    const int64_t i = ulist[u];
    const float* x = X + i * d;
    uint64_t best = KEY_NONE;
    // walk the candidate bits PER at a time; this lane's slot is lane / G
    int w = 0;
    uint64_t m = umask[u * mw];
    const int slot = lane / G;
    for (;;) {
      int got = 0, j = 0;
      while (got < PER) {
        while (m == 0 && w + 1 < mw) m = umask[u * mw + (++w)];
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
    if (lane == 0) lab_new[i] = (int32_t)key_idx(best);
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

int make_map(CUtensorMap* tm, const void* ptr, int64_t rows, int dp, int box_rows) {
  auto fn = encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is unavailable from the driver");
    return ST_ECUDA;
  }
  cuuint64_t dims[2] = {(cuuint64_t)dp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)dp * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d) for rows=%lld dp=%d box_rows=%d", (int)r, (long long)rows, dp,
              box_rows);
    return ST_ECUDA;
  }
  return ST_OK;
}

}  // namespace

// Per-call state of the tensor-core Lloyd tier: the BF16 copy of X is made
// once per k-means call; the centre copy every iteration.
struct TcLloydState {
  bool split = false;
  int dp = 0, kp = 0, kc = 0, mw = 0, stages = 0;
  size_t smem = 0;
  Scratch xhi, xlo, xnrm2, xnrm, chi, clo, cnrm2, cnrm, ulist, umask, ucount, rescored_total;
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
  const size_t a_bytes = BM * BK * 2, b_bytes = (size_t)st->kp * BK * 2;
  const size_t stage_bytes = (st->split ? 2 : 1) * (a_bytes + b_bytes);
  int stages = (int)((200 * 1024) / stage_bytes);
  stages = std::max(2, std::min(8, stages));
  st->stages = stages;
  st->smem = 1024 + stages * stage_bytes + 8 * (2 * stages + 5) + 16 + 8 * st->kp;
  if (st->smem > 227 * 1024) {
    set_error("tensor-core Lloyd tile does not fit shared memory (k=%d)", p.k);
    return ST_ENOTSUP;
  }
  const size_t xb = (size_t)n * st->dp * 2;
  FUELG_TRY(st->xhi.alloc(xb, stream));
  if (st->split) FUELG_TRY(st->xlo.alloc(xb, stream));
  FUELG_TRY(st->xnrm2.alloc(sizeof(float) * n, stream));
  FUELG_TRY(st->xnrm.alloc(sizeof(float) * n, stream));
  const size_t cb = (size_t)st->kp * st->dp * 2;
  FUELG_TRY(st->chi.alloc(cb, stream));
  if (st->split) FUELG_TRY(st->clo.alloc(cb, stream));
  FUELG_TRY(st->cnrm2.alloc(sizeof(float) * st->kp, stream));
  FUELG_TRY(st->cnrm.alloc(sizeof(float) * st->kp, stream));
  FUELG_TRY(st->ulist.alloc(sizeof(int32_t) * n, stream));
  FUELG_TRY(st->umask.alloc(sizeof(uint64_t) * n * st->mw, stream));
  FUELG_TRY(st->ucount.alloc(sizeof(int32_t), stream));
  FUELG_TRY(st->rescored_total.alloc(sizeof(unsigned long long), stream));
  FUELG_CUDA(cudaMemsetAsync(st->rescored_total.p, 0, sizeof(unsigned long long), stream));
  if (st->split)
    prep_rows_kernel<true><<<4 * 152, 256, 0, stream>>>(p.X, n, n, p.d, st->dp, st->xhi.as<__nv_bfloat16>(),
                                                         st->xlo.as<__nv_bfloat16>(), st->xnrm2.as<float>(),
                                                         st->xnrm.as<float>());
  else
    prep_rows_kernel<false><<<4 * 152, 256, 0, stream>>>(p.X, n, n, p.d, st->dp, st->xhi.as<__nv_bfloat16>(),
                                                          nullptr, st->xnrm2.as<float>(), st->xnrm.as<float>()); ::fuelg::note_launch();
  FUELG_CUDA(cudaGetLastError());
  FUELG_TRY(make_map(&st->tmA, st->xhi.p, n, st->dp, BM));
  FUELG_TRY(make_map(&st->tmB, st->chi.p, st->kp, st->dp, st->kp));
  if (st->split) {
    FUELG_TRY(make_map(&st->tmAlo, st->xlo.p, n, st->dp, BM));
    FUELG_TRY(make_map(&st->tmBlo, st->clo.p, st->kp, st->dp, st->kp));
  } else {
    st->tmAlo = st->tmA;
    st->tmBlo = st->tmB;
  }
  auto kern = st->split ? lloyd_tc_kernel<true> : lloyd_tc_kernel<false>;
  FUELG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)st->smem));
  return ST_OK;
}

int lloyd_assign_tc(const LloydParams& p, TcLloydState* st, const float* centers, bool first, int32_t* lab_new,
                    int* dev_status, cudaStream_t stream) {
  const int64_t n = p.n;
  // centre copies and norms for this iteration (padded rows are zero)
  if (st->split)
    prep_rows_kernel<true><<<(st->kp + 7) / 8, 256, 0, stream>>>(centers, st->kp, p.k, p.d, st->dp,
                                                                 st->chi.as<__nv_bfloat16>(), st->clo.as<__nv_bfloat16>(),
                                                                 st->cnrm2.as<float>(), st->cnrm.as<float>());
  else
    prep_rows_kernel<false><<<(st->kp + 7) / 8, 256, 0, stream>>>(centers, st->kp, p.k, p.d, st->dp,
                                                                  st->chi.as<__nv_bfloat16>(), nullptr,
                                                                  st->cnrm2.as<float>(), st->cnrm.as<float>()); ::fuelg::note_launch();
  FUELG_CUDA(cudaMemsetAsync(st->ucount.p, 0, sizeof(int32_t), stream));
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
  a.cn = st->cnrm.as<float>();
  a.lab_new = lab_new;
  a.ulist = st->ulist.as<int32_t>();
  a.umask = st->umask.as<uint64_t>();
  a.ucount = st->ucount.as<int32_t>();
  a.mw = st->mw;
  // Error-bound constants (see the file comment): operand rounding u = 2^-8
  // per BF16 value (2^-16 residual for hi+lo), FP32 accumulation of KP
  // (3*KP for hi+lo) products bounded by KP * 2^-23 of sum|x_i c_i| <= |x||c|,
  // epilogue roundings within 2^-21 (|x|^2 + |c|^2), and fuel's own f32 sum of
  // d squares within (d + 4) 2^-24 of the distance.
  const double KP = (double)st->kc * BK;
  const double u8 = std::ldexp(1.0, -8), u23 = std::ldexp(1.0, -23);
  const double prod = st->split ? 3.1 * std::ldexp(1.0, -16) : (2 * u8 + u8 * u8);
  const double acc = (st->split ? 3.0 : 1.0) * KP * u23 * (1.0 + 2 * u8);
  a.alpha = (float)(2.0 * (prod + acc) * 1.01);
  a.beta = (float)std::ldexp(1.0, -21);
  a.gamma = (float)((p.d + 4) * std::ldexp(1.0, -24) * 1.01);
  // instruction descriptor: D=F32, A=B=BF16, K-major both, N=kp, M=128
  a.idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(st->kp >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
  uint32_t cols = 32;
  while (cols < (uint32_t)(2 * st->kp)) cols <<= 1;
  a.tmem_cols = cols;
  a.status = dev_status;
  a.cancel = cancel_word_device();
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t ntiles = (n + BM - 1) / BM;
  const int grid = (int)std::min<int64_t>(ntiles, sms);
  HotTimer* ht = hot_timer();
  if (ht) ht->begin(stream);
  if (st->split)
    lloyd_tc_kernel<true><<<grid, kTcThreads, st->smem, stream>>>(st->tmA, st->tmAlo, st->tmB, st->tmBlo, a);
  else
    lloyd_tc_kernel<false><<<grid, kTcThreads, st->smem, stream>>>(st->tmA, st->tmAlo, st->tmB, st->tmBlo, a); ::fuelg::note_launch();
  if (ht) ht->end(stream);
  FUELG_CUDA(cudaGetLastError());
  const int rgrid = 4 * sms;
  const int kind = first ? KIND_PAIRWISE : KIND_SQDIST;
  if (kind == KIND_PAIRWISE) {
    if (p.order == ORDER_X86)
      rescore_kernel<KIND_PAIRWISE, ORDER_X86><<<rgrid, 256, 0, stream>>>(p.X, centers, p.d, st->mw, a.ulist, a.umask,
                                                                         a.ucount, a.lab_new, st->rescored_total.as<unsigned long long>());
    else
      rescore_kernel<KIND_PAIRWISE, ORDER_ARM><<<rgrid, 256, 0, stream>>>(p.X, centers, p.d, st->mw, a.ulist, a.umask,
                                                                         a.ucount, a.lab_new, st->rescored_total.as<unsigned long long>()); ::fuelg::note_launch();
  } else {
    if (p.order == ORDER_X86)
      rescore_kernel<KIND_SQDIST, ORDER_X86><<<rgrid, 256, 0, stream>>>(p.X, centers, p.d, st->mw, a.ulist, a.umask,
                                                                       a.ucount, a.lab_new, st->rescored_total.as<unsigned long long>());
    else
      rescore_kernel<KIND_SQDIST, ORDER_ARM><<<rgrid, 256, 0, stream>>>(p.X, centers, p.d, st->mw, a.ulist, a.umask,
                                                                       a.ucount, a.lab_new, st->rescored_total.as<unsigned long long>()); ::fuelg::note_launch();
  }
FUELG_CUDA(cudaGetLastError());
  return ST_OK;
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
