// fuelg_pairwise.cu -- all pairwise distances of one point set, the GPU form
// of fuel.search.pairwise_distances (python/fuel/search.py:92-150 ->
// _compute_pairwise_distances[_condensed]_f32, python/mod.rs:74-124).
//
// Forms (src/api/condensed_distance_matrix.rs:16-48, square_distance_matrix.rs:11-40):
//   condensed: the lower triangle, pair (i, j) with j < i at i (i - 1) / 2 + j;
//   square:    the symmetric n x n matrix (diagonal: distance(x_i, x_i) = 0).
// Every value is fuel's SquaredEuclidean / Euclidean distance(x_i, x_j)
// (src/distance/squared_euclidean.rs:16-39 on x86 with FMA, 99-133 otherwise,
// euclidean.rs:7-9): eight lane accumulators over d & ~7, summed in lane
// order, then the tail -- the same operation sequence as the kNN scan
// (exact_dist_scalar<KIND_KNN, order>), so results are bit-identical.
// (x_i - x_j)^2 == (x_j - x_i)^2 exactly, so the mirrored half of the square
// form is the same value.
//
// Kernels: one CTA per tile of the lower tile triangle (row tile >= column
// tile), 256 threads.  d <= 128 (pairwise_rows_kernel): 64 x 64 tiles, whole
// rows of both blocks in shared memory, 4 x 4 pairs per thread computed lane by
// lane -- lane l's sum over the 8-blocks is finished before it is added to the
// running total, which is the reference's order (acc_0 + acc_1 + ... + acc_7,
// then the tail) with 2 registers per pair instead of 9.  Larger d
// (pairwise_kernel): 32 x 32 tiles, 64-column chunks, 2 x 2 pairs with 8 lane
// accumulators each.  Small d is bound by FP32 issue and the output writes
// (HBM), large d by FP32 issue.
#include <cmath>

#include "../../include/fuelg.h"
#include "fuelg_common.cuh"
#include "fuelg_internal.h"

namespace fuelg {
namespace {

constexpr int PT = 32;      // tile edge (points)
constexpr int PC = 64;      // dims per staged chunk (a multiple of 8)
constexpr int PS = PC + 4;  // staged row stride (floats): 16-byte rows, rotated banks

template <int ORDER, int METRIC, int FORM>
__global__ void __launch_bounds__(256) pairwise_kernel(const float* __restrict__ X, int64_t n, int d,
                                                       int64_t ntb, float* __restrict__ out) {
  constexpr bool FMA8 = ORDER == ORDER_X86;
  __shared__ __align__(16) float sa[PT * PS];
  __shared__ __align__(16) float sb[PT * PS];
  __shared__ float st[PT][PT + 1];  // square form: the tile, for the mirrored (transposed) write
  // tile t of the lower tile triangle -> (bi, bj), bj <= bi
  const int64_t t = blockIdx.x;
  int64_t bi = (int64_t)((std::sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while (bi * (bi + 1) / 2 > t) bi--;
  while ((bi + 1) * (bi + 2) / 2 <= t) bi++;
  const int64_t bj = t - bi * (bi + 1) / 2;
  if (bi >= ntb) return;
  const int64_t i0 = bi * PT, j0 = bj * PT;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int r0 = 2 * ty, c0 = 2 * tx;  // this thread: rows i0 + r0 + {0,1}, cols j0 + c0 + {0,1}
  float acc[2][2][8];
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++)
#pragma unroll
      for (int l = 0; l < 8; l++) acc[a][b][l] = 0.0f;
  const int sd = d & ~7;
  for (int k0 = 0; k0 < sd; k0 += PC) {
    const int kw = min(PC, sd - k0);  // a multiple of 8
    __syncthreads();
    for (int e = threadIdx.x; e < PT * PC; e += 256) {
      const int r = e / PC, c = e - r * PC;
      const int64_t gi = i0 + r, gj = j0 + r;
      sa[r * PS + c] = (c < kw && gi < n) ? __ldg(X + gi * d + k0 + c) : 0.0f;
      sb[r * PS + c] = (c < kw && gj < n) ? __ldg(X + gj * d + k0 + c) : 0.0f;
    }
    __syncthreads();
    for (int g = 0; g < kw; g += 8) {
      float va[2][8], vb[2][8];
#pragma unroll
      for (int a = 0; a < 2; a++) {
        const float4 p = *reinterpret_cast<const float4*>(sa + (r0 + a) * PS + g);
        const float4 q = *reinterpret_cast<const float4*>(sa + (r0 + a) * PS + g + 4);
        va[a][0] = p.x, va[a][1] = p.y, va[a][2] = p.z, va[a][3] = p.w;
        va[a][4] = q.x, va[a][5] = q.y, va[a][6] = q.z, va[a][7] = q.w;
      }
#pragma unroll
      for (int b = 0; b < 2; b++) {
        const float4 p = *reinterpret_cast<const float4*>(sb + (c0 + b) * PS + g);
        const float4 q = *reinterpret_cast<const float4*>(sb + (c0 + b) * PS + g + 4);
        vb[b][0] = p.x, vb[b][1] = p.y, vb[b][2] = p.z, vb[b][3] = p.w;
        vb[b][4] = q.x, vb[b][5] = q.y, vb[b][6] = q.z, vb[b][7] = q.w;
      }
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++)
#pragma unroll
          for (int l = 0; l < 8; l++) {
            const float df = __fsub_rn(va[a][l], vb[b][l]);
            acc[a][b][l] = FMA8 ? __fmaf_rn(df, df, acc[a][b][l]) : __fadd_rn(sq_rn(df), acc[a][b][l]);
          }
    }
  }
  float res[2][2];
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++) {
      const int64_t gi = i0 + r0 + a, gj = j0 + c0 + b;
      float s = acc[a][b][0];
#pragma unroll
      for (int l = 1; l < 8; l++) s = __fadd_rn(s, acc[a][b][l]);
      if (gi < n && gj < n)
        for (int k = sd; k < d; k++) {
          const float df = __fsub_rn(__ldg(X + gi * d + k), __ldg(X + gj * d + k));
          s = FMA8 ? __fmaf_rn(df, df, s) : __fadd_rn(s, sq_rn(df));
        }
      res[a][b] = METRIC == METRIC_EUCLIDEAN ? __fsqrt_rn(s) : s;
    }
  if (FORM == FUELG_PAIRWISE_CONDENSED) {
#pragma unroll
    for (int a = 0; a < 2; a++) {
      const int64_t gi = i0 + r0 + a;
#pragma unroll
      for (int b = 0; b < 2; b++) {
        const int64_t gj = j0 + c0 + b;
        if (gi < n && gj < gi) out[gi * (gi - 1) / 2 + gj] = res[a][b];
      }
    }
  } else {
#pragma unroll
    for (int a = 0; a < 2; a++) {
      const int64_t gi = i0 + r0 + a;
#pragma unroll
      for (int b = 0; b < 2; b++) {
        const int64_t gj = j0 + c0 + b;
        if (gi < n && gj < n) out[gi * n + gj] = res[a][b];
        st[r0 + a][c0 + b] = res[a][b];
      }
    }
    if (bi != bj) {  // the mirrored tile (j, i), written row by row through shared memory
      __syncthreads();
      for (int e = threadIdx.x; e < PT * PT; e += 256) {
        const int rj = e / PT, ci = e - rj * PT;
        const int64_t gj = j0 + rj, gi = i0 + ci;
        if (gj < n && gi < n) out[gj * n + gi] = st[ci][rj];
      }
    }
  }
}

constexpr int PR = 64;      // rows-kernel tile edge
constexpr int kRowsMaxD = 128;

template <int ORDER, int METRIC, int FORM>
__global__ void __launch_bounds__(256) pairwise_rows_kernel(const float* __restrict__ X, int64_t n, int d,
                                                            int64_t ntb, float* __restrict__ out) {
  constexpr bool FMA8 = ORDER == ORDER_X86;
  extern __shared__ float rs[];  // [2][PR][d + 1]: row block i, row block j
  __shared__ float st[PR][PR + 1];
  const int S = d + 1;  // odd stride: the 16 rows a half-warp reads sit in different banks
  float* sa = rs;
  float* sb = rs + PR * S;
  const int64_t t = blockIdx.x;
  int64_t bi = (int64_t)((std::sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while (bi * (bi + 1) / 2 > t) bi--;
  while ((bi + 1) * (bi + 2) / 2 <= t) bi++;
  const int64_t bj = t - bi * (bi + 1) / 2;
  if (bi >= ntb) return;
  const int64_t i0 = bi * PR, j0 = bj * PR;
  for (int e = threadIdx.x; e < PR * d; e += 256) {
    const int r = e / d, c = e - r * d;
    const int64_t gi = i0 + r, gj = j0 + r;
    sa[r * S + c] = gi < n ? __ldg(X + gi * d + c) : 0.0f;
    sb[r * S + c] = gj < n ? __ldg(X + gj * d + c) : 0.0f;
  }
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // rows ty + 16a, cols tx + 16b
  const int sd = d & ~7;
  float sum[4][4];
#pragma unroll 1
  for (int l = 0; l < 8; l++) {
    float acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = 0; b < 4; b++) acc[a][b] = 0.0f;
    for (int c = l; c < sd; c += 8) {
      float xa[4], yb[4];
#pragma unroll
      for (int a = 0; a < 4; a++) xa[a] = sa[(ty + 16 * a) * S + c];
#pragma unroll
      for (int b = 0; b < 4; b++) yb[b] = sb[(tx + 16 * b) * S + c];
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
          const float df = __fsub_rn(xa[a], yb[b]);
          acc[a][b] = FMA8 ? __fmaf_rn(df, df, acc[a][b]) : __fadd_rn(sq_rn(df), acc[a][b]);
        }
    }
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = 0; b < 4; b++) sum[a][b] = l == 0 ? acc[a][b] : __fadd_rn(sum[a][b], acc[a][b]);
  }
  for (int c = sd; c < d; c++) {
    float xa[4], yb[4];
#pragma unroll
    for (int a = 0; a < 4; a++) xa[a] = sa[(ty + 16 * a) * S + c];
#pragma unroll
    for (int b = 0; b < 4; b++) yb[b] = sb[(tx + 16 * b) * S + c];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = 0; b < 4; b++) {
        const float df = __fsub_rn(xa[a], yb[b]);
        sum[a][b] = FMA8 ? __fmaf_rn(df, df, sum[a][b]) : __fadd_rn(sum[a][b], sq_rn(df));
      }
  }
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const int64_t gi = i0 + ty + 16 * a;
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const int64_t gj = j0 + tx + 16 * b;
      const float v = METRIC == METRIC_EUCLIDEAN ? __fsqrt_rn(sum[a][b]) : sum[a][b];
      if (FORM == FUELG_PAIRWISE_CONDENSED) {
        if (gi < n && gj < gi) out[gi * (gi - 1) / 2 + gj] = v;
      } else {
        if (gi < n && gj < n) out[gi * n + gj] = v;
        st[ty + 16 * a][tx + 16 * b] = v;
      }
    }
  }
  if (FORM == FUELG_PAIRWISE_SQUARE && bi != bj) {  // the mirrored tile (j, i), row by row
    __syncthreads();
    for (int e = threadIdx.x; e < PR * PR; e += 256) {
      const int rj = e / PR, ci = e - rj * PR;
      const int64_t gj = j0 + rj, gi = i0 + ci;
      if (gj < n && gi < n) out[gj * n + gi] = st[ci][rj];
    }
  }
}

}  // namespace

int pairwise_launch(const float* X, int64_t n, int d, int metric, int order, int form, float* out,
                    cudaStream_t stream) {
  if (n < 2 && form == FUELG_PAIRWISE_CONDENSED) return ST_OK;
  if (n < 1) return ST_OK;
  const bool rows = d <= kRowsMaxD;
  const int64_t ntb = (n + (rows ? PR : PT) - 1) / (rows ? PR : PT);
  const int64_t tiles = ntb * (ntb + 1) / 2;
  if (tiles > 0x7fffffffll) {
    set_error("pairwise: %lld points need more tiles than one launch holds", (long long)n);
    return ST_ENOTSUP;
  }
  HotTimer* ht = hot_timer();
  if (ht) ht->begin(stream);
  const size_t rsm = (size_t)2 * PR * (d + 1) * sizeof(float);
  auto launch = [&](auto kr, auto kc) -> int {
    if (rows) {
      FUELG_CUDA(cudaFuncSetAttribute(kr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm));
      kr<<<(unsigned)tiles, 256, rsm, stream>>>(X, n, d, ntb, out);
    } else {
      kc<<<(unsigned)tiles, 256, 0, stream>>>(X, n, d, ntb, out);
    }
    return ST_OK;
  };
#define FUELG_PW(O, M, F) FUELG_TRY(launch(pairwise_rows_kernel<O, M, F>, pairwise_kernel<O, M, F>))
  const bool x86 = order == ORDER_X86, eu = metric == METRIC_EUCLIDEAN, cond = form == FUELG_PAIRWISE_CONDENSED;
  if (x86 && eu && cond) FUELG_PW(ORDER_X86, METRIC_EUCLIDEAN, FUELG_PAIRWISE_CONDENSED);
  else if (x86 && eu) FUELG_PW(ORDER_X86, METRIC_EUCLIDEAN, FUELG_PAIRWISE_SQUARE);
  else if (x86 && cond) FUELG_PW(ORDER_X86, METRIC_SQEUCLIDEAN, FUELG_PAIRWISE_CONDENSED);
  else if (x86) FUELG_PW(ORDER_X86, METRIC_SQEUCLIDEAN, FUELG_PAIRWISE_SQUARE);
  else if (eu && cond) FUELG_PW(ORDER_ARM, METRIC_EUCLIDEAN, FUELG_PAIRWISE_CONDENSED);
  else if (eu) FUELG_PW(ORDER_ARM, METRIC_EUCLIDEAN, FUELG_PAIRWISE_SQUARE);
  else if (cond) FUELG_PW(ORDER_ARM, METRIC_SQEUCLIDEAN, FUELG_PAIRWISE_CONDENSED);
  else FUELG_PW(ORDER_ARM, METRIC_SQEUCLIDEAN, FUELG_PAIRWISE_SQUARE);
#undef FUELG_PW
  ::fuelg::note_launch();
  if (ht) ht->end(stream);
  FUELG_CUDA(cudaGetLastError());
  return ST_OK;
}

}  // namespace fuelg
