// fuelg_prep.cuh -- f32 rows -> the BF16 operand copies of the tensor-core
// Lloyd screen, shared by the point preparation (fuelg_tc.cu) and the centre
// update that writes the next pass's centre copies (fuelg_sums.cu).
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace fuelg {

// Element (r, c) of a BF16 copy with rows padded to dp.  With tile_kc > 0 the
// copy is tile-major -- [row tile of 128][K chunk of 64][128 rows][64 columns]
// -- so that every TMA box the screen loads is one contiguous 16 KB block of
// HBM; dp is then tile_kc * 64.
__device__ __forceinline__ int64_t prep_offset(int64_t r, int c, int dp, int tile_kc) {
  if (tile_kc == 0) return r * dp + c;
  return (((r >> 7) * tile_kc + (c >> 6)) * 128 + (r & 127)) * 64 + (c & 63);
}

// One row by one warp: BF16 hi (and lo = BF16(x - hi)) with the row padded to
// dp (a multiple of 8, zero filled; an invalid row is all zeros), plus
// ||x||^2 and ||x||.  Four columns per lane per step; the squared norm is an
// FP32 sum of at most 4*ceil(dp/128) terms per lane and a 5-level tree, so its
// relative error is below (ceil(d/32) + 9) 2^-24 -- the beta term of the
// screen's error bound.  `vec`: xr is 16-byte aligned and d % 4 == 0.  The
// copies hold fl(scale * x) (scale 1: x itself); the norms are those of x.
// Returns whether this lane saw a negative value.
template <bool SPLIT>
__device__ __forceinline__ bool prep_row(const float* __restrict__ xr, int64_t r, bool v, bool vec, int d, int dp,
                                         int tile_kc, __nv_bfloat16* __restrict__ hi,
                                         __nv_bfloat16* __restrict__ lo, float* __restrict__ nrm2,
                                         float* __restrict__ nrm, int lane, float scale = 1.0f) {
  float acc = 0.0f;
  bool anyneg = false;
  // up to 8 chunks of 4 values per lane are loaded before any is used (the
  // loads overlap), then converted in order (the norm chain keeps its order)
  for (int cb = 4 * lane; cb < dp; cb += 128 * 8) {
    float x8[8][4];
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const int c0 = cb + 128 * u;
      if (v && vec && c0 + 3 < d) {
        const float4 t = __ldg(reinterpret_cast<const float4*>(xr + c0));
        x8[u][0] = t.x, x8[u][1] = t.y, x8[u][2] = t.z, x8[u][3] = t.w;
      } else {
#pragma unroll
        for (int q = 0; q < 4; q++) x8[u][q] = (v && c0 + q < d) ? __ldg(xr + c0 + q) : 0.0f;
      }
    }
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const int c0 = cb + 128 * u;
      if (c0 >= dp) break;
      const float* x4 = x8[u];
      float t4[4];
#pragma unroll
      for (int q = 0; q < 4; q++) t4[q] = __fmul_rn(scale, x4[q]);
      __nv_bfloat162 h01 = __floats2bfloat162_rn(t4[0], t4[1]);
      __nv_bfloat162 h23 = __floats2bfloat162_rn(t4[2], t4[3]);
      uint2 hpack;
      hpack.x = *reinterpret_cast<uint32_t*>(&h01);
      hpack.y = *reinterpret_cast<uint32_t*>(&h23);
      const int64_t off = prep_offset(r, c0, dp, tile_kc);
      *reinterpret_cast<uint2*>(hi + off) = hpack;
      if (SPLIT) {
        const float2 f01 = __bfloat1622float2(h01), f23 = __bfloat1622float2(h23);
        __nv_bfloat162 l01 = __floats2bfloat162_rn(t4[0] - f01.x, t4[1] - f01.y);
        __nv_bfloat162 l23 = __floats2bfloat162_rn(t4[2] - f23.x, t4[3] - f23.y);
        uint2 lpack;
        lpack.x = *reinterpret_cast<uint32_t*>(&l01);
        lpack.y = *reinterpret_cast<uint32_t*>(&l23);
        *reinterpret_cast<uint2*>(lo + off) = lpack;
      }
#pragma unroll
      for (int q = 0; q < 4; q++) {
        acc = fmaf(x4[q], x4[q], acc);
        anyneg |= x4[q] < 0.0f;
      }
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if (lane == 0) {
    nrm2[r] = acc;
    nrm[r] = sqrtf(acc);
  }
  return anyneg;
}

// Where the centre update writes the next pass's screen operands: the BF16
// centre rows (row-major, dp columns, kp rows of which k are real) and norms.
struct CentrePrep {
  __nv_bfloat16* hi = nullptr;  // nullptr: no copies to write
  __nv_bfloat16* lo = nullptr;  // split tier only
  float* nrm2 = nullptr;  // ||c||^2 as two halves: nrm2[j] + nrm2[kp + j]
  int dp = 0, kp = 0;
  int32_t* zero_word = nullptr;  // cleared for the next pass (the screen's undecided-point counter)
  float scale = 1.0f;            // the copies hold fl(scale * c)
};

}  // namespace fuelg
