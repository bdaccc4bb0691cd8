// fuelg_exact.cuh -- exact fixed-point arithmetic on f32 data for the
// centroid sums: every finite f32 x is I(x) * 2^unit with a 24-bit integer
// mantissa; at a common scale 2^e_lo (the lowest set bit over the data) the
// sums of I(x) are exact integers, and a mean is rounded once to f32.
#pragma once
#include <cstdint>

namespace fuelg {

__device__ __forceinline__ void f32_parts(float x, uint32_t& mant, int& lsb, int& msb, bool& zero, bool& bad) {
  const uint32_t b = __float_as_uint(x);
  const uint32_t eb = (b >> 23) & 0xffu;
  const uint32_t m = b & 0x7fffffu;
  zero = (b & 0x7fffffffu) == 0;
  bad = eb == 0xffu;
  if (eb == 0) {  // subnormal: m * 2^-149
    mant = m;
    lsb = m ? -149 + __ffs((int)m) - 1 : 0;
    msb = m ? -149 + 31 - __clz((int)m) : 0;
  } else {
    mant = m | 0x800000u;
    lsb = (int)eb - 150 + __ffs((int)mant) - 1;
    msb = (int)eb - 127;
  }
}

// Two's complement of +-I(x) modulo 2^128 (callers use the low 32L bits).
__device__ __forceinline__ unsigned __int128 fixed_of(float x, int e_lo, bool negate) {
  uint32_t mant;
  int l, h;
  bool z, b;
  f32_parts(x, mant, l, h, z, b);
  if (z) return 0;
  const uint32_t bits = __float_as_uint(x);
  const int eb = (int)((bits >> 23) & 0xffu);
  const int unit = (eb == 0 ? -149 : eb - 150);  // weight of mantissa bit 0
  const int sh = unit - e_lo;
  unsigned __int128 v = sh >= 0 ? ((unsigned __int128)mant << sh) : (unsigned __int128)(mant >> (-sh));
  const bool neg = ((bits >> 31) != 0) != negate;
  return neg ? (unsigned __int128)0 - v : v;
}

// Correctly rounded (RNE) f32 of A * 2^e / cnt for A > 0 (normal range).
__device__ __forceinline__ float rn_ratio_f32(unsigned __int128 A, unsigned long long cnt, int e) {
  const int bitsA = A >> 64 ? 128 - __clzll((long long)(unsigned long long)(A >> 64))
                            : 64 - __clzll((long long)(unsigned long long)A);
  const int bitsC = 64 - __clzll((long long)cnt);
  int sh = 0;
  if (bitsA - bitsC < 27) sh = 27 - (bitsA - bitsC);
  const unsigned __int128 A2 = A << sh;
  // exact quotient and remainder: one 64-bit division when A2 fits 64 bits (the
  // common case), else long division by 32-bit digits (cnt < 2^32), else the
  // generic 128-bit division
  unsigned __int128 q, r;
  if ((A2 >> 64) == 0) {
    const unsigned long long a64 = (unsigned long long)A2;
    const unsigned long long q64 = a64 / cnt;
    q = q64;
    r = a64 - q64 * cnt;
  } else if ((cnt >> 32) == 0) {
    unsigned long long rr = 0;
    q = 0;
#pragma unroll
    for (int w = 3; w >= 0; w--) {
      const unsigned long long cur = (rr << 32) | (unsigned long long)(uint32_t)(A2 >> (32 * w));
      const unsigned long long qw = cur / cnt;  // < 2^32: rr < cnt < 2^32
      rr = cur - qw * cnt;
      q = (q << 32) | qw;
    }
    r = rr;
  } else {
    q = A2 / cnt;
    r = A2 - q * cnt;
  }
  const int p = q >> 64 ? 128 - __clzll((long long)(unsigned long long)(q >> 64))
                        : 64 - __clzll((long long)(unsigned long long)q);
  const int drop = p - 24;
  unsigned long long mant = (unsigned long long)(q >> drop);
  const unsigned __int128 rem = q & (((unsigned __int128)1 << drop) - 1);
  const unsigned __int128 half = (unsigned __int128)1 << (drop - 1);
  if (rem > half || (rem == half && (r != 0 || (mant & 1)))) mant += 1;
  return ldexpf((float)mant, drop + e - sh);
}

}  // namespace fuelg
