// Conversions between binary64 and binary32, and exact halving of a binary64
// value, on the integer pipe.
//
// On this GPU the hardware conversions between binary64 and binary32 issue at
// the binary64 rate (measured: about 1.5-1.9 per SM per clock, like DADD),
// against about 60 integer operations per SM per clock, so stages that convert
// every cell spend binary64-pipe time on them.  These helpers give the same
// results as the hardware instructions -- round to nearest, ties to even, for
// binary64 -> binary32, exact the other way; the same infinities and zeros
// (with their signs); subnormals handled -- from bit manipulation alone.  NaNs
// convert to NaNs (their payloads are not kept).
#pragma once
#include <cstdint>

namespace pfgb {

// binary64 -> binary32, round to nearest even
__device__ __forceinline__ float d2f_rn(double d) {
  const uint64_t b = (uint64_t)__double_as_longlong(d);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ff);
  const uint64_t m = b & 0x000FFFFFFFFFFFFFull;
  if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m ? 0x00400000u : 0u));
  const int ef = e - 1023 + 127;             // binary32 exponent field if the result is normal
  if (ef >= 0xff) return __uint_as_float(sign | 0x7f800000u);
  const uint64_t M = e ? (m | (1ull << 52)) : m;   // 53-bit significand (double subnormals: tiny)
  if (ef >= 1) {
    // keep 24 bits; the 29 below decide the rounding; a carry out of the mantissa moves
    // into the exponent field (up to infinity) by the integer addition itself
    const uint32_t kept = (uint32_t)(M >> 29);
    const uint32_t rest = (uint32_t)M & 0x1FFFFFFFu;
    uint32_t u = ((uint32_t)ef << 23) + (kept & 0x7FFFFFu);
    u += (rest > 0x10000000u || (rest == 0x10000000u && (kept & 1u))) ? 1u : 0u;
    return __uint_as_float(sign | u);
  }
  // binary32 subnormal (or zero): significand = M * 2^(e - 1075) / 2^-149 = M >> (29 + 1 - ef)
  const int sh = 30 - ef;                    // >= 30
  if (sh >= 64) return __uint_as_float(sign); // below half the smallest subnormal: rounds to zero
  const uint32_t kept = (uint32_t)(M >> sh);
  const uint64_t rest = M & ((1ull << sh) - 1ull);
  const uint64_t half = 1ull << (sh - 1);
  const uint32_t u = kept + ((rest > half || (rest == half && (kept & 1u))) ? 1u : 0u);
  return __uint_as_float(sign | u);          // a carry to 2^23 is the smallest normal, as it should be
}

// binary32 -> binary64 (exact)
__device__ __forceinline__ double f2d(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint64_t sign = (uint64_t)(b & 0x80000000u) << 32;
  const uint32_t e = (b >> 23) & 0xffu;
  uint32_t m = b & 0x7FFFFFu;
  if (e == 0xffu) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull | (m ? (1ull << 51) : 0ull)));
  if (e == 0u) {
    if (m == 0u) return __longlong_as_double((long long)sign);
    const int k = __clz(m) - 8;              // shifts that bring the leading one to bit 23
    m = (m << k) & 0x7FFFFFu;
    const uint64_t ed = (uint64_t)(1 - k - 127 + 1023);
    return __longlong_as_double((long long)(sign | (ed << 52) | ((uint64_t)m << 29)));
  }
  const uint64_t ed = (uint64_t)(e - 127 + 1023);
  return __longlong_as_double((long long)(sign | (ed << 52) | ((uint64_t)m << 29)));
}

// x * 0.5, exactly as the binary64 multiplication rounds it: one less in the exponent
// field for normal values that stay normal; the multiplication for the rest (zeros,
// subnormals, the smallest normals, infinities, NaNs)
__device__ __forceinline__ double half_exact(double x) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
  if (e > 1u && e < 0x7ffu) return __longlong_as_double((long long)(b - (1ull << 52)));
  return __dmul_rn(x, 0.5);
}

}  // namespace pfgb
