// Correctly rounded binary64 division a / d by a fixed positive divisor d,
// computed on the integer pipe.
//
// GB300 issues binary64 arithmetic at about 1.6 thread-instructions per clock
// per SM and an IEEE division costs about seven of those; integer multiply-add
// issues at about 60.  The stencils divide every difference by dx or dy, so
// the quotient is formed from the operands' integer significands instead:
//
//   a = ma * 2^(ea-1075), d = md * 2^(ed-1075), ma, md in [2^52, 2^53)
//   Q = floor(ma * 2^55 / md) in [2^54, 2^56)
//
// Q is estimated as floor(ma * R / 2^61) with the precomputed reciprocal
// R = floor(2^116 / md) (exact integer division on the host).  The estimate is
// Q or Q-1 (its error is below ma / 2^61 < 2^-8), so one comparison of the
// exact remainder rem = ma*2^55 - Q*md against md fixes it.  The result is then
// rounded to nearest, ties to even, from Q, the round bit and the sticky
// bit (lower bits of Q, or rem != 0), including subnormal results.  This is the
// classical division by an invariant integer (multiply by a scaled reciprocal,
// correct with the remainder) applied to the significands; it returns exactly
// what IEEE division returns, which the tests check against the hardware
// division on every operand class.
#pragma once
#include <cstdint>

namespace pfgb {

struct DivConst {
  uint64_t md;    // divisor significand (53 bits), never a power of two here
  uint64_t R;     // floor(2^116 / md), in (2^63, 2^64)
  int ed;         // divisor biased exponent field (normal: 1..2046)
  int ok;         // 1 when d is positive, normal and not a power of two
};

#ifndef __CUDACC_RTC__
// Host-side preparation.
inline DivConst make_divconst(double d) {
  DivConst c;
  c.md = 0;
  c.R = 0;
  c.ed = 0;
  c.ok = 0;
  uint64_t bits;
  static_assert(sizeof(bits) == sizeof(d), "binary64");
  __builtin_memcpy(&bits, &d, sizeof(d));
  const int ef = (int)((bits >> 52) & 0x7ff);
  const uint64_t frac = bits & 0x000FFFFFFFFFFFFFull;
  if ((bits >> 63) || ef == 0 || ef == 0x7ff || frac == 0) return c;   // sign, subnormal, inf/nan, pow2
  c.md = frac | (1ull << 52);
  unsigned __int128 num = (unsigned __int128)1 << 116;
  c.R = (uint64_t)(num / c.md);
  c.ed = ef;
  c.ok = 1;
  return c;
}
#endif

__device__ __forceinline__ double div_const(double a, const DivConst& c) {
  const uint64_t bits = (uint64_t)__double_as_longlong(a);
  const uint64_t sign = bits & 0x8000000000000000ull;
  const int ef = (int)((bits >> 52) & 0x7ff);
  uint64_t ma = bits & 0x000FFFFFFFFFFFFFull;
  if (ef == 0x7ff) return a;                   // inf / d = inf, NaN stays NaN
  int ea;
  if (ef == 0) {
    if (ma == 0) return a;                     // +-0 / d = +-0
    const int lz = __clzll(ma) - 11;           // bring the leading one to bit 52
    ma <<= lz;
    ea = 1 - lz;
  } else {
    ma |= (1ull << 52);
    ea = ef;
  }
  // quotient estimate and exact remainder
  const uint64_t plo = ma * c.R;
  const uint64_t phi = __umul64hi(ma, c.R);
  uint64_t Q = (phi << 3) | (plo >> 61);
  uint64_t rem = (ma << 55) - Q * c.md;        // exact: the true value is below 2^54
  if (rem >= c.md) {
    Q += 1;
    rem -= c.md;
  }
  // value = (Q + rem/md) * 2^(e0) with e0 = ea - ed - 55 (unbiased exponents)
  const int e0 = ea - c.ed - 55;
  const int msb = 63 - __clzll(Q);             // 54 or 55
  const int E = e0 + msb;                      // exponent of the leading bit
  const int lsb = (E >= -1022) ? E - 52 : -1074;
  const int s = lsb - e0;                      // >= 2
  uint64_t mant, rbit;
  bool sticky;
  if (s < 64) {
    mant = Q >> s;
    rbit = (Q >> (s - 1)) & 1ull;
    sticky = (Q & ((1ull << (s - 1)) - 1ull)) != 0ull;
  } else {                                     // everything below the subnormal LSB
    mant = 0ull;
    rbit = (s == 64) ? (Q >> 63) : 0ull;
    sticky = (s == 64) ? ((Q << 1) != 0ull) : (Q != 0ull);
  }
  sticky = sticky || (rem != 0ull);
  if (rbit && (sticky || (mant & 1ull))) mant += 1ull;
  uint64_t r;
  if (E >= -1022) {
    if (E > 1023) return __longlong_as_double((long long)(sign | 0x7ff0000000000000ull));
    r = ((uint64_t)(E + 1022) << 52) + mant;   // the hidden bit carries into the exponent
    if ((r >> 52) >= 0x7ffull) r = 0x7ff0000000000000ull;
  } else {
    r = mant;                                  // subnormal; a carry to 2^52 is the smallest normal
  }
  return __longlong_as_double((long long)(sign | r));
}

}  // namespace pfgb
