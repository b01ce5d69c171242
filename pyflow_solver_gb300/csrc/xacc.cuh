// Exactly rounded, order-independent reductions on the integer pipe.
//
// The pressure CG of the reference is cut off at lin_maxiter on a non-symmetric
// operator, so the rounding of its dot products changes u, v and p far above
// 1e-10.  Every reduction here therefore returns the exactly rounded value of
// the exact mathematical sum (products taken exactly), which is independent of
// tile shape, grid size, batching and launch order.  The CPU oracle defines the
// same values (math.fsum over exact TwoProduct splits).
//
// Representation: a fixed-point "superaccumulator" of XA_DIGITS signed 64-bit
// digits; digit k weighs 2^(32k + XA_LSB).  Digits are carry-save (any int64),
// so CTAs add into them with plain atomicAdd and one finaliser normalises.
//
// Per CTA: the threads agree on a bound of the largest term's top bit, and
// each thread adds its terms (a*b products as exact 106-bit integers; a plain
// double is the product with 1.0) into a signed 256-bit window anchored
// XA_HEADROOM bits above that bound.  Terms whose low bits would fall below
// the window take a slow path: shared-memory atomics into a full-range CTA
// superaccumulator.  Both are flushed into the global slot with int64
// atomics; the last CTA to finish (atomic ticket) rounds the result to double
// (round to nearest, ties to even) and clears the slot for reuse.
//
// Binary64 arithmetic on GB300 issues at ~1.6 ops/clk/SM versus ~60 integer
// ops/clk/SM, so all of this is integer arithmetic.
#pragma once
#include <cstdint>

namespace pfgb {

constexpr int XA_DIGITS = 72;
constexpr int XA_LSB = -1184;          // weight of digit 0 is 2^-1184
constexpr int XA_WLIMBS = 8;           // CTA window: 8 x 32-bit limbs
constexpr int XA_HEADROOM = 14;        // carry + sign bits kept above the CTA max

// flags
constexpr unsigned XA_NAN = 1u, XA_PINF = 2u, XA_NINF = 4u, XA_INEXACT = 8u, XA_OVERFLOW = 16u;

struct XASlot {                  // one reduction site in global memory (zeroed at allocation)
  long long digit[XA_DIGITS];
  unsigned int ticket;           // CTAs finished
  unsigned int flags;
  double result;                 // value of the last completed reduction
  unsigned int result_flags;     // flags of the last completed reduction
  int lo_inv;                    // XA_DIGITS - lowest digit written (0: none), atomicMax
  int hi_p1;                     // highest digit written + 1 (0: none), atomicMax
  int pad;
};

struct XTerm {                   // value = (-1)^neg * M * 2^e,  M = m3:m2:m1:m0 < 2^106
  uint32_t m[4];
  int e;
  int top;                       // absolute position of the top bit of M*2^e (INT_MIN for zero)
  bool neg;
};

// Decompose a double into (sign, 53-bit integer mantissa, exponent of its LSB).
// Returns 0 finite, 1 NaN, 2 +inf, 3 -inf.
__device__ __forceinline__ int xa_unpack(double a, uint64_t& m, int& e, bool& neg) {
  uint64_t bits = (uint64_t)__double_as_longlong(a);
  neg = (bits >> 63) != 0;
  int ex = (int)((bits >> 52) & 0x7ff);
  m = bits & 0x000FFFFFFFFFFFFFull;
  if (ex == 0x7ff) return m ? 1 : (neg ? 3 : 2);
  if (ex == 0) { e = 1 - 1075; }
  else { m |= (1ull << 52); e = ex - 1075; }
  return 0;
}

__device__ __forceinline__ void xa_special(int kind, unsigned& flags) {
  if (kind == 1) flags |= XA_NAN;
  else if (kind == 2) flags |= XA_PINF;
  else if (kind == 3) flags |= XA_NINF;
}

// Window base digit for a CTA whose largest term top bit is `top`
// (absolute exponent).  Window digits are [k0, k0+8).
__device__ __forceinline__ int xa_window_digit(int top) {
  int need = top + 1 + XA_HEADROOM - XA_LSB;            // grid bits needed up to the window top
  int kt = (need + 31) >> 5;
  return kt - XA_WLIMBS;
}

// Shift the 4-limb mantissa left by r (0..31) bits into 5 limbs.
__device__ __forceinline__ void xa_shift_limbs(const uint32_t m[4], int r, uint32_t sh[5]) {
  sh[0] = m[0] << r;
  sh[1] = __funnelshift_l(m[0], m[1], r);
  sh[2] = __funnelshift_l(m[1], m[2], r);
  sh[3] = __funnelshift_l(m[2], m[3], r);
  sh[4] = (r == 0) ? 0u : (m[3] >> (32 - r));
}

// Slow path: add a term into a full-range shared-memory superaccumulator.
__device__ __forceinline__ void xa_slow_add(long long* sacc, const XTerm& t, unsigned& flags) {
  int pos = t.e - XA_LSB;                       // bit position of M's LSB on the grid
  uint32_t m[4] = {t.m[0], t.m[1], t.m[2], t.m[3]};
  if (pos < 0) {
    // bits below the grid (below 2^-1184) are dropped
    int drop = -pos;
    flags |= XA_INEXACT;
    if (drop >= 128) return;
    uint32_t s[4];
    int qd = drop >> 5, rd = drop & 31;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int src = i + qd;
      uint32_t lo = (src < 4) ? m[src] : 0u;
      uint32_t hi = (src + 1 < 4) ? m[src + 1] : 0u;
      s[i] = (rd == 0) ? lo : __funnelshift_r(lo, hi, rd);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) m[i] = s[i];
    pos = 0;
  }
  int q = pos >> 5, r = pos & 31;
  uint32_t sh[5];
  xa_shift_limbs(m, r, sh);
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    if (sh[j] == 0u) continue;
    int d = q + j;
    if (d >= XA_DIGITS) { flags |= XA_OVERFLOW; continue; }
    long long v = (long long)sh[j];
    atomicAdd((unsigned long long*)&sacc[d], (unsigned long long)(t.neg ? -v : v));
  }
}

// ---- per-thread accumulation --------------------------------------------------
//
// A thread adds its terms into a signed 256-bit two's complement window of
// eight 32-bit limbs; limb j is digit k0 + j of the slot.  A term a*b is the
// exact integer product of the two 53-bit significands (four 32-bit partial
// products), moved to its place by a funnel shift (the bit offset) and a
// three-stage limb rotation (the limb offset, 0..4), and added with one carry
// chain; a negative term is added as its complement with a carry-in of one.
// Nothing branches on the term but the rare cases (a NaN or infinite operand,
// a term whose low bits fall below the window).

// Upper bound of the top bit of |a*b| (the product's LSB exponent plus 105);
// INT_MIN when an operand is NaN or infinite (those only set flags).
__device__ __forceinline__ int xa_prod_top(double a, double b) {
  const int efa = (int)(((uint32_t)__double2hiint(a) >> 20) & 0x7ffu);
  const int efb = (int)(((uint32_t)__double2hiint(b) >> 20) & 0x7ffu);
  if (efa == 0x7ff || efb == 0x7ff) return INT_MIN;
  return max(efa, 1) + max(efb, 1) - 2150 + 105;
}

// One thread's share of one reduction.
struct XAcc {
  uint32_t w[XA_WLIMBS];
  unsigned flags;
  int slow;       // a term went to the shared full-range accumulator
  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int j = 0; j < XA_WLIMBS; ++j) w[j] = 0u;
    flags = 0u;
    slow = 0;
  }
};

// NaN and infinity flags of a product with a non-finite operand (inf * 0 is NaN).
__device__ __forceinline__ void xa_special_prod(double a, double b, unsigned& flags) {
  uint64_t ma, mb; int ea, eb; bool sa, sb;
  const int ka = xa_unpack(a, ma, ea, sa);
  const int kb = xa_unpack(b, mb, eb, sb);
  if (ka == 1 || kb == 1) { flags |= XA_NAN; return; }
  const bool zero_other = ka ? (kb == 0 && mb == 0) : (ma == 0);
  if (zero_other) { flags |= XA_NAN; return; }
  flags |= (sa != sb) ? XA_NINF : XA_PINF;
}

// x += a*b (SQUARE: b is a, and the term is never negative).  k0 is the CTA's
// window digit (xa_window_digit of the largest xa_prod_top of the CTA's terms).
template <bool SQUARE = false>
__device__ __forceinline__ void xa_acc_prod(XAcc& x, long long* sacc, int k0, double a, double b) {
  const uint32_t ha = (uint32_t)__double2hiint(a), la = (uint32_t)__double2loint(a);
  const uint32_t hb = SQUARE ? ha : (uint32_t)__double2hiint(b);
  const uint32_t lb = SQUARE ? la : (uint32_t)__double2loint(b);
  const int efa = (int)((ha >> 20) & 0x7ffu), efb = (int)((hb >> 20) & 0x7ffu);
  if (efa == 0x7ff || efb == 0x7ff) {
    xa_special_prod(a, SQUARE ? a : b, x.flags);
    return;
  }
  const uint32_t a1 = (ha & 0xfffffu) | (efa ? 0x100000u : 0u);
  const uint32_t b1 = SQUARE ? a1 : ((hb & 0xfffffu) | (efb ? 0x100000u : 0u));
  // M = a*b significands = p00 + mid 2^32 + p11 2^64 (< 2^106)
  const uint64_t p00 = (uint64_t)la * lb;
  const uint64_t mid = SQUARE ? (((uint64_t)la * a1) << 1) : ((uint64_t)la * b1 + (uint64_t)a1 * lb);   // < 2^54
  const uint64_t p11 = (uint64_t)a1 * b1;                                                             // < 2^42
  uint32_t m1, m2, m3;
  asm("add.cc.u32 %0, %3, %4;\n\taddc.cc.u32 %1, %5, %6;\n\taddc.u32 %2, %7, 0;"
      : "=r"(m1), "=r"(m2), "=r"(m3)
      : "r"((uint32_t)(p00 >> 32)), "r"((uint32_t)mid), "r"((uint32_t)(mid >> 32)), "r"((uint32_t)p11),
        "r"((uint32_t)(p11 >> 32)));
  const uint32_t m0 = (uint32_t)p00;
  const int e = max(efa, 1) + max(efb, 1) - 2150;          // weight of M's LSB
  const int s = e - (32 * k0 + XA_LSB);                      // its bit offset in the window
  const bool neg = !SQUARE && ((ha ^ hb) >> 31);
  if (s < 0 || k0 < 0 || k0 + XA_WLIMBS > XA_DIGITS) {
    if ((m0 | m1 | m2 | m3) == 0u) return;
    XTerm t;
    t.m[0] = m0; t.m[1] = m1; t.m[2] = m2; t.m[3] = m3;
    t.e = e;
    t.top = e + 105;
    t.neg = neg;
    xa_slow_add(sacc, t, x.flags);
    x.slow = 1;
    return;
  }
  // s <= 135 here (the term lies at least XA_HEADROOM bits below the window top),
  // so the limb offset q is at most 4 and nothing is shifted past limb 7
  const int r = s & 31, q = s >> 5;
  uint32_t v[XA_WLIMBS];
  v[0] = m0 << r;
  v[1] = __funnelshift_l(m0, m1, r);
  v[2] = __funnelshift_l(m1, m2, r);
  v[3] = __funnelshift_l(m2, m3, r);
  v[4] = __funnelshift_l(m3, 0u, r);
  v[5] = v[6] = v[7] = 0u;
#pragma unroll
  for (int k = 1; k <= 4; k <<= 1) {
    const bool c = (q & k) != 0;
#pragma unroll
    for (int j = XA_WLIMBS - 1; j >= 0; --j) v[j] = c ? (j >= k ? v[j - k] : 0u) : v[j];
  }
  uint32_t* w = x.w;
  if (SQUARE) {
    asm("add.cc.u32 %0, %0, %8;\n\taddc.cc.u32 %1, %1, %9;\n\t"
        "addc.cc.u32 %2, %2, %10;\n\taddc.cc.u32 %3, %3, %11;\n\t"
        "addc.cc.u32 %4, %4, %12;\n\taddc.cc.u32 %5, %5, %13;\n\t"
        "addc.cc.u32 %6, %6, %14;\n\taddc.u32 %7, %7, %15;"
        : "+r"(w[0]), "+r"(w[1]), "+r"(w[2]), "+r"(w[3]), "+r"(w[4]), "+r"(w[5]), "+r"(w[6]), "+r"(w[7])
        : "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]));
  } else {
    // w += (v ^ mask) + (mask & 1): the carry-in comes from mask + mask
    const uint32_t mask = neg ? 0xffffffffu : 0u;
    asm("{\n\t.reg .u32 t;\n\tadd.cc.u32 t, %8, %8;\n\t"
        "addc.cc.u32 %0, %0, %9;\n\taddc.cc.u32 %1, %1, %10;\n\t"
        "addc.cc.u32 %2, %2, %11;\n\taddc.cc.u32 %3, %3, %12;\n\t"
        "addc.cc.u32 %4, %4, %13;\n\taddc.cc.u32 %5, %5, %14;\n\t"
        "addc.cc.u32 %6, %6, %15;\n\taddc.u32 %7, %7, %16;\n\t}"
        : "+r"(w[0]), "+r"(w[1]), "+r"(w[2]), "+r"(w[3]), "+r"(w[4]), "+r"(w[5]), "+r"(w[6]), "+r"(w[7])
        : "r"(mask), "r"(v[0] ^ mask), "r"(v[1] ^ mask), "r"(v[2] ^ mask), "r"(v[3] ^ mask), "r"(v[4] ^ mask),
          "r"(v[5] ^ mask), "r"(v[6] ^ mask), "r"(v[7] ^ mask));
  }
}

// x += a (exactly: the product a * 1.0)
__device__ __forceinline__ void xa_acc_val(XAcc& x, long long* sacc, int k0, double a) {
  xa_acc_prod<false>(x, sacc, k0, a, 1.0);
}

// Block-wide max of an int (all threads get it). `red` is >= 32 ints of smem.
__device__ __forceinline__ int xa_block_max(int v, int* red) {
  v = __reduce_max_sync(0xffffffffu, v);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  int r = (lane < nw) ? red[lane] : INT_MIN;
  r = __reduce_max_sync(0xffffffffu, r);
  return r;
}

// Two block-wide maxima with one barrier. `red` is >= 64 ints of smem that no
// earlier code of the kernel uses.
__device__ __forceinline__ void xa_block_max2(int& v0, int& v1, int* red) {
  v0 = __reduce_max_sync(0xffffffffu, v0);
  v1 = __reduce_max_sync(0xffffffffu, v1);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  if (lane == 0) {
    red[wid] = v0;
    red[32 + wid] = v1;
  }
  __syncthreads();
  v0 = __reduce_max_sync(0xffffffffu, (lane < nw) ? red[lane] : INT_MIN);
  v1 = __reduce_max_sync(0xffffffffu, (lane < nw) ? red[32 + lane] : INT_MIN);
}

// Warp sum of the eight signed digits of the lanes' windows, reduce-scattered
// (each shuffle level halves the digits a lane carries): every fourth lane
// returns the warp sum of digit *digit.
__device__ __forceinline__ long long xa_warp_digits(const XAcc& x, int* digit) {
  const int lane = threadIdx.x & 31;
  long long d[XA_WLIMBS];
#pragma unroll
  for (int j = 0; j < XA_WLIMBS - 1; ++j) d[j] = (long long)x.w[j];
  d[XA_WLIMBS - 1] = (long long)(int)x.w[XA_WLIMBS - 1];   // the sign limb
  const bool u16 = (lane & 16) != 0, u8 = (lane & 8) != 0, u4 = (lane & 4) != 0;
  long long d4[4], d2[2], d1;
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const long long send = u16 ? d[m] : d[m + 4];
    const long long keep = u16 ? d[m + 4] : d[m];
    d4[m] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int m = 0; m < 2; ++m) {
    const long long send = u8 ? d4[m] : d4[m + 2];
    const long long keep = u8 ? d4[m + 2] : d4[m];
    d2[m] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
  {
    const long long send = u4 ? d2[0] : d2[1];
    const long long keep = u4 ? d2[1] : d2[0];
    d1 = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
  d1 += __shfl_xor_sync(0xffffffffu, d1, 2);
  d1 += __shfl_xor_sync(0xffffffffu, d1, 1);
  *digit = (u16 ? 4 : 0) + (u8 ? 2 : 0) + (u4 ? 1 : 0);
  return d1;
}

// One warp adds the CTA's window sums (wred: XA_WLIMBS per warp) into digits
// k0..k0+7 of the slot and widens the slot's span of written digits once.
// Returns whether this lane made an atomic update.
__device__ __forceinline__ int xa_warp_flush(XASlot* slot, int k0, const long long* wred, int nw) {
  const int lane = threadIdx.x & 31;
  long long s = 0;
  if (lane < XA_WLIMBS)
    for (int w = 0; w < nw; ++w) s += wred[w * XA_WLIMBS + lane];
  const int dig = k0 + lane;
  const bool inr = dig >= 0 && dig < XA_DIGITS;
  int did = 0;
  if (s != 0) {
    if (inr) atomicAdd((unsigned long long*)&slot->digit[dig], (unsigned long long)s);
    else atomicOr(&slot->flags, XA_OVERFLOW);
    did = 1;
  }
  const unsigned m = __ballot_sync(0xffffffffu, s != 0 && inr);
  if (lane == 0 && m) {
    atomicMax(&slot->lo_inv, XA_DIGITS - (k0 + __ffs(m) - 1));
    atomicMax(&slot->hi_p1, k0 + 32 - __clz(m));
    did = 1;
  }
  return did;
}

// The CTA's shared-memory superaccumulator of slow-path terms into the slot.
__device__ __forceinline__ int xa_flush_slow(XASlot* slot, const long long* sacc) {
  int did = 0;
  for (int k = threadIdx.x; k < XA_DIGITS; k += blockDim.x) {
    const long long s = sacc[k];
    if (s != 0) {
      atomicAdd((unsigned long long*)&slot->digit[k], (unsigned long long)s);
      atomicMax(&slot->lo_inv, XA_DIGITS - k);
      atomicMax(&slot->hi_p1, k + 1);
      did = 1;
    }
  }
  return did;
}

// Sum the CTA's windows into digits k0..k0+7 of the global slot, flush the
// slow-path accumulator and OR the flags.  `wred` is smem of XA_WLIMBS x
// (warps) long longs.  Must be called by all threads of the CTA.
__device__ __forceinline__ void xa_acc_commit(XASlot* slot, const XAcc& x, int k0, long long* sacc, int any_slow,
                                              long long* wred) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  int my_digit;
  const long long d1 = xa_warp_digits(x, &my_digit);
  const unsigned flags = __reduce_or_sync(0xffffffffu, x.flags);
  __shared__ unsigned s_flags;
  if (threadIdx.x == 0) s_flags = 0u;
  __syncthreads();
  if ((lane & 3) == 0) wred[wid * XA_WLIMBS + my_digit] = d1;
  if (lane == 0 && flags) atomicOr(&s_flags, flags);
  __syncthreads();
  int did_atomic = 0;
  if (wid == 0) did_atomic = xa_warp_flush(slot, k0, wred, nw);
  if (any_slow) did_atomic |= xa_flush_slow(slot, sacc);
  if (threadIdx.x == 0 && s_flags) {
    atomicOr(&slot->flags, s_flags);
    did_atomic = 1;
  }
  // make this thread's atomics visible before the CTA takes its ticket
  if (did_atomic) __threadfence();
}

// Shared state of a two-slot commit; zero() runs before the CTA's first barrier
// of the reduction.
struct XCommit2 {
  unsigned flags[2];
  int slow;
  __device__ __forceinline__ void zero() {
    if (threadIdx.x == 0) {
      flags[0] = flags[1] = 0u;
      slow = 0;
    }
  }
};

// A warp's share of one window: the warp sum of digit `digit` (every fourth
// lane), and the warp's flags and slow-path bit.
struct XWarpPart {
  long long sum;
  int digit;
  unsigned flags;
  int slow;
};

__device__ __forceinline__ XWarpPart xa_warp_part(const XAcc& x) {
  XWarpPart p;
  p.sum = xa_warp_digits(x, &p.digit);
  p.flags = __reduce_or_sync(0xffffffffu, x.flags);
  p.slow = (int)__reduce_or_sync(0xffffffffu, (unsigned)x.slow);
  return p;
}

// Two slots at once with one barrier: warp 0 flushes the first window, warp 1
// the second.  `wred` holds 2 x XA_WLIMBS x (warps) long longs.  The CTA needs
// at least two warps.
__device__ __forceinline__ void xa_acc_commit2(XASlot* s0, const XWarpPart& p0, int k0, long long* sacc0, XASlot* s1,
                                               const XWarpPart& p1, int k1, long long* sacc1, long long* wred,
                                               XCommit2& cs) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  if ((lane & 3) == 0) {
    wred[wid * XA_WLIMBS + p0.digit] = p0.sum;
    wred[(nw + wid) * XA_WLIMBS + p1.digit] = p1.sum;
  }
  if (lane == 0) {
    if (p0.flags) atomicOr(&cs.flags[0], p0.flags);
    if (p1.flags) atomicOr(&cs.flags[1], p1.flags);
    const int slow = p0.slow | (p1.slow << 1);
    if (slow) atomicOr(&cs.slow, slow);
  }
  __syncthreads();
  int did_atomic = 0;
  if (wid == 0) did_atomic = xa_warp_flush(s0, k0, wred, nw);
  else if (wid == 1) did_atomic = xa_warp_flush(s1, k1, wred + nw * XA_WLIMBS, nw);
  const int any_slow = cs.slow;
  if (any_slow & 1) did_atomic |= xa_flush_slow(s0, sacc0);
  if (any_slow & 2) did_atomic |= xa_flush_slow(s1, sacc1);
  if (threadIdx.x == 0 && cs.flags[0]) {
    atomicOr(&s0->flags, cs.flags[0]);
    did_atomic = 1;
  }
  if (threadIdx.x == 32 && cs.flags[1]) {
    atomicOr(&s1->flags, cs.flags[1]);
    did_atomic = 1;
  }
  // make this thread's atomics visible before the CTA takes its ticket
  if (did_atomic) __threadfence();
}

// Round the superaccumulator to double (round to nearest, ties to even).
// Only digits [lo, hi] can be non-zero.  Single thread.
static __device__ __noinline__ double xa_round(const long long* dg, int lo, int hi, unsigned flags) {
  if (flags & XA_NAN) return __longlong_as_double(0x7ff8000000000000ll);
  if ((flags & XA_PINF) && (flags & XA_NINF)) return __longlong_as_double(0x7ff8000000000000ll);
  if (flags & XA_PINF) return __longlong_as_double(0x7ff0000000000000ll);
  if (flags & XA_NINF) return __longlong_as_double((long long)0xfff0000000000000ull);
  if (hi < lo) return 0.0;
  // normalise digits lo..top into [0, 2^32) with a signed final carry; the
  // span is widened by three digits so that every carry lands inside it
  const int top = (hi + 3 < XA_DIGITS) ? hi + 3 : XA_DIGITS - 1;
  uint32_t v[XA_DIGITS];
  long long carry = 0;
  for (int k = lo; k <= top; ++k) {
    long long x = (k <= hi ? dg[k] : 0) + carry;   // |dg| < 2^62: no overflow
    v[k] = (uint32_t)x;
    carry = x >> 32;
  }
  bool neg = carry < 0;
  if (carry != 0 && carry != -1) flags |= XA_OVERFLOW;
  if (neg) {                        // two's complement negate of the span
    uint32_t c = 1;
    for (int k = lo; k <= top; ++k) {
      uint32_t x = ~v[k] + c;
      c = (c && x == 0u) ? 1u : 0u;
      v[k] = x;
    }
  }
  if (flags & XA_OVERFLOW)
    return __longlong_as_double(neg ? (long long)0xfff0000000000000ull : 0x7ff0000000000000ll);
  int h = -1;
  for (int k = top; k >= lo; --k) if (v[k]) { h = k; break; }
  if (h < 0) return 0.0;
  auto digit = [&](int k) -> uint64_t { return (k >= lo && k <= top) ? v[k] : 0u; };
  int msb = 32 * h + 31 - __clz(v[h]);          // grid bit index of the leading one
  int E = msb + XA_LSB;                          // value in [2^E, 2^(E+1))
  int lsb = (E >= -1022) ? E - 52 : -1074;       // weight of the double's LSB
  int b0 = lsb - XA_LSB;                         // grid bit index of that LSB (>= 110)
  uint64_t mant;
  {
    int q = b0 >> 5, r = b0 & 31;
    uint64_t lo64 = digit(q) | (digit(q + 1) << 32);
    uint64_t part = (r == 0) ? lo64 : ((lo64 >> r) | (digit(q + 2) << (64 - r)));
    int nb = msb - b0 + 1;
    mant = (nb >= 64) ? part : (part & ((1ull << nb) - 1ull));
  }
  const int rb = b0 - 1;
  const uint32_t rbit = (uint32_t)((digit(rb >> 5) >> (rb & 31)) & 1u);
  bool sticky = false;
  {
    int q = rb >> 5, r = rb & 31;   // bits [0, rb) are sticky
    for (int k = lo; k < q && !sticky; ++k) sticky = v[k] != 0u;
    if (!sticky && r) sticky = (digit(q) & ((1ull << r) - 1ull)) != 0u;
  }
  if (rbit && (sticky || (mant & 1ull))) mant += 1ull;
  uint64_t bits;
  if (E >= -1022) bits = ((uint64_t)(E + 1022) << 52) + mant;   // hidden bit carries into the exponent
  else bits = mant;                                             // subnormal (rounding may reach 2^-1022)
  if ((bits >> 52) >= 0x7ffull) bits = 0x7ff0000000000000ull;
  if (neg) bits |= 0x8000000000000000ull;
  return __longlong_as_double((long long)bits);
}

// Called by every CTA after its xa_acc_commit calls for `nslots` slots: the last
// CTA rounds and clears them.  Returns true in the (single) finalising CTA, with
// results written into slot->result.  All threads of the CTA must call.
__device__ __forceinline__ bool xa_finish(XASlot* const* slots, int nslots, unsigned nctas) {
  __shared__ unsigned s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned t = atomicAdd(&slots[0]->ticket, 1u);
    s_last = (t == nctas - 1) ? 1u : 0u;
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  if (threadIdx.x < nslots) {
    XASlot* s = slots[threadIdx.x];
    const int li = *(volatile int*)&s->lo_inv, hp = *(volatile int*)&s->hi_p1;
    const int lo = li ? XA_DIGITS - li : 0, hi = hp - 1;
    long long dg[XA_DIGITS];
    for (int k = lo; k <= hi; ++k) dg[k] = *(volatile long long*)&s->digit[k];
    unsigned fl = *(volatile unsigned*)&s->flags;
    s->result = xa_round(dg, lo, hi, fl);
    s->result_flags = fl;
    for (int k = lo; k <= hi; ++k) s->digit[k] = 0;
    s->flags = 0u;
    s->lo_inv = 0;
    s->hi_p1 = 0;
  }
  if (threadIdx.x == 0) slots[0]->ticket = 0u;
  __syncthreads();
  __threadfence();
  return true;
}

}  // namespace pfgb
