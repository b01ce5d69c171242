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
// Per CTA: every thread turns its terms (a*b products as exact 106-bit
// integers, or plain doubles) into (mantissa, exponent) pairs, the CTA agrees on
// the largest top bit, and each thread adds its terms into an 8-limb (256-bit)
// two's complement window anchored just above that bit.  Terms whose low bits
// would fall below the window take a slow path: shared-memory atomics into a
// full-range CTA superaccumulator.  Both are flushed into the global slot with
// int64 atomics; the last CTA to finish (atomic ticket) rounds the result to
// double (round to nearest, ties to even) and clears the slot for reuse.
//
// FP64 work on GB300 issues at ~1.6 ops/clk/SM versus ~60 integer ops/clk/SM,
// so all of this is integer arithmetic.
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

__device__ __forceinline__ int xa_bitlen64(uint64_t x) { return x ? 64 - __clzll(x) : 0; }

__device__ __forceinline__ void xa_zero(XTerm& t) {
  t.m[0] = t.m[1] = t.m[2] = t.m[3] = 0u; t.e = 0; t.top = INT_MIN; t.neg = false;
}

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

// Exact term for the product a*b.
__device__ __forceinline__ void xa_term_prod(double a, double b, XTerm& t, unsigned& flags) {
  uint64_t ma, mb; int ea, eb; bool sa, sb;
  int ka = xa_unpack(a, ma, ea, sa);
  int kb = xa_unpack(b, mb, eb, sb);
  xa_zero(t);
  if (ka | kb) {
    if (ka == 1 || kb == 1) { flags |= XA_NAN; return; }
    // at least one infinity and no NaN: inf*0 is NaN
    bool zero_other = (ka ? (mb == 0) : (ma == 0));
    if (zero_other) { flags |= XA_NAN; return; }
    flags |= ((sa != sb) ? XA_NINF : XA_PINF);
    return;
  }
  if (ma == 0 || mb == 0) return;
  uint64_t lo = ma * mb;
  uint64_t hi = __umul64hi(ma, mb);
  t.m[0] = (uint32_t)lo; t.m[1] = (uint32_t)(lo >> 32);
  t.m[2] = (uint32_t)hi; t.m[3] = (uint32_t)(hi >> 32);
  t.e = ea + eb;
  t.neg = sa != sb;
  int bl = hi ? 64 + xa_bitlen64(hi) : xa_bitlen64(lo);
  t.top = t.e + bl - 1;
}

// Exact term for the product of two binary32 values (48-bit significand product).
__device__ __forceinline__ void xa_term_prod_f32(float a, float b, XTerm& t, unsigned& flags) {
  const uint32_t ba = __float_as_uint(a), bb = __float_as_uint(b);
  const int efa = (int)((ba >> 23) & 0xff), efb = (int)((bb >> 23) & 0xff);
  uint32_t ma = ba & 0x7fffffu, mb = bb & 0x7fffffu;
  const bool sa = (ba >> 31) != 0, sb = (bb >> 31) != 0;
  xa_zero(t);
  if (efa == 0xff || efb == 0xff) {
    if ((efa == 0xff && ma) || (efb == 0xff && mb)) { flags |= XA_NAN; return; }
    const bool zero_other = (efa == 0xff) ? (efb == 0 && mb == 0) : (efa == 0 && ma == 0);
    if (zero_other) { flags |= XA_NAN; return; }
    flags |= (sa != sb) ? XA_NINF : XA_PINF;
    return;
  }
  int ea, eb;
  if (efa == 0) { ea = 1 - 150; } else { ma |= 0x800000u; ea = efa - 150; }
  if (efb == 0) { eb = 1 - 150; } else { mb |= 0x800000u; eb = efb - 150; }
  if (ma == 0u || mb == 0u) return;
  const uint64_t prod = (uint64_t)ma * (uint64_t)mb;
  t.m[0] = (uint32_t)prod;
  t.m[1] = (uint32_t)(prod >> 32);
  t.e = ea + eb;
  t.neg = sa != sb;
  t.top = t.e + xa_bitlen64(prod) - 1;
}

// Exact term for a single double (used for sums of rounded values).
__device__ __forceinline__ void xa_term_val(double a, XTerm& t, unsigned& flags) {
  uint64_t ma; int ea; bool sa;
  int ka = xa_unpack(a, ma, ea, sa);
  xa_zero(t);
  if (ka) { xa_special(ka, flags); return; }
  if (ma == 0) return;
  t.m[0] = (uint32_t)ma; t.m[1] = (uint32_t)(ma >> 32);
  t.e = ea; t.neg = sa;
  t.top = ea + xa_bitlen64(ma) - 1;
}

// Thread-local 256-bit windows: positive and negative terms accumulate into
// separate unsigned windows (no sign branches); the CTA commit subtracts them.
struct XWin { uint32_t w[XA_WLIMBS]; };

__device__ __forceinline__ void xwin_clear(XWin& w) {
#pragma unroll
  for (int i = 0; i < XA_WLIMBS; ++i) w.w[i] = 0u;
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

// acc += sh placed at limb offset q (0..7); limbs that would land above limb 7
// are zero because every term's top bit lies below the window top.  The carry
// flag does not survive between asm statements, so each offset has its own chain.
__device__ __forceinline__ void xwin_add_at(XWin& acc, const uint32_t sh[5], int q) {
  uint32_t* a = acc.w;
  switch (q) {
    case 0:
      asm("add.cc.u32 %0, %0, %8;\n\taddc.cc.u32 %1, %1, %9;\n\t"
          "addc.cc.u32 %2, %2, %10;\n\taddc.cc.u32 %3, %3, %11;\n\t"
          "addc.cc.u32 %4, %4, %12;\n\taddc.cc.u32 %5, %5, 0;\n\t"
          "addc.cc.u32 %6, %6, 0;\n\taddc.u32 %7, %7, 0;"
          : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4]), "+r"(a[5]), "+r"(a[6]), "+r"(a[7])
          : "r"(sh[0]), "r"(sh[1]), "r"(sh[2]), "r"(sh[3]), "r"(sh[4]));
      break;
    case 1:
      asm("add.cc.u32 %0, %0, %7;\n\taddc.cc.u32 %1, %1, %8;\n\t"
          "addc.cc.u32 %2, %2, %9;\n\taddc.cc.u32 %3, %3, %10;\n\t"
          "addc.cc.u32 %4, %4, %11;\n\taddc.cc.u32 %5, %5, 0;\n\t"
          "addc.u32 %6, %6, 0;"
          : "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4]), "+r"(a[5]), "+r"(a[6]), "+r"(a[7])
          : "r"(sh[0]), "r"(sh[1]), "r"(sh[2]), "r"(sh[3]), "r"(sh[4]));
      break;
    case 2:
      asm("add.cc.u32 %0, %0, %6;\n\taddc.cc.u32 %1, %1, %7;\n\t"
          "addc.cc.u32 %2, %2, %8;\n\taddc.cc.u32 %3, %3, %9;\n\t"
          "addc.cc.u32 %4, %4, %10;\n\taddc.u32 %5, %5, 0;"
          : "+r"(a[2]), "+r"(a[3]), "+r"(a[4]), "+r"(a[5]), "+r"(a[6]), "+r"(a[7])
          : "r"(sh[0]), "r"(sh[1]), "r"(sh[2]), "r"(sh[3]), "r"(sh[4]));
      break;
    case 3:
      asm("add.cc.u32 %0, %0, %5;\n\taddc.cc.u32 %1, %1, %6;\n\t"
          "addc.cc.u32 %2, %2, %7;\n\taddc.cc.u32 %3, %3, %8;\n\t"
          "addc.u32 %4, %4, %9;"
          : "+r"(a[3]), "+r"(a[4]), "+r"(a[5]), "+r"(a[6]), "+r"(a[7])
          : "r"(sh[0]), "r"(sh[1]), "r"(sh[2]), "r"(sh[3]), "r"(sh[4]));
      break;
    case 4:  // sh[4] is zero: the term's top bit is below 256
      asm("add.cc.u32 %0, %0, %4;\n\taddc.cc.u32 %1, %1, %5;\n\t"
          "addc.cc.u32 %2, %2, %6;\n\taddc.u32 %3, %3, %7;"
          : "+r"(a[4]), "+r"(a[5]), "+r"(a[6]), "+r"(a[7])
          : "r"(sh[0]), "r"(sh[1]), "r"(sh[2]), "r"(sh[3]));
      break;
    case 5:
      asm("add.cc.u32 %0, %0, %3;\n\taddc.cc.u32 %1, %1, %4;\n\t"
          "addc.u32 %2, %2, %5;"
          : "+r"(a[5]), "+r"(a[6]), "+r"(a[7])
          : "r"(sh[0]), "r"(sh[1]), "r"(sh[2]));
      break;
    case 6:
      asm("add.cc.u32 %0, %0, %2;\n\taddc.u32 %1, %1, %3;"
          : "+r"(a[6]), "+r"(a[7])
          : "r"(sh[0]), "r"(sh[1]));
      break;
    default:
      a[7] += sh[0];
      break;
  }
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

// Add a term to the thread windows (anchored at digit k0) or the slow path.
__device__ __forceinline__ void xa_add(XWin& pos, XWin& neg, long long* sacc, int k0,
                                       const XTerm& t, unsigned& flags, int& slow_used) {
  if (t.top == INT_MIN) return;
  int s = t.e - (32 * k0 + XA_LSB);            // shift relative to the window bottom
  if (s < 0 || k0 < 0 || k0 + XA_WLIMBS > XA_DIGITS) {
    xa_slow_add(sacc, t, flags);
    slow_used = 1;
    return;
  }
  uint32_t sh[5];
  xa_shift_limbs(t.m, s & 31, sh);
  xwin_add_at(t.neg ? neg : pos, sh, s >> 5);
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

// Reduce the per-thread windows of the CTA into digits k0..k0+7 of the global
// slot, flush the slow-path accumulator, and OR the flags.  `wred` is smem of
// XA_WLIMBS*32 long longs.  Must be called by all threads of the CTA.
__device__ __forceinline__ void xa_cta_commit(XASlot* slot, const XWin& pos, const XWin& neg, int k0,
                                              long long* sacc, int any_slow,
                                              unsigned flags, long long* wred) {
  long long d[XA_WLIMBS];
#pragma unroll
  for (int j = 0; j < XA_WLIMBS; ++j) d[j] = (long long)(uint64_t)pos.w[j] - (long long)(uint64_t)neg.w[j];
#pragma unroll
  for (int j = 0; j < XA_WLIMBS; ++j) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d[j] += __shfl_xor_sync(0xffffffffu, d[j], o);
  }
  flags = __reduce_or_sync(0xffffffffu, flags);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int nw = (blockDim.x + 31) >> 5;
  __shared__ unsigned s_flags;
  if (threadIdx.x == 0) s_flags = 0u;
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int j = 0; j < XA_WLIMBS; ++j) wred[wid * XA_WLIMBS + j] = d[j];
    if (flags) atomicOr(&s_flags, flags);
  }
  __syncthreads();
  int did_atomic = 0;
  if (threadIdx.x < XA_WLIMBS) {
    long long s = 0;
    for (int w = 0; w < nw; ++w) s += wred[w * XA_WLIMBS + threadIdx.x];
    int dig = k0 + threadIdx.x;
    if (s != 0) {
      if (dig >= 0 && dig < XA_DIGITS) {
        atomicAdd((unsigned long long*)&slot->digit[dig], (unsigned long long)s);
        atomicMax(&slot->lo_inv, XA_DIGITS - dig);
        atomicMax(&slot->hi_p1, dig + 1);
      } else {
        atomicOr(&slot->flags, XA_OVERFLOW);
      }
      did_atomic = 1;
    }
  }
  if (any_slow) {
    for (int k = threadIdx.x; k < XA_DIGITS; k += blockDim.x) {
      long long s = sacc[k];
      if (s != 0) {
        atomicAdd((unsigned long long*)&slot->digit[k], (unsigned long long)s);
        atomicMax(&slot->lo_inv, XA_DIGITS - k);
        atomicMax(&slot->hi_p1, k + 1);
        did_atomic = 1;
      }
    }
  }
  if (threadIdx.x == 0 && s_flags) {
    atomicOr(&slot->flags, s_flags);
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

// Called by every CTA after its xa_cta_commit calls for `nslots` slots: the last
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

// Convenience: a per-thread accumulation context for one reduction.
struct XCtx {
  XWin pos, neg;
  unsigned flags;
  int slow;
  int k0;
  __device__ __forceinline__ void clear() { xwin_clear(pos); xwin_clear(neg); flags = 0u; slow = 0; k0 = 0; }
  __device__ __forceinline__ void add(long long* sacc, const XTerm& t) { xa_add(pos, neg, sacc, k0, t, flags, slow); }
};

}  // namespace pfgb
