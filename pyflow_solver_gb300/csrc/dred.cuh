// Deterministic binary64 sums over the tiles of one instance.
//
// Each tile (a CTA, or a 256-thread group of a persistent CTA) reduces its
// values with a fixed shuffle tree, writes the tile's partial to
// part[r * nt + tile], and the last tile of the instance to arrive (an atomic
// ticket) adds the nt partials in tile order with a fixed tree as well.  The
// result depends only on the instance's values and its tiling, not on timing
// or on the other instances of a batch.
//
// Sums of binary32 products use float-float accumulation: each product is
// split exactly into p + e (e = fma(a, b, -p)) and added into an unevaluated
// pair hi + lo with error-free transformations, about 44 significant bits --
// the accuracy of a binary64 sum at a binary32 instruction cost (the binary64
// pipe of this GPU issues at a small fraction of the binary32 rate).  The
// pairs are combined by a fixed shuffle tree; each warp's pair is rounded to
// binary64 and the tile's partial is the binary64 sum of its warps in order.
//
// X is the execution context (tid(), sync()) of persist.cuh; NT threads.
#pragma once
#include <cuda_runtime.h>

namespace pfgb {

template <int NT>
struct DRedSmem {
  double w[4][NT / 32];
  int last;
};

struct FF {
  float hi, lo;
};

__device__ __forceinline__ FF ff_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return FF{s, e};
}

__device__ __forceinline__ FF ff_renorm(float hi, float lo) {
  const float s = hi + lo;
  return FF{s, lo - (s - hi)};
}

__device__ __forceinline__ void ff_add_prod(FF& acc, float a, float b) {
  const float p = a * b;
  const float pe = fmaf(a, b, -p);
  const FF t = ff_two_sum(acc.hi, p);
  acc = ff_renorm(t.hi, t.lo + (acc.lo + pe));
}

__device__ __forceinline__ FF ff_merge(FF a, FF b) {
  const FF t = ff_two_sum(a.hi, b.hi);
  return ff_renorm(t.hi, t.lo + (a.lo + b.lo));
}

__device__ __forceinline__ FF ff_warp_sum(FF x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    FF y;
    y.hi = __shfl_xor_sync(0xffffffffu, x.hi, o);
    y.lo = __shfl_xor_sync(0xffffffffu, x.lo, o);
    x = ff_merge(x, y);
  }
  return x;
}

// Sum over the tile of per-warp binary64 values already in sm.w[r][warp];
// valid in tid 0.  The NT/32 values of each r are added by a fixed tree over
// the lanes of warp 0 (lane r * NT/32 + warp), so the R sums take log2(NT/32)
// dependent additions instead of a serial chain.
template <int R, int NT, class X>
__device__ __forceinline__ void dred_warps(const X& x, double (&v)[R], DRedSmem<NT>& sm) {
  constexpr int NW = NT / 32;
  static_assert(R * NW <= 32 && (NW & (NW - 1)) == 0, "one lane of warp 0 per value and warp");
  x.sync();
  if (x.tid() < 32) {
    const int lane = x.tid(), r = lane / NW, w = lane % NW;
    double a = (r < R) ? sm.w[r][w] : 0.0;
#pragma unroll
    for (int o = NW / 2; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = __shfl_sync(0xffffffffu, a, q * NW);
  }
  x.sync();
}

// Warp sums of R values per lane: a reduce-scatter for R = 2 and 4 (each of the
// first shuffle levels halves the values a lane carries), a plain tree otherwise.
// Returns the lane's sum and sets *r to the value it belongs to; the lanes with
// (lane % (32 / R)) == 0 hold the warp's total of value lane / (32 / R).
template <int R>
__device__ __forceinline__ double dred_warp_scatter(const double (&v)[R], int lane, int* r) {
  if constexpr (R == 2) {
    const bool up = (lane & 16) != 0;
    double a = (up ? v[1] : v[0]) + __shfl_xor_sync(0xffffffffu, up ? v[0] : v[1], 16);
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    *r = up ? 1 : 0;
    return a;
  } else if constexpr (R == 4) {
    const bool u16 = (lane & 16) != 0, u8 = (lane & 8) != 0;
    const double a0 = (u16 ? v[2] : v[0]) + __shfl_xor_sync(0xffffffffu, u16 ? v[0] : v[2], 16);
    const double a1 = (u16 ? v[3] : v[1]) + __shfl_xor_sync(0xffffffffu, u16 ? v[1] : v[3], 16);
    double a = (u8 ? a1 : a0) + __shfl_xor_sync(0xffffffffu, u8 ? a0 : a1, 8);
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    *r = (u16 ? 2 : 0) + (u8 ? 1 : 0);
    return a;
  } else {
    static_assert(R == 1, "warp sums of 1, 2 or 4 values");
    double a = v[0];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    *r = 0;
    return a;
  }
}

// Sum of v over the tile (fixed order); valid in tid 0.
template <int R, int NT, class X>
__device__ __forceinline__ void dred_block(const X& x, double (&v)[R], DRedSmem<NT>& sm) {
  const int lane = x.tid() & 31, warp = x.tid() >> 5;
  int r;
  const double a = dred_warp_scatter<R>(v, lane, &r);
  if ((lane & (32 / R - 1)) == 0) sm.w[r][warp] = a;
  dred_warps<R, NT>(x, v, sm);
}

// The tile's partials (in tid 0) into the instance's sums: true in every
// thread of the tile that completes them; out[] is then valid in tid 0.
template <int R, int NT, class X>
__device__ __forceinline__ bool dred_finish(const X& x, const double (&d)[R], double* part, int nt, int tile,
                                            unsigned* ticket, double (&out)[R], DRedSmem<NT>& sm) {
  if (x.tid() == 0) {
#pragma unroll
    for (int r = 0; r < R; ++r) part[(long)r * nt + tile] = d[r];
    __threadfence();
    sm.last = (atomicAdd(ticket, 1u) == (unsigned)(nt - 1)) ? 1 : 0;
  }
  x.sync();
  if (!sm.last) return false;
  __threadfence();
  double s[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    s[r] = 0.0;
    for (int k = x.tid(); k < nt; k += NT) s[r] += __ldcg(&part[(long)r * nt + k]);
  }
  dred_block<R, NT>(x, s, sm);
  if (x.tid() == 0) {
#pragma unroll
    for (int r = 0; r < R; ++r) out[r] = s[r];
    atomicExch(ticket, 0u);
  }
  return true;
}

// binary64 values
template <int R, int NT, class X>
__device__ __forceinline__ bool dred_sum(const X& x, double (&v)[R], double* part, int nt, int tile, unsigned* ticket,
                                         double (&out)[R], DRedSmem<NT>& sm) {
  dred_block<R, NT>(x, v, sm);
  return dred_finish<R, NT>(x, v, part, nt, tile, ticket, out, sm);
}

// float-float values
template <int R, int NT, class X>
__device__ __forceinline__ bool dred_sum_ff(const X& x, FF (&v)[R], double* part, int nt, int tile, unsigned* ticket,
                                            double (&out)[R], DRedSmem<NT>& sm) {
  const int lane = x.tid() & 31, warp = x.tid() >> 5;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const FF a = ff_warp_sum(v[r]);
    if (lane == 0) sm.w[r][warp] = (double)a.hi + (double)a.lo;
  }
  double d[R];
#pragma unroll
  for (int r = 0; r < R; ++r) d[r] = 0.0;
  dred_warps<R, NT>(x, d, sm);
  return dred_finish<R, NT>(x, d, part, nt, tile, ticket, out, sm);
}

}  // namespace pfgb
