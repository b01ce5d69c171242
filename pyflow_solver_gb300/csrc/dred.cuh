// Deterministic binary64 sums over the tiles of one instance.
//
// Each CTA reduces its values with a fixed shuffle tree, writes the tile's
// partial to part[r * nt + tile], and the last CTA of the instance to arrive
// (an atomic ticket) adds the nt partials in tile order with a fixed tree as
// well.  The result depends only on the instance's values and its tiling, not
// on timing or on the other instances of a batch.  Binary32 products are exact
// in binary64, so a dot of binary32 vectors is a sum of exact terms.
#pragma once
#include <cuda_runtime.h>

namespace pfgb {

template <int NT>
struct DRedSmem {
  double w[4][NT / 32];
  int last;
};

// Sum of v over the CTA (fixed order); valid in thread 0.
template <int R, int NT>
__device__ __forceinline__ void dred_block(double (&v)[R], DRedSmem<NT>& sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    double x = v[r];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sm.w[r][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      double s = sm.w[r][0];
      for (int k = 1; k < NT / 32; ++k) s += sm.w[r][k];
      v[r] = s;
    }
  }
  __syncthreads();
}

// All threads of the CTA call this.  Returns true in every thread of the CTA
// that completes the instance's sums; out[] is then valid in thread 0.
template <int R, int NT>
__device__ __forceinline__ bool dred_sum(double (&v)[R], double* part, int nt, int tile, unsigned* ticket,
                                         double (&out)[R], DRedSmem<NT>& sm) {
  dred_block<R, NT>(v, sm);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int r = 0; r < R; ++r) part[(long)r * nt + tile] = v[r];
    __threadfence();
    sm.last = (atomicAdd(ticket, 1u) == (unsigned)(nt - 1)) ? 1 : 0;
  }
  __syncthreads();
  if (!sm.last) return false;
  __threadfence();
  double s[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    s[r] = 0.0;
    for (int k = threadIdx.x; k < nt; k += NT) s[r] += __ldcg(&part[(long)r * nt + k]);
  }
  dred_block<R, NT>(s, sm);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int r = 0; r < R; ++r) out[r] = s[r];
    *ticket = 0u;
  }
  return true;
}

}  // namespace pfgb

namespace pfgb {

// ---- float-float accumulation -------------------------------------------------
//
// Sums of binary32 products on the binary32 pipe: each product is split
// exactly into p + e (e = fma(a, b, -p)) and added into an unevaluated pair
// hi + lo with error-free transformations, about 44 significant bits -- the
// accuracy of a binary64 sum at a binary32 instruction cost (the binary64 pipe
// of this GPU issues at a small fraction of the binary32 rate).  The pairs are
// combined by a fixed shuffle tree, then each warp's pair is rounded to
// binary64 and the CTA partial is the binary64 sum of its warps in order.

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

// CTA sums of float-float values, then the instance's sum over tiles as dred_sum.
template <int R, int NT>
__device__ __forceinline__ bool dred_sum_ff(FF (&v)[R], double* part, int nt, int tile, unsigned* ticket,
                                            double (&out)[R], DRedSmem<NT>& sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    FF x = v[r];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      FF y;
      y.hi = __shfl_xor_sync(0xffffffffu, x.hi, o);
      y.lo = __shfl_xor_sync(0xffffffffu, x.lo, o);
      x = ff_merge(x, y);
    }
    if (lane == 0) sm.w[r][warp] = (double)x.hi + (double)x.lo;
  }
  __syncthreads();
  double d[R];
#pragma unroll
  for (int r = 0; r < R; ++r) d[r] = 0.0;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      double s = sm.w[r][0];
      for (int k = 1; k < NT / 32; ++k) s += sm.w[r][k];
      d[r] = s;
    }
  }
  __syncthreads();
  // d[] holds the CTA sums in thread 0: the rest is dred_sum without its block step
  if (threadIdx.x == 0) {
#pragma unroll
    for (int r = 0; r < R; ++r) part[(long)r * nt + tile] = d[r];
    __threadfence();
    sm.last = (atomicAdd(ticket, 1u) == (unsigned)(nt - 1)) ? 1 : 0;
  }
  __syncthreads();
  if (!sm.last) return false;
  __threadfence();
  double s[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    s[r] = 0.0;
    for (int k = threadIdx.x; k < nt; k += NT) s[r] += __ldcg(&part[(long)r * nt + k]);
  }
  dred_block<R, NT>(s, sm);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int r = 0; r < R; ++r) out[r] = s[r];
    *ticket = 0u;
  }
  return true;
}

}  // namespace pfgb
