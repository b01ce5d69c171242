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
