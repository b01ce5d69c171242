// Execution contexts of the mixed-precision phase functions, and the bounded
// grid barrier of the persistent solve.
//
// A phase function (one tile of one kernel of the V-cycle or the PCG) is
// written once against a context that supplies its thread index, its barrier
// and its global loads:
//   * CtaCtx   -- the tile is a whole 256-thread CTA of an ordinary launch;
//   * GroupCtx -- the tile is one of the four 256-thread groups of a
//     1024-thread CTA of the persistent kernel, synchronised by its own named
//     barrier; loads of arrays written earlier in the same launch go through
//     L2 (ld.global.cg), since the SM's L1 is not coherent with other SMs.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace pfgb {
namespace mixed {

struct CtaCtx {
  __device__ __forceinline__ int tid() const { return threadIdx.x; }
  __device__ __forceinline__ void sync() const { __syncthreads(); }
  template <typename T>
  __device__ __forceinline__ T ld(const T* p) const { return *p; }
  __device__ __forceinline__ View2<const double> view(const double* p, long ld) const {
    return View2<const double>{p, ld};
  }
};

struct GroupCtx {
  int g;    // group 0..3 of the CTA
  __device__ __forceinline__ int tid() const { return threadIdx.x & 255; }
  __device__ __forceinline__ void sync() const {
    asm volatile("bar.sync %0, 256;" ::"r"(g + 1) : "memory");
  }
  template <typename T>
  __device__ __forceinline__ T ld(const T* p) const { return __ldcg(p); }
  __device__ __forceinline__ View2Cg<double> view(const double* p, long ld) const { return View2Cg<double>{p, ld}; }
};

// Grid-wide barrier of a cooperative launch with a bounded wait.  Every CTA
// calls it the same number of times.  The arrival counter only grows: a CTA
// arriving as number a waits until the counter reaches the next multiple of
// the grid size (release on arrival, acquire on the polls, so the writes of
// every CTA before the barrier are visible to every CTA after it).  A CTA that
// waits longer than the limit (or finds the error flag set) marks the error
// and returns false; its caller leaves the kernel, and every other CTA fails
// its next barrier at once.  The counter is zeroed before each launch.
struct GridBar {
  unsigned count;
  unsigned pad0;
  int err;
  int pad1;
};

constexpr unsigned long long GRID_SPIN_LIMIT = 1ull << 22;

__device__ __forceinline__ bool grid_sync(GridBar* gb) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    if (*(volatile int*)&gb->err) {
      ok = 0;
    } else {
      const unsigned n = gridDim.x;
      unsigned arrived;
      asm volatile("atom.add.release.gpu.u32 %0, [%1], 1;" : "=r"(arrived) : "l"(&gb->count) : "memory");
      const unsigned target = (arrived / n + 1) * n;
      unsigned long long spins = 0;
      while (true) {
        unsigned cur;
        asm volatile("ld.acquire.gpu.u32 %0, [%1];" : "=r"(cur) : "l"(&gb->count) : "memory");
        if ((int)(cur - target) >= 0) break;
        if (++spins > GRID_SPIN_LIMIT || *(volatile int*)&gb->err) {
          atomicExch(&gb->err, 1);
          ok = 0;
          break;
        }
        __nanosleep(20);
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

}  // namespace mixed
}  // namespace pfgb
