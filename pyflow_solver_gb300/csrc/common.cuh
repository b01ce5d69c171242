// Shared device helpers for the PyFlow projection step on GB300 (sm_103a).
//
// Every binary64 operation that must reproduce the reference's NumPy
// arithmetic is written with the IEEE round-to-nearest intrinsics
// (__dadd_rn, __dsub_rn, __dmul_rn, __ddiv_rn), which are never contracted
// into FMAs, and the translation units are also compiled with -fmad=false.
#pragma once
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#include "idiv.cuh"

namespace pfgb {

__device__ __forceinline__ double ADD(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double SUB(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double MUL(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double DIV(double a, double b) { return __ddiv_rn(a, b); }

// -a (a sign flip: exact, and no binary64-pipe instruction)
__device__ __forceinline__ double neg_exact(double a) {
  return __hiloint2double(__double2hiint(a) ^ (int)0x80000000, __double2loint(a));
}

// Division by a grid spacing.  When the spacing is a power of two the quotient
// equals the product with its (exact) reciprocal for every operand, so the
// cheaper multiply is used; otherwise the integer-pipe division by an invariant
// divisor (idiv.cuh), which returns the IEEE quotient.
struct Spacing {
  double h;      // the spacing
  double rh;     // 1/h, exact when pow2
  int pow2;
  DivConst dc;   // valid (dc.ok) for positive normal spacings that are not powers of two
};

__device__ __forceinline__ double DIVH(double a, const Spacing& s) {
  if (s.pow2) return __dmul_rn(a, s.rh);
  if (s.dc.ok) return div_const(a, s.dc);
  return __ddiv_rn(a, s.h);
}

// Host-side preparation of a spacing.
inline Spacing spacing_for(double h) {
  Spacing s;
  s.h = h;
  s.pow2 = 0;
  s.rh = 0.0;
  int e;
  double m = std::frexp(h, &e);
  if (h > 0.0 && m == 0.5 && e - 1 >= -1022 && e - 1 <= 1022) {   // h = 2^(e-1), 1/h normal
    s.pow2 = 1;
    s.rh = std::ldexp(1.0, -(e - 1));
  }
  s.dc = make_divconst(h);
  return s;
}

// A 2-D row-major view: element (j, i) at p[j*ld + i].
template <typename T>
struct View2 {
  T* p;
  long ld;
  __device__ __forceinline__ T& operator()(int j, int i) const { return p[(long)j * ld + i]; }
};

// The same view with loads through L2 (ld.global.cg): for arrays that other
// SMs wrote earlier in the same launch.
template <typename T>
struct View2Cg {
  const T* p;
  long ld;
  __device__ __forceinline__ T operator()(int j, int i) const { return __ldcg(p + (long)j * ld + i); }
};

// Programmatic dependent launch, in two halves: pdl_launch lets the graph's
// next kernel start launching; pdl_wait waits until this kernel's predecessor
// has completed and its writes are visible.  Between the two a kernel reads only
// what no kernel writes (tile tables and instance descriptors, which the host
// writes before a launch), so those loads overlap the predecessor's tail.  Every
// kernel of a step graph begins with them (no-ops for a kernel that was not
// launched as a programmatic dependent).
__device__ __forceinline__ void pdl_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_enter() {
  pdl_launch();
  pdl_wait();
}

// A descriptor copied into shared memory by the CTA as 8-byte words (read-only
// path): called between pdl_launch and pdl_wait, the caller synchronises the CTA
// after pdl_wait.
template <typename T>
__device__ __forceinline__ void stage_desc(const T* src, T* dst) {
  static_assert(sizeof(T) % 8 == 0 && alignof(T) >= 8, "descriptor copied as 8-byte words");
  const unsigned long long* s = reinterpret_cast<const unsigned long long*>(src);
  unsigned long long* d = reinterpret_cast<unsigned long long*>(dst);
  for (int k = threadIdx.x; k < (int)(sizeof(T) / 8); k += blockDim.x) d[k] = __ldg(s + k);
}

// Ordered bit pattern of a non-negative double (NaN sorts above +inf), for
// exact max reductions with 64-bit integer atomics.
__device__ __forceinline__ unsigned long long abs_bits(double a) {
  return (unsigned long long)__double_as_longlong(a) & 0x7FFFFFFFFFFFFFFFull;
}

__device__ __forceinline__ int isfinite_d(double a) {
  return ((unsigned long long)__double_as_longlong(a) & 0x7FF0000000000000ull) != 0x7FF0000000000000ull;
}

// Python's min(a, b): returns b only when b < a (NaN-aware exactly like CPython).
__device__ __forceinline__ double py_min(double a, double b) { return (b < a) ? b : a; }
// Python's max(a, b): returns b only when b > a.
__device__ __forceinline__ double py_max(double a, double b) { return (b > a) ? b : a; }

}  // namespace pfgb
