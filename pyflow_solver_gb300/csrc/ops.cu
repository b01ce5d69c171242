// Array operators of the reference as stand-alone device kernels, the pressure
// operators, and exactly rounded dot products / sums (see xacc.cuh).
#include <string>

#include "icvt.cuh"
#include "pfgb_internal.h"
#include "stencil.cuh"
#include "xacc.cuh"

namespace pfgb {

constexpr int OT = 256;

struct OpGeo {
  int nx, ny;
  Grid2 g;
  double dx, dy;     // raw spacings (central divergence divides by 2*dx etc.)
};

static Spacing spacing_of(double h) { return spacing_for(h); }

static OpGeo make_geo(int nx, int ny, double dx, double dy) {
  OpGeo G;
  G.nx = nx;
  G.ny = ny;
  G.g.nx = nx;
  G.g.ny = ny;
  G.g.sx = spacing_of(dx);
  G.g.sy = spacing_of(dy);
  G.dx = dx;
  G.dy = dy;
  return G;
}

__global__ void k_gradient(OpGeo G, const double* p, long ldp, double* gx, double* gy, long ldo) {
  int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (i >= G.nx || j >= G.ny) return;
  View2<const double> P{p, ldp};
  gx[(long)j * ldo + i] = grad_x(P, j, i, G.g);
  gy[(long)j * ldo + i] = grad_y(P, j, i, G.g);
}

__global__ void k_divergence(OpGeo G, const double* u, const double* v, long ldi, double* d, long ldo) {
  int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (i >= G.nx || j >= G.ny) return;
  View2<const double> U{u, ldi}, V{v, ldi};
  d[(long)j * ldo + i] = div_coherent_at(U, V, j, i, G.g);
}

__global__ void k_laplacian(OpGeo G, const double* p, long ldp, double* l, long ldo) {
  int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (i >= G.nx || j >= G.ny) return;
  View2<const double> P{p, ldp};
  l[(long)j * ldo + i] = lap_coherent_at(P, j, i, G.g);
}

__global__ void k_div_central(OpGeo G, const double* u, const double* v, long ldi, double* d, long ldo) {
  int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (i >= G.nx || j >= G.ny) return;
  View2<const double> U{u, ldi}, V{v, ldi};
  d[(long)j * ldo + i] = div_central_at(U, V, j, i, G.nx, G.ny, G.dx, G.dy);
}

__global__ void k_advect(OpGeo G, int scheme, const double* u, const double* v, const double* f, long ldi,
                         double* c, long ldo) {
  int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (i >= G.nx || j >= G.ny) return;
  View2<const double> U{u, ldi}, V{v, ldi}, F{f, ldi};
  c[(long)j * ldo + i] = (scheme == PFGB_SCHEME_QUICK) ? advect_quick_at(U, V, F, j, i, G.g)
                                                       : advect_upwind_at(U, V, F, j, i, G.g);
}

__global__ void k_apply_op(OpGeo G, int op, const double* x, double* y) {
  int i = blockIdx.x * 32 + (threadIdx.x & 31), j = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (i >= G.nx || j >= G.ny) return;
  View2<const double> X{x, G.nx};
  double val;
  if (op == PFGB_OP_NEG_LAPLACIAN_PINNED) {
    val = (i == 0 && j == 0) ? X(0, 0) : -lap_coherent_at(X, j, i, G.g);
  } else {
    bool ring = i == 0 || j == 0 || i == G.nx - 1 || j == G.ny - 1;
    val = ring ? X(j, i) : lap_coherent_at(X, j, i, G.g);
  }
  y[(long)j * G.nx + i] = val;
}

// out[i] = a[i] / d through the spacing division used by the stencils
// (method 0) or the hardware IEEE division (method 1).
__global__ void k_div_by(const double* a, double* out, long n, Spacing s, int method) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = method ? __ddiv_rn(a[i], s.h) : DIVH(a[i], s);
}

// ---- exactly rounded dot / sum over a contiguous vector --------------------
constexpr int XPT = 8;   // elements per thread

__global__ void __launch_bounds__(OT) k_xdot(const double* a, const double* b, long n, int mode, XASlot* slot) {
  __shared__ long long sacc[XA_DIGITS];
  __shared__ long long wred[(OT / 32) * XA_WLIMBS];
  __shared__ int ired[32];
  for (int k = threadIdx.x; k < XA_DIGITS; k += OT) sacc[k] = 0;
  long base = (long)blockIdx.x * OT * XPT;
  double va[XPT], vb[XPT];
  int top = INT_MIN;
#pragma unroll
  for (int k = 0; k < XPT; ++k) {
    long idx = base + (long)k * OT + threadIdx.x;
    va[k] = 0.0;
    vb[k] = 1.0;                  // a plain sum is the sum of the products with 1
    if (idx < n) {
      va[k] = a[idx];
      if (mode == 0) vb[k] = b[idx];
    }
    top = max(top, xa_prod_top(va[k], vb[k]));
  }
  top = xa_block_max(top, ired);
  const int k0 = xa_window_digit(top);
  XAcc x;
  x.clear();
#pragma unroll
  for (int k = 0; k < XPT; ++k) xa_acc_prod<false>(x, sacc, k0, va[k], vb[k]);
  const int anyslow = __syncthreads_or(x.slow);
  xa_acc_commit(slot, x, k0, sacc, anyslow, wred);
  XASlot* sl[1] = {slot};
  xa_finish(sl, 1, gridDim.x);
}

static int xreduce(const double* a, const double* b, long n, int mode, double* result, cudaStream_t s) {
  if (n < 0) return set_error(PFGB_EINVAL, "negative length");
  if (n == 0) {
    *result = 0.0;
    return PFGB_OK;
  }
  long nblocks = (n + (long)OT * XPT - 1) / ((long)OT * XPT);
  if (nblocks > 0x7fffffffL) return set_error(PFGB_EINVAL, "vector too long");
  XASlot* slot = nullptr;
  cudaError_t e = cudaMallocAsync(&slot, sizeof(XASlot), s);
  if (e != cudaSuccess) return set_error(PFGB_ENOMEM, "cudaMallocAsync of the reduction slot failed");
  cudaMemsetAsync(slot, 0, sizeof(XASlot), s);
  k_xdot<<<(unsigned)nblocks, OT, 0, s>>>(a, b, n, mode, slot);
  e = cudaGetLastError();
  double r = 0.0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&r, &slot->result, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(slot, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("exact reduction failed: ") + cudaGetErrorString(e));
  *result = r;
  return PFGB_OK;
}

// Exactly rounded a.b (mode 0) or sum(a) (mode 1) of device vectors, to the host (synchronises s).
int exact_reduce(const double* a, const double* b, long n, int mode, double* result, cudaStream_t s) {
  return xreduce(a, b, n, mode, result, s);
}

// ---- self-test of the integer-pipe conversions (icvt.cuh) -----------------------

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}

__device__ __forceinline__ bool same_f(float a, float b) {
  return (a != a && b != b) || __float_as_uint(a) == __float_as_uint(b);
}
__device__ __forceinline__ bool same_d(double a, double b) {
  return (a != a && b != b) || __double_as_longlong(a) == __double_as_longlong(b);
}

// sample k: a random 64-bit pattern; every fourth one has its exponent drawn near the
// binary32 range (normal, subnormal, overflow and rounding boundaries); k < 64: specials
__global__ void k_icvt_check(long n, unsigned long long* bad) {
  const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  uint64_t r = mix64((uint64_t)k + 0x9e3779b97f4a7c15ull);
  if ((k & 3) == 0) {
    const uint64_t e = 1023 - 160 + (mix64(r) % 300);       // 2^-160 .. 2^140
    r = (r & 0x800FFFFFFFFFFFFFull) | (e << 52);
    if ((k & 15) == 0) r &= ~0x000000000FFFFFFFull | (mix64(r) & 0x10000000ull);   // exact halfway / ties
  }
  if (k < 64) {
    const uint64_t sp[16] = {0ull, 0x8000000000000000ull, 0x7FF0000000000000ull, 0xFFF0000000000000ull,
                             0x7FF8000000000000ull, 0x0000000000000001ull, 0x0010000000000000ull,
                             0x0020000000000000ull, 0x47EFFFFFE0000000ull, 0x47EFFFFFF0000000ull,
                             0x47EFFFFFEFFFFFFFull, 0x3690000000000000ull, 0x36A0000000000000ull,
                             0x3680000000000000ull, 0x380FFFFFF0000000ull, 0x380FFFFFE0000000ull};
    r = sp[k & 15] ^ ((k >> 4) ? (1ull << 63) : 0ull);
  }
  const double d = __longlong_as_double((long long)r);
  unsigned long long miss = 0;
  if (!same_f(d2f_rn(d), __double2float_rn(d))) miss |= 1;
  const float f = __uint_as_float((uint32_t)r ^ (uint32_t)(r >> 32));
  if (!same_d(f2d(f), (double)f)) miss |= 2;
  if (!same_d(half_exact(d), __dmul_rn(d, 0.5))) miss |= 4;
  if (miss) atomicAdd(bad + (miss & 1 ? 0 : (miss & 2 ? 1 : 2)), 1ull);
}

int icvt_selftest(long n, cudaStream_t s, long long* mismatches) {
  unsigned long long* bad = nullptr;
  if (cudaMallocAsync(&bad, 3 * sizeof(unsigned long long), s) != cudaSuccess)
    return set_error(PFGB_ENOMEM, "cudaMallocAsync of the self-test counters failed");
  cudaMemsetAsync(bad, 0, 3 * sizeof(unsigned long long), s);
  if (n > 0) k_icvt_check<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, bad);
  unsigned long long h[3] = {0, 0, 0};
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, bad, sizeof(h), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(bad, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("conversion self-test: ") + cudaGetErrorString(e));
  for (int k = 0; k < 3; ++k) mismatches[k] = (long long)h[k];
  return PFGB_OK;
}

static int check_grid(int nx, int ny) {
  if (nx < 2 || ny < 2) return set_error(PFGB_EINVAL, "nx and ny must be >= 2");
  return PFGB_OK;
}

static int launch_status(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return PFGB_OK;
}

}  // namespace pfgb

using namespace pfgb;

static dim3 op_grid(int nx, int ny) { return dim3((nx + 31) / 32, (ny + 7) / 8); }

extern "C" int pfgb_gradient_coherent(const double* p, long ldp, double* gx, double* gy, long ldo, int nx, int ny,
                                      double dx, double dy, void* stream) {
  if (int rc = check_grid(nx, ny)) return rc;
  k_gradient<<<op_grid(nx, ny), OT, 0, (cudaStream_t)stream>>>(make_geo(nx, ny, dx, dy), p, ldp, gx, gy, ldo);
  return launch_status("gradient_coherent");
}

extern "C" int pfgb_divergence_coherent(const double* u, const double* v, long ldi, double* div, long ldo, int nx,
                                        int ny, double dx, double dy, void* stream) {
  if (int rc = check_grid(nx, ny)) return rc;
  k_divergence<<<op_grid(nx, ny), OT, 0, (cudaStream_t)stream>>>(make_geo(nx, ny, dx, dy), u, v, ldi, div, ldo);
  return launch_status("divergence_coherent");
}

extern "C" int pfgb_laplacian_coherent(const double* p, long ldp, double* lap, long ldo, int nx, int ny, double dx,
                                       double dy, void* stream) {
  if (int rc = check_grid(nx, ny)) return rc;
  k_laplacian<<<op_grid(nx, ny), OT, 0, (cudaStream_t)stream>>>(make_geo(nx, ny, dx, dy), p, ldp, lap, ldo);
  return launch_status("laplacian_coherent");
}

extern "C" int pfgb_divergence_central(const double* u, const double* v, long ldi, double* div, long ldo, int nx,
                                       int ny, double dx, double dy, void* stream) {
  if (int rc = check_grid(nx, ny)) return rc;
  k_div_central<<<op_grid(nx, ny), OT, 0, (cudaStream_t)stream>>>(make_geo(nx, ny, dx, dy), u, v, ldi, div, ldo);
  return launch_status("divergence_central");
}

extern "C" int pfgb_advect(int scheme, const double* u, const double* v, const double* f, long ldi, double* conv,
                           long ldo, int nx, int ny, double dx, double dy, void* stream) {
  if (int rc = check_grid(nx, ny)) return rc;
  if (scheme != PFGB_SCHEME_UPWIND && scheme != PFGB_SCHEME_QUICK) return set_error(PFGB_EINVAL, "unknown scheme");
  k_advect<<<op_grid(nx, ny), OT, 0, (cudaStream_t)stream>>>(make_geo(nx, ny, dx, dy), scheme, u, v, f, ldi, conv, ldo);
  return launch_status("advect");
}

extern "C" int pfgb_apply_operator(int op, const double* x, double* y, int nx, int ny, double dx, double dy,
                                   void* stream) {
  if (int rc = check_grid(nx, ny)) return rc;
  if (op != PFGB_OP_NEG_LAPLACIAN_PINNED && op != PFGB_OP_LAPLACIAN_DIRICHLET) return set_error(PFGB_EINVAL, "unknown operator");
  k_apply_op<<<op_grid(nx, ny), OT, 0, (cudaStream_t)stream>>>(make_geo(nx, ny, dx, dy), op, x, y);
  return launch_status("apply_operator");
}

extern "C" int pfgb_xdot(const double* a, const double* b, long n, double* result, void* stream) {
  return xreduce(a, b, n, 0, result, (cudaStream_t)stream);
}

extern "C" int pfgb_xsum(const double* a, long n, double* result, void* stream) {
  return xreduce(a, a, n, 1, result, (cudaStream_t)stream);
}

extern "C" int pfgb_div_by_constant(const double* a, double* out, long n, double d, int method, void* stream) {
  if (n < 0 || !(d > 0.0)) return set_error(PFGB_EINVAL, "n must be >= 0 and d > 0");
  if (n == 0) return PFGB_OK;
  long blocks = (n + OT - 1) / OT;
  if (blocks > 0x7fffffffL) return set_error(PFGB_EINVAL, "vector too long");
  k_div_by<<<(unsigned)blocks, OT, 0, (cudaStream_t)stream>>>(a, out, n, spacing_for(d), method);
  return launch_status("div_by_constant");
}

extern "C" int pfgb_selftest_conversions(long samples, void* stream, long long* mismatches) {
  if (!mismatches || samples < 0 || samples > (1L << 31)) return set_error(PFGB_EINVAL, "invalid self-test arguments");
  return icvt_selftest(samples, (cudaStream_t)stream, mismatches);
}
