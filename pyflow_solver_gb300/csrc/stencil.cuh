// Point-wise forms of the reference's array operators (binary64, reference
// evaluation order).  Arrays are interior fields of shape (ny, nx), row = y.
//
//   gradient_coherent     src/pyflow/numerics/core_ops_coherent.py:45-61
//   divergence_coherent   src/pyflow/numerics/core_ops_coherent.py:63-79
//   laplacian_coherent    src/pyflow/numerics/core_ops_coherent.py:81-84
//   divergence (central)  src/pyflow/numerics/fluid_ops.py:8-28
//   advect_quick          src/pyflow/numerics/operators/advection.py:45-84
//   advect_upwind         src/pyflow/numerics/operators/advection.py:17-43
//
// The reference's coherent divergence adds its x part to a zero field before
// the y part ((0 + x) + y); that differs from x + y only in the sign of a zero
// result, which never changes a value downstream (every consumer is a product,
// a difference, an exactly rounded sum or a comparison), so it is written x + y.
#pragma once
#include "icvt.cuh"
#include "common.cuh"

namespace pfgb {

struct Grid2 {
  int nx, ny;
  Spacing sx, sy;
};

// forward difference gradient, zero on the high boundary (V: any 2-D view)
template <class V>
__device__ __forceinline__ double grad_x(V p, int j, int i, const Grid2& g) {
  return (i < g.nx - 1) ? DIVH(SUB(p(j, i + 1), p(j, i)), g.sx) : 0.0;
}
template <class V>
__device__ __forceinline__ double grad_y(V p, int j, int i, const Grid2& g) {
  return (j < g.ny - 1) ? DIVH(SUB(p(j + 1, i), p(j, i)), g.sy) : 0.0;
}

// backward difference divergence, zero exterior flux on the low boundary
__device__ __forceinline__ double div_coherent_at(View2<const double> u, View2<const double> v,
                                                  int j, int i, const Grid2& g) {
  double xp = (i >= 1) ? DIVH(SUB(u(j, i), u(j, i - 1)), g.sx) : DIVH(u(j, 0), g.sx);
  double yp = (j >= 1) ? DIVH(SUB(v(j, i), v(j - 1, i)), g.sy) : DIVH(v(0, i), g.sy);
  return ADD(xp, yp);
}

// laplacian_coherent = divergence_coherent(gradient_coherent(p))
template <class V>
__device__ __forceinline__ double lap_coherent_at(V p, int j, int i, const Grid2& g) {
  double gxi = grad_x(p, j, i, g);
  double xp = (i >= 1) ? DIVH(SUB(gxi, grad_x(p, j, i - 1, g)), g.sx) : DIVH(gxi, g.sx);
  double gyj = grad_y(p, j, i, g);
  double yp = (j >= 1) ? DIVH(SUB(gyj, grad_y(p, j - 1, i, g)), g.sy) : DIVH(gyj, g.sy);
  return ADD(xp, yp);
}

// central divergence with one-sided edges; the last column of rows
// 1..ny-2 is left at zero exactly as the reference leaves it
__device__ __forceinline__ double div_central_at(View2<const double> u, View2<const double> v,
                                                 int j, int i, int nx, int ny, double dx, double dy) {
  const int L = nx - 1, T = ny - 1;
  const double dx2 = MUL(2.0, dx), dy2 = MUL(2.0, dy);
  if (j == 0 && i == 0) return ADD(DIV(SUB(u(0, 1), u(0, 0)), dx), DIV(SUB(v(1, 0), v(0, 0)), dy));
  if (j == 0 && i == L) return ADD(DIV(SUB(u(0, L), u(0, L - 1)), dx), DIV(SUB(v(1, L), v(0, L)), dy));
  if (j == T && i == 0) return ADD(DIV(SUB(u(T, 1), u(T, 0)), dx), DIV(SUB(v(T, 0), v(T - 1, 0)), dy));
  if (j == T && i == L) return ADD(DIV(SUB(u(T, L), u(T, L - 1)), dx), DIV(SUB(v(T, L), v(T - 1, L)), dy));
  if (j == 0) return ADD(DIV(SUB(u(0, i + 1), u(0, i - 1)), dx2), DIV(SUB(v(1, i), v(0, i)), dy));
  if (j == T) return ADD(DIV(SUB(u(T, i + 1), u(T, i - 1)), dx2), DIV(SUB(v(T, i), v(T - 1, i)), dy));
  if (i == 0) return ADD(DIV(SUB(u(j, 1), u(j, 0)), dx), DIV(SUB(v(j + 1, 0), v(j - 1, 0)), dy2));
  if (i == L) return 0.0;
  return ADD(DIV(SUB(u(j, i + 1), u(j, i - 1)), dx2), DIV(SUB(v(j + 1, i), v(j - 1, i)), dy2));
}

// The same with dx = dy = 1 (the step's continuity and safeguard norms): a
// quotient by 1 is the dividend and a quotient by 2 equals the product with
// 0.5 (both exact, or rounded alike when subnormal), so no division is issued;
// the product is an exponent decrement on the integer pipe wherever the result
// stays normal (half_exact).
template <class UV, class VV>
__device__ __forceinline__ double div_central_unit(UV u, VV v, int j, int i, int nx, int ny) {
  const int L = nx - 1, T = ny - 1;
  if (j == 0 && i == 0) return ADD(SUB(u(0, 1), u(0, 0)), SUB(v(1, 0), v(0, 0)));
  if (j == 0 && i == L) return ADD(SUB(u(0, L), u(0, L - 1)), SUB(v(1, L), v(0, L)));
  if (j == T && i == 0) return ADD(SUB(u(T, 1), u(T, 0)), SUB(v(T, 0), v(T - 1, 0)));
  if (j == T && i == L) return ADD(SUB(u(T, L), u(T, L - 1)), SUB(v(T, L), v(T - 1, L)));
  if (j == 0) return ADD(half_exact(SUB(u(0, i + 1), u(0, i - 1))), SUB(v(1, i), v(0, i)));
  if (j == T) return ADD(half_exact(SUB(u(T, i + 1), u(T, i - 1))), SUB(v(T, i), v(T - 1, i)));
  if (i == 0) return ADD(SUB(u(j, 1), u(j, 0)), half_exact(SUB(v(j + 1, 0), v(j - 1, 0))));
  if (i == L) return 0.0;
  return ADD(half_exact(SUB(u(j, i + 1), u(j, i - 1))), half_exact(SUB(v(j + 1, i), v(j - 1, i))));
}

// ((3/8)*a + (6/8)*b) - (1/8)*c
__device__ __forceinline__ double quick3(double a, double b, double c) {
  return SUB(ADD(MUL(0.375, a), MUL(0.75, b)), MUL(0.125, c));
}

__device__ __forceinline__ int clampi(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

// QUICK convective derivative of f at (j, i): edge padding by clamping indices
__device__ __forceinline__ double advect_quick_at(View2<const double> u, View2<const double> v,
                                                  View2<const double> f, int j, int i, const Grid2& g) {
  const int L = g.nx - 1, T = g.ny - 1;
  const double uc = u(j, i), vc = v(j, i);
  const double fm2 = f(j, clampi(i - 2, 0, L)), fm1 = f(j, clampi(i - 1, 0, L));
  const double f0 = f(j, i), fp1 = f(j, clampi(i + 1, 0, L));
  const double gm2 = f(clampi(j - 2, 0, T), i), gm1 = f(clampi(j - 1, 0, T), i);
  const double gp1 = f(clampi(j + 1, 0, T), i);
  double pe, pw, pn, ps;
  if (uc >= 0.0) { pe = quick3(fp1, f0, fm1); pw = quick3(f0, fm1, fm2); }
  else { pe = quick3(fm1, f0, fp1); pw = quick3(fm2, fm1, f0); }
  if (vc >= 0.0) { pn = quick3(gp1, f0, gm1); ps = quick3(f0, gm1, gm2); }
  else { pn = quick3(gm1, f0, gp1); ps = quick3(gm2, gm1, f0); }
  return ADD(DIVH(SUB(MUL(uc, pe), MUL(uc, pw)), g.sx), DIVH(SUB(MUL(vc, pn), MUL(vc, ps)), g.sy));
}

// first-order upwind convective derivative of f at (j, i)
__device__ __forceinline__ double advect_upwind_at(View2<const double> u, View2<const double> v,
                                                   View2<const double> f, int j, int i, const Grid2& g) {
  const int L = g.nx - 1, T = g.ny - 1;
  const double uc = u(j, i), vc = v(j, i), f0 = f(j, i);
  double fx, fy;
  if (uc > 0.0) fx = (i > 0) ? DIVH(SUB(f0, f(j, i - 1)), g.sx) : DIVH(SUB(f0, f0), g.sx);
  else fx = DIVH(SUB(f(j, (i + 1 <= L) ? i + 1 : i), f0), g.sx);
  if (vc > 0.0) fy = (j > 0) ? DIVH(SUB(f0, f(j - 1, i)), g.sy) : DIVH(SUB(f0, f0), g.sy);
  else fy = DIVH(SUB(f((j + 1 <= T) ? j + 1 : j, i), f0), g.sy);
  return ADD(MUL(uc, fx), MUL(vc, fy));
}

}  // namespace pfgb
