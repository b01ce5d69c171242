// Plain binary64 projection step of the 2-D lid-driven cavity on one GPU.
//
// Kernel sequence of one step (reference: src/pyflow/solvers/solver.py:15-193,
// src/pyflow/solvers/pressure_solver.py:95-219, scipy.sparse.linalg.cg):
//
//   k_prestep      max|u|, max|v|, ||div_central(u,v;1,1)||^2        solver.py:25-26,45
//   k_dt           dt / CFL / divergence-trend safeguard (1 thread)    solver.py:27-62
//   k_predict      u* = u - dt*conv(u), v* likewise (QUICK / upwind)    solver.py:73-95
//   k_rhs          b = -div_c(u*,v*)/max(dt,1e-14), sum(b), ||div||^2  pressure_solver.py:116-126
//   k_cg_init      b -= mean(b); b[0] = 0; r = b; ||b||^2; r.z          pressure_solver.py:127-128
//   { k_cg_matvec  p = z + beta p; q = A p; p.q                         scipy cg loop
//     k_cg_update  x += alpha p; r -= alpha q; r.r; r.z } x maxiter
//   k_post_resid   ||b - A x||^2                                        interface.py:48-49
//   k_pin_correct  p = x - x[0]; u -= dt grad_c p; lid; sums (u-u_old)^2 pressure_solver.py:147-157, solver.py:104-109
//   k_post_diag    ||div_c||^2, ||A p - b||^2, ||div_central||^2         pressure_solver.py:165-178, solver.py:111
//   k_gather       one StepOut64 record for the host
//
// Every CG kernel returns at once when the device control block says the
// solve is done, so a fixed launch sequence reproduces scipy's early exit.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "graph.cuh"
#include "mixed.cuh"
#include "pfgb_internal.h"
#include "stencil.cuh"
#include "step64.cuh"

namespace pfgb {

constexpr int NT = 256;       // threads per CTA (1-D blocks)
constexpr int TX = 32;        // tile width (one warp per tile row)
constexpr int TY = 16;        // tile height of the CG kernels (2 rows per thread)
constexpr int RPT = TY / (NT / TX);   // rows per thread in the CG kernels (4)
constexpr int PB_Y = NT / TX;         // tile height of the per-cell kernels (8)

struct Geo64 {
  int nx, ny;
  long ld;            // pitch of the work vectors (doubles)
  long lds;           // pitch of the state arrays (nx + 2)
  Grid2 g;
  double invd;        // interior Jacobi entry 1/(2/dx^2 + 2/dy^2)
  int jacobi;
};

__device__ __forceinline__ double jacobi_apply(const Geo64& G, int j, int i, double r) {
  if (!G.jacobi) return r;
  bool ring = (i == 0) || (i == G.nx - 1) || (j == 0) || (j == G.ny - 1);
  return ring ? r : MUL(G.invd, r);
}

// ---------------------------------------------------------------------------
// Reduction tail shared by the kernels: one slot per call.
__device__ __forceinline__ void reduce_terms(XASlot* slot, const XTerm* t, int nt, unsigned fl,
                                             long long* sacc, long long* wred, int* ired) {
  int top = INT_MIN;
  for (int k = 0; k < nt; ++k) top = max(top, t[k].top);
  top = xa_block_max(top, ired);
  XCtx c;
  c.clear();
  c.flags = fl;
  c.k0 = xa_window_digit(top);
  for (int k = 0; k < nt; ++k) c.add(sacc, t[k]);
  int anyslow = __syncthreads_or(c.slow);
  xa_cta_commit(slot, c.pos, c.neg, c.k0, sacc, anyslow, c.flags, wred);
}

__device__ __forceinline__ void zero_sacc(long long* sacc) {
  for (int k = threadIdx.x; k < XA_DIGITS; k += blockDim.x) sacc[k] = 0;
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NT) k_prestep(Geo64 G, const double* __restrict__ u, const double* __restrict__ v,
                                                 XASlot* slots, Ctrl64* ctrl) {
  __shared__ long long sacc[XA_DIGITS];
  __shared__ long long wred[(NT / 32) * XA_WLIMBS];
  __shared__ int ired[32];
  zero_sacc(sacc);
  const int i = blockIdx.x * TX + (threadIdx.x & 31);
  const int j = blockIdx.y * PB_Y + (threadIdx.x >> 5);
  View2<const double> U{u, G.lds}, V{v, G.lds};
  XTerm t;
  xa_zero(t);
  unsigned fl = 0u;
  unsigned long long ub = 0ull, vb = 0ull;
  if (i < G.nx && j < G.ny) {
    ub = abs_bits(U(j, i));
    vb = abs_bits(V(j, i));
    double d = div_central_at(U, V, j, i, G.nx, G.ny, 1.0, 1.0);
    xa_term_prod(d, d, t, fl);
  }
  for (int o = 16; o > 0; o >>= 1) {
    ub = max(ub, __shfl_xor_sync(0xffffffffu, ub, o));
    vb = max(vb, __shfl_xor_sync(0xffffffffu, vb, o));
  }
  if ((threadIdx.x & 31) == 0) {
    if (ub) atomicMax(&ctrl->umax_bits, ub);
    if (vb) atomicMax(&ctrl->vmax_bits, vb);
  }
  reduce_terms(&slots[S_DIVC_BEFORE], &t, 1, fl, sacc, wred, ired);
  XASlot* sl[1] = {&slots[S_DIVC_BEFORE]};
  if (xa_finish(sl, 1, gridDim.x * gridDim.y) && threadIdx.x == 0) {
    double um = __longlong_as_double((long long)*(volatile unsigned long long*)&ctrl->umax_bits);
    double vm = __longlong_as_double((long long)*(volatile unsigned long long*)&ctrl->vmax_bits);
    ctrl->umax = ADD(um, 1e-12);
    ctrl->vmax = ADD(vm, 1e-12);
    ctrl->umax_bits = 0ull;
    ctrl->vmax_bits = 0ull;
    ctrl->div_before = __dsqrt_rn(slots[S_DIVC_BEFORE].result);
  }
}

// dt selection, exactly the Python float sequence of solver.py:25-62.
struct DtArgs {
  double dx, dy, cfl_target, growth, nu;
};

__global__ void k_dt(DtArgs a, const StepIn* __restrict__ in_d, Ctrl64* ctrl) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const StepIn in = *in_d;
  const double umax = ctrl->umax, vmax = ctrl->vmax;
  const double dt_cfl_u = DIV(MUL(a.cfl_target, a.dx), umax);
  const double dt_cfl_v = DIV(MUL(a.cfl_target, a.dy), vmax);
  const double dt_cfl = py_min(dt_cfl_u, dt_cfl_v);
  const double dt_diff = DIV(MUL(0.25, py_min(MUL(a.dx, a.dx), MUL(a.dy, a.dy))), py_max(a.nu, 1e-12));
  const double dt_cand = py_min(dt_cfl, dt_diff);
  const double lim = MUL(in.dt_prev, a.growth);
  double dt = (dt_cand > lim) ? lim : dt_cand;
  // history: previous entries then the new baseline, keep the last five
  double h[6];
  int n = in.hist_len;
  for (int k = 0; k < n; ++k) h[k] = in.hist[k];
  h[n++] = ctrl->div_before;
  int safeguard = 0;
  if (n >= 3) {
    double x = h[n - 3], y = h[n - 2], z = h[n - 1];
    if (x > 0.0 && y > MUL(x, 1.01) && z > MUL(y, 1.01)) {
      dt = MUL(dt, 0.5);
      safeguard = 1;
    }
  }
  ctrl->dt = dt;
  ctrl->safeguard = safeguard;
  ctrl->cfl = py_max(DIV(MUL(umax, dt), a.dx), DIV(MUL(vmax, dt), a.dy));
  ctrl->dtm = py_max(dt, 1e-14);
}

// dt given by the caller of a stand-alone projection
__global__ void k_set_dt(double dt, Ctrl64* ctrl) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  ctrl->dt = dt;
  ctrl->dtm = py_max(dt, 1e-14);
  ctrl->safeguard = 0;
}

// predictor: u* = u - dt*conv_u(u,v), v* likewise (solver.py:73-95)
__global__ void __launch_bounds__(NT) k_predict(Geo64 G, const double* __restrict__ u, const double* __restrict__ v,
                                                 double* __restrict__ us, double* __restrict__ vs, int scheme,
                                                 const Ctrl64* __restrict__ ctrl) {
  const int i = blockIdx.x * TX + (threadIdx.x & 31);
  const int j = blockIdx.y * PB_Y + (threadIdx.x >> 5);
  if (i >= G.nx || j >= G.ny) return;
  View2<const double> U{u, G.lds}, V{v, G.lds};
  const double dt = ctrl->dt;
  double u0 = U(j, i), v0 = V(j, i), un, vn;
  if (scheme == 2) {            // advection disabled: u* = u_old
    un = u0; vn = v0;
  } else if (scheme == 1) {     // QUICK
    un = SUB(u0, MUL(dt, advect_quick_at(U, V, U, j, i, G.g)));
    vn = SUB(v0, MUL(dt, advect_quick_at(U, V, V, j, i, G.g)));
  } else {                      // upwind
    un = SUB(u0, MUL(dt, advect_upwind_at(U, V, U, j, i, G.g)));
    vn = SUB(v0, MUL(dt, advect_upwind_at(U, V, V, j, i, G.g)));
  }
  us[(long)j * G.ld + i] = un;
  vs[(long)j * G.ld + i] = vn;
}

// RHS: b = -div_c(u*,v*)/max(dt,1e-14); sum(b); ||div_c(u*,v*)||^2
__global__ void __launch_bounds__(NT) k_rhs(Geo64 G, const double* __restrict__ us, const double* __restrict__ vs,
                                             long usld, double* __restrict__ b, XASlot* slots,
                                             const Ctrl64* __restrict__ ctrl) {
  __shared__ long long sacc0[XA_DIGITS], sacc1[XA_DIGITS];
  __shared__ long long wred[(NT / 32) * XA_WLIMBS];
  __shared__ int ired[32];
  zero_sacc(sacc0);
  zero_sacc(sacc1);
  const int i = blockIdx.x * TX + (threadIdx.x & 31);
  const int j = blockIdx.y * PB_Y + (threadIdx.x >> 5);
  XTerm t0, t1;
  xa_zero(t0);
  xa_zero(t1);
  unsigned f0 = 0u, f1 = 0u;
  if (i < G.nx && j < G.ny) {
    View2<const double> US{us, usld}, VS{vs, usld};
    double d = div_coherent_at(US, VS, j, i, G.g);
    double bv = DIV(-d, ctrl->dtm);
    b[(long)j * G.ld + i] = bv;
    xa_term_val(bv, t0, f0);
    xa_term_prod(d, d, t1, f1);
  }
  reduce_terms(&slots[S_BSUM], &t0, 1, f0, sacc0, wred, ired);
  reduce_terms(&slots[S_DIVSTAR], &t1, 1, f1, sacc1, wred, ired);
  XASlot* sl[2] = {&slots[S_BSUM], &slots[S_DIVSTAR]};
  xa_finish(sl, 2, gridDim.x * gridDim.y);
}

struct CGArgs {
  double rtol;
  int maxiter;
  double n_cells;     // N as a double (exact)
};

// adjust = 1 (projection): b -= mean(b); b[0] = 0.  Then r = b; x = 0;
// ||b||^2; r.(M r).  adjust = 0 (operator interface): b is used as given.
__global__ void __launch_bounds__(NT) k_cg_init(Geo64 G, CGArgs A, int adjust, double* __restrict__ b,
                                                 double* __restrict__ r, double* __restrict__ x, XASlot* slots,
                                                 Ctrl64* ctrl, cudaGraphConditionalHandle cond, int use_cond) {
  __shared__ long long sacc0[XA_DIGITS], sacc1[XA_DIGITS];
  __shared__ long long wred[(NT / 32) * XA_WLIMBS];
  __shared__ int ired[32];
  zero_sacc(sacc0);
  zero_sacc(sacc1);
  const int i = blockIdx.x * TX + (threadIdx.x & 31);
  const int j = blockIdx.y * PB_Y + (threadIdx.x >> 5);
  const double mean = adjust ? DIV(slots[S_BSUM].result, A.n_cells) : 0.0;
  XTerm t0, t1;
  xa_zero(t0);
  xa_zero(t1);
  unsigned f0 = 0u, f1 = 0u;
  if (i < G.nx && j < G.ny) {
    long o = (long)j * G.ld + i;
    double bv = b[o];
    if (adjust) {
      bv = SUB(bv, mean);
      if (i == 0 && j == 0) bv = 0.0;
      b[o] = bv;
    }
    r[o] = bv;
    x[o] = 0.0;
    xa_term_prod(bv, bv, t0, f0);
    xa_term_prod(bv, jacobi_apply(G, j, i, bv), t1, f1);
  }
  reduce_terms(&slots[S_BB], &t0, 1, f0, sacc0, wred, ired);
  reduce_terms(&slots[S_RZ0], &t1, 1, f1, sacc1, wred, ired);
  XASlot* sl[2] = {&slots[S_BB], &slots[S_RZ0]};
  if (xa_finish(sl, 2, gridDim.x * gridDim.y) && threadIdx.x == 0) {
    double bb = slots[S_BB].result;
    double bnrm2 = __dsqrt_rn(bb);
    ctrl->mean = mean;
    ctrl->bnrm2 = bnrm2;
    ctrl->atol = py_max(0.0, MUL(A.rtol, bnrm2));
    ctrl->iter = 0;
    ctrl->info = 0;
    ctrl->zero_rhs = 0;
    ctrl->nan_flag = 0u;
    ctrl->rr = bb;
    ctrl->rho = slots[S_RZ0].result;
    ctrl->rho_prev = 0.0;
    ctrl->pq = 0.0;
    if (bnrm2 == 0.0) {              // scipy: return b, 0
      ctrl->done = 1;
      ctrl->zero_rhs = 1;
    } else if (A.maxiter <= 0) {     // empty loop: info = maxiter = 0
      ctrl->done = 1;
    } else if (__dsqrt_rn(bb) < ctrl->atol) {
      ctrl->done = 1;
    } else {
      ctrl->done = 0;
    }
    if (use_cond) cudaGraphSetConditional(cond, ctrl->done ? 0u : 1u);
  }
}

// p_new = z + beta*p_old (p_new = z at k = 0); q = A p_new; p_new.q
// OP 0: A = -lap_c with row 0 = identity (normal projection);
// OP 1: A = lap_c with identity rows on the boundary ring (manufactured mode).
// The iteration index k is read from the control block and selects the
// ping-pong buffers: iteration k reads p[k & 1] and writes p[(k + 1) & 1].
template <int OP>
__global__ void __launch_bounds__(NT) k_cg_matvec(Geo64 G, const double* __restrict__ r, double* p0, double* p1,
                                                   double* __restrict__ q, XASlot* slots, Ctrl64* ctrl) {
  if (*(volatile int*)&ctrl->done) return;
  const int k = *(volatile int*)&ctrl->iter;
  const double* __restrict__ pold = (k & 1) ? p1 : p0;
  double* __restrict__ pnew = (k & 1) ? p0 : p1;
  __shared__ double pn[TY + 2][TX + 2];
  __shared__ double gxs[TY][TX + 1];
  __shared__ double gys[TY + 1][TX];
  __shared__ long long sacc[XA_DIGITS];
  __shared__ long long wred[(NT / 32) * XA_WLIMBS];
  __shared__ int ired[32];
  zero_sacc(sacc);
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const double beta = (k > 0) ? ctrl->beta : 0.0;
  for (int idx = threadIdx.x; idx < (TY + 2) * (TX + 2); idx += NT) {
    int jj = idx / (TX + 2) - 1, ii = idx % (TX + 2) - 1;
    int gj = j0 + jj, gi = i0 + ii;
    bool corner = (jj < 0 || jj >= TY) && (ii < 0 || ii >= TX);
    double val = 0.0;
    if (!corner && gj >= 0 && gj < G.ny && gi >= 0 && gi < G.nx) {
      long o = (long)gj * G.ld + gi;
      double z = jacobi_apply(G, gj, gi, r[o]);
      val = (k == 0) ? z : ADD(MUL(pold[o], beta), z);
    }
    pn[jj + 1][ii + 1] = val;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < TY * (TX + 1); idx += NT) {
    int jj = idx / (TX + 1), ii = idx % (TX + 1) - 1;
    int gj = j0 + jj, gi = i0 + ii;
    double gv = 0.0;
    if (gj < G.ny && gi >= 0 && gi < G.nx - 1) gv = DIVH(SUB(pn[jj + 1][ii + 2], pn[jj + 1][ii + 1]), G.g.sx);
    gxs[jj][ii + 1] = gv;
  }
  for (int idx = threadIdx.x; idx < (TY + 1) * TX; idx += NT) {
    int jj = idx / TX - 1, ii = idx % TX;
    int gj = j0 + jj, gi = i0 + ii;
    double gv = 0.0;
    if (gi < G.nx && gj >= 0 && gj < G.ny - 1) gv = DIVH(SUB(pn[jj + 2][ii + 1], pn[jj + 1][ii + 1]), G.g.sy);
    gys[jj + 1][ii] = gv;
  }
  __syncthreads();
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  XTerm t[RPT];
  unsigned fl = 0u;
#pragma unroll
  for (int rr = 0; rr < RPT; ++rr) {
    xa_zero(t[rr]);
    int jj = ty + rr * PB_Y;
    int gj = j0 + jj, gi = i0 + tx;
    if (gj < G.ny && gi < G.nx) {
      double gxi = gxs[jj][tx + 1];
      double xp = (gi >= 1) ? DIVH(SUB(gxi, gxs[jj][tx]), G.g.sx) : DIVH(gxi, G.g.sx);
      double gyj = gys[jj + 1][tx];
      double yp = (gj >= 1) ? DIVH(SUB(gyj, gys[jj][tx]), G.g.sy) : DIVH(gyj, G.g.sy);
      double pv = pn[jj + 1][tx + 1];
      double qv;
      if (OP == 0) qv = (gi == 0 && gj == 0) ? pv : -ADD(xp, yp);
      else qv = (gi == 0 || gj == 0 || gi == G.nx - 1 || gj == G.ny - 1) ? pv : ADD(xp, yp);
      long o = (long)gj * G.ld + gi;
      q[o] = qv;
      pnew[o] = pv;
      xa_term_prod(pv, qv, t[rr], fl);
    }
  }
  reduce_terms(&slots[S_PQ], t, RPT, fl, sacc, wred, ired);
  XASlot* sl[1] = {&slots[S_PQ]};
  if (xa_finish(sl, 1, gridDim.x * gridDim.y) && threadIdx.x == 0) {
    const double pq = slots[S_PQ].result;
    ctrl->pq = pq;
    ctrl->alpha = DIV(ctrl->rho, pq);
  }
}

// x += alpha p; r -= alpha q; r.r; r.(M r)
__global__ void __launch_bounds__(NT) k_cg_update(Geo64 G, CGArgs A, const double* p0, const double* p1,
                                                   const double* __restrict__ q, double* __restrict__ x,
                                                   double* __restrict__ r, XASlot* slots, Ctrl64* ctrl,
                                                   cudaGraphConditionalHandle cond, int use_cond) {
  if (*(volatile int*)&ctrl->done) return;
  const int k = *(volatile int*)&ctrl->iter;
  const double* __restrict__ p = (k & 1) ? p0 : p1;    // the buffer this iteration's matvec wrote
  __shared__ long long sacc0[XA_DIGITS], sacc1[XA_DIGITS];
  __shared__ long long wred[(NT / 32) * XA_WLIMBS];
  __shared__ int ired[32];
  zero_sacc(sacc0);
  zero_sacc(sacc1);
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const double alpha = ctrl->alpha;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  XTerm trr[RPT], trz[RPT];
  unsigned f0 = 0u, f1 = 0u;
#pragma unroll
  for (int rr = 0; rr < RPT; ++rr) {
    xa_zero(trr[rr]);
    xa_zero(trz[rr]);
    int gj = j0 + ty + rr * PB_Y, gi = i0 + tx;
    if (gj < G.ny && gi < G.nx) {
      long o = (long)gj * G.ld + gi;
      double xv = ADD(x[o], MUL(alpha, p[o]));
      double rv = SUB(r[o], MUL(alpha, q[o]));
      x[o] = xv;
      r[o] = rv;
      xa_term_prod(rv, rv, trr[rr], f0);
      xa_term_prod(rv, jacobi_apply(G, gj, gi, rv), trz[rr], f1);
    }
  }
  reduce_terms(&slots[S_RR], trr, RPT, f0, sacc0, wred, ired);
  reduce_terms(&slots[S_RZ], trz, RPT, f1, sacc1, wred, ired);
  XASlot* sl[2] = {&slots[S_RR], &slots[S_RZ]};
  if (xa_finish(sl, 2, gridDim.x * gridDim.y) && threadIdx.x == 0) {
    double rr = slots[S_RR].result;
    ctrl->rr = rr;
    ctrl->rho_prev = ctrl->rho;
    ctrl->rho = slots[S_RZ].result;
    ctrl->beta = DIV(ctrl->rho, ctrl->rho_prev);
    int it = k + 1;
    ctrl->iter = it;
    if (it >= A.maxiter) {
      ctrl->done = 1;
      ctrl->info = A.maxiter;
    } else if (__dsqrt_rn(rr) < ctrl->atol) {
      ctrl->done = 1;
      ctrl->info = 0;
    }
    if (use_cond && ctrl->done) cudaGraphSetConditional(cond, 0u);
  }
}

// The pressure operators at one cell.
template <int OP>
__device__ __forceinline__ double apply_A(View2<const double> X, int j, int i, const Grid2& g) {
  if (OP == 0) {
    if (i == 0 && j == 0) return X(0, 0);
    return -lap_coherent_at(X, j, i, g);
  }
  if (i == 0 || j == 0 || i == g.nx - 1 || j == g.ny - 1) return X(j, i);
  return lap_coherent_at(X, j, i, g);
}

// ||b - A x||^2 (the true residual of interface.solve)
template <int OP>
__global__ void __launch_bounds__(NT) k_post_resid(Geo64 G, const double* __restrict__ b, const double* __restrict__ x,
                                                    XASlot* slots) {
  __shared__ long long sacc[XA_DIGITS];
  __shared__ long long wred[(NT / 32) * XA_WLIMBS];
  __shared__ int ired[32];
  zero_sacc(sacc);
  const int i = blockIdx.x * TX + (threadIdx.x & 31);
  const int j = blockIdx.y * PB_Y + (threadIdx.x >> 5);
  XTerm t;
  xa_zero(t);
  unsigned fl = 0u;
  if (i < G.nx && j < G.ny) {
    View2<const double> X{x, G.ld};
    double rv = SUB(b[(long)j * G.ld + i], apply_A<OP>(X, j, i, G.g));
    xa_term_prod(rv, rv, t, fl);
  }
  reduce_terms(&slots[S_RES], &t, 1, fl, sacc, wred, ired);
  XASlot* sl[1] = {&slots[S_RES]};
  xa_finish(sl, 1, gridDim.x * gridDim.y);
}

struct LidArgs {
  int has_lid;
  double lid;
};

// p = x - x[0] into the state; u = u* - dt*gx(p).
// mode 0 (full step): u* lives in us/vs (pitch usld) and keeps the pre-lid
//   corrected velocity for the divergence diagnostic; the state gets the lid
//   on its top interior row and the sums of (u-u_old)^2 are formed.
// mode 1 (projection only): us/vs are the state's own u/v, corrected in place.
__global__ void __launch_bounds__(NT) k_pin_correct(Geo64 G, LidArgs L, int mode, const double* __restrict__ x,
                                                     double* us, double* vs, long usld, double* u, double* v,
                                                     double* __restrict__ p, XASlot* slots, Ctrl64* ctrl) {
  __shared__ long long sacc0[XA_DIGITS], sacc1[XA_DIGITS];
  __shared__ long long wred[(NT / 32) * XA_WLIMBS];
  __shared__ int ired[32];
  zero_sacc(sacc0);
  zero_sacc(sacc1);
  const int i = blockIdx.x * TX + (threadIdx.x & 31);
  const int j = blockIdx.y * PB_Y + (threadIdx.x >> 5);
  XTerm t0, t1;
  xa_zero(t0);
  xa_zero(t1);
  unsigned f0 = 0u, f1 = 0u;
  int bad = 0;
  if (i < G.nx && j < G.ny) {
    const double dt = ctrl->dt;
    const double x0 = x[0];
    View2<const double> X{x, G.ld};
    const double pv = SUB(X(j, i), x0);
    const double gx = (i < G.nx - 1) ? DIVH(SUB(SUB(X(j, i + 1), x0), pv), G.g.sx) : 0.0;
    const double gy = (j < G.ny - 1) ? DIVH(SUB(SUB(X(j + 1, i), x0), pv), G.g.sy) : 0.0;
    long o = (long)j * usld + i;
    long os = (long)j * G.lds + i;
    const double uc = SUB(us[o], MUL(dt, gx));
    const double vc = SUB(vs[o], MUL(dt, gy));
    us[o] = uc;
    vs[o] = vc;
    p[os] = pv;
    if (mode == 0) {
      const double uf = (L.has_lid && j == G.ny - 1) ? L.lid : uc;
      const double du = SUB(uf, u[os]);
      const double dv = SUB(vc, v[os]);
      u[os] = uf;
      v[os] = vc;
      xa_term_val(MUL(du, du), t0, f0);
      xa_term_val(MUL(dv, dv), t1, f1);
      bad = !(isfinite_d(uf) && isfinite_d(vc) && isfinite_d(pv));
    } else {
      bad = !(isfinite_d(uc) && isfinite_d(vc) && isfinite_d(pv));
    }
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&ctrl->nan_flag, 1u);
  reduce_terms(&slots[S_RU], &t0, 1, f0, sacc0, wred, ired);
  reduce_terms(&slots[S_RV], &t1, 1, f1, sacc1, wred, ired);
  XASlot* sl[2] = {&slots[S_RU], &slots[S_RV]};
  xa_finish(sl, 2, gridDim.x * gridDim.y);
}

// ||div_c(u_corr)||^2, ||A p - b||^2, ||div_central(u,v;1,1)||^2
__global__ void __launch_bounds__(NT) k_post_diag(Geo64 G, const double* __restrict__ us, const double* __restrict__ vs,
                                                   long usld, const double* __restrict__ b, const double* __restrict__ u,
                                                   const double* __restrict__ v, const double* __restrict__ p,
                                                   XASlot* slots) {
  __shared__ long long sacc0[XA_DIGITS], sacc1[XA_DIGITS], sacc2[XA_DIGITS];
  __shared__ long long wred[(NT / 32) * XA_WLIMBS];
  __shared__ int ired[32];
  zero_sacc(sacc0);
  zero_sacc(sacc1);
  zero_sacc(sacc2);
  const int i = blockIdx.x * TX + (threadIdx.x & 31);
  const int j = blockIdx.y * PB_Y + (threadIdx.x >> 5);
  XTerm t0, t1, t2;
  xa_zero(t0);
  xa_zero(t1);
  xa_zero(t2);
  unsigned f0 = 0u, f1 = 0u, f2 = 0u;
  if (i < G.nx && j < G.ny) {
    View2<const double> US{us, usld}, VS{vs, usld};
    View2<const double> U{u, G.lds}, V{v, G.lds}, P{p, G.lds};
    double d = div_coherent_at(US, VS, j, i, G.g);
    xa_term_prod(d, d, t0, f0);
    double lr = SUB(apply_A<0>(P, j, i, G.g), b[(long)j * G.ld + i]);
    xa_term_prod(lr, lr, t1, f1);
    double c = div_central_at(U, V, j, i, G.nx, G.ny, 1.0, 1.0);
    xa_term_prod(c, c, t2, f2);
  }
  reduce_terms(&slots[S_DIVAFTER], &t0, 1, f0, sacc0, wred, ired);
  reduce_terms(&slots[S_LINRES], &t1, 1, f1, sacc1, wred, ired);
  reduce_terms(&slots[S_CONT], &t2, 1, f2, sacc2, wred, ired);
  XASlot* sl[3] = {&slots[S_DIVAFTER], &slots[S_LINRES], &slots[S_CONT]};
  xa_finish(sl, 3, gridDim.x * gridDim.y);
}

__global__ void k_gather(const XASlot* slots, const Ctrl64* ctrl, StepOut64* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  out->umax = ctrl->umax;
  out->vmax = ctrl->vmax;
  out->div_before = ctrl->div_before;
  out->dt = ctrl->dt;
  out->cfl = ctrl->cfl;
  out->safeguard = ctrl->safeguard;
  out->cg_iters = ctrl->zero_rhs ? 0 : ctrl->iter;
  out->cg_info = ctrl->info;
  out->nan_flag = (int)ctrl->nan_flag;
  out->divstar2 = slots[S_DIVSTAR].result;
  out->bnrm2 = ctrl->bnrm2;
  out->res2 = slots[S_RES].result;
  out->ru2 = slots[S_RU].result;
  out->rv2 = slots[S_RV].result;
  out->divafter2 = slots[S_DIVAFTER].result;
  out->linres2 = slots[S_LINRES].result;
  out->cont2 = slots[S_CONT].result;
  unsigned f = 0u;
  for (int s = 0; s < S_COUNT; ++s) f |= slots[s].result_flags;
  out->flags_or = f;
  out->refine_passes = ctrl->refine_passes;
}

// ---------------------------------------------------------------------------
// Host driver of one instance.

static long round_up(long a, long m) { return (a + m - 1) / m * m; }

static Spacing make_spacing(double h) { return spacing_for(h); }

struct Instance64 {
  pfgb_params P;
  Geo64 G;
  CGArgs A;
  DtArgs D;
  LidArgs L;
  char* ws = nullptr;
  double *us, *vs, *b, *x, *r, *p[2], *q;
  XASlot* slots;
  Ctrl64* ctrl;
  StepIn* in_d;
  StepIn* in_h = nullptr;     // pinned staging of the per-step inputs
  StepOut64* out_d;
  StepOut64* out_h = nullptr;
  // mixed-precision pressure solve (precision 1)
  mixed::Solver* mix = nullptr;
  // the whole step as one CUDA graph (CG loop = WHILE conditional node)
  int use_graph = 1;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const double* g_u = nullptr;
  const double* g_v = nullptr;
  const double* g_p = nullptr;
  // optional per-launch timing of k_cg_matvec (benchmark roofline)
  int profiling = 0;
  std::vector<cudaEvent_t> ev;
  int ev_used = 0;
};

int instance64_create(const pfgb_params* prm, Instance64** out) {
  if (prm->nx < 2 || prm->ny < 2) return set_error(PFGB_EINVAL, "nx and ny must be >= 2 (the reference's central divergence indexes two columns and rows)");
  if (prm->nx > (1 << 20) || prm->ny > (1 << 20)) return set_error(PFGB_EINVAL, "grid side above 2^20");
  if (!(prm->dx > 0.0) || !(prm->dy > 0.0)) return set_error(PFGB_EINVAL, "dx and dy must be positive");
  Instance64* I = new Instance64();
  I->P = *prm;
  Geo64& G = I->G;
  G.nx = prm->nx;
  G.ny = prm->ny;
  G.ld = round_up(prm->nx, 32);
  G.lds = prm->nx + 2;
  G.g.nx = prm->nx;
  G.g.ny = prm->ny;
  G.g.sx = make_spacing(prm->dx);
  G.g.sy = make_spacing(prm->dy);
  G.invd = prm->jacobi_interior;
  G.jacobi = prm->enable_jacobi;
  I->A.rtol = prm->lin_tol;
  I->A.maxiter = prm->lin_maxiter;
  I->A.n_cells = (double)prm->nx * (double)prm->ny;
  I->D.dx = prm->dx;
  I->D.dy = prm->dy;
  I->D.cfl_target = prm->cfl_target;
  I->D.growth = prm->cfl_growth;
  I->D.nu = prm->nu;
  I->L.has_lid = prm->has_lid;
  I->L.lid = prm->lid_velocity;
  size_t vec = (size_t)G.ld * G.ny * sizeof(double);
  size_t bytes = 8 * vec + S_COUNT * sizeof(XASlot) + sizeof(Ctrl64) + sizeof(StepIn) + sizeof(StepOut64) + 2048;
  if (cudaMalloc(&I->ws, bytes) != cudaSuccess) {
    delete I;
    return set_error(PFGB_ECUDA, "cudaMalloc of the workspace failed");
  }
  if (cudaMemset(I->ws, 0, bytes) != cudaSuccess) {
    cudaFree(I->ws);
    delete I;
    return set_error(PFGB_ECUDA, "cudaMemset of the workspace failed");
  }
  char* c = I->ws;
  auto take = [&](size_t n) { char* r = c; c += (n + 255) / 256 * 256; return r; };
  I->us = (double*)take(vec);
  I->vs = (double*)take(vec);
  I->b = (double*)take(vec);
  I->x = (double*)take(vec);
  I->r = (double*)take(vec);
  I->p[0] = (double*)take(vec);
  I->p[1] = (double*)take(vec);
  I->q = (double*)take(vec);
  I->slots = (XASlot*)take(S_COUNT * sizeof(XASlot));
  I->ctrl = (Ctrl64*)take(sizeof(Ctrl64));
  I->in_d = (StepIn*)take(sizeof(StepIn));
  I->out_d = (StepOut64*)take(sizeof(StepOut64));
  if (cudaMallocHost(&I->out_h, sizeof(StepOut64)) != cudaSuccess ||
      cudaMallocHost(&I->in_h, sizeof(StepIn)) != cudaSuccess) {
    cudaFree(I->ws);
    delete I;
    return set_error(PFGB_ECUDA, "cudaMallocHost failed");
  }
  if (prm->precision == 1) {
    const double tol_out = prm->mixed_tol_outer > 0.0 ? prm->mixed_tol_outer : prm->lin_tol;
    const double tol_in = prm->mixed_tol_inner > 0.0 ? prm->mixed_tol_inner : 1e-5;
    const int mo = prm->mixed_max_outer > 0 ? prm->mixed_max_outer : 8;
    const int mi = prm->mixed_max_inner > 0 ? prm->mixed_max_inner : 50;
    int rc = mixed::solver_create(prm->nx, prm->ny, prm->dx, prm->dy, G.ld, tol_out, tol_in, mo, mi, &I->mix);
    if (rc) {
      instance64_destroy(I);
      return rc;
    }
  }
  *out = I;
  return PFGB_OK;
}

void instance64_destroy(Instance64* I) {
  if (!I) return;
  if (I->mix) mixed::solver_destroy(I->mix);
  for (cudaEvent_t e : I->ev) cudaEventDestroy(e);
  if (I->exec) cudaGraphExecDestroy(I->exec);
  if (I->graph) cudaGraphDestroy(I->graph);
  if (I->ws) cudaFree(I->ws);
  if (I->out_h) cudaFreeHost(I->out_h);
  if (I->in_h) cudaFreeHost(I->in_h);
  delete I;
}

size_t instance64_workspace_bytes(const Instance64* I) {
  size_t vec = (size_t)I->G.ld * I->G.ny * sizeof(double);
  return 8 * vec + S_COUNT * sizeof(XASlot) + sizeof(Ctrl64) + sizeof(StepIn) + sizeof(StepOut64) + 2048;
}

// Projection stage on u*, v* (pitch usld): RHS, CG, pin, correction, diagnostics.
static void enqueue_projection(Instance64* I, const Geo64& G, int mode, double* us, double* vs, long usld,
                               double* ui, double* vi, double* pi, cudaStream_t s) {
  dim3 gp((G.nx + TX - 1) / TX, (G.ny + PB_Y - 1) / PB_Y);
  dim3 gc((G.nx + TX - 1) / TX, (G.ny + TY - 1) / TY);
  k_rhs<<<gp, NT, 0, s>>>(G, us, vs, usld, I->b, I->slots, I->ctrl);
  k_cg_init<<<gp, NT, 0, s>>>(G, I->A, 1, I->b, I->r, I->x, I->slots, I->ctrl, 0ull, 0);
  for (int k = 0; k < I->A.maxiter; ++k) {
    const bool timed = I->profiling && (size_t)(2 * k + 1) < I->ev.size();
    if (timed) cudaEventRecord(I->ev[2 * k], s);
    k_cg_matvec<0><<<gc, NT, 0, s>>>(G, I->r, I->p[0], I->p[1], I->q, I->slots, I->ctrl);
    if (timed) {
      cudaEventRecord(I->ev[2 * k + 1], s);
      I->ev_used = k + 1;
    }
    k_cg_update<<<gc, NT, 0, s>>>(G, I->A, I->p[0], I->p[1], I->q, I->x, I->r, I->slots, I->ctrl, 0ull, 0);
  }
  k_post_resid<0><<<gp, NT, 0, s>>>(G, I->b, I->x, I->slots);
  k_pin_correct<<<gp, NT, 0, s>>>(G, I->L, mode, I->x, us, vs, usld, ui, vi, pi, I->slots, I->ctrl);
  k_post_diag<<<gp, NT, 0, s>>>(G, us, vs, usld, I->b, ui, vi, pi, I->slots);
  k_gather<<<1, 32, 0, s>>>(I->slots, I->ctrl, I->out_d);
}

// Enqueue the whole step on `s` (no host synchronisation).
int instance64_enqueue(Instance64* I, double* u, double* v, double* p, long lds, const StepIn& in, cudaStream_t s) {
  const Geo64& G = I->G;
  if (lds != G.lds) return set_error(PFGB_EINVAL, "state pitch must be nx + 2");
  double* ui = u + lds + 1;   // interior pointers of the ghosted state arrays
  double* vi = v + lds + 1;
  double* pi = p + lds + 1;
  dim3 gp((G.nx + TX - 1) / TX, (G.ny + PB_Y - 1) / PB_Y);
  *I->in_h = in;
  cudaMemcpyAsync(I->in_d, I->in_h, sizeof(StepIn), cudaMemcpyHostToDevice, s);
  k_prestep<<<gp, NT, 0, s>>>(G, ui, vi, I->slots, I->ctrl);
  k_dt<<<1, 32, 0, s>>>(I->D, I->in_d, I->ctrl);
  k_predict<<<gp, NT, 0, s>>>(G, ui, vi, I->us, I->vs, I->P.scheme, I->ctrl);
  enqueue_projection(I, G, 0, I->us, I->vs, G.ld, ui, vi, pi, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
  return PFGB_OK;
}

// Build the step graph for the given state arrays.
static int build_step_graph(Instance64* I, double* ui, double* vi, double* pi) {
  if (I->exec) {
    cudaGraphExecDestroy(I->exec);
    I->exec = nullptr;
  }
  if (I->graph) {
    cudaGraphDestroy(I->graph);
    I->graph = nullptr;
  }
  cudaError_t e = cudaGraphCreate(&I->graph, 0);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("cudaGraphCreate: ") + cudaGetErrorString(e));
  const Geo64& G = I->G;
  dim3 gp((G.nx + TX - 1) / TX, (G.ny + PB_Y - 1) / PB_Y);
  dim3 gc((G.nx + TX - 1) / TX, (G.ny + TY - 1) / TY);
  GraphChain c(I->graph);
  c.kernel(k_prestep, gp, dim3(NT), G, (const double*)ui, (const double*)vi, I->slots, I->ctrl);
  c.kernel(k_dt, dim3(1), dim3(32), I->D, (const StepIn*)I->in_d, I->ctrl);
  c.kernel(k_predict, gp, dim3(NT), G, (const double*)ui, (const double*)vi, I->us, I->vs, I->P.scheme,
           (const Ctrl64*)I->ctrl);
  c.kernel(k_rhs, gp, dim3(NT), G, (const double*)I->us, (const double*)I->vs, G.ld, I->b, I->slots,
           (const Ctrl64*)I->ctrl);
  cudaGraphConditionalHandle cond = 0;
  GraphChain body(nullptr);
  if (I->mix) {
    // b is finished (mean removed, b[0] = 0) by the CG init; the refinement solves A x = b
    c.kernel(k_cg_init, gp, dim3(NT), G, I->A, 1, I->b, I->r, I->x, I->slots, I->ctrl, cond, 0);
    if (int rc = mixed::append_solve(c, I->mix, I->b, I->x, I->ctrl, I->A.maxiter)) return rc;
  } else {
    // every conditional handle must belong to a conditional node: create it only here
    e = cudaGraphConditionalHandleCreate(&cond, I->graph, 1u, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("conditional handle: ") + cudaGetErrorString(e));
    c.kernel(k_cg_init, gp, dim3(NT), G, I->A, 1, I->b, I->r, I->x, I->slots, I->ctrl, cond, 1);
    body = c.while_loop_with(cond);
    body.kernel(k_cg_matvec<0>, gc, dim3(NT), G, (const double*)I->r, I->p[0], I->p[1], I->q, I->slots, I->ctrl);
    body.kernel(k_cg_update, gc, dim3(NT), G, I->A, (const double*)I->p[0], (const double*)I->p[1],
                (const double*)I->q, I->x, I->r, I->slots, I->ctrl, cond, 1);
  }
  c.kernel(k_post_resid<0>, gp, dim3(NT), G, (const double*)I->b, (const double*)I->x, I->slots);
  c.kernel(k_pin_correct, gp, dim3(NT), G, I->L, 0, (const double*)I->x, I->us, I->vs, G.ld, ui, vi, pi, I->slots,
           I->ctrl);
  c.kernel(k_post_diag, gp, dim3(NT), G, (const double*)I->us, (const double*)I->vs, G.ld, (const double*)I->b,
           (const double*)ui, (const double*)vi, (const double*)pi, I->slots);
  c.kernel(k_gather, dim3(1), dim3(32), (const XASlot*)I->slots, (const Ctrl64*)I->ctrl, I->out_d);
  if (c.status() != cudaSuccess || (!I->mix && body.status() != cudaSuccess)) {
    cudaError_t be = c.status() != cudaSuccess ? c.status() : body.status();
    return set_error(PFGB_ECUDA, std::string("building the step graph: ") + cudaGetErrorString(be));
  }
  e = cudaGraphInstantiate(&I->exec, I->graph, 0);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  I->g_u = ui;
  I->g_v = vi;
  I->g_p = pi;
  return PFGB_OK;
}

static void copy_out(const StepOut64& o, pfgb_step_out* out) {
  out->umax = o.umax;
  out->vmax = o.vmax;
  out->div_before = o.div_before;
  out->dt = o.dt;
  out->cfl = o.cfl;
  out->safeguard = o.safeguard;
  out->cg_iterations = o.cg_iters;
  out->cg_info = o.cg_info;
  out->nan_detected = o.nan_flag;
  out->divstar_sq = o.divstar2;
  out->bnorm = o.bnrm2;
  out->res_sq = o.res2;
  out->ru_sq = o.ru2;
  out->rv_sq = o.rv2;
  out->divafter_sq = o.divafter2;
  out->linres_sq = o.linres2;
  out->cont_sq = o.cont2;
  out->reduction_flags = o.flags_or;
  out->refine_passes = o.refine_passes;
}

static int read_out(Instance64* I, cudaStream_t s, pfgb_step_out* out) {
  cudaError_t e = cudaMemcpyAsync(I->out_h, I->out_d, sizeof(StepOut64), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("step failed: ") + cudaGetErrorString(e));
  copy_out(*I->out_h, out);
  return PFGB_OK;
}

// Stand-alone projection (solve_pressure_poisson, normal mode) on the state.
int instance64_project(Instance64* I, double* u, double* v, double* p, long lds, double dt, cudaStream_t s,
                       pfgb_step_out* out) {
  if (I->mix) return set_error(PFGB_ESTATE, "pfgb_project runs the binary64 path only");
  const Geo64& G = I->G;
  if (lds != G.lds) return set_error(PFGB_EINVAL, "state pitch must be nx + 2");
  double* ui = u + lds + 1;
  double* vi = v + lds + 1;
  double* pi = p + lds + 1;
  k_set_dt<<<1, 32, 0, s>>>(dt, I->ctrl);
  enqueue_projection(I, G, 1, ui, vi, lds, ui, vi, pi, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
  return read_out(I, s, out);
}

// Mixed-precision step with direct launches (host loop control).
static int mixed_step_direct(Instance64* I, double* u, double* v, double* p, long lds, const StepIn& in,
                             cudaStream_t s, pfgb_step_out* out) {
  const Geo64& G = I->G;
  if (lds != G.lds) return set_error(PFGB_EINVAL, "state pitch must be nx + 2");
  double* ui = u + lds + 1;
  double* vi = v + lds + 1;
  double* pi = p + lds + 1;
  dim3 gp((G.nx + TX - 1) / TX, (G.ny + PB_Y - 1) / PB_Y);
  *I->in_h = in;
  cudaMemcpyAsync(I->in_d, I->in_h, sizeof(StepIn), cudaMemcpyHostToDevice, s);
  k_prestep<<<gp, NT, 0, s>>>(G, ui, vi, I->slots, I->ctrl);
  k_dt<<<1, 32, 0, s>>>(I->D, I->in_d, I->ctrl);
  k_predict<<<gp, NT, 0, s>>>(G, ui, vi, I->us, I->vs, I->P.scheme, I->ctrl);
  k_rhs<<<gp, NT, 0, s>>>(G, I->us, I->vs, G.ld, I->b, I->slots, I->ctrl);
  k_cg_init<<<gp, NT, 0, s>>>(G, I->A, 1, I->b, I->r, I->x, I->slots, I->ctrl, 0ull, 0);
  if (int rc = mixed::run_direct(I->mix, I->b, I->x, I->ctrl, I->A.maxiter, s)) return rc;
  k_post_resid<0><<<gp, NT, 0, s>>>(G, I->b, I->x, I->slots);
  k_pin_correct<<<gp, NT, 0, s>>>(G, I->L, 0, I->x, I->us, I->vs, G.ld, ui, vi, pi, I->slots, I->ctrl);
  k_post_diag<<<gp, NT, 0, s>>>(G, I->us, I->vs, G.ld, I->b, ui, vi, pi, I->slots);
  k_gather<<<1, 32, 0, s>>>(I->slots, I->ctrl, I->out_d);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
  return read_out(I, s, out);
}

int instance64_step(Instance64* I, double* u, double* v, double* p, long lds, const StepIn& in, cudaStream_t s,
                    pfgb_step_out* out) {
  if (I->mix && (!I->use_graph || I->profiling)) return mixed_step_direct(I, u, v, p, lds, in, s, out);
  if (I->use_graph && !I->profiling) {
    if (lds != I->G.lds) return set_error(PFGB_EINVAL, "state pitch must be nx + 2");
    double* ui = u + lds + 1;
    double* vi = v + lds + 1;
    double* pi = p + lds + 1;
    if (!I->exec || I->g_u != ui || I->g_v != vi || I->g_p != pi) {
      if (int rc = build_step_graph(I, ui, vi, pi)) return rc;
    }
    *I->in_h = in;
    cudaError_t e = cudaMemcpyAsync(I->in_d, I->in_h, sizeof(StepIn), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaGraphLaunch(I->exec, s);
    if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("graph launch: ") + cudaGetErrorString(e));
    return read_out(I, s, out);
  }
  int rc = instance64_enqueue(I, u, v, p, lds, in, s);
  if (rc) return rc;
  return read_out(I, s, out);
}

int instance64_set_graph(Instance64* I, int on) {
  I->use_graph = on ? 1 : 0;
  return PFGB_OK;
}

// Per-launch timing of the matvec kernel in the following steps.
int instance64_set_profiling(Instance64* I, int on) {
  if (on && I->ev.empty()) {
    int n = 2 * (I->A.maxiter > 0 ? I->A.maxiter : 1);
    I->ev.resize(n);
    for (int k = 0; k < n; ++k)
      if (cudaEventCreate(&I->ev[k]) != cudaSuccess) return set_error(PFGB_ECUDA, "cudaEventCreate failed");
  }
  I->profiling = on;
  I->ev_used = 0;
  return PFGB_OK;
}

// Sum of the matvec launch durations of the last (synchronised) step.  Launches
// that returned at once because the solve had converged are included.
int instance64_profile_result(Instance64* I, double* ms, int* launches) {
  double tot = 0.0;
  for (int k = 0; k < I->ev_used; ++k) {
    float t = 0.f;
    cudaError_t e = cudaEventElapsedTime(&t, I->ev[2 * k], I->ev[2 * k + 1]);
    if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("event timing: ") + cudaGetErrorString(e));
    tot += t;
  }
  *ms = tot;
  *launches = I->ev_used;
  return PFGB_OK;
}

// FP64 issue-rate probe: independent DFMA chains on every SM.
__global__ void k_probe_fp64(double* out, double a, double b, int n) {
  double x0 = a + threadIdx.x, x1 = x0 + 1.0, x2 = x0 + 2.0, x3 = x0 + 3.0;
#pragma unroll 16
  for (int i = 0; i < n; ++i) {
    x0 = fma(x0, b, a); x1 = fma(x1, b, a); x2 = fma(x2, b, a); x3 = fma(x3, b, a);
  }
  out[(long)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}

int probe_fp64(cudaStream_t s, double* tops) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256, n = 2048;
  double* buf = nullptr;
  if (cudaMallocAsync(&buf, (size_t)blocks * threads * sizeof(double), s) != cudaSuccess)
    return set_error(PFGB_ENOMEM, "probe buffer allocation failed");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0, s);
    k_probe_fp64<<<blocks, threads, 0, s>>>(buf, 1.0, 0.9999999, n);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(buf, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("probe failed: ") + cudaGetErrorString(e));
  // one DFMA = one FP64 instruction (2 flops); report instructions per second
  *tops = 4.0 * n * (double)blocks * threads / (best * 1e-3) / 1e12;
  return PFGB_OK;
}

// ---------------------------------------------------------------------------
// Operator-interface CG (x0 = 0) on contiguous vectors of nx*ny doubles.
int cg_solve_run(int op, const double* b, double* x, int nx, int ny, double dx, double dy, int precond,
                 double invd, double tol, int maxiter, cudaStream_t s, pfgb_solve_out* out) {
  if (nx < 2 || ny < 2) return set_error(PFGB_EINVAL, "nx and ny must be >= 2");
  if (op != PFGB_OP_NEG_LAPLACIAN_PINNED && op != PFGB_OP_LAPLACIAN_DIRICHLET) return set_error(PFGB_EINVAL, "unknown operator");
  if (maxiter < 0) return set_error(PFGB_EINVAL, "maxiter must be >= 0");
  Geo64 G;
  G.nx = nx;
  G.ny = ny;
  G.ld = nx;
  G.lds = nx + 2;
  G.g.nx = nx;
  G.g.ny = ny;
  G.g.sx = make_spacing(dx);
  G.g.sy = make_spacing(dy);
  G.invd = invd;
  G.jacobi = precond;
  CGArgs A;
  A.rtol = tol;
  A.maxiter = maxiter;
  A.n_cells = (double)nx * (double)ny;
  size_t vec = (size_t)nx * ny * sizeof(double);
  size_t vecr = (vec + 255) / 256 * 256;
  size_t bytes = 4 * vecr + S_COUNT * sizeof(XASlot) + 256 + sizeof(Ctrl64) + 256;
  char* ws = nullptr;
  cudaError_t e = cudaMallocAsync(&ws, bytes, s);
  if (e != cudaSuccess) return set_error(PFGB_ENOMEM, "cudaMallocAsync of the CG workspace failed");
  cudaMemsetAsync(ws, 0, bytes, s);
  double* r = (double*)ws;
  double* p0 = (double*)(ws + vecr);
  double* p1 = (double*)(ws + 2 * vecr);
  double* q = (double*)(ws + 3 * vecr);
  XASlot* slots = (XASlot*)(ws + 4 * vecr);
  Ctrl64* ctrl = (Ctrl64*)(ws + 4 * vecr + ((S_COUNT * sizeof(XASlot) + 255) / 256 * 256));
  dim3 gp((nx + TX - 1) / TX, (ny + PB_Y - 1) / PB_Y);
  dim3 gc((nx + TX - 1) / TX, (ny + TY - 1) / TY);
  k_cg_init<<<gp, NT, 0, s>>>(G, A, 0, const_cast<double*>(b), r, x, slots, ctrl, 0ull, 0);
  for (int k = 0; k < maxiter; ++k) {
    if (op == PFGB_OP_NEG_LAPLACIAN_PINNED)
      k_cg_matvec<0><<<gc, NT, 0, s>>>(G, r, p0, p1, q, slots, ctrl);
    else
      k_cg_matvec<1><<<gc, NT, 0, s>>>(G, r, p0, p1, q, slots, ctrl);
    k_cg_update<<<gc, NT, 0, s>>>(G, A, p0, p1, q, x, r, slots, ctrl, 0ull, 0);
  }
  if (op == PFGB_OP_NEG_LAPLACIAN_PINNED)
    k_post_resid<0><<<gp, NT, 0, s>>>(G, b, x, slots);
  else
    k_post_resid<1><<<gp, NT, 0, s>>>(G, b, x, slots);
  Ctrl64 hc;
  double res2 = 0.0;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hc, ctrl, sizeof(Ctrl64), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&res2, &slots[S_RES].result, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(ws, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("cg solve failed: ") + cudaGetErrorString(e));
  out->info = hc.info;
  out->iterations = hc.zero_rhs ? 0 : hc.iter;
  out->bnorm = hc.bnrm2;
  out->res_sq = res2;
  return PFGB_OK;
}

}  // namespace pfgb

namespace pfgb {

// ---------------------------------------------------------------------------
// Allocation-free variant of the operator-interface CG.
//
// Some callers cannot allocate device memory at the moment they need a solve:
// a real-time loop that must not stall on cudaMalloc/cudaFree (both can
// synchronise the whole device), or an embedding application that reserved the
// device memory for its own pool and admits no third-party allocation.  For them the work vectors, reduction slots and
// control block of the CG live in one file-scope device array of fixed size,
// reserved once when the library's module is loaded on a device and held until
// the process exits.  Its limit is NOALLOC_MAX_CELLS = 262,144 cells
// (512 x 512), about 8.4 MiB per device.
namespace noalloc {

constexpr long NOALLOC_MAX_CELLS = 1L << 18;

struct Scratch {
  double r[NOALLOC_MAX_CELLS];
  double p0[NOALLOC_MAX_CELLS];
  double p1[NOALLOC_MAX_CELLS];
  double q[NOALLOC_MAX_CELLS];
  XASlot slots[S_COUNT];
  Ctrl64 ctrl;
};

static __device__ __align__(256) Scratch g_scratch;

constexpr int MAX_DEVICES = 64;
static std::mutex g_mu;
static Scratch* g_addr[MAX_DEVICES] = {};

// Device address of g_scratch on the current device (looked up once per device).
static int scratch_address(Scratch** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= MAX_DEVICES) return set_error(PFGB_EINVAL, "device index beyond the scratch table");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess)
      return set_error(PFGB_ECUDA, std::string("cudaGetSymbolAddress of the CG scratch: ") + cudaGetErrorString(e));
    g_addr[dev] = static_cast<Scratch*>(p);
  }
  *out = g_addr[dev];
  return PFGB_OK;
}

}  // namespace noalloc

int cg_solve_noalloc_run(int op, const double* b, double* x, int nx, int ny, double dx, double dy, int precond,
                         double invd, double tol, int maxiter, cudaStream_t s, pfgb_solve_out* out) {
  using namespace noalloc;
  if (nx < 2 || ny < 2) return set_error(PFGB_EINVAL, "nx and ny must be >= 2");
  if ((long)nx * (long)ny > NOALLOC_MAX_CELLS)
    return set_error(PFGB_EINVAL, "nx*ny exceeds the 262144-cell limit of the allocation-free CG scratch");
  if (op != PFGB_OP_NEG_LAPLACIAN_PINNED && op != PFGB_OP_LAPLACIAN_DIRICHLET) return set_error(PFGB_EINVAL, "unknown operator");
  if (maxiter < 0) return set_error(PFGB_EINVAL, "maxiter must be >= 0");
  Scratch* S = nullptr;
  if (int rc = scratch_address(&S)) return rc;
  Geo64 G;
  G.nx = nx;
  G.ny = ny;
  G.ld = nx;
  G.lds = nx + 2;
  G.g.nx = nx;
  G.g.ny = ny;
  G.g.sx = make_spacing(dx);
  G.g.sy = make_spacing(dy);
  G.invd = invd;
  G.jacobi = precond;
  CGArgs A;
  A.rtol = tol;
  A.maxiter = maxiter;
  A.n_cells = (double)nx * (double)ny;
  // the slots and the control block must start from zero on every call
  cudaError_t e = cudaMemsetAsync(S->slots, 0, sizeof(S->slots) + sizeof(S->ctrl), s);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("clearing the CG scratch: ") + cudaGetErrorString(e));
  XASlot* slots = S->slots;
  Ctrl64* ctrl = &S->ctrl;
  dim3 gp((nx + TX - 1) / TX, (ny + PB_Y - 1) / PB_Y);
  dim3 gc((nx + TX - 1) / TX, (ny + TY - 1) / TY);
  k_cg_init<<<gp, NT, 0, s>>>(G, A, 0, const_cast<double*>(b), S->r, x, slots, ctrl, 0ull, 0);
  for (int k = 0; k < maxiter; ++k) {
    if (op == PFGB_OP_NEG_LAPLACIAN_PINNED)
      k_cg_matvec<0><<<gc, NT, 0, s>>>(G, S->r, S->p0, S->p1, S->q, slots, ctrl);
    else
      k_cg_matvec<1><<<gc, NT, 0, s>>>(G, S->r, S->p0, S->p1, S->q, slots, ctrl);
    k_cg_update<<<gc, NT, 0, s>>>(G, A, S->p0, S->p1, S->q, x, S->r, slots, ctrl, 0ull, 0);
  }
  if (op == PFGB_OP_NEG_LAPLACIAN_PINNED)
    k_post_resid<0><<<gp, NT, 0, s>>>(G, b, x, slots);
  else
    k_post_resid<1><<<gp, NT, 0, s>>>(G, b, x, slots);
  Ctrl64 hc;
  double res2 = 0.0;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hc, ctrl, sizeof(Ctrl64), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&res2, &slots[S_RES].result, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("allocation-free cg solve failed: ") + cudaGetErrorString(e));
  out->info = hc.info;
  out->iterations = hc.zero_rhs ? 0 : hc.iter;
  out->bnorm = hc.bnrm2;
  out->res_sq = res2;
  return PFGB_OK;
}

}  // namespace pfgb
