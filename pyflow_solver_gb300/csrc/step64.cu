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
#include <cstddef>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <algorithm>
#include <vector>

#include "dred.cuh"
#include "graph.cuh"
#include "mixed.cuh"
#include "persist.cuh"
#include "pfgb_internal.h"
#include "stencil.cuh"
#include "step64.cuh"

namespace pfgb {

constexpr int NT = 256;       // threads per CTA (1-D blocks)
constexpr int TX = 32;        // tile width (one warp per tile row)
constexpr int TY = 16;        // tile height of the CG kernels (2 rows per thread)
constexpr int RPT = TY / (NT / TX);   // rows per thread in the CG kernels (2)
constexpr int PB_Y = NT / TX;         // tile height of the per-cell kernels (8)
constexpr int PB_R = 4;               // the mixed-form per-cell kernels: 32 x 32 tiles, 4 rows per thread
constexpr int TY_M = PB_R * PB_Y;

__device__ __forceinline__ double jacobi_apply(const Geo64& G, int j, int i, double r) {
  if (!G.jacobi) return r;
  bool ring = (i == 0) || (i == G.nx - 1) || (j == 0) || (j == G.ny - 1);
  return ring ? r : MUL(G.invd, r);
}

// ---------------------------------------------------------------------------
// Reduction tails shared by the kernels.  A CTA's share of the exactly rounded
// sum of a[k]*b[k], k < N (SQUARE: b is a) goes into `slot`; cells outside the
// grid pass a = 0.  A plain sum passes b = 1.
template <int N, bool SQUARE>
__device__ __forceinline__ void reduce_prods(XASlot* slot, const double* a, const double* b, long long* sacc,
                                             long long* wred, int* ired) {
  int top = INT_MIN;
#pragma unroll
  for (int k = 0; k < N; ++k) top = max(top, xa_prod_top(a[k], SQUARE ? a[k] : b[k]));
  top = xa_block_max(top, ired);
  const int k0 = xa_window_digit(top);
  XAcc x;
  x.clear();
#pragma unroll
  for (int k = 0; k < N; ++k) xa_acc_prod<SQUARE>(x, sacc, k0, a[k], SQUARE ? a[k] : b[k]);
  const int anyslow = __syncthreads_or(x.slow);
  xa_acc_commit(slot, x, k0, sacc, anyslow, wred);
}

// Two such sums with one block-wide maximum and one commit barrier.  `ired`
// holds 64 ints that no earlier code of the kernel uses; `wred` holds
// 2 x XA_WLIMBS x (warps) long longs.
template <int N, bool SQ0, bool SQ1>
__device__ __forceinline__ void reduce_prods2(XASlot* s0, const double* a0, const double* b0, long long* sacc0,
                                              XASlot* s1, const double* a1, const double* b1, long long* sacc1,
                                              long long* wred, int* ired) {
  __shared__ XCommit2 cs;
  cs.zero();
  int t0 = INT_MIN, t1 = INT_MIN;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    t0 = max(t0, xa_prod_top(a0[k], SQ0 ? a0[k] : b0[k]));
    t1 = max(t1, xa_prod_top(a1[k], SQ1 ? a1[k] : b1[k]));
  }
  xa_block_max2(t0, t1, ired);
  const int k0 = xa_window_digit(t0), k1 = xa_window_digit(t1);
  // one window at a time: the first is folded into its warp digit sums before
  // the second is formed, which keeps the live registers of one window
  XAcc x;
  x.clear();
#pragma unroll
  for (int k = 0; k < N; ++k) xa_acc_prod<SQ0>(x, sacc0, k0, a0[k], SQ0 ? a0[k] : b0[k]);
  XWarpPart w0 = xa_warp_part(x);
  x.clear();
#pragma unroll
  for (int k = 0; k < N; ++k) xa_acc_prod<SQ1>(x, sacc1, k1, a1[k], SQ1 ? a1[k] : b1[k]);
  XWarpPart w1 = xa_warp_part(x);
  xa_acc_commit2(s0, w0, k0, sacc0, s1, w1, k1, sacc1, wred, cs);
}

__device__ __forceinline__ void zero_sacc(long long* sacc) {
  for (int k = threadIdx.x; k < XA_DIGITS; k += blockDim.x) sacc[k] = 0;
}

// The CTA's tile and instance: the instance's descriptor is staged in shared
// memory before the wait on the predecessor.  Every CTA of an inactive instance
// returns.
#define TILE_PROLOGUE                                             \
  pdl_launch();                                                   \
  __shared__ InstDesc sdesc_;                                     \
  const Tile tl = TL[blockIdx.x];                                 \
  stage_desc(ID + tl.inst, &sdesc_);                              \
  pdl_wait();                                                     \
  __syncthreads();                                                \
  const InstDesc& D = sdesc_;                                     \
  if (!D.active) return;                                          \
  const Geo64 G = D.G;

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NT) k_prestep(const InstDesc* __restrict__ ID, const Tile* __restrict__ TL) {
  TILE_PROLOGUE
  __shared__ long long sacc[XA_DIGITS];
  __shared__ long long wred[2 * (NT / 32) * XA_WLIMBS];
  __shared__ int ired[64];
  zero_sacc(sacc);
  XASlot* slots = D.slots;
  Ctrl64* ctrl = D.ctrl;
  const int i = tl.i0 + (threadIdx.x & 31);
  const int j = tl.j0 + (threadIdx.x >> 5);
  View2<const double> U{D.ui, G.lds}, V{D.vi, G.lds};
  double d = 0.0;
  unsigned long long ub = 0ull, vb = 0ull;
  if (i < G.nx && j < G.ny) {
    ub = abs_bits(U(j, i));
    vb = abs_bits(V(j, i));
    d = div_central_unit(U, V, j, i, G.nx, G.ny);
  }
  for (int o = 16; o > 0; o >>= 1) {
    ub = max(ub, __shfl_xor_sync(0xffffffffu, ub, o));
    vb = max(vb, __shfl_xor_sync(0xffffffffu, vb, o));
  }
  if ((threadIdx.x & 31) == 0) {
    if (ub) atomicMax(&ctrl->umax_bits, ub);
    if (vb) atomicMax(&ctrl->vmax_bits, vb);
  }
  reduce_prods<1, true>(&slots[S_DIVC_BEFORE], &d, &d, sacc, wred, ired);
  XASlot* sl[1] = {&slots[S_DIVC_BEFORE]};
  if (xa_finish(sl, 1, D.nt_pc) && threadIdx.x == 0) {
    double um = __longlong_as_double((long long)*(volatile unsigned long long*)&ctrl->umax_bits);
    double vm = __longlong_as_double((long long)*(volatile unsigned long long*)&ctrl->vmax_bits);
    ctrl->umax = ADD(um, 1e-12);
    ctrl->vmax = ADD(vm, 1e-12);
    ctrl->umax_bits = 0ull;
    ctrl->vmax_bits = 0ull;
    ctrl->div_before = __dsqrt_rn(slots[S_DIVC_BEFORE].result);
  }
}

// dt selection, exactly the Python float sequence of solver.py:25-62 (one thread per instance)
__device__ __forceinline__ void dt_one(const InstDesc& Dd) {
  const DtArgs a = Dd.D;
  const StepIn in = *Dd.in;
  Ctrl64* ctrl = Dd.ctrl;
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
  int nh = in.hist_len;
  for (int q = 0; q < nh; ++q) h[q] = in.hist[q];
  h[nh++] = ctrl->div_before;
  int safeguard = 0;
  if (nh >= 3) {
    double x = h[nh - 3], y = h[nh - 2], z = h[nh - 1];
    if (x > 0.0 && y > MUL(x, 1.01) && z > MUL(y, 1.01)) {
      dt = MUL(dt, 0.5);
      safeguard = 1;
    }
  }
  ctrl->dt = dt;
  ctrl->safeguard = safeguard;
  ctrl->cfl = py_max(DIV(MUL(umax, dt), a.dx), DIV(MUL(vmax, dt), a.dy));
  ctrl->dtm = py_max(dt, 1e-14);
  ctrl->rdtm = 1.0 / ctrl->dtm;
}

__global__ void k_dt(const InstDesc* __restrict__ ID, int n) {
  pdl_enter();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const InstDesc& Dd = ID[k];
  if (!Dd.active) return;
  dt_one(Dd);
}

// dt given by the caller of a stand-alone projection (instance 0)
__global__ void k_set_dt(const InstDesc* __restrict__ ID, double dt) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  Ctrl64* ctrl = ID[0].ctrl;
  ctrl->dt = dt;
  ctrl->dtm = py_max(dt, 1e-14);
  ctrl->rdtm = 1.0 / ctrl->dtm;
  ctrl->safeguard = 0;
}

// predictor: u* = u - dt*conv_u(u,v), v* likewise (solver.py:73-95)
__global__ void __launch_bounds__(NT) k_predict(const InstDesc* __restrict__ ID, const Tile* __restrict__ TL) {
  TILE_PROLOGUE
  const int i = tl.i0 + (threadIdx.x & 31);
  const int j = tl.j0 + (threadIdx.x >> 5);
  if (i >= G.nx || j >= G.ny) return;
  View2<const double> U{D.ui, G.lds}, V{D.vi, G.lds};
  const double dt = D.ctrl->dt;
  double u0 = U(j, i), v0 = V(j, i), un, vn;
  if (D.scheme == 2) {            // advection disabled: u* = u_old
    un = u0; vn = v0;
  } else if (D.scheme == 1) {     // QUICK
    un = SUB(u0, MUL(dt, advect_quick_at(U, V, U, j, i, G.g)));
    vn = SUB(v0, MUL(dt, advect_quick_at(U, V, V, j, i, G.g)));
  } else {                        // upwind
    un = SUB(u0, MUL(dt, advect_upwind_at(U, V, U, j, i, G.g)));
    vn = SUB(v0, MUL(dt, advect_upwind_at(U, V, V, j, i, G.g)));
  }
  D.us[(long)j * D.usld + i] = un;
  D.vs[(long)j * D.usld + i] = vn;
}

// RHS: b = -div_c(u*,v*)/max(dt,1e-14); sum(b); ||div_c(u*,v*)||^2
__global__ void __launch_bounds__(NT) k_rhs(const InstDesc* __restrict__ ID, const Tile* __restrict__ TL) {
  TILE_PROLOGUE
  __shared__ long long sacc0[XA_DIGITS], sacc1[XA_DIGITS];
  __shared__ long long wred[2 * (NT / 32) * XA_WLIMBS];
  __shared__ int ired[64];
  zero_sacc(sacc0);
  zero_sacc(sacc1);
  XASlot* slots = D.slots;
  const int i = tl.i0 + (threadIdx.x & 31);
  const int j = tl.j0 + (threadIdx.x >> 5);
  double d = 0.0, bv = 0.0;
  const double one = 1.0;
  if (i < G.nx && j < G.ny) {
    View2<const double> US{D.us, D.usld}, VS{D.vs, D.usld};
    d = div_coherent_at(US, VS, j, i, G.g);
    bv = DIV(-d, D.ctrl->dtm);
    D.b[(long)j * G.ld + i] = bv;
  }
  reduce_prods2<1, false, true>(&slots[S_BSUM], &bv, &one, sacc0, &slots[S_DIVSTAR], &d, &d, sacc1, wred, ired);
  XASlot* sl[2] = {&slots[S_BSUM], &slots[S_DIVSTAR]};
  xa_finish(sl, 2, D.nt_pc);
}

// adjust = 1 (projection): b -= mean(b); b[0] = 0.  Then r = b; x = 0;
// ||b||^2; r.(M r).  adjust = 0 (operator interface): b is used as given.
// Instances that start iterating are counted in the loop control.
__global__ void __launch_bounds__(NT) k_cg_init(const InstDesc* __restrict__ ID, const Tile* __restrict__ TL,
                                                 LoopCtl* lc) {
  TILE_PROLOGUE
  __shared__ long long sacc0[XA_DIGITS], sacc1[XA_DIGITS];
  __shared__ long long wred[2 * (NT / 32) * XA_WLIMBS];
  __shared__ int ired[64];
  zero_sacc(sacc0);
  zero_sacc(sacc1);
  XASlot* slots = D.slots;
  Ctrl64* ctrl = D.ctrl;
  const CGArgs A = D.A;
  const int i = tl.i0 + (threadIdx.x & 31);
  const int j = tl.j0 + (threadIdx.x >> 5);
  const double mean = D.adjust ? DIV(slots[S_BSUM].result, A.n_cells) : 0.0;
  double bv = 0.0, zv = 0.0;
  if (i < G.nx && j < G.ny) {
    long o = (long)j * G.ld + i;
    bv = D.b[o];
    if (D.adjust) {
      bv = SUB(bv, mean);
      if (i == 0 && j == 0) bv = 0.0;
      D.b[o] = bv;
    }
    D.r[o] = bv;
    D.x[o] = 0.0;
    zv = jacobi_apply(G, j, i, bv);
    if (D.z) D.z[o] = zv;
  }
  reduce_prods2<1, true, false>(&slots[S_BB], &bv, &bv, sacc0, &slots[S_RZ0], &bv, &zv, sacc1, wred, ired);
  XASlot* sl[2] = {&slots[S_BB], &slots[S_RZ0]};
  if (xa_finish(sl, 2, D.nt_pc) && threadIdx.x == 0) {
    double bb = slots[S_BB].result;
    double bnrm2 = __dsqrt_rn(bb);
    ctrl->mean = mean;
    ctrl->bnrm2 = bnrm2;
    ctrl->atol = py_max(0.0, MUL(A.rtol, bnrm2));
    ctrl->iter = 0;
    ctrl->info = 0;
    ctrl->zero_rhs = 0;
    ctrl->nan_flag = 0u;
    ctrl->refine_passes = 0;
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
      if (lc) atomicAdd(&lc->active, 1);
    }
  }
}

// Arms a WHILE loop: its condition is "some instance still iterates".
__global__ void k_loop_arm(LoopCtl* lc, cudaGraphConditionalHandle cond, int use_cond) {
  pdl_enter();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  lc->guard = 0;
  lc->tripped = 0;
  if (use_cond) cudaGraphSetConditional(cond, lc->active > 0 ? 1u : 0u);
}

// Last node of a WHILE body: stops the loop after guard_max trips in any case.
__global__ void k_loop_guard(LoopCtl* lc, cudaGraphConditionalHandle cond, int use_cond) {
  pdl_enter();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int g = ++lc->guard;
  if (g >= lc->guard_max && lc->active > 0) {
    lc->tripped = 1;
    if (use_cond) cudaGraphSetConditional(cond, 0u);
  }
}

// p_new = z + beta*p_old (p_new = z at k = 0); q = A p_new; p_new.q
// OP 0: A = -lap_c with row 0 = identity (normal projection);
// OP 1: A = lap_c with identity rows on the boundary ring (manufactured mode).
// The iteration index k is read from the control block and selects the
// ping-pong buffers: iteration k reads p[k & 1] and writes p[(k + 1) & 1].
// R: rows per thread (the tile is 32 x 8R cells); the autotuner picks R per handle.
template <int OP, int R = RPT>
__global__ void __launch_bounds__(NT, 5) k_cg_matvec(const InstDesc* __restrict__ ID, const Tile* __restrict__ TL) {
  constexpr int TYv = R * PB_Y;
  TILE_PROLOGUE
  Ctrl64* ctrl = D.ctrl;
  if (*(volatile int*)&ctrl->done) return;
  __shared__ double pn[TYv + 2][TX + 2];
  __shared__ double gxs[TYv][TX + 1];
  __shared__ double gys[TYv + 1][TX];
  __shared__ long long sacc[XA_DIGITS];
  __shared__ long long wred[2 * (NT / 32) * XA_WLIMBS];
  __shared__ int ired[64];
  zero_sacc(sacc);
  XASlot* slots = D.slots;
  const int k = *(volatile int*)&ctrl->iter;
  const double* __restrict__ pold = (k & 1) ? D.p1 : D.p0;
  double* __restrict__ pnew = (k & 1) ? D.p0 : D.p1;
  const double* __restrict__ r = D.r;
  const double* __restrict__ zs = D.z;     // M r as the last update wrote it (null: formed here)
  const int i0 = tl.i0, j0 = tl.j0;
  const double beta = (k > 0) ? ctrl->beta : 0.0;
  for (int idx = threadIdx.x; idx < (TYv + 2) * (TX + 2); idx += NT) {
    int jj = idx / (TX + 2) - 1, ii = idx % (TX + 2) - 1;
    int gj = j0 + jj, gi = i0 + ii;
    bool corner = (jj < 0 || jj >= TYv) && (ii < 0 || ii >= TX);
    double val = 0.0;
    if (!corner && gj >= 0 && gj < G.ny && gi >= 0 && gi < G.nx) {
      long o = (long)gj * G.ld + gi;
      const double z = zs ? zs[o] : jacobi_apply(G, gj, gi, r[o]);
      val = (k == 0) ? z : ADD(MUL(pold[o], beta), z);
    }
    pn[jj + 1][ii + 1] = val;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < TYv * (TX + 1); idx += NT) {
    int jj = idx / (TX + 1), ii = idx % (TX + 1) - 1;
    int gj = j0 + jj, gi = i0 + ii;
    double gv = 0.0;
    if (gj < G.ny && gi >= 0 && gi < G.nx - 1) gv = DIVH(SUB(pn[jj + 1][ii + 2], pn[jj + 1][ii + 1]), G.g.sx);
    gxs[jj][ii + 1] = gv;
  }
  for (int idx = threadIdx.x; idx < (TYv + 1) * TX; idx += NT) {
    int jj = idx / TX - 1, ii = idx % TX;
    int gj = j0 + jj, gi = i0 + ii;
    double gv = 0.0;
    if (gi < G.nx && gj >= 0 && gj < G.ny - 1) gv = DIVH(SUB(pn[jj + 2][ii + 1], pn[jj + 1][ii + 1]), G.g.sy);
    gys[jj + 1][ii] = gv;
  }
  __syncthreads();
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  double pa[R], qa[R];
#pragma unroll
  for (int rr = 0; rr < R; ++rr) {
    pa[rr] = 0.0;
    qa[rr] = 0.0;
    int jj = ty + rr * PB_Y;
    int gj = j0 + jj, gi = i0 + tx;
    if (gj < G.ny && gi < G.nx) {
      double gxi = gxs[jj][tx + 1];
      double xp = (gi >= 1) ? DIVH(SUB(gxi, gxs[jj][tx]), G.g.sx) : DIVH(gxi, G.g.sx);
      double gyj = gys[jj + 1][tx];
      double yp = (gj >= 1) ? DIVH(SUB(gyj, gys[jj][tx]), G.g.sy) : DIVH(gyj, G.g.sy);
      double pv = pn[jj + 1][tx + 1];
      double qv;
      if (OP == 0) qv = (gi == 0 && gj == 0) ? pv : neg_exact(ADD(xp, yp));
      else qv = (gi == 0 || gj == 0 || gi == G.nx - 1 || gj == G.ny - 1) ? pv : ADD(xp, yp);
      long o = (long)gj * G.ld + gi;
      D.q[o] = qv;
      pnew[o] = pv;
      pa[rr] = pv;
      qa[rr] = qv;
    }
  }
  reduce_prods<R, false>(&slots[S_PQ], pa, qa, sacc, wred, ired);
  XASlot* sl[1] = {&slots[S_PQ]};
  if (xa_finish(sl, 1, D.nt_cg) && threadIdx.x == 0) {
    const double pq = slots[S_PQ].result;
    ctrl->pq = pq;
    ctrl->alpha = DIV(ctrl->rho, pq);
  }
}

// x += alpha p; r -= alpha q; r.r; r.(M r).  An instance that finishes
// leaves the loop control's active count; the last one stops the loop.
template <int R = RPT>
__global__ void __launch_bounds__(NT, R == 1 ? 6 : 5) k_cg_update(const InstDesc* __restrict__ ID, const Tile* __restrict__ TL,
                                                   LoopCtl* lc, cudaGraphConditionalHandle cond, int use_cond) {
  TILE_PROLOGUE
  Ctrl64* ctrl = D.ctrl;
  if (*(volatile int*)&ctrl->done) return;
  __shared__ long long sacc0[XA_DIGITS], sacc1[XA_DIGITS];
  __shared__ long long wred[2 * (NT / 32) * XA_WLIMBS];
  __shared__ int ired[64];
  zero_sacc(sacc0);
  zero_sacc(sacc1);
  XASlot* slots = D.slots;
  const CGArgs A = D.A;
  const int k = *(volatile int*)&ctrl->iter;
  const double* __restrict__ p = (k & 1) ? D.p0 : D.p1;    // the buffer this iteration's matvec wrote
  const int i0 = tl.i0, j0 = tl.j0;
  const double alpha = ctrl->alpha;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  double ra[R], za[R];
#pragma unroll
  for (int rr = 0; rr < R; ++rr) {
    ra[rr] = 0.0;
    za[rr] = 0.0;
    int gj = j0 + ty + rr * PB_Y, gi = i0 + tx;
    if (gj < G.ny && gi < G.nx) {
      long o = (long)gj * G.ld + gi;
      double xv = ADD(D.x[o], MUL(alpha, p[o]));
      double rv = SUB(D.r[o], MUL(alpha, D.q[o]));
      D.x[o] = xv;
      D.r[o] = rv;
      ra[rr] = rv;
      za[rr] = jacobi_apply(G, gj, gi, rv);
      if (D.z) D.z[o] = za[rr];
    }
  }
  reduce_prods2<R, true, false>(&slots[S_RR], ra, ra, sacc0, &slots[S_RZ], ra, za, sacc1, wred, ired);
  XASlot* sl[2] = {&slots[S_RR], &slots[S_RZ]};
  if (xa_finish(sl, 2, D.nt_cg) && threadIdx.x == 0) {
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
    if (ctrl->done && lc) {
      if (atomicSub(&lc->active, 1) == 1 && use_cond) cudaGraphSetConditional(cond, 0u);
    }
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
__global__ void __launch_bounds__(NT) k_post_resid(const InstDesc* __restrict__ ID, const Tile* __restrict__ TL) {
  TILE_PROLOGUE
  __shared__ long long sacc[XA_DIGITS];
  __shared__ long long wred[2 * (NT / 32) * XA_WLIMBS];
  __shared__ int ired[64];
  zero_sacc(sacc);
  XASlot* slots = D.slots;
  const int i = tl.i0 + (threadIdx.x & 31);
  const int j = tl.j0 + (threadIdx.x >> 5);
  double rv = 0.0;
  if (i < G.nx && j < G.ny) {
    View2<const double> X{D.x, G.ld};
    rv = SUB(D.b[(long)j * G.ld + i], apply_A<OP>(X, j, i, G.g));
  }
  reduce_prods<1, true>(&slots[S_RES], &rv, &rv, sacc, wred, ired);
  XASlot* sl[1] = {&slots[S_RES]};
  xa_finish(sl, 1, D.nt_pc);
}

// p = x - x[0] into the state; u = u* - dt*gx(p).
// mode 0 (full step): u* lives in us/vs and keeps the pre-lid corrected
//   velocity for the divergence diagnostic; the state gets the lid on its top
//   interior row and the sums of (u-u_old)^2 are formed.
// mode 1 (projection only): us/vs are the state's own u/v, corrected in place.
__global__ void __launch_bounds__(NT) k_pin_correct(const InstDesc* __restrict__ ID, const Tile* __restrict__ TL) {
  TILE_PROLOGUE
  __shared__ long long sacc0[XA_DIGITS], sacc1[XA_DIGITS];
  __shared__ long long wred[2 * (NT / 32) * XA_WLIMBS];
  __shared__ int ired[64];
  zero_sacc(sacc0);
  zero_sacc(sacc1);
  XASlot* slots = D.slots;
  Ctrl64* ctrl = D.ctrl;
  const LidArgs L = D.L;
  const int i = tl.i0 + (threadIdx.x & 31);
  const int j = tl.j0 + (threadIdx.x >> 5);
  double du2 = 0.0, dv2 = 0.0;
  const double one = 1.0;
  int bad = 0;
  if (i < G.nx && j < G.ny) {
    const double dt = ctrl->dt;
    const double* __restrict__ x = D.x;
    const double x0 = x[0];
    View2<const double> X{x, G.ld};
    const double pv = SUB(X(j, i), x0);
    const double gx = (i < G.nx - 1) ? DIVH(SUB(SUB(X(j, i + 1), x0), pv), G.g.sx) : 0.0;
    const double gy = (j < G.ny - 1) ? DIVH(SUB(SUB(X(j + 1, i), x0), pv), G.g.sy) : 0.0;
    long o = (long)j * D.usld + i;
    long os = (long)j * G.lds + i;
    const double uc = SUB(D.us[o], MUL(dt, gx));
    const double vc = SUB(D.vs[o], MUL(dt, gy));
    D.us[o] = uc;
    D.vs[o] = vc;
    D.pi[os] = pv;
    if (D.mode == 0) {
      const double uf = (L.has_lid && j == G.ny - 1) ? L.lid : uc;
      const double du = SUB(uf, D.ui[os]);
      const double dv = SUB(vc, D.vi[os]);
      D.ui[os] = uf;
      D.vi[os] = vc;
      du2 = MUL(du, du);
      dv2 = MUL(dv, dv);
      bad = !(isfinite_d(uf) && isfinite_d(vc) && isfinite_d(pv));
    } else {
      bad = !(isfinite_d(uc) && isfinite_d(vc) && isfinite_d(pv));
    }
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&ctrl->nan_flag, 1u);
  reduce_prods2<1, false, false>(&slots[S_RU], &du2, &one, sacc0, &slots[S_RV], &dv2, &one, sacc1, wred, ired);
  XASlot* sl[2] = {&slots[S_RU], &slots[S_RV]};
  xa_finish(sl, 2, D.nt_pc);
}

// ||div_c(u_corr)||^2, ||A p - b||^2, ||div_central(u,v;1,1)||^2
__global__ void __launch_bounds__(NT) k_post_diag(const InstDesc* __restrict__ ID, const Tile* __restrict__ TL) {
  TILE_PROLOGUE
  __shared__ long long sacc0[XA_DIGITS], sacc1[XA_DIGITS], sacc2[XA_DIGITS];
  __shared__ long long wred[2 * (NT / 32) * XA_WLIMBS];
  __shared__ int ired[64];
  zero_sacc(sacc0);
  zero_sacc(sacc1);
  zero_sacc(sacc2);
  XASlot* slots = D.slots;
  const int i = tl.i0 + (threadIdx.x & 31);
  const int j = tl.j0 + (threadIdx.x >> 5);
  double d = 0.0, lr = 0.0, c = 0.0;
  if (i < G.nx && j < G.ny) {
    View2<const double> US{D.us, D.usld}, VS{D.vs, D.usld};
    View2<const double> U{D.ui, G.lds}, V{D.vi, G.lds}, P{D.pi, G.lds};
    d = div_coherent_at(US, VS, j, i, G.g);
    lr = SUB(apply_A<0>(P, j, i, G.g), D.b[(long)j * G.ld + i]);
    c = div_central_unit(U, V, j, i, G.nx, G.ny);
  }
  reduce_prods2<1, true, true>(&slots[S_DIVAFTER], &d, &d, sacc0, &slots[S_LINRES], &lr, &lr, sacc1, wred, ired);
  reduce_prods<1, true>(&slots[S_CONT], &c, &c, sacc2, wred, ired);
  XASlot* sl[3] = {&slots[S_DIVAFTER], &slots[S_LINRES], &slots[S_CONT]};
  xa_finish(sl, 3, D.nt_pc);
}

// ---------------------------------------------------------------------------
// The same kernels for the mixed-precision form.  The arithmetic of every cell
// is the binary64 code above, except that divisions by the spacing and by dt
// are products with the reciprocal; the sums are deterministic binary64 sums
// over the instance's tiles (dred.cuh) instead of exactly rounded ones.  Both
// differences are at the level of one rounding, far inside the 1e-6 the mixed
// form is held to, and keep a result identical alone and in any batch.

using StepRed = DRedSmem<NT>;
#define STEP_RED(R, vals, outv) dred_sum<R, NT>(mixed::CtaCtx{}, vals, D.part, D.nt_m, tl.loc, D.ticket, outv, rsm)
#define M_ROWS(...)                                         \
  for (int r_ = 0; r_ < PB_R; ++r_) {                       \
    const int j = tl.j0 + (threadIdx.x >> 5) + r_ * PB_Y;   \
    __VA_ARGS__                                             \
  }

struct RecipGrid {
  double rx, ry;
};
__device__ __forceinline__ RecipGrid recips(const Geo64& G) { return RecipGrid{G.rdx, G.rdy}; }

__device__ __forceinline__ double gx_r(View2<const double> p, int j, int i, int nx, double rx) {
  return (i < nx - 1) ? MUL(SUB(p(j, i + 1), p(j, i)), rx) : 0.0;
}
__device__ __forceinline__ double gy_r(View2<const double> p, int j, int i, int ny, double ry) {
  return (j < ny - 1) ? MUL(SUB(p(j + 1, i), p(j, i)), ry) : 0.0;
}
__device__ __forceinline__ double div_c_r(View2<const double> u, View2<const double> v, int j, int i,
                                          const RecipGrid& r) {
  const double xp = (i >= 1) ? MUL(SUB(u(j, i), u(j, i - 1)), r.rx) : MUL(u(j, 0), r.rx);
  const double yp = (j >= 1) ? MUL(SUB(v(j, i), v(j - 1, i)), r.ry) : MUL(v(0, i), r.ry);
  return ADD(xp, yp);
}
__device__ __forceinline__ double neg_lap_pinned_r(View2<const double> p, int j, int i, int nx, int ny,
                                                   const RecipGrid& r) {
  if (i == 0 && j == 0) return p(0, 0);
  const double gxi = gx_r(p, j, i, nx, r.rx);
  const double xp = (i >= 1) ? MUL(SUB(gxi, gx_r(p, j, i - 1, nx, r.rx)), r.rx) : MUL(gxi, r.rx);
  const double gyj = gy_r(p, j, i, ny, r.ry);
  const double yp = (j >= 1) ? MUL(SUB(gyj, gy_r(p, j - 1, i, ny, r.ry)), r.ry) : MUL(gyj, r.ry);
  return -ADD(xp, yp);
}

// max|u|, max|v| and ||div_central(u, v; 1, 1)||^2 (the safeguard's baseline)
__global__ void __launch_bounds__(NT) k_prestep_m(const InstDesc* __restrict__ ID, const Tile* __restrict__ TL) {
  TILE_PROLOGUE
  __shared__ StepRed rsm;
  Ctrl64* ctrl = D.ctrl;
  const int i = tl.i0 + (threadIdx.x & 31);
  View2<const double> U{D.ui, G.lds}, V{D.vi, G.lds};
  double v[1] = {0.0}, out[1];
  unsigned long long ub = 0ull, vb = 0ull;
  M_ROWS({
    if (i < G.nx && j < G.ny) {
      ub = max(ub, abs_bits(U(j, i)));
      vb = max(vb, abs_bits(V(j, i)));
      const double d = div_central_unit(U, V, j, i, G.nx, G.ny);
      v[0] += d * d;
    }
  })
  for (int o = 16; o > 0; o >>= 1) {
    ub = max(ub, __shfl_xor_sync(0xffffffffu, ub, o));
    vb = max(vb, __shfl_xor_sync(0xffffffffu, vb, o));
  }
  if ((threadIdx.x & 31) == 0) {
    if (ub) atomicMax(&ctrl->umax_bits, ub);
    if (vb) atomicMax(&ctrl->vmax_bits, vb);
  }
  if (STEP_RED(1, v, out) && threadIdx.x == 0) {
    const double um = __longlong_as_double((long long)*(volatile unsigned long long*)&ctrl->umax_bits);
    const double vm = __longlong_as_double((long long)*(volatile unsigned long long*)&ctrl->vmax_bits);
    ctrl->umax = ADD(um, 1e-12);
    ctrl->vmax = ADD(vm, 1e-12);
    ctrl->umax_bits = 0ull;
    ctrl->vmax_bits = 0ull;
    D.slots[S_DIVC_BEFORE].result = out[0];
    ctrl->div_before = sqrt(out[0]);
    dt_one(D);     // the instance's dt, CFL and safeguard (k_dt of the binary64 form)
  }
}

// Predictor of the mixed form: the convective derivative in binary32 on
// binary32 copies of u and v, the update u* = u - dt conv in binary64.  The
// rounding of the inputs perturbs conv by about eps32 |f| / dx, so dt conv by
// about CFL eps32 |f| (CFL <= 0.5): a few 1e-8 of the field, inside the 1e-6 the
// mixed form is held to.  Same stencils, clamping and sign tests as advection.py.
__device__ __forceinline__ float q_comb(float dp, float d0, float dm, bool pos) {
  // phi_e - phi_w of the QUICK interpolants from the three face differences
  return pos ? (0.375f * dp + 0.75f * d0) - 0.125f * dm : (0.375f * dm + 0.75f * d0) - 0.125f * dp;
}

__global__ void __launch_bounds__(NT) k_predict_m(const InstDesc* __restrict__ ID, const Tile* __restrict__ TL) {
  TILE_PROLOGUE
  __shared__ float su[TY_M + 4][TX + 4], sv[TY_M + 4][TX + 4];
  const int i0 = tl.i0, j0 = tl.j0;
  View2<const double> U{D.ui, G.lds}, V{D.vi, G.lds};
  const int L = G.nx - 1, T = G.ny - 1;
  // u and v as binary32 on a 2-cell halo; outside the grid the clamped (edge-padded) values
  for (int idx = threadIdx.x; idx < (TY_M + 4) * (TX + 4); idx += NT) {
    const int jj = idx / (TX + 4) - 2, ii = idx % (TX + 4) - 2;
    const int gj = clampi(j0 + jj, 0, T), gi = clampi(i0 + ii, 0, L);
    su[jj + 2][ii + 2] = d2f_rn(U(gj, gi));      // the conversions on the integer pipe (icvt.cuh)
    sv[jj + 2][ii + 2] = d2f_rn(V(gj, gi));
  }
  __syncthreads();
  const double dt = D.ctrl->dt;
  const float rdx = (float)G.rdx, rdy = (float)G.rdy;
  const int i = i0 + (threadIdx.x & 31);
  const int tx = threadIdx.x & 31;
  double ub[PB_R], vb[PB_R];
#pragma unroll
  for (int r = 0; r < PB_R; ++r) {
    const int j = j0 + (threadIdx.x >> 5) + r * PB_Y;
    const bool in = i < G.nx && j < G.ny;
    ub[r] = in ? U(j, i) : 0.0;
    vb[r] = in ? V(j, i) : 0.0;
  }
  double* __restrict__ us = D.us;
  double* __restrict__ vs = D.vs;
#pragma unroll
  for (int r_ = 0; r_ < PB_R; ++r_) {
    const int j = j0 + (threadIdx.x >> 5) + r_ * PB_Y;
    if (i < G.nx && j < G.ny) {
      const int lj = j - j0 + 2, li = tx + 2;
      const double u0 = ub[r_], v0 = vb[r_];
      double un = u0, vn = v0;
      if (D.scheme != 2) {
        const float uc = su[lj][li], vc = sv[lj][li];
        float cu, cv;
        if (D.scheme == 1) {
          auto conv = [&](float (*f)[TX + 4]) {
            // clamped neighbours: the staged halo already holds the edge values
            const float fx_p = f[lj][li + 1] - f[lj][li], fx_0 = f[lj][li] - f[lj][li - 1],
                        fx_m = f[lj][li - 1] - f[lj][li - 2];
            const float fy_p = f[lj + 1][li] - f[lj][li], fy_0 = f[lj][li] - f[lj - 1][li],
                        fy_m = f[lj - 1][li] - f[lj - 2][li];
            return uc * q_comb(fx_p, fx_0, fx_m, uc >= 0.f) * rdx + vc * q_comb(fy_p, fy_0, fy_m, vc >= 0.f) * rdy;
          };
          cu = conv(su);
          cv = conv(sv);
        } else {
          auto conv = [&](float (*f)[TX + 4]) {
            const float f0 = f[lj][li];
            const float fx = (uc > 0.f) ? ((i > 0) ? f0 - f[lj][li - 1] : 0.f) : f[lj][li + 1] - f0;
            const float fy = (vc > 0.f) ? ((j > 0) ? f0 - f[lj - 1][li] : 0.f) : f[lj + 1][li] - f0;
            return uc * (fx * rdx) + vc * (fy * rdy);
          };
          cu = conv(su);
          cv = conv(sv);
        }
        un = SUB(u0, MUL(dt, f2d(cu)));
        vn = SUB(v0, MUL(dt, f2d(cv)));
      }
      us[(long)j * D.usld + i] = un;
      vs[(long)j * D.usld + i] = vn;
    }
  }
}

// b = -div_c(u*, v*) / max(dt, 1e-14); sum(b) (for the mean) and ||div_c||^2
__global__ void __launch_bounds__(NT) k_rhs_m(const InstDesc* __restrict__ ID, const Tile* __restrict__ TL) {
  TILE_PROLOGUE
  __shared__ StepRed rsm;
  const int i = tl.i0 + (threadIdx.x & 31);
  const RecipGrid rg = recips(G);
  const double rdt = D.ctrl->rdtm;
  View2<const double> US{D.us, D.usld}, VS{D.vs, D.usld};
  double v[2] = {0.0, 0.0}, out[2];
  double dv[PB_R];
#pragma unroll
  for (int r = 0; r < PB_R; ++r) {
    const int j = tl.j0 + (threadIdx.x >> 5) + r * PB_Y;
    dv[r] = (i < G.nx && j < G.ny) ? div_c_r(US, VS, j, i, rg) : 0.0;
  }
  double* __restrict__ b = D.b;
#pragma unroll
  for (int r = 0; r < PB_R; ++r) {
    const int j = tl.j0 + (threadIdx.x >> 5) + r * PB_Y;
    if (i < G.nx && j < G.ny) {
      const double bv = MUL(-dv[r], rdt);
      b[(long)j * G.ld + i] = bv;
      v[0] += bv;
      v[1] += dv[r] * dv[r];
    }
  }
  if (STEP_RED(2, v, out) && threadIdx.x == 0) {
    D.slots[S_BSUM].result = out[0];
    D.slots[S_DIVSTAR].result = out[1];
  }
}

// Append this step's Ru (sqrt(sum (u - u_old)^2) / max(1, N), as the host forms it) to
// the instance's series and run the steady-state test on the last `window` entries.
__device__ __noinline__ void steady_update(const InstDesc& Dd, double ru2, StepOut64* out) {
  SteadyRing* sr = Dd.steady;
  out->steady = 0;
  out->steady_slope = __longlong_as_double(0x7ff8000000000000LL);
  if (!sr || Dd.mode != 0) return;
  const int W = sr->window;
  if (W <= 0) return;
  const double n = fmax(1.0, Dd.A.n_cells);
  const double ru = sqrt(ru2) / n;
  const int k = sr->count;
  sr->y[k % STEADY_MAX_WINDOW] = ru > 0.0 ? log10(ru) : __longlong_as_double(0x7ff8000000000000LL);
  sr->count = k + 1;
  if (k + 1 < W) return;
  double sy = 0.0, sxy = 0.0;
  bool ok = true;
  for (int m = 0; m < W; ++m) {
    const double v = sr->y[(k - W + 1 + m) % STEADY_MAX_WINDOW];
    ok = ok && (v == v);
    sy += v;
    sxy = fma((double)m, v, sxy);
  }
  if (!ok) return;
  // sum (x - xm)^2 over x = 0 .. W - 1 is W (W^2 - 1) / 12
  const double w = (double)W, xm = 0.5 * (w - 1.0), sxx = w * (w * w - 1.0) / 12.0;
  const double slope = (sxy - xm * sy) / sxx;
  out->steady_slope = slope;
  out->steady = fabs(slope) < sr->tol ? 1 : 0;
}

// one StepOut64 record of instance Dd for the host
__device__ __forceinline__ void gather_one(const InstDesc& Dd, const int* trip, const int* gb_err) {
  const XASlot* slots = Dd.slots;
  const Ctrl64* ctrl = Dd.ctrl;
  StepOut64* out = Dd.out;
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
  out->loop_status = (*trip ? 1 : 0) | ((gb_err && *gb_err) ? 2 : 0);
  steady_update(Dd, out->ru2, out);
}

// The correction and the step's closing diagnostics of the mixed form, in one pass:
// p = x - x[0]; u* = u* - dt gx(p), v* likewise (the products with the reciprocal
// spacings); the lid; the state u, v, p; the sums of (u - u_old)^2 and (v - v_old)^2;
// then ||div_c(u*, v*)||^2 of the corrected u* and ||div_central(u, v; 1, 1)||^2 of the
// new state, the solve's summary and the step record.  The divergences read the
// corrected fields on the tile's one-cell ring too: those are formed here again from x
// and the predictor's u*, v* with the operations of their own tile, so no second pass
// is needed, and the corrected u* is not written back (nothing reads it after the
// diagnostics).  Every sum is accumulated and reduced as the two passes did.
constexpr int CD_W = TX + 3;                  // x on columns i0-1 .. i0+33
__global__ void __launch_bounds__(NT, 3) k_correct_diag_m(const InstDesc* __restrict__ ID, const Tile* __restrict__ TL,
                                                          const mixed::MixDesc* __restrict__ MD, const int* trip,
                                                          const int* gb_err) {
  TILE_PROLOGUE
  __shared__ double sx[TY_M + 3][CD_W];       // x - x[0] at rows j0-1 .. j0+33, columns i0-1 .. i0+33
  __shared__ double su[TY_M][TX + 2];         // corrected u*, rows j0 .. j0+31, columns i0-1 .. i0+32
  __shared__ double sv[TY_M + 2][TX];         // corrected v*, rows j0-1 .. j0+32, columns i0 .. i0+31
  __shared__ StepRed rsm;
  Ctrl64* ctrl = D.ctrl;
  const LidArgs L = D.L;
  const RecipGrid rg = recips(G);
  const int i0 = tl.i0, j0 = tl.j0;
  const int tx = threadIdx.x & 31, i = i0 + tx;
  const double dt = ctrl->dt;
  const double* __restrict__ xs = D.x;
  const double* __restrict__ us = D.us;
  const double* __restrict__ vs = D.vs;
  double* __restrict__ ui = D.ui;
  double* __restrict__ vi = D.vi;
  double* __restrict__ pi = D.pi;
  const double x0 = xs[0];
  for (int idx = threadIdx.x; idx < (TY_M + 3) * CD_W; idx += NT) {
    const int jj = idx / CD_W - 1, ii = idx % CD_W - 1;
    const int gj = j0 + jj, gi = i0 + ii;
    sx[jj + 1][ii + 1] = (gj >= 0 && gj < G.ny && gi >= 0 && gi < G.nx) ? SUB(xs[(long)gj * G.ld + gi], x0) : 0.0;
  }
  __syncthreads();
  // the correction at (j, c) of a cell whose x - x[0] (the pinned pressure, formed
  // once per staged cell) is at sx[j - j0 + 1][c - i0 + 1]
  auto ucorr = [&](int j, int c, double u1) {
    const double pv = sx[j - j0 + 1][c - i0 + 1];
    const double gx = (c < G.nx - 1) ? MUL(SUB(sx[j - j0 + 1][c - i0 + 2], pv), rg.rx) : 0.0;
    return SUB(u1, MUL(dt, gx));
  };
  auto vcorr = [&](int j, int c, double v1) {
    const double pv = sx[j - j0 + 1][c - i0 + 1];
    const double gy = (j < G.ny - 1) ? MUL(SUB(sx[j - j0 + 2][c - i0 + 1], pv), rg.ry) : 0.0;
    return SUB(v1, MUL(dt, gy));
  };
  double v[2] = {0.0, 0.0};
  int bad = 0;
#pragma unroll 1
  for (int h = 0; h < PB_R; h += 2) {
    double u1[2], v1[2], u0[2], v0[2];
    bool in[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int j = j0 + (threadIdx.x >> 5) + (h + r) * PB_Y;
      in[r] = i < G.nx && j < G.ny;
      if (in[r]) {
        const long o = (long)j * D.usld + i, os = (long)j * G.lds + i;
        u1[r] = us[o];
        v1[r] = vs[o];
        u0[r] = ui[os];
        v0[r] = vi[os];
      }
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int j = j0 + (threadIdx.x >> 5) + (h + r) * PB_Y;
      if (in[r]) {
        const double pv = sx[j - j0 + 1][tx + 1];
        const double uc = ucorr(j, i, u1[r]);
        const double vc = vcorr(j, i, v1[r]);
        su[j - j0][tx + 1] = uc;
        sv[j - j0 + 1][tx] = vc;
        const long os = (long)j * G.lds + i;
        pi[os] = pv;
        const double uf = (L.has_lid && j == G.ny - 1) ? L.lid : uc;
        const double du = SUB(uf, u0[r]);
        const double dv = SUB(vc, v0[r]);
        ui[os] = uf;
        vi[os] = vc;
        v[0] += du * du;
        v[1] += dv * dv;
        bad |= !(isfinite_d(uf) && isfinite_d(vc) && isfinite_d(pv));
      }
    }
  }
  // the ring: u* of columns i0-1 and i0+32, v* of rows j0-1 and j0+32 (threads 0..127)
  if (threadIdx.x < 4 * 32) {
    const int side = threadIdx.x >> 5, k = threadIdx.x & 31;
    if (side < 2) {
      const int c = side == 0 ? i0 - 1 : i0 + TX, j = j0 + k;
      if (c >= 0 && c < G.nx && j < G.ny) su[k][side == 0 ? 0 : TX + 1] = ucorr(j, c, us[(long)j * D.usld + c]);
    } else {
      const int j = side == 2 ? j0 - 1 : j0 + TY_M, c = i0 + k;
      if (j >= 0 && j < G.ny && c < G.nx) sv[side == 2 ? 0 : TY_M + 1][k] = vcorr(j, c, vs[(long)j * D.usld + c]);
    }
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&ctrl->nan_flag, 1u);
  // the divergences of the corrected fields (u* before the lid, the state after it)
  struct SU {
    const double (*a)[TX + 2];
    int j0, i0;
    __device__ double operator()(int j, int c) const { return a[j - j0][c - i0 + 1]; }
  };
  struct SV {
    const double (*a)[TX];
    int j0, i0;
    __device__ double operator()(int j, int c) const { return a[j - j0 + 1][c - i0]; }
  };
  struct SUL {
    SU s;
    int top, lid_on;
    double lid;
    __device__ double operator()(int j, int c) const { return (lid_on && j == top) ? lid : s(j, c); }
  };
  const SU US{su, j0, i0};
  const SV VS{sv, j0, i0};
  const SUL U{US, G.ny - 1, L.has_lid, L.lid};
  double w[2] = {0.0, 0.0};
  M_ROWS({
    if (i < G.nx && j < G.ny) {
      const double xp = (i >= 1) ? MUL(SUB(US(j, i), US(j, i - 1)), rg.rx) : MUL(US(j, 0), rg.rx);
      const double yp = (j >= 1) ? MUL(SUB(VS(j, i), VS(j - 1, i)), rg.ry) : MUL(VS(0, i), rg.ry);
      const double d = ADD(xp, yp);
      const double c = div_central_unit(U, VS, j, i, G.nx, G.ny);
      w[0] += d * d;
      w[1] += c * c;
    }
  })
  // the two pairs of sums, each formed as a two-value reduction, with one arrival
  dred_block<2, NT>(mixed::CtaCtx{}, v, rsm);
  dred_block<2, NT>(mixed::CtaCtx{}, w, rsm);
  double* part = D.part;
  const int nt = D.nt_m;
  if (threadIdx.x == 0) {
    part[tl.loc] = v[0];
    part[nt + tl.loc] = v[1];
    part[2 * nt + tl.loc] = w[0];
    part[3 * nt + tl.loc] = w[1];
    __threadfence();
    rsm.last = (atomicAdd(D.ticket, 1u) == (unsigned)(nt - 1)) ? 1 : 0;
  }
  __syncthreads();
  if (!rsm.last) return;
  __threadfence();
  double s1[2] = {0.0, 0.0}, s2[2] = {0.0, 0.0};
  for (int k = threadIdx.x; k < nt; k += NT) {
    s1[0] += __ldcg(&part[k]);
    s1[1] += __ldcg(&part[nt + k]);
    s2[0] += __ldcg(&part[2 * nt + k]);
    s2[1] += __ldcg(&part[3 * nt + k]);
  }
  dred_block<2, NT>(mixed::CtaCtx{}, s1, rsm);
  dred_block<2, NT>(mixed::CtaCtx{}, s2, rsm);
  if (threadIdx.x == 0) {
    atomicExch(D.ticket, 0u);
    // the instance's last tile: the solve's summary, the norms, then its step record
    D.slots[S_RU].result = s1[0];
    D.slots[S_RV].result = s1[1];
    mixed::mx_finish_one(MD[tl.inst]);
    D.slots[S_DIVAFTER].result = s2[0];
    // ||A p - b||^2: p is the refinement's x exactly (x[0] stays 0), so this is the
    // refinement's final binary64 residual, which the solve has already formed
    D.slots[S_LINRES].result = D.slots[S_RES].result;
    D.slots[S_CONT].result = s2[1];
    __threadfence();
    gather_one(D, trip, gb_err);
  }
}

// one StepOut64 record per instance
__global__ void k_gather(const InstDesc* __restrict__ ID, int n, const int* trip, const int* gb_err) {
  pdl_enter();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const InstDesc& Dd = ID[k];
  if (!Dd.active) return;
  gather_one(Dd, trip, gb_err);
}

// ---------------------------------------------------------------------------
// Host driver of one instance.


static long round_up(long a, long m) { return (a + m - 1) / m * m; }

static Spacing make_spacing(double h) { return spacing_for(h); }

// tiles of height th covering an nx x ny grid of instance k
static void add_tiles(std::vector<Tile>& v, int k, int nx, int ny, int th) {
  int loc = 0;
  for (int j0 = 0; j0 < ny; j0 += th)
    for (int i0 = 0; i0 < nx; i0 += TX) v.push_back(Tile{k, i0, j0, loc++});
}

static int count_tiles(int nx, int ny, int th) { return ((nx + TX - 1) / TX) * ((ny + th - 1) / th); }

// Per-tile partial sums of an instance: three rows over its 32 x 8 tiles (the binary64
// stages), four rows over its 32 x 32 tiles (the mixed form's correction and diagnostics).
static size_t part_doubles(int nx, int ny) {
  return std::max(3 * (size_t)count_tiles(nx, ny, PB_Y), 4 * (size_t)count_tiles(nx, ny, TY_M));
}

constexpr int NVAR = 3;                          // CG tile variants: rows per thread 1, 2, 4
constexpr int VAR_R[NVAR] = {1, 2, 4};

static Geo64 make_geo(int nx, int ny, long ld, double dx, double dy, double invd, int jacobi) {
  Geo64 G;
  G.nx = nx;
  G.ny = ny;
  G.ld = ld;
  G.lds = nx + 2;
  G.g.nx = nx;
  G.g.ny = ny;
  G.g.sx = make_spacing(dx);
  G.g.sy = make_spacing(dy);
  G.invd = invd;
  G.jacobi = jacobi;
  G.rdx = 1.0 / dx;
  G.rdy = 1.0 / dy;
  return G;
}

// A batch of n independent cavity instances (n = 1 for a single cavity).
struct Instance64 {
  int n = 0;
  std::vector<pfgb_params> P;
  std::vector<InstDesc> hd;          // host copy of the descriptors
  InstDesc* dd = nullptr;            // device descriptors
  Tile* tpc = nullptr;               // per-cell tiles (32 x 8)
  Tile* tpcm = nullptr;              // per-cell tiles of the mixed form (32 x 32)
  int ntpcm = 0;
  Tile* tcg = nullptr;               // CG tiles of the selected variant
  int ntpc = 0, ntcg = 0;
  // CG tile variants 32 x 8R (R = 1, 2, 4 rows per thread); the autotuner selects one
  Tile* tcgv[NVAR] = {};
  int ntcgv[NVAR] = {};
  std::vector<int> ntcg_inst[NVAR];  // per-instance CG tile counts of each variant
  int cg_var = 1;
  LoopCtl* lc = nullptr;
  int maxiter_max = 0;
  char* ws = nullptr;
  size_t ws_bytes = 0;
  StepIn* in_d = nullptr;
  StepIn* in_h = nullptr;            // pinned staging of the per-step inputs
  StepOut64* out_d = nullptr;
  StepOut64* out_h = nullptr;
  bool desc_dirty = true;
  // mixed-precision pressure solve of every instance (precision 1)
  mixed::Batch* mix = nullptr;
  // the whole step as one CUDA graph (CG loop = WHILE conditional node)
  int use_graph = 1;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_mode = -1;               // 0 step, 1 projection
  // per-kernel timing of the following steps (benchmark profiling; direct launches)
  int profiling = 0;
  KProf kp;
  KProf* prof() { return profiling ? &kp : nullptr; }
};

// where the step's loop guards report, and the bounded waits (the persistent solve's
// barrier, the TMA matvec's copies)
static const int* loop_trip(const Instance64* I) { return I->mix ? &I->mix->loop->tripped : &I->lc->tripped; }
static const int* loop_gb_err(const Instance64* I) { return I->mix ? &I->mix->loop->gb.err : nullptr; }

static int validate_params(const pfgb_params* prm) {
  if (prm->nx < 2 || prm->ny < 2) return set_error(PFGB_EINVAL, "nx and ny must be >= 2 (the reference's central divergence indexes two columns and rows)");
  if (prm->nx > (1 << 20) || prm->ny > (1 << 20)) return set_error(PFGB_EINVAL, "grid side above 2^20");
  if (!(prm->dx > 0.0) || !(prm->dy > 0.0)) return set_error(PFGB_EINVAL, "dx and dy must be positive");
  if (prm->lin_maxiter < 0) return set_error(PFGB_EINVAL, "lin_maxiter must be >= 0");
  return PFGB_OK;
}

int instance64_create_batch(const pfgb_params* prms, int n, Instance64** out) {
  if (n < 1) return set_error(PFGB_EINVAL, "batch size must be >= 1");
  for (int k = 0; k < n; ++k)
    if (int rc = validate_params(&prms[k])) return rc;
  for (int k = 1; k < n; ++k)
    if (prms[k].precision != prms[0].precision) return set_error(PFGB_EINVAL, "all instances of a batch share one precision");
  Instance64* I = new Instance64();
  I->n = n;
  I->P.assign(prms, prms + n);
  I->hd.resize(n);
  // workspace layout: per instance 8 vectors + slots + ctrl; then descriptors, tiles, loop control, in/out
  std::vector<size_t> vec(n);
  size_t bytes = 0;
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  std::vector<Tile> tpc, tpcm, tcgv[NVAR];
  for (int k = 0; k < n; ++k) {
    const long ld = round_up(prms[k].nx, 32);
    vec[k] = up((size_t)ld * prms[k].ny * sizeof(double));
    bytes += 9 * vec[k] + up(S_COUNT * sizeof(XASlot)) + up(sizeof(Ctrl64)) + up(sizeof(SteadyRing)) +
             up(part_doubles(prms[k].nx, prms[k].ny) * sizeof(double)) + up(sizeof(unsigned));
    add_tiles(tpc, k, prms[k].nx, prms[k].ny, PB_Y);
    add_tiles(tpcm, k, prms[k].nx, prms[k].ny, TY_M);
    for (int v = 0; v < NVAR; ++v) {
      add_tiles(tcgv[v], k, prms[k].nx, prms[k].ny, VAR_R[v] * PB_Y);
      I->ntcg_inst[v].push_back(count_tiles(prms[k].nx, prms[k].ny, VAR_R[v] * PB_Y));
    }
    I->maxiter_max = std::max(I->maxiter_max, prms[k].lin_maxiter);
  }
  I->ntpc = (int)tpc.size();
  I->ntpcm = (int)tpcm.size();
  bytes += up(n * sizeof(InstDesc)) + up(tpc.size() * sizeof(Tile)) + up(tpcm.size() * sizeof(Tile)) +
           up(sizeof(LoopCtl)) + up(n * sizeof(StepIn)) + up(n * sizeof(StepOut64));
  for (int v = 0; v < NVAR; ++v) {
    I->ntcgv[v] = (int)tcgv[v].size();
    bytes += up(tcgv[v].size() * sizeof(Tile));
  }
  if (cudaMalloc(&I->ws, bytes) != cudaSuccess) {
    delete I;
    return set_error(PFGB_ENOMEM, "cudaMalloc of the workspace failed");
  }
  I->ws_bytes = bytes;
  if (cudaMemset(I->ws, 0, bytes) != cudaSuccess) {
    cudaFree(I->ws);
    delete I;
    return set_error(PFGB_ECUDA, "cudaMemset of the workspace failed");
  }
  char* c = I->ws;
  auto take = [&](size_t b) { char* r = c; c += up(b); return r; };
  for (int k = 0; k < n; ++k) {
    const pfgb_params& prm = prms[k];
    InstDesc& D = I->hd[k];
    const long ld = round_up(prm.nx, 32);
    D.G = make_geo(prm.nx, prm.ny, ld, prm.dx, prm.dy, prm.jacobi_interior, prm.enable_jacobi);
    D.A.rtol = prm.lin_tol;
    D.A.maxiter = prm.lin_maxiter;
    D.A.n_cells = (double)prm.nx * (double)prm.ny;
    D.D.dx = prm.dx;
    D.D.dy = prm.dy;
    D.D.cfl_target = prm.cfl_target;
    D.D.growth = prm.cfl_growth;
    D.D.nu = prm.nu;
    D.L.has_lid = prm.has_lid;
    D.L.lid = prm.lid_velocity;
    D.scheme = prm.scheme;
    D.adjust = 1;
    D.mode = 0;
    D.active = 1;
    D.ui = D.vi = D.pi = nullptr;
    D.us = (double*)take(vec[k]);
    D.vs = (double*)take(vec[k]);
    D.usld = ld;
    D.b = (double*)take(vec[k]);
    D.x = (double*)take(vec[k]);
    D.r = (double*)take(vec[k]);
    D.p0 = (double*)take(vec[k]);
    D.p1 = (double*)take(vec[k]);
    D.q = (double*)take(vec[k]);
    D.z = (double*)take(vec[k]);
    D.slots = (XASlot*)take(S_COUNT * sizeof(XASlot));
    D.ctrl = (Ctrl64*)take(sizeof(Ctrl64));
    D.nt_pc = count_tiles(prm.nx, prm.ny, PB_Y);
    D.nt_m = count_tiles(prm.nx, prm.ny, TY_M);
    D.nt_cg = I->ntcg_inst[I->cg_var][k];
    D.part = (double*)take(part_doubles(prm.nx, prm.ny) * sizeof(double));
    D.ticket = (unsigned*)take(sizeof(unsigned));
    D.steady = (SteadyRing*)take(sizeof(SteadyRing));   // zeroed: the test is off
  }
  I->dd = (InstDesc*)take(n * sizeof(InstDesc));
  I->tpc = (Tile*)take(tpc.size() * sizeof(Tile));
  I->tpcm = (Tile*)take(tpcm.size() * sizeof(Tile));
  for (int v = 0; v < NVAR; ++v) I->tcgv[v] = (Tile*)take(tcgv[v].size() * sizeof(Tile));
  I->tcg = I->tcgv[I->cg_var];
  I->ntcg = I->ntcgv[I->cg_var];
  I->lc = (LoopCtl*)take(sizeof(LoopCtl));
  I->in_d = (StepIn*)take(n * sizeof(StepIn));
  I->out_d = (StepOut64*)take(n * sizeof(StepOut64));
  for (int k = 0; k < n; ++k) {
    I->hd[k].in = I->in_d + k;
    I->hd[k].out = I->out_d + k;
  }
  cudaError_t e = cudaMemcpy(I->tpc, tpc.data(), tpc.size() * sizeof(Tile), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(I->tpcm, tpcm.data(), tpcm.size() * sizeof(Tile), cudaMemcpyHostToDevice);
  for (int v = 0; v < NVAR; ++v)
    if (e == cudaSuccess) e = cudaMemcpy(I->tcgv[v], tcgv[v].data(), tcgv[v].size() * sizeof(Tile), cudaMemcpyHostToDevice);
  LoopCtl lc0 = {0, 0, I->maxiter_max + 1, 0};
  if (e == cudaSuccess) e = cudaMemcpy(I->lc, &lc0, sizeof(LoopCtl), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMallocHost(&I->out_h, n * sizeof(StepOut64));
  if (e == cudaSuccess) e = cudaMallocHost(&I->in_h, n * sizeof(StepIn));
  if (e != cudaSuccess) {
    instance64_destroy(I);
    return set_error(PFGB_ECUDA, std::string("batch set-up: ") + cudaGetErrorString(e));
  }
  if (prms[0].precision == 1) {
    std::vector<mixed::MixParams> mp(n);
    for (int k = 0; k < n; ++k) {
      const pfgb_params& prm = prms[k];
      mixed::MixParams& m = mp[k];
      m.nx = prm.nx;
      m.ny = prm.ny;
      m.dx = prm.dx;
      m.dy = prm.dy;
      m.ld64 = I->hd[k].G.ld;
      m.tol_out = prm.mixed_tol_outer > 0.0 ? prm.mixed_tol_outer : prm.lin_tol;
      m.tol_in = prm.mixed_tol_inner > 0.0 ? prm.mixed_tol_inner : 1e-5;
      m.max_outer = prm.mixed_max_outer > 0 ? prm.mixed_max_outer : 8;
      m.max_inner = prm.mixed_max_inner > 0 ? prm.mixed_max_inner : 50;
      m.b = I->hd[k].b;
      m.bsum = &I->hd[k].slots[S_BSUM].result;
      m.res_out = &I->hd[k].slots[S_RES].result;
      m.x = I->hd[k].x;
      // the pressure field of the bound state, read through the descriptor (rebound every step)
      m.pprev = reinterpret_cast<const double* const*>(reinterpret_cast<const char*>(I->dd + k) + offsetof(InstDesc, pi));
      m.ldp = I->hd[k].G.lds;
      m.warm = prm.mixed_cold_start ? 0 : 1;
      m.ctrl64 = I->hd[k].ctrl;
      // the instance's activity flag inside the device descriptor table
      m.active = reinterpret_cast<const int*>(reinterpret_cast<const char*>(I->dd + k) + offsetof(InstDesc, active));
      m.maxiter_report = prm.lin_maxiter;
    }
    int rc = mixed::batch_create(mp.data(), n, &I->mix);
    if (rc) {
      instance64_destroy(I);
      return rc;
    }
  }
  *out = I;
  return PFGB_OK;
}

int instance64_create(const pfgb_params* prm, Instance64** out) { return instance64_create_batch(prm, 1, out); }

void instance64_destroy(Instance64* I) {
  if (!I) return;
  if (I->mix) mixed::batch_destroy(I->mix);
  if (I->exec) cudaGraphExecDestroy(I->exec);
  if (I->graph) cudaGraphDestroy(I->graph);
  if (I->ws) cudaFree(I->ws);
  if (I->out_h) cudaFreeHost(I->out_h);
  if (I->in_h) cudaFreeHost(I->in_h);
  delete I;
}

size_t instance64_workspace_bytes(const Instance64* I) {
  return I->ws_bytes + (I->mix ? I->mix->ws_bytes : 0);
}

int instance64_count(const Instance64* I) { return I->n; }

// Point instance k at its state arrays and mark the descriptors for upload.
static int bind_state(Instance64* I, int k, double* u, double* v, double* p, long lds, int mode, int active) {
  InstDesc& D = I->hd[k];
  if (active && lds != D.G.lds) return set_error(PFGB_EINVAL, "state pitch must be nx + 2");
  double* ui = active ? u + lds + 1 : nullptr;   // interior pointers of the ghosted state arrays
  double* vi = active ? v + lds + 1 : nullptr;
  double* pi = active ? p + lds + 1 : nullptr;
  double* us = mode == 0 ? D.us : ui;            // projection only: correct the state in place
  double* vs = mode == 0 ? D.vs : vi;
  const long usld = mode == 0 ? D.G.ld : lds;
  if (D.ui != ui || D.vi != vi || D.pi != pi || D.mode != mode || D.active != active || D.usld != usld ||
      (mode == 1 && (D.us != us || D.vs != vs))) {
    D.ui = ui;
    D.vi = vi;
    D.pi = pi;
    D.mode = mode;
    D.active = active;
    if (mode == 1) {
      D.us = us;
      D.vs = vs;
    }
    D.usld = usld;
    I->desc_dirty = true;
  }
  return PFGB_OK;
}

static int upload_desc(Instance64* I, cudaStream_t s) {
  if (!I->desc_dirty) return PFGB_OK;
  cudaError_t e = cudaMemcpyAsync(I->dd, I->hd.data(), I->n * sizeof(InstDesc), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("descriptor upload: ") + cudaGetErrorString(e));
  // the host array may change before the copy runs: wait for it
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("descriptor upload: ") + cudaGetErrorString(e));
  I->desc_dirty = false;
  return PFGB_OK;
}

__global__ void k_loop_reset(LoopCtl* lc) {
  pdl_enter();
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    lc->active = 0;
    lc->guard = 0;
    lc->tripped = 0;
  }
}

// The CG kernel pair of tile variant var.
template <int OP>
static void launch_matvec(int var, int grid, cudaStream_t s, const InstDesc* dd, const Tile* t) {
  if (var == 0) k_cg_matvec<OP, 1><<<grid, NT, 0, s>>>(dd, t);
  else if (var == 2) k_cg_matvec<OP, 4><<<grid, NT, 0, s>>>(dd, t);
  else k_cg_matvec<OP, 2><<<grid, NT, 0, s>>>(dd, t);
}
static void launch_update(int var, int grid, cudaStream_t s, const InstDesc* dd, const Tile* t) {
  if (var == 0) k_cg_update<1><<<grid, NT, 0, s>>>(dd, t, nullptr, 0ull, 0);
  else if (var == 2) k_cg_update<4><<<grid, NT, 0, s>>>(dd, t, nullptr, 0ull, 0);
  else k_cg_update<2><<<grid, NT, 0, s>>>(dd, t, nullptr, 0ull, 0);
}

// Direct launches of the projection stage (host loop bound = largest maxiter).
static void enqueue_projection(Instance64* I, cudaStream_t s) {
  KProf* kp = I->prof();
  PFGB_TIMED(kp, "k_rhs", -1, s, k_rhs<<<I->ntpc, NT, 0, s>>>(I->dd, I->tpc));
  PFGB_TIMED(kp, "k_cg_init", -1, s, k_cg_init<<<I->ntpc, NT, 0, s>>>(I->dd, I->tpc, nullptr));
  for (int k = 0; k < I->maxiter_max; ++k) {
    PFGB_TIMED(kp, "k_cg_matvec", -1, s, launch_matvec<0>(I->cg_var, I->ntcg, s, I->dd, I->tcg));
    PFGB_TIMED(kp, "k_cg_update", -1, s, launch_update(I->cg_var, I->ntcg, s, I->dd, I->tcg));
  }
  PFGB_TIMED(kp, "k_post_resid", -1, s, k_post_resid<0><<<I->ntpc, NT, 0, s>>>(I->dd, I->tpc));
  PFGB_TIMED(kp, "k_pin_correct", -1, s, k_pin_correct<<<I->ntpc, NT, 0, s>>>(I->dd, I->tpc));
  PFGB_TIMED(kp, "k_post_diag", -1, s, k_post_diag<<<I->ntpc, NT, 0, s>>>(I->dd, I->tpc));
  PFGB_TIMED(kp, "k_gather", -1, s, k_gather<<<(I->n + 31) / 32, 32, 0, s>>>(I->dd, I->n, loop_trip(I), loop_gb_err(I)));
}

static void enqueue_prologue(Instance64* I, cudaStream_t s) {
  KProf* kp = I->prof();
  if (I->mix) PFGB_TIMED(kp, "k_prestep_m", -1, s, k_prestep_m<<<I->ntpcm, NT, 0, s>>>(I->dd, I->tpcm));
  else PFGB_TIMED(kp, "k_prestep", -1, s, k_prestep<<<I->ntpc, NT, 0, s>>>(I->dd, I->tpc));
  if (!I->mix) PFGB_TIMED(kp, "k_dt", -1, s, k_dt<<<(I->n + 31) / 32, 32, 0, s>>>(I->dd, I->n));
  if (I->mix) PFGB_TIMED(kp, "k_predict_m", -1, s, k_predict_m<<<I->ntpcm, NT, 0, s>>>(I->dd, I->tpcm));
  else PFGB_TIMED(kp, "k_predict", -1, s, k_predict<<<I->ntpc, NT, 0, s>>>(I->dd, I->tpc));
}

// Build the step graph (mode 0: full step; mode 1: stand-alone projection).
static int build_graph(Instance64* I, int mode) {
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
  const dim3 gp(I->ntpc), gc(I->ntcg), g1((I->n + 31) / 32), gm(I->ntpcm);
  GraphChain c(I->graph, I->use_graph == 1);
  if (mode == 0) {
    if (I->mix) c.kernel(k_prestep_m, gm, dim3(NT), (const InstDesc*)I->dd, (const Tile*)I->tpcm);
    else c.kernel(k_prestep, gp, dim3(NT), (const InstDesc*)I->dd, (const Tile*)I->tpc);
    if (!I->mix) c.kernel(k_dt, g1, dim3(32), (const InstDesc*)I->dd, I->n);
    if (I->mix) c.kernel(k_predict_m, gm, dim3(NT), (const InstDesc*)I->dd, (const Tile*)I->tpcm);
    else c.kernel(k_predict, gp, dim3(NT), (const InstDesc*)I->dd, (const Tile*)I->tpc);
  }
  if (I->mix) c.kernel(k_rhs_m, gm, dim3(NT), (const InstDesc*)I->dd, (const Tile*)I->tpcm);
  else c.kernel(k_rhs, gp, dim3(NT), (const InstDesc*)I->dd, (const Tile*)I->tpc);
  GraphChain body(nullptr);
  if (I->mix) {
    // the refinement removes b's mean, pins b[0], solves A x = b and leaves ||b - A x||^2
    if (int rc = mixed::append_solve(c, I->mix)) return rc;
  } else {
    cudaGraphConditionalHandle cond = 0;
    // every conditional handle must belong to a conditional node: create it only here
    e = cudaGraphConditionalHandleCreate(&cond, I->graph, 0u, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("conditional handle: ") + cudaGetErrorString(e));
    c.kernel(k_loop_reset, dim3(1), dim3(32), I->lc);
    c.kernel(k_cg_init, gp, dim3(NT), (const InstDesc*)I->dd, (const Tile*)I->tpc, I->lc);
    c.kernel(k_loop_arm, dim3(1), dim3(32), I->lc, cond, 1);
    body = c.while_loop_with(cond);
    auto mv = I->cg_var == 0 ? k_cg_matvec<0, 1> : (I->cg_var == 2 ? k_cg_matvec<0, 4> : k_cg_matvec<0, 2>);
    auto up = I->cg_var == 0 ? k_cg_update<1> : (I->cg_var == 2 ? k_cg_update<4> : k_cg_update<2>);
    body.kernel(mv, gc, dim3(NT), (const InstDesc*)I->dd, (const Tile*)I->tcg);
    body.kernel(up, gc, dim3(NT), (const InstDesc*)I->dd, (const Tile*)I->tcg, I->lc, cond, 1);
    body.kernel(k_loop_guard, dim3(1), dim3(32), I->lc, cond, 1);
  }
  if (!I->mix) c.kernel(k_post_resid<0>, gp, dim3(NT), (const InstDesc*)I->dd, (const Tile*)I->tpc);
  if (I->mix) {
    c.kernel(k_correct_diag_m, gm, dim3(NT), (const InstDesc*)I->dd, (const Tile*)I->tpcm,
             (const mixed::MixDesc*)I->mix->dd, loop_trip(I), loop_gb_err(I));
  } else {
    c.kernel(k_pin_correct, gp, dim3(NT), (const InstDesc*)I->dd, (const Tile*)I->tpc);
    c.kernel(k_post_diag, gp, dim3(NT), (const InstDesc*)I->dd, (const Tile*)I->tpc);
  }
  if (!I->mix) c.kernel(k_gather, g1, dim3(32), (const InstDesc*)I->dd, I->n, loop_trip(I), loop_gb_err(I));
  if (c.status() != cudaSuccess || (!I->mix && body.status() != cudaSuccess)) {
    cudaError_t be = c.status() != cudaSuccess ? c.status() : body.status();
    return set_error(PFGB_ECUDA, std::string("building the step graph: ") + cudaGetErrorString(be));
  }
  if (std::getenv("PFGB_GRAPH_DEBUG"))
    std::fprintf(stderr, "pfgb graph: %d programmatic edges in the top chain; last refusal: %s\n", c.n_prog_,
                 cudaGetErrorString(c.last_prog_err_));
  e = cudaGraphInstantiate(&I->exec, I->graph, 0);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  I->graph_mode = mode;
  return PFGB_OK;
}

// Turn instance k's device-side steady-state test on (window >= 2 entries of the Ru
// series, slope tolerance tol) or off (window 0); either way its series restarts
// from the tracker's seed 1.0 (log10 = 0).
int instance64_set_steady(Instance64* I, int k, int window, double tol) {
  if (k < 0 || k >= I->n) return set_error(PFGB_EINVAL, "instance index out of range");
  if (window != 0 && (window < 2 || window > STEADY_MAX_WINDOW))
    return set_error(PFGB_EINVAL, "steady window must be 0 (off) or between 2 and 1024 steps");
  if (!(tol >= 0.0)) return set_error(PFGB_EINVAL, "steady slope tolerance must be >= 0");
  struct {
    int window, count;
    double tol, y0;
  } head = {window, 1, tol, 0.0};
  static_assert(offsetof(SteadyRing, y) == 2 * sizeof(int) + sizeof(double), "SteadyRing header layout");
  const cudaError_t e = cudaMemcpy(I->hd[k].steady, &head, sizeof(head), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("steady set-up: ") + cudaGetErrorString(e));
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
  out->steady = o.steady;
  out->steady_slope = o.steady_slope;
}

static int read_out(Instance64* I, cudaStream_t s, pfgb_step_out* out) {
  cudaError_t e = cudaMemcpyAsync(I->out_h, I->out_d, I->n * sizeof(StepOut64), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("step failed: ") + cudaGetErrorString(e));
  if (I->use_graph && !I->profiling) {
    // the loop status rides in the records (every active instance's carries the same word)
    int st = 0;
    for (int k = 0; k < I->n; ++k)
      if (I->hd[k].active) st |= I->out_h[k].loop_status;
    if (st & 2)
      return set_error(PFGB_ESTATE, "a bounded device wait gave up: the persistent solve's grid barrier (its CTAs "
                                    "were not co-resident) or the TMA matvec's wait for a halo copy");
    if (st & 1) return set_error(PFGB_ESTATE, "a loop guard stopped the step (an instance did not report completion)");
  }
  for (int k = 0; k < I->n; ++k)
    if (I->hd[k].active) copy_out(I->out_h[k], &out[k]);
  return PFGB_OK;
}

// A few tens of microseconds of device work ahead of the next launches (profiling:
// the first timed kernel then does not absorb the host's launch latency).
__global__ void k_pad64(float* sink, int n) {
  float x = (float)threadIdx.x;
  for (int i = 0; i < n; ++i) x = fmaf(x, 1.0000001f, 0.5f);
  if (x == -1.f) *sink = x;
}
static void pad_stream(Instance64* I, cudaStream_t s) {
  k_pad64<<<1, 32, 0, s>>>(reinterpret_cast<float*>(I->out_d), 20000);
}

// Run one step (mode 0) or projection (mode 1) for the bound instances.
static int run(Instance64* I, int mode, cudaStream_t s, pfgb_step_out* out) {
  if (int rc = upload_desc(I, s)) return rc;
  cudaError_t e = cudaMemcpyAsync(I->in_d, I->in_h, I->n * sizeof(StepIn), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("step input upload: ") + cudaGetErrorString(e));
  if (I->use_graph && !I->profiling) {
    if (!I->exec || I->graph_mode != mode)
      if (int rc = build_graph(I, mode)) return rc;
    e = cudaGraphLaunch(I->exec, s);
    if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("graph launch: ") + cudaGetErrorString(e));
    return read_out(I, s, out);
  }
  KProf* kp = I->prof();
  if (kp) {
    kp->clear();
    if (I->mix) I->mix->kp = kp;
    pad_stream(I, s);
  }
  if (mode == 0) enqueue_prologue(I, s);
  if (I->mix) {
    PFGB_TIMED(kp, "k_rhs_m", -1, s, k_rhs_m<<<I->ntpcm, NT, 0, s>>>(I->dd, I->tpcm));
    if (int rc = mixed::run_direct(I->mix, s)) return rc;
    PFGB_TIMED(kp, "k_correct_diag_m", -1, s,
               k_correct_diag_m<<<I->ntpcm, NT, 0, s>>>(I->dd, I->tpcm, I->mix->dd, loop_trip(I), loop_gb_err(I)));
  } else {
    enqueue_projection(I, s);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
  return read_out(I, s, out);
}

int instance64_step(Instance64* I, double* u, double* v, double* p, long lds, const StepIn& in, cudaStream_t s,
                    pfgb_step_out* out) {
  if (int rc = bind_state(I, 0, u, v, p, lds, 0, 1)) return rc;
  I->in_h[0] = in;
  return run(I, 0, s, out);
}

// Batch step: instance k uses us[k]... (null u[k] leaves instance k out of this step).
int instance64_batch_step(Instance64* I, double* const* u, double* const* v, double* const* p, const StepIn* in,
                          cudaStream_t s, pfgb_step_out* out) {
  for (int k = 0; k < I->n; ++k) {
    const int act = (u[k] && v[k] && p[k]) ? 1 : 0;
    if (int rc = bind_state(I, k, u[k], v[k], p[k], I->hd[k].G.lds, 0, act)) return rc;
    I->in_h[k] = in[k];
  }
  return run(I, 0, s, out);
}

// Stand-alone projection (solve_pressure_poisson, normal mode) on the state.
int instance64_project(Instance64* I, double* u, double* v, double* p, long lds, double dt, cudaStream_t s,
                       pfgb_step_out* out) {
  if (I->mix) return set_error(PFGB_ESTATE, "pfgb_project runs the binary64 path only");
  if (I->n != 1) return set_error(PFGB_ESTATE, "pfgb_project takes a single-instance handle");
  if (int rc = bind_state(I, 0, u, v, p, lds, 1, 1)) return rc;
  if (int rc = upload_desc(I, s)) return rc;
  k_set_dt<<<1, 32, 0, s>>>(I->dd, dt);
  return run(I, 1, s, out);
}

// New physical parameters for instance k of a batch (a new request in a slot).
// The grid (nx, ny, dx, dy), the precision and the preconditioner stay; the
// iteration limit may not exceed the batch's largest one (the loop guard).
int instance64_set_params(Instance64* I, int k, const pfgb_params* prm) {
  if (k < 0 || k >= I->n) return set_error(PFGB_EINVAL, "instance index out of range");
  const pfgb_params& o = I->P[k];
  if (prm->nx != o.nx || prm->ny != o.ny || prm->dx != o.dx || prm->dy != o.dy || prm->precision != o.precision ||
      prm->enable_jacobi != o.enable_jacobi || prm->jacobi_interior != o.jacobi_interior)
    return set_error(PFGB_EINVAL, "a slot keeps its grid, spacing, precision and preconditioner");
  if (prm->lin_maxiter < 0 || prm->lin_maxiter > I->maxiter_max)
    return set_error(PFGB_EINVAL, "lin_maxiter above the batch's largest");
  if (prm->scheme < 0 || prm->scheme > 2) return set_error(PFGB_EINVAL, "unknown advection scheme");
  if (I->mix) {
    const double tol_out = prm->mixed_tol_outer > 0.0 ? prm->mixed_tol_outer : prm->lin_tol;
    const double tol_in = prm->mixed_tol_inner > 0.0 ? prm->mixed_tol_inner : 1e-5;
    const int max_outer = prm->mixed_max_outer > 0 ? prm->mixed_max_outer : 8;
    const int max_inner = prm->mixed_max_inner > 0 ? prm->mixed_max_inner : 50;
    if (int rc = mixed::set_tolerances(I->mix, k, tol_out, tol_in, max_outer, max_inner, prm->mixed_cold_start ? 0 : 1,
                                       prm->lin_maxiter))
      return rc;
  }
  InstDesc& D = I->hd[k];
  D.A.rtol = prm->lin_tol;
  D.A.maxiter = prm->lin_maxiter;
  D.D.cfl_target = prm->cfl_target;
  D.D.growth = prm->cfl_growth;
  D.D.nu = prm->nu;
  D.L.has_lid = prm->has_lid;
  D.L.lid = prm->lid_velocity;
  D.scheme = prm->scheme;
  I->P[k] = *prm;
  I->desc_dirty = true;
  return PFGB_OK;
}

// ---- CG tile autotuner ----------------------------------------------------------
//
// The CG kernel pair (matvec + update) comes in three tile shapes, 32 x 8R cells
// with R = 1, 2, 4 rows per thread.  The exact reductions make the result
// independent of the shape, so the choice is free: the tuner times each
// variant on this handle's own instances and keeps the fastest.

__global__ void k_tune_fill(const InstDesc* __restrict__ ID, const Tile* __restrict__ TL) {
  TILE_PROLOGUE
  const int i = tl.i0 + (threadIdx.x & 31), j = tl.j0 + (threadIdx.x >> 5);
  if (i >= G.nx || j >= G.ny) return;
  const long o = (long)j * G.ld + i;
  const double a = 0.5 + 1e-3 * (double)((i * 7919 + j * 104729) % 1000);
  D.r[o] = a;
  D.p0[o] = 1.0 - a;
  D.p1[o] = a - 0.25;
  D.x[o] = 0.0;
}

__global__ void k_tune_arm(const InstDesc* __restrict__ ID, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  Ctrl64* c = ID[k].ctrl;
  c->done = 0;
  c->iter = 0;
  c->beta = 0.5;
  c->alpha = 1e-3;
  c->rho = 1.0;
  c->atol = -1.0;
}

static void set_cg_variant(Instance64* I, int v) {
  I->cg_var = v;
  I->tcg = I->tcgv[v];
  I->ntcg = I->ntcgv[v];
  for (int k = 0; k < I->n; ++k) I->hd[k].nt_cg = I->ntcg_inst[v][k];
  I->desc_dirty = true;
  if (I->exec) {
    cudaGraphExecDestroy(I->exec);
    I->exec = nullptr;
  }
  if (I->graph) {
    cudaGraphDestroy(I->graph);
    I->graph = nullptr;
  }
  I->graph_mode = -1;
}

int instance64_set_cg_variant(Instance64* I, int v) {
  if (v < 0 || v >= NVAR) return set_error(PFGB_EINVAL, "CG tile variant must be 0, 1 or 2");
  set_cg_variant(I, v);
  return PFGB_OK;
}

static void drop_graph(Instance64* I) {
  if (I->exec) {
    cudaGraphExecDestroy(I->exec);
    I->exec = nullptr;
  }
  if (I->graph) {
    cudaGraphDestroy(I->graph);
    I->graph = nullptr;
  }
  I->graph_mode = -1;
}

int instance64_set_mixed_variant(Instance64* I, int variant) {
  if (!I->mix) return set_error(PFGB_EINVAL, "launch variants of the mixed solve need precision 1");
  if (int rc = mixed::set_variant(I->mix, variant)) return rc;
  drop_graph(I);
  return PFGB_OK;
}

int instance64_autotune(Instance64* I, cudaStream_t s, int* chosen, double* us) {
  if (I->mix) {  // the mixed solve: its launch shapes (matvec form, coarse CTA width)
    if (int rc = upload_desc(I, s)) return rc;
    if (int rc = mixed::tune(I->mix, s, chosen, us)) return rc;
    drop_graph(I);
    return PFGB_OK;
  }
  std::vector<InstDesc> saved = I->hd;
  for (int k = 0; k < I->n; ++k) {
    I->hd[k].active = 1;
    I->hd[k].A.maxiter = 1 << 30;
  }
  float best = 1e30f;
  int best_v = I->cg_var;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaError_t err = cudaSuccess;
  for (int v = 0; v < NVAR && err == cudaSuccess; ++v) {
    for (int k = 0; k < I->n; ++k) I->hd[k].nt_cg = I->ntcg_inst[v][k];
    err = cudaMemcpyAsync(I->dd, I->hd.data(), I->n * sizeof(InstDesc), cudaMemcpyHostToDevice, s);
    if (err != cudaSuccess) break;
    k_tune_fill<<<I->ntpc, NT, 0, s>>>(I->dd, I->tpc);
    k_tune_arm<<<(I->n + 127) / 128, 128, 0, s>>>(I->dd, I->n);
    for (int w = 0; w < 2; ++w) {
      launch_matvec<0>(v, I->ntcgv[v], s, I->dd, I->tcgv[v]);
      launch_update(v, I->ntcgv[v], s, I->dd, I->tcgv[v]);
    }
    const int reps = 10;
    cudaEventRecord(e0, s);
    for (int w = 0; w < reps; ++w) {
      launch_matvec<0>(v, I->ntcgv[v], s, I->dd, I->tcgv[v]);
      launch_update(v, I->ntcgv[v], s, I->dd, I->tcgv[v]);
    }
    cudaEventRecord(e1, s);
    err = cudaEventSynchronize(e1);
    if (err != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const float per = 1e3f * ms / reps;
    if (us) us[v] = per;
    if (per < best) {
      best = per;
      best_v = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  I->hd = saved;
  if (err == cudaSuccess) err = cudaGetLastError();
  if (err != cudaSuccess) {
    I->desc_dirty = true;
    return set_error(PFGB_ECUDA, std::string("autotune: ") + cudaGetErrorString(err));
  }
  set_cg_variant(I, best_v);
  if (chosen) *chosen = best_v;
  return PFGB_OK;
}

int instance64_matvec_form(const Instance64* I, int* tma) {
  *tma = I->mix ? mixed::matvec_form(I->mix) : 0;
  return PFGB_OK;
}

int instance64_set_persistent(Instance64* I, int on) {
  if (!I->mix) return PFGB_OK;
  mixed::set_persistent(I->mix, on);
  drop_graph(I);
  return PFGB_OK;
}

int instance64_set_graph(Instance64* I, int on) {
  const int m = (on == 2) ? 2 : (on ? 1 : 0);
  if (m != I->use_graph) {
    if (I->exec) {
      cudaGraphExecDestroy(I->exec);
      I->exec = nullptr;
    }
    if (I->graph) {
      cudaGraphDestroy(I->graph);
      I->graph = nullptr;
    }
    I->graph_mode = -1;
  }
  I->use_graph = m;
  return PFGB_OK;
}

// Per-kernel timing of the following steps (direct launches, events around each).
int instance64_set_profiling(Instance64* I, int on) {
  I->profiling = on ? 1 : 0;
  I->kp.clear();
  if (I->mix) I->mix->kp = on ? &I->kp : nullptr;
  return PFGB_OK;
}

// Per-kernel sums of the last (synchronised) profiled step.
int instance64_profile_kernels(Instance64* I, std::vector<KTime>& out) {
  if (!I->kp.ok) return set_error(PFGB_ECUDA, "profiling events could not be created or recorded");
  const cudaError_t e = kprof_collect(I->kp, out);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("event timing: ") + cudaGetErrorString(e));
  return PFGB_OK;
}

// Sum of the pressure-matvec launch durations of the last (synchronised) profiled
// step (the persistent solve as a whole where that form runs).  Launches that
// returned at once because the solve had converged are included.
int instance64_profile_result(Instance64* I, double* ms, int* launches) {
  std::vector<KTime> kt;
  if (int rc = instance64_profile_kernels(I, kt)) return rc;
  *ms = 0.0;
  *launches = 0;
  for (const KTime& k : kt)
    if (k.name == "k_cg_matvec" || k.name == "k_mx_matvec" || k.name == "k_mx_matvec_tma" || k.name == "k_mx_persist") {
      *ms += k.ms;
      *launches += k.launches;
    }
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
// tiles of one instance written on the device (no host allocation)
__global__ void k_fill_tiles(Tile* t, int nx, int ny, int th) {
  const int ntx = (nx + TX - 1) / TX, nty = (ny + th - 1) / th;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ntx * nty; k += gridDim.x * blockDim.x)
    t[k] = Tile{0, (k % ntx) * TX, (k / ntx) * th, 0};
}

// Descriptor of the one-instance operator-interface solve (b and x contiguous).
static InstDesc op_solve_desc(const double* b, double* x, int nx, int ny, double dx, double dy, int precond,
                              double invd, double tol, int maxiter, double* r, double* p0, double* p1, double* q,
                              XASlot* slots, Ctrl64* ctrl) {
  InstDesc D = {};
  D.G = make_geo(nx, ny, nx, dx, dy, invd, precond);
  D.A.rtol = tol;
  D.A.maxiter = maxiter;
  D.A.n_cells = (double)nx * (double)ny;
  D.adjust = 0;
  D.mode = 1;
  D.active = 1;
  D.b = const_cast<double*>(b);
  D.x = x;
  D.r = r;
  D.p0 = p0;
  D.p1 = p1;
  D.q = q;
  D.slots = slots;
  D.ctrl = ctrl;
  D.nt_pc = count_tiles(nx, ny, PB_Y);
  D.nt_cg = count_tiles(nx, ny, TY);
  return D;
}

static void op_solve_launch(int op, const InstDesc* dd, const Tile* tpc, int ntpc, const Tile* tcg, int ntcg,
                            int maxiter, cudaStream_t s) {
  k_cg_init<<<ntpc, NT, 0, s>>>(dd, tpc, nullptr);
  for (int k = 0; k < maxiter; ++k) {
    if (op == PFGB_OP_NEG_LAPLACIAN_PINNED)
      k_cg_matvec<0><<<ntcg, NT, 0, s>>>(dd, tcg);
    else
      k_cg_matvec<1><<<ntcg, NT, 0, s>>>(dd, tcg);
    k_cg_update<<<ntcg, NT, 0, s>>>(dd, tcg, nullptr, 0ull, 0);
  }
  if (op == PFGB_OP_NEG_LAPLACIAN_PINNED)
    k_post_resid<0><<<ntpc, NT, 0, s>>>(dd, tpc);
  else
    k_post_resid<1><<<ntpc, NT, 0, s>>>(dd, tpc);
}

int cg_solve_run(int op, const double* b, double* x, int nx, int ny, double dx, double dy, int precond,
                 double invd, double tol, int maxiter, cudaStream_t s, pfgb_solve_out* out) {
  if (nx < 2 || ny < 2) return set_error(PFGB_EINVAL, "nx and ny must be >= 2");
  if (op != PFGB_OP_NEG_LAPLACIAN_PINNED && op != PFGB_OP_LAPLACIAN_DIRICHLET) return set_error(PFGB_EINVAL, "unknown operator");
  if (maxiter < 0) return set_error(PFGB_EINVAL, "maxiter must be >= 0");
  const int ntpc = count_tiles(nx, ny, PB_Y), ntcg = count_tiles(nx, ny, TY);
  auto up = [](size_t v) { return (v + 255) / 256 * 256; };
  const size_t vecr = up((size_t)nx * ny * sizeof(double));
  const size_t o_slots = 4 * vecr, o_ctrl = o_slots + up(S_COUNT * sizeof(XASlot));
  const size_t o_desc = o_ctrl + up(sizeof(Ctrl64)), o_tpc = o_desc + up(sizeof(InstDesc));
  const size_t o_tcg = o_tpc + up(ntpc * sizeof(Tile)), bytes = o_tcg + up(ntcg * sizeof(Tile));
  char* ws = nullptr;
  cudaError_t e = cudaMallocAsync(&ws, bytes, s);
  if (e != cudaSuccess) return set_error(PFGB_ENOMEM, "cudaMallocAsync of the CG workspace failed");
  cudaMemsetAsync(ws, 0, o_desc, s);
  XASlot* slots = (XASlot*)(ws + o_slots);
  Ctrl64* ctrl = (Ctrl64*)(ws + o_ctrl);
  InstDesc* dd = (InstDesc*)(ws + o_desc);
  Tile* tpc = (Tile*)(ws + o_tpc);
  Tile* tcg = (Tile*)(ws + o_tcg);
  const InstDesc hd = op_solve_desc(b, x, nx, ny, dx, dy, precond, invd, tol, maxiter, (double*)ws,
                                    (double*)(ws + vecr), (double*)(ws + 2 * vecr), (double*)(ws + 3 * vecr), slots,
                                    ctrl);
  cudaMemcpyAsync(dd, &hd, sizeof(InstDesc), cudaMemcpyHostToDevice, s);
  k_fill_tiles<<<64, 256, 0, s>>>(tpc, nx, ny, PB_Y);
  k_fill_tiles<<<64, 256, 0, s>>>(tcg, nx, ny, TY);
  op_solve_launch(op, dd, tpc, ntpc, tcg, ntcg, maxiter, s);
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
// reserved on a device when the library's module is loaded there and held until
// the process exits.  Its limit is NOALLOC_MAX_CELLS = 262,144 cells
// (512 x 512); the array is about 8.5 MiB per device (sizeof(Scratch), pinned
// below by a static_assert).
namespace noalloc {

constexpr long NOALLOC_MAX_CELLS = 1L << 18;

constexpr int NOALLOC_MAX_TILES = 32768;   // per-cell plus CG tiles of one grid

struct Scratch {
  double r[NOALLOC_MAX_CELLS];
  double p0[NOALLOC_MAX_CELLS];
  double p1[NOALLOC_MAX_CELLS];
  double q[NOALLOC_MAX_CELLS];
  XASlot slots[S_COUNT];
  Ctrl64 ctrl;
  InstDesc desc;
  Tile tiles[NOALLOC_MAX_TILES];
};

static_assert(sizeof(Scratch) > 8.5 * 1024 * 1024 && sizeof(Scratch) < 8.6 * 1024 * 1024,
              "the documented size of the allocation-free CG scratch (about 8.5 MiB)");

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
  const int ntpc = count_tiles(nx, ny, PB_Y), ntcg = count_tiles(nx, ny, TY);
  if (ntpc + ntcg > NOALLOC_MAX_TILES)
    return set_error(PFGB_EINVAL, "grid shape needs more tiles than the allocation-free CG scratch holds");
  Scratch* S = nullptr;
  if (int rc = scratch_address(&S)) return rc;
  // the slots and the control block (and any padding between them) must start from
  // zero on every call
  cudaError_t e = cudaMemsetAsync(S->slots, 0, offsetof(Scratch, desc) - offsetof(Scratch, slots), s);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("clearing the CG scratch: ") + cudaGetErrorString(e));
  XASlot* slots = S->slots;
  Ctrl64* ctrl = &S->ctrl;
  const InstDesc hd = op_solve_desc(b, x, nx, ny, dx, dy, precond, invd, tol, maxiter, S->r, S->p0, S->p1, S->q,
                                    slots, ctrl);
  // the descriptor goes through a host stack copy: no allocation
  cudaMemcpyAsync(&S->desc, &hd, sizeof(InstDesc), cudaMemcpyHostToDevice, s);
  k_fill_tiles<<<64, 256, 0, s>>>(S->tiles, nx, ny, PB_Y);
  k_fill_tiles<<<64, 256, 0, s>>>(S->tiles + ntpc, nx, ny, TY);
  op_solve_launch(op, &S->desc, S->tiles, ntpc, S->tiles + ntpc, ntcg, maxiter, s);
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
