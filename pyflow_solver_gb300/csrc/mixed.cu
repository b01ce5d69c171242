// Mixed-precision pressure solve: FP64 iterative refinement around an FP32
// multigrid-preconditioned CG.
//
// The reference's system A x = b (A = -lap_c with row 0 replaced by the
// identity, b mean-free with b[0] = 0; src/pyflow/solvers/pressure_solver.py:97-128)
// has x[0] = 0, and its rows k != 0 form the SPD matrix -lap_c without row and
// column 0.  The refinement keeps x and the residual r = b - A x in binary64
// (the reference stencil); each correction e solves the equivalent singular
// Neumann system -lap_c e = r~ in binary32, where r~ equals r except
// r~_0 = -sum_{k != 0} r_k (which makes it consistent), and is shifted by -e[0]
// so that x[0] stays 0.  The inner solve is CG preconditioned by a
// cell-centred geometric multigrid V-cycle: bilinear prolongation P (weights
// 3/4, 1/4 per coarsened axis, reflected at the Neumann walls), restriction
// R = P^T, coarse operators rediscretised consistently with R = P^T; both axes
// are halved where the face coefficients are balanced, only the strongly
// coupled one where they differ by more than 2x (semi-coarsening, for cells
// longer in one direction); two Chebyshev-weighted Jacobi sweeps before and after; every
// level of at most 4096 cells inside one CTA, whose bottom level is solved by
// its pseudo-inverse.  The cycle is symmetric (R = P^T, adjoint smoothing,
// symmetric bottom solve), as PCG requires.
// Dot products are float-float sums of exactly split binary32 products per
// CTA and binary64 across CTAs in a fixed order (dred.cuh); alpha, beta and
// every norm of the refinement are binary64.
//
// Both loops are WHILE conditional nodes of the step graph: the inner loop
// stops at ||r_in|| <= tol_in ||r~|| or max_inner iterations, the outer loop
// at ||b - A x|| <= tol_out ||b|| or max_outer passes.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstdio>
#include <string>
#include <vector>

#include "dred.cuh"
#include "graph.cuh"
#include "icvt.cuh"
#include "mixed.cuh"
#include "persist.cuh"
#include "pfgb_internal.h"
#include "stencil.cuh"
#include "step64.cuh"

namespace pfgb {
namespace mixed {

constexpr int MT = 256;
constexpr double REACH_REL = 3e-7;           // the first pass's deepest relative aim
constexpr int REACH_WAIT = 8;                // steps before aiming again after a miss
constexpr int BX = 32, BY = 32;              // a tile: 32 x 32 cells, each thread a column of 4
constexpr int RPT = BY / (MT / 32);

__device__ __forceinline__ float mg_diag(const Lvl& L, int j, int i) {
  float d = 0.f;
  if (i > 0) d += L.cx;
  if (i < L.nx - 1) d += L.cx;
  if (j > 0) d += L.cy;
  if (j < L.ny - 1) d += L.cy;
  return d;
}

// sum of c * u over the existing neighbours of (j, i), reading u(jj, ii) via `at`
template <typename F>
__device__ __forceinline__ float mg_nsum(const Lvl& L, int j, int i, F at) {
  float s = 0.f;
  if (i > 0) s = fmaf(L.cx, at(j, i - 1), s);
  if (i < L.nx - 1) s = fmaf(L.cx, at(j, i + 1), s);
  if (j > 0) s = fmaf(L.cy, at(j - 1, i), s);
  if (j < L.ny - 1) s = fmaf(L.cy, at(j + 1, i), s);
  return s;
}

// The interior forms of the tile phases.  A tile whose region with a halo of h
// cells keeps at least one cell away from every wall has no wall cell in it:
// every cell has four neighbours, the full diagonal and, on a coarsened axis,
// both parents.  Those forms run the per-cell arithmetic of the general form
// operation for operation (the diagonal summed in the same order, the same fma
// chains), so both give the same bits; what goes is the per-cell wall logic.
__device__ __forceinline__ bool tile_interior(const MTile& tl, int nx, int ny, int h) {
  return tl.i0 - h >= 1 && tl.j0 - h >= 1 && tl.i0 + BX + h <= nx - 1 && tl.j0 + BY + h <= ny - 1;
}

// the diagonal of a cell with four neighbours, summed as mg_diag sums it
__device__ __forceinline__ float mg_diag_in(const Lvl& L) {
  float d = 0.f;
  d += L.cx;
  d += L.cx;
  d += L.cy;
  d += L.cy;
  return d;
}

template <bool IN>
__device__ __forceinline__ float lv_diag(const Lvl& L, float din, int j, int i) {
  return IN ? din : mg_diag(L, j, i);
}

template <bool IN, typename F>
__device__ __forceinline__ float lv_nsum(const Lvl& L, int j, int i, F at) {
  if (!IN) return mg_nsum(L, j, i, at);
  float s = 0.f;
  s = fmaf(L.cx, at(j, i - 1), s);
  s = fmaf(L.cx, at(j, i + 1), s);
  s = fmaf(L.cy, at(j - 1, i), s);
  s = fmaf(L.cy, at(j + 1, i), s);
  return s;
}

// Bilinear prolongation along each coarsened axis (3/4 parent + 1/4 neighbour,
// all of the parent at a wall; an axis that is not coarsened (factor 1) is
// copied) and its transpose.  A level may halve both axes or, for cells much
// longer in one direction, only the strongly coupled one (semi-coarsening).
struct PAxis {
  int p, p2;       // parent, second parent
  float w, w2;     // their weights (w2 = 0: no second parent)
};

template <int K>
__device__ __forceinline__ PAxis prolong_axis(int i, int nc) {
  if (K == 1) return PAxis{i, i, 1.f, 0.f};
  const int I = i >> 1, I2 = (i & 1) ? I + 1 : I - 1;
  const bool h = I2 >= 0 && I2 < nc;
  return PAxis{I, h ? I2 : I, h ? 0.75f : 1.f, h ? 0.25f : 0.f};
}

// value at fine cell (j, i) of P e on a coarse level of nx x ny cells, the
// coarse values read through at(J, I)
template <int KX, int KY, class AT>
__device__ __forceinline__ float prolong_k(AT at, int nx, int ny, int j, int i) {
  const PAxis ax = prolong_axis<KX>(i, nx), ay = prolong_axis<KY>(j, ny);
  float v = ax.w * ay.w * at(ay.p, ax.p);
  if (KX == 2 && ax.w2 != 0.f) v = fmaf(ax.w2 * ay.w, at(ay.p, ax.p2), v);
  if (KY == 2 && ay.w2 != 0.f) v = fmaf(ax.w * ay.w2, at(ay.p2, ax.p), v);
  if (KX == 2 && KY == 2 && ax.w2 != 0.f && ay.w2 != 0.f) v = fmaf(ax.w2 * ay.w2, at(ay.p2, ax.p2), v);
  return v;
}

template <class AT>
__device__ __forceinline__ float prolong_val(AT at, int nx, int ny, int kx, int ky, int j, int i) {
  if (kx == 2 && ky == 2) return prolong_k<2, 2>(at, nx, ny, j, i);
  if (kx == 2) return prolong_k<2, 1>(at, nx, ny, j, i);
  return prolong_k<1, 2>(at, nx, ny, j, i);
}

// weight with which fine index i (offset d = i - 2I in {-1, 0, 1, 2}) enters coarse I (R = P^T)
__device__ __forceinline__ float rweight(int d, int I, int nc) {
  if (d == -1) return (I - 1 >= 0) ? 0.25f : 0.f;
  if (d == 2) return (I + 1 < nc) ? 0.25f : 0.f;
  if (d == 0) return (I == 0) ? 1.f : 0.75f;
  return (I == nc - 1) ? 1.f : 0.75f;          // d == 1
}

// (P^T w) at coarse cell (J, I): fine value (j, i) at w[(j - j0) * ld + (i - i0)], coarse
// level nx x ny, factors KX, KY
template <int KX, int KY>
__device__ __forceinline__ float restrict_k(const float* w, long ld, int j0, int i0, int nx, int ny, int J, int I) {
  float s = 0.f;
#pragma unroll
  for (int dj = (KY == 2 ? -1 : 0); dj <= (KY == 2 ? 2 : 0); ++dj) {
    const float wy = KY == 2 ? rweight(dj, J, ny) : 1.f;
    if (wy == 0.f) continue;
    const int j = KY * J + dj;
    float row = 0.f;
#pragma unroll
    for (int di = (KX == 2 ? -1 : 0); di <= (KX == 2 ? 2 : 0); ++di) {
      const float wx = KX == 2 ? rweight(di, I, nx) : 1.f;
      if (wx == 0.f) continue;
      row = fmaf(wx, w[(long)(j - j0) * ld + (KX * I + di - i0)], row);
    }
    s = fmaf(wy, row, s);
  }
  return s;
}

__device__ __forceinline__ float restrict_val(const float* w, long ld, int j0, int i0, int nx, int ny, int kx, int ky,
                                              int J, int I) {
  if (kx == 2 && ky == 2) return restrict_k<2, 2>(w, ld, j0, i0, nx, ny, J, I);
  if (kx == 2) return restrict_k<2, 1>(w, ld, j0, i0, nx, ny, J, I);
  return restrict_k<1, 2>(w, ld, j0, i0, nx, ny, J, I);
}

// prolong_k and restrict_k for cells away from the walls (both parents, weights
// 3/4 and 1/4 on a coarsened axis), in the same operation order
template <int KX, int KY, class AT>
__device__ __forceinline__ float prolong_k_in(AT at, int j, int i) {
  const int I = KX == 2 ? (i >> 1) : i, I2 = KX == 2 ? ((i & 1) ? I + 1 : I - 1) : i;
  const int J = KY == 2 ? (j >> 1) : j, J2 = KY == 2 ? ((j & 1) ? J + 1 : J - 1) : j;
  const float wx = KX == 2 ? 0.75f : 1.f, wy = KY == 2 ? 0.75f : 1.f;
  float v = wx * wy * at(J, I);
  if (KX == 2) v = fmaf(0.25f * wy, at(J, I2), v);
  if (KY == 2) v = fmaf(wx * 0.25f, at(J2, I), v);
  if (KX == 2 && KY == 2) v = fmaf(0.25f * 0.25f, at(J2, I2), v);
  return v;
}

template <bool IN, class AT>
__device__ __forceinline__ float prolong_lv(AT at, int nx, int ny, int kx, int ky, int j, int i) {
  if (!IN) return prolong_val(at, nx, ny, kx, ky, j, i);
  if (kx == 2 && ky == 2) return prolong_k_in<2, 2>(at, j, i);
  if (kx == 2) return prolong_k_in<2, 1>(at, j, i);
  return prolong_k_in<1, 2>(at, j, i);
}

template <int KX, int KY>
__device__ __forceinline__ float restrict_k_in(const float* w, long ld, int j0, int i0, int J, int I) {
  float s = 0.f;
#pragma unroll
  for (int dj = (KY == 2 ? -1 : 0); dj <= (KY == 2 ? 2 : 0); ++dj) {
    const float wy = KY == 2 ? ((dj == -1 || dj == 2) ? 0.25f : 0.75f) : 1.f;
    const int j = KY * J + dj;
    float row = 0.f;
#pragma unroll
    for (int di = (KX == 2 ? -1 : 0); di <= (KX == 2 ? 2 : 0); ++di) {
      const float wx = KX == 2 ? ((di == -1 || di == 2) ? 0.25f : 0.75f) : 1.f;
      row = fmaf(wx, w[(long)(j - j0) * ld + (KX * I + di - i0)], row);
    }
    s = fmaf(wy, row, s);
  }
  return s;
}

template <bool IN>
__device__ __forceinline__ float restrict_lv(const float* w, long ld, int j0, int i0, int nx, int ny, int kx, int ky,
                                             int J, int I) {
  if (!IN) return restrict_val(w, ld, j0, i0, nx, ny, kx, ky, J, I);
  if (kx == 2 && ky == 2) return restrict_k_in<2, 2>(w, ld, j0, i0, J, I);
  if (kx == 2) return restrict_k_in<2, 1>(w, ld, j0, i0, J, I);
  return restrict_k_in<1, 2>(w, ld, j0, i0, J, I);
}

// ---- phases ---------------------------------------------------------------
//
// Each phase function processes one 32 x 32 tile of one instance, written once
// against an execution context (persist.cuh): the ordinary kernels below run it
// as a 256-thread CTA, the persistent kernel as a 256-thread group.  The caller
// has checked that the instance is live: it has not sat the step out or left
// the loop the phase belongs to (gate 0: the refinement loop, 1: the inner PCG).

__device__ __forceinline__ bool mx_live(const MixDesc& M, int gate) {
  // the three flags are loaded together (one round trip, not a chain of three)
  const MixCtrl* c = M.ctrl;
  const int act = *M.active;
  const int od = *(volatile const int*)&c->outer_done;
  const int id = gate ? *(volatile const int*)&c->inner_done : 0;
  return act && !od && !id;
}

using RedSmem = DRedSmem<MT>;

// control-block fields written by the finalising tile of an earlier phase
template <typename T>
__device__ __forceinline__ T cget(const T* p) {
  return __ldcg(p);
}

// rho = r.z of a V-cycle's result; beta = rho / rho_prev after the first inner iteration
__device__ __forceinline__ void set_rho(MixCtrl* ctrl, double rz) {
  if (cget(&ctrl->inner) > 0) ctrl->beta = rz / cget(&ctrl->rho);
  ctrl->rho = rz;
}

// level-0 right-hand side (the PCG residual) of the current inner iteration
__device__ __forceinline__ float* f_cur(const MixDesc& M) {
  return (cget(&M.ctrl->inner) & 1) ? M.f0b : M.lev[0].f;
}

// the rows ty of the tile that this thread owns (ty = warp, warp + 8, ...)
#define MX_ROWS_X(...)                                      \
  for (int r_ = 0; r_ < RPT; ++r_) {                        \
    const int ty = (x.tid() >> 5) + r_ * (MT / 32);         \
    __VA_ARGS__                                             \
  }

// an instance-wide sum of R values per tile (M.part holds MAX_RED per tile)
template <int R, class X>
__device__ __forceinline__ bool x_red(const X& x, const MixDesc& M, const MTile& tl, double (&v)[R], double (&out)[R],
                                      RedSmem& rsm) {
  static_assert(R <= MAX_RED, "reduction wider than the partial-sum array");
  return dred_sum<R, MT>(x, v, M.part, M.nt0, tl.loc, M.ticket, out, rsm);
}
template <int R, class X>
__device__ __forceinline__ bool x_red(const X& x, const MixDesc& M, const MTile& tl, FF (&v)[R], double (&out)[R],
                                      RedSmem& rsm) {
  static_assert(R <= MAX_RED, "reduction wider than the partial-sum array");
  return dred_sum_ff<R, MT>(x, v, M.part, M.nt0, tl.loc, M.ticket, out, rsm);
}
#define X_RED(R, vals, outv) x_red<R>(x, M, tl, vals, outv, rsm)
#define X_RED_FF(R, vals, outv) x_red<R>(x, M, tl, vals, outv, rsm)

constexpr int H3 = 3;
struct DownSmem {
  float sf[BY + 2 * H3][BX + 2 * H3];   // f on the 3-cell halo
  float s1[BY + 2 * H3][BX + 2 * H3];
  float s2[BY + 4][BX + 4];
  float rs[BY + 2][BX + 2];
};
struct PostSmem {
  float w0[BY + 4][BX + 4];
  float w1[BY + 2][BX + 2];
  float sf[BY + 2][BX + 2];             // f on the 1-cell halo
  float cs[BY + 6][BX + 6];             // the coarse values the tile's prolongation reads
  RedSmem rsm;
};
struct MatvecSmem {
  float pn[BY + 2][BX + 2];
  RedSmem rsm;
};
struct UpdDownSmem;
union TileSmem;

// Down-sweep of level l, fused: two damped-Jacobi sweeps from u = 0 (t = S(S(0))
// for A u = f), the residual r = f - A t, and its restriction f_{l+1} = P^T r.
// The tile computes the first sweep on a 3-cell halo, t on 2 and r on 1, so
// every coarse cell whose fine patch lies in the tile is complete; only t
// goes back to memory (the up-sweep needs it).
template <bool IN, class X>
__device__ __forceinline__ void ph_down_t(const X& x, const MixDesc& M, const MTile& tl, int l, Smooth sw,
                                        DownSmem& sm) {
  Lvl L = M.lev[l];
  const Lvl C = M.lev[l + 1];
  if (l == 0) L.f = f_cur(M);
  const int i0 = tl.i0, j0 = tl.j0;
  const float din = mg_diag_in(L);
  auto inside = [&](int gj, int gi) { return IN || (gj >= 0 && gj < L.ny && gi >= 0 && gi < L.nx); };
  {
    // every load of the halo first, then the stores
    constexpr int HW = BX + 2 * H3, HN = (BY + 2 * H3) * HW, NI = (HN + MT - 1) / MT;
    float fv[NI];
#pragma unroll
    for (int t = 0; t < NI; ++t) {
      const int idx = x.tid() + t * MT;
      const int gj = j0 + idx / HW - H3, gi = i0 + idx % HW - H3;
      fv[t] = 0.f;
      if ((t < NI - 1 || idx < HN) && inside(gj, gi)) fv[t] = x.ld(L.f + (long)gj * L.ld + gi);
    }
#pragma unroll
    for (int t = 0; t < NI; ++t) {
      const int idx = x.tid() + t * MT;
      if (t < NI - 1 || idx < HN) {
        const int jj = idx / HW - H3, ii = idx % HW - H3;
        const int gj = j0 + jj, gi = i0 + ii;
        float v = 0.f;
        if (inside(gj, gi)) v = __fdividef(sw.w1 * fv[t], lv_diag<IN>(L, din, gj, gi));
        sm.sf[jj + H3][ii + H3] = fv[t];
        sm.s1[jj + H3][ii + H3] = v;
      }
    }
  }
  x.sync();
  for (int idx = x.tid(); idx < (BY + 4) * (BX + 4); idx += MT) {
    const int jj = idx / (BX + 4) - 2, ii = idx % (BX + 4) - 2;
    const int gj = j0 + jj, gi = i0 + ii;
    float v = 0.f;
    if (inside(gj, gi)) {
      auto at = [&](int j, int i) { return sm.s1[j - j0 + H3][i - i0 + H3]; };
      v = fmaf(1.f - sw.w2, sm.s1[jj + H3][ii + H3],
               __fdividef(sw.w2 * (sm.sf[jj + H3][ii + H3] + lv_nsum<IN>(L, gj, gi, at)), lv_diag<IN>(L, din, gj, gi)));
    }
    sm.s2[jj + 2][ii + 2] = v;
  }
  x.sync();
  for (int idx = x.tid(); idx < (BY + 2) * (BX + 2); idx += MT) {
    const int jj = idx / (BX + 2) - 1, ii = idx % (BX + 2) - 1;
    const int gj = j0 + jj, gi = i0 + ii;
    float v = 0.f;
    if (inside(gj, gi)) {
      auto at = [&](int j, int i) { return sm.s2[j - j0 + 2][i - i0 + 2]; };
      const float t = sm.s2[jj + 2][ii + 2];
      v = sm.sf[jj + H3][ii + H3] - (lv_diag<IN>(L, din, gj, gi) * t - lv_nsum<IN>(L, gj, gi, at));
      if (jj >= 0 && jj < BY && ii >= 0 && ii < BX) L.t[(long)gj * L.ld + gi] = t;
    }
    sm.rs[jj + 1][ii + 1] = v;
  }
  x.sync();
  // coarse cells of this tile: (32 / kx) x (32 / ky)
  const int cw = BX / L.kx, chh = BY / L.ky;
  const int I0 = i0 / L.kx, J0 = j0 / L.ky;
  for (int idx = x.tid(); idx < cw * chh; idx += MT) {
    const int jj = idx / cw, ii = idx - jj * cw;
    const int I = I0 + ii, J = J0 + jj;
    // sm.rs holds r at fine rows j0 - 1 .. j0 + BY and columns i0 - 1 .. i0 + BX
    if (IN || (I < C.nx && J < C.ny))
      C.f[(long)J * C.ld + I] = restrict_lv<IN>(&sm.rs[0][0], BX + 2, j0 - 1, i0 - 1, C.nx, C.ny, L.kx, L.ky, J, I);
  }
}

template <class X>
__device__ __forceinline__ void ph_down(const X& x, const MixDesc& M, const MTile& tl, int l, Smooth sw,
                                        DownSmem& sm) {
  if (M.interior && tile_interior(tl, M.lev[l].nx, M.lev[l].ny, H3)) ph_down_t<true>(x, M, tl, l, sw, sm);
  else ph_down_t<false>(x, M, tl, l, sw, sm);
}

// u_l = S(S(t_l + P u_{l+1})) with the bilinear P; on level 0 also rho = r.z
template <bool IN, class X>
__device__ __forceinline__ void ph_post_t(const X& x, const MixDesc& M, const MTile& tl, int l, Smooth sw,
                                        PostSmem& sm) {
  Lvl F = M.lev[l];
  const Lvl C = M.lev[l + 1];
  if (l == 0) F.f = f_cur(M);
  RedSmem& rsm = sm.rsm;
  const int i0 = tl.i0, j0 = tl.j0;
  const float din = mg_diag_in(F);
  // every global load first (t on the 2-cell halo, f on 1, the coarse patch the
  // prolongation reads: its parents of fine cells i0-2 .. i0+BX+1, at most 38 x 38),
  // then the prolongation from shared memory
  const int Ilo = max(0, max(0, i0 - 2) / F.kx - 1), Ihi = min(C.nx - 1, (i0 + BX + 1) / F.kx + 1);
  const int Jlo = max(0, max(0, j0 - 2) / F.ky - 1), Jhi = min(C.ny - 1, (j0 + BY + 1) / F.ky + 1);
  const int cw = Ihi - Ilo + 1, ch = Jhi - Jlo + 1;
  {
    // all of these loads are issued before the first store
    constexpr int HW = BX + 4, HN = (BY + 4) * HW, NI = (HN + MT - 1) / MT;
    // the coarse patch: one axis coarsened at least, so at most 38 x 20 parents
    constexpr int NC = ((BY + 6) * (BX / 2 + 4) + MT - 1) / MT;
    const int cn = cw * ch;
    float tv[NI], fv[NI], cv[NC];
#pragma unroll
    for (int t = 0; t < NI; ++t) {
      const int idx = x.tid() + t * MT;
      const int jj = idx / HW - 2, ii = idx % HW - 2;
      const int gj = j0 + jj, gi = i0 + ii;
      tv[t] = 0.f;
      fv[t] = 0.f;
      if ((t < NI - 1 || idx < HN) && (IN || (gj >= 0 && gj < F.ny && gi >= 0 && gi < F.nx))) {
        const long o = (long)gj * F.ld + gi;
        tv[t] = x.ld(F.t + o);
        if (jj >= -1 && jj <= BY && ii >= -1 && ii <= BX) fv[t] = x.ld(F.f + o);
      }
    }
#pragma unroll
    for (int t = 0; t < NC; ++t) {
      const int idx = x.tid() + t * MT;
      cv[t] = 0.f;
      if (idx < cn) {
        const int r = idx / cw, c = idx - r * cw;
        cv[t] = x.ld(C.u + (long)(Jlo + r) * C.ld + Ilo + c);
      }
    }
#pragma unroll
    for (int t = 0; t < NI; ++t) {
      const int idx = x.tid() + t * MT;
      if (t < NI - 1 || idx < HN) {
        const int jj = idx / HW - 2, ii = idx % HW - 2;
        sm.w0[jj + 2][ii + 2] = tv[t];
        if (jj >= -1 && jj <= BY && ii >= -1 && ii <= BX) sm.sf[jj + 1][ii + 1] = fv[t];
      }
    }
#pragma unroll
    for (int t = 0; t < NC; ++t) {
      const int idx = x.tid() + t * MT;
      if (idx < cn) {
        const int r = idx / cw, c = idx - r * cw;
        sm.cs[r][c] = cv[t];
      }
    }
    for (int idx = x.tid() + NC * MT; idx < cn; idx += MT) {
      const int r = idx / cw, c = idx - r * cw;
      sm.cs[r][c] = x.ld(C.u + (long)(Jlo + r) * C.ld + Ilo + c);
    }
  }
  x.sync();
  auto cat = [&sm, Ilo, Jlo](int J, int I) { return sm.cs[J - Jlo][I - Ilo]; };
  for (int idx = x.tid(); idx < (BY + 4) * (BX + 4); idx += MT) {
    const int jj = idx / (BX + 4) - 2, ii = idx % (BX + 4) - 2;
    const int gj = j0 + jj, gi = i0 + ii;
    if (IN || (gj >= 0 && gj < F.ny && gi >= 0 && gi < F.nx))
      sm.w0[jj + 2][ii + 2] = sm.w0[jj + 2][ii + 2] + prolong_lv<IN>(cat, C.nx, C.ny, F.kx, F.ky, gj, gi);
  }
  x.sync();
  for (int idx = x.tid(); idx < (BY + 2) * (BX + 2); idx += MT) {
    const int jj = idx / (BX + 2) - 1, ii = idx % (BX + 2) - 1;
    const int gj = j0 + jj, gi = i0 + ii;
    float v = 0.f;
    if (IN || (gj >= 0 && gj < F.ny && gi >= 0 && gi < F.nx)) {
      auto at = [&](int j, int i) { return sm.w0[j - j0 + 2][i - i0 + 2]; };
      const float d = lv_diag<IN>(F, din, gj, gi);
      v = fmaf(1.f - sw.w2, sm.w0[jj + 2][ii + 2], __fdividef(sw.w2 * (sm.sf[jj + 1][ii + 1] + lv_nsum<IN>(F, gj, gi, at)), d));
    }
    sm.w1[jj + 1][ii + 1] = v;
  }
  x.sync();
  const int tx = x.tid() & 31;
  FF acc[1] = {{0.f, 0.f}};
  MX_ROWS_X({
    const int gi = i0 + tx, gj = j0 + ty;
    if (IN || (gi < F.nx && gj < F.ny)) {
      auto at = [&](int j, int i) { return sm.w1[j - j0 + 1][i - i0 + 1]; };
      const float d = lv_diag<IN>(F, din, gj, gi);
      const float fv = sm.sf[ty + 1][tx + 1];
      const float v = fmaf(1.f - sw.w1, sm.w1[ty + 1][tx + 1], __fdividef(sw.w1 * (fv + lv_nsum<IN>(F, gj, gi, at)), d));
      F.u[(long)gj * F.ld + gi] = v;
      if (l == 0) ff_add_prod(acc[0], fv, v);
    }
  })
  // level 0: z = u is complete in this tile; rho = r.z of the PCG
  if (l == 0) {
    double out[1];
    if (X_RED_FF(1, acc, out) && x.tid() == 0) set_rho(M.ctrl, out[0]);
  }
}

template <class X>
__device__ __forceinline__ void ph_post(const X& x, const MixDesc& M, const MTile& tl, int l, Smooth sw,
                                        PostSmem& sm) {
  if (M.interior && tile_interior(tl, M.lev[l].nx, M.lev[l].ny, 2)) ph_post_t<true>(x, M, tl, l, sw, sm);
  else ph_post_t<false>(x, M, tl, l, sw, sm);
}

// -A x at a cell k != 0 of the refinement's operator: the reference's coherent
// Laplacian (src/pyflow/numerics/core_ops_coherent.py:81-84, forward-difference
// gradient then backward-difference divergence), written as the difference of a
// cell's two face differences times 1/dx^2 (and 1/dy^2): ((p_e - p_c) - (p_c - p_w))
// / dx^2 + ... , a face missing at a wall counting as zero, as the reference's
// gradient is zero there.  The face differences of neighbouring values are exact
// (Sterbenz) wherever the values are within a factor of two, so this form rounds no
// worse than the reference's two divisions per face; it takes 9 binary64 operations
// instead of 13 on this GPU's narrow binary64 pipe.  The operator differs from the
// reference's by roundings, which move the solution of the system by about
// cond(A) x 1e-16 -- far below the refinement's tolerance -- and the stopping test is
// taken on this same operator.
template <class V>
__device__ __forceinline__ double lap_recip_at(V p, int j, int i, const Geo& G) {
  const int L = G.nx - 1, T = G.ny - 1;
  const double pc = p(j, i);
  const double de = (i < L) ? __dsub_rn(p(j, i + 1), pc) : 0.0;
  const double dw = (i >= 1) ? __dsub_rn(pc, p(j, i - 1)) : 0.0;
  const double dn = (j < T) ? __dsub_rn(p(j + 1, i), pc) : 0.0;
  const double ds = (j >= 1) ? __dsub_rn(pc, p(j - 1, i)) : 0.0;
  const double xp = __dmul_rn((i >= 1) ? __dsub_rn(de, dw) : de, G.rdx2);
  const double yp = __dmul_rn((j >= 1) ? __dsub_rn(dn, ds) : dn, G.rdy2);
  return __dadd_rn(xp, yp);
}

// the previous pressure as a 2-D view (loads through L2)
struct PrevView {
  const double* p;
  long ld;
  __device__ __forceinline__ double operator()(int j, int i) const { return __ldcg(p + (long)j * ld + i); }
};

// b -= mean(b), b[0] = 0 (pressure_solver.py:127-128, the mean from the exactly
// rounded sum as in the binary64 path); ||b||^2 and sum(b).  Cold start: x = 0,
// r64 = b.  Warm start: x = p_prev - p_prev[0] (the state's pressure, which the
// step has not yet replaced) and r64 = b - A x with the pinned operator, plus
// ||r64||^2 and sum(r64); the finalising tile keeps it when
// ||r64|| <= ||b|| and otherwise marks the solve cold (the first pass then
// restarts from x = 0, r = b).  Counts the instances that refine.
template <class X>
__device__ __forceinline__ void ph_init(const X& x, const MixDesc& M, const MTile& tl, MixLoop* ml, RedSmem& rsm) {
  const Geo G = M.G;
  MixCtrl* ctrl = M.ctrl;
  // the mean, divided once for the tile (the reduction's scratch carries it)
  if (x.tid() == 0) rsm.w[0][0] = __ddiv_rn(cget(M.bsum), M.n_cells);
  x.sync();
  const double mean = rsm.w[0][0];
  x.sync();
  const bool warm = cget(&ctrl->warm) != 0;
  const double* P = warm ? *M.pprev : nullptr;
  const PrevView Pv{P, M.ldp};
  const double p0 = P ? __ldcg(P) : 0.0;
  const int i = tl.i0 + (x.tid() & 31);
  double v[4] = {0.0, 0.0, 0.0, 0.0}, out[4];
  MX_ROWS_X({
    const int j = tl.j0 + ty;
    if (i < G.nx && j < G.ny) {
      const long o = (long)j * G.ld + i;
      const double bv = (i == 0 && j == 0) ? 0.0 : __dsub_rn(x.ld(M.b + o), mean);
      M.b[o] = bv;
      v[0] += bv * bv;
      v[1] += bv;
      if (P) {
        // x0 = p - p[0]; A x0 = -lap(p) away from the pinned cell (differences do not see the
        // shift, up to a rounding the refinement's own residual corrects)
        const double xv = __dsub_rn(Pv(j, i), p0);
        const double ax = (i == 0 && j == 0) ? xv : -lap_recip_at(Pv, j, i, G);
        const double rv = __dsub_rn(bv, ax);
        M.x[o] = xv;
        M.r64[o] = rv;
        v[2] += rv * rv;
        v[3] += rv;
      } else {
        M.x[o] = 0.0;
        M.r64[o] = bv;
      }
    }
  })
  if (X_RED(4, v, out) && x.tid() == 0) {
    M.ctrl64->mean = mean;
    M.ctrl64->nan_flag = 0u;
    const double bb = out[0];
    ctrl->bnorm = sqrt(bb);
    ctrl->tol_abs_out = cget(&ctrl->tol_out) * ctrl->bnorm;
    ctrl->outer = 0;
    ctrl->inner = 0;
    ctrl->inner_total = 0;
    ctrl->inner_done = 1;
    bool done;
    if (P && out[2] <= bb) {            // the warm guess is no worse than zero (false for a NaN)
      ctrl->cold = 0;
      ctrl->rr64 = out[2];
      ctrl->sum64 = out[3];
      done = !(sqrt(out[2]) > ctrl->tol_abs_out);
    } else {                            // from zero; a rejected warm guess still takes one pass to reset x
      ctrl->cold = P ? 1 : 0;
      ctrl->rr64 = bb;
      ctrl->sum64 = out[1];
      done = !P && bb == 0.0;
    }
    ctrl->converged = done ? 1 : 0;
    ctrl->outer_done = done ? 1 : 0;
    if (!done) atomicAdd(&ml->outer_active, 1);
  }
}

// r~ = float(r64) with r~_0 = -sum_{k != 0} r64_k; e = 0; ||r~||^2; starts an inner solve.
// The first pass of a cold-marked solve takes r64 = b and resets x = 0 instead.
// The inner solve stops at ||r_in|| <= max(tol_in ||r~||, tol_abs_out / 4): a
// quarter of the outer target is as far as this pass needs to go.  When the outer
// target is within REACH_REL ||r~|| -- about as deep as binary32 corrections still
// improve the binary64 residual -- the first pass of a solve may instead aim there
// (or at the quarter, if higher): on a warm start that often finishes the solve in
// one pass.  Whether it did is seen
// at the end of the pass (ph_resid); an instance whose first pass aimed at the
// target and missed it goes back to tol_in for REACH_WAIT steps, then tries
// again, so grids too large for binary32 to get there lose at most an occasional
// iteration.
template <class X>
__device__ __forceinline__ void ph_prep(const X& x, const MixDesc& M, const MTile& tl, MixLoop* ml, RedSmem& rsm) {
  const Geo G = M.G;
  const Lvl L0 = M.lev[0];
  MixCtrl* ctrl = M.ctrl;
  const bool first = cget(&ctrl->outer) == 0;
  const bool restart = cget(&ctrl->cold) != 0 && first;
  const double* rsrc = restart ? M.b : M.r64;
  const int i = tl.i0 + (x.tid() & 31);
  FF v[1] = {{0.f, 0.f}};
  double out[1];
  MX_ROWS_X({
    const int j = tl.j0 + ty;
    if (i < G.nx && j < G.ny) {
      if (restart) M.x[(long)j * G.ld + i] = 0.0;
      const double rv = (i == 0 && j == 0) ? -(cget(&ctrl->sum64) - x.ld(rsrc)) : x.ld(rsrc + (long)j * G.ld + i);
      const float rf = d2f_rn(rv);                 // on the integer pipe (icvt.cuh)
      L0.f[(long)j * L0.ld + i] = rf;
      M.e[(long)j * L0.ld + i] = 0.f;
      ff_add_prod(v[0], rf, rf);
    }
  })
  if (X_RED_FF(1, v, out) && x.tid() == 0) {
    const double rt = sqrt(out[0]);
    ctrl->rt_norm = rt;
    const double target = cget(&ctrl->tol_abs_out), quarter = 0.25 * target;
    const bool reach = first && cget(&ctrl->reach) != 0 && REACH_REL * rt <= target;
    ctrl->reach_tried = reach ? 1 : 0;
    ctrl->tol_abs_in = reach ? fmax(REACH_REL * rt, quarter) : fmax(cget(&ctrl->tol_in) * rt, quarter);
    ctrl->inner = 0;
    ctrl->inner_done = rt > 0.0 ? 0 : 1;
    if (rt > 0.0) atomicAdd(&ml->inner_active, 1);
  }
}

// p_new = z (first) or z + beta p_old; q = A p_new (binary32 Neumann operator); p.q
template <bool IN, class X>
__device__ __forceinline__ void ph_matvec_t(const X& x, const MixDesc& M, const MTile& tl, MatvecSmem& sm) {
  RedSmem& rsm = sm.rsm;
  const Lvl L0 = M.lev[0];
  MixCtrl* ctrl = M.ctrl;
  const float* z = L0.u;
  const int k = cget(&ctrl->inner);
  const float* pold = (k & 1) ? M.p1 : M.p0;
  float* pnew = (k & 1) ? M.p0 : M.p1;
  const float beta = (float)cget(&ctrl->beta);
  const int i0 = tl.i0, j0 = tl.j0;
  const float din = mg_diag_in(L0);
  // every load of the halo first (all in flight together), then the stores
  constexpr int HW = BX + 2, HN = (BY + 2) * HW, NI = (HN + MT - 1) / MT;
  auto inside = [&](int gj, int gi) { return IN || (gj >= 0 && gj < L0.ny && gi >= 0 && gi < L0.nx); };
  float zv[NI], pv0[NI];
#pragma unroll
  for (int t = 0; t < NI; ++t) {
    const int idx = x.tid() + t * MT;
    const int gj = j0 + idx / HW - 1, gi = i0 + idx % HW - 1;
    zv[t] = 0.f;
    pv0[t] = 0.f;
    if ((t < NI - 1 || idx < HN) && inside(gj, gi)) {
      const long o = (long)gj * L0.ld + gi;
      zv[t] = x.ld(z + o);
      if (k != 0) pv0[t] = x.ld(pold + o);
    }
  }
#pragma unroll
  for (int t = 0; t < NI; ++t) {
    const int idx = x.tid() + t * MT;
    if (t < NI - 1 || idx < HN) {
      const int jj = idx / HW - 1, ii = idx % HW - 1;
      float v = 0.f;
      if (inside(j0 + jj, i0 + ii)) v = (k == 0) ? zv[t] : fmaf(beta, pv0[t], zv[t]);
      sm.pn[jj + 1][ii + 1] = v;
    }
  }
  x.sync();
  const int tx = x.tid() & 31;
  const int gi = i0 + tx;
  FF v[1] = {{0.f, 0.f}};
  double out[1];
  MX_ROWS_X({
    const int gj = j0 + ty;
    if (IN || (gi < L0.nx && gj < L0.ny)) {
      auto at = [&](int j, int i) { return sm.pn[j - j0 + 1][i - i0 + 1]; };
      const float pv = sm.pn[ty + 1][tx + 1];
      const float qv = lv_diag<IN>(L0, din, gj, gi) * pv - lv_nsum<IN>(L0, gj, gi, at);
      const long o = (long)gj * L0.ld + gi;
      pnew[o] = pv;
      M.q[o] = qv;
      ff_add_prod(v[0], pv, qv);
    }
  })
  if (X_RED_FF(1, v, out) && x.tid() == 0) {
    ctrl->pq = out[0];
    ctrl->alpha = cget(&ctrl->rho) / out[0];
  }
}

template <class X>
__device__ __forceinline__ void ph_matvec(const X& x, const MixDesc& M, const MTile& tl, MatvecSmem& sm) {
  if (M.interior && tile_interior(tl, M.lev[0].nx, M.lev[0].ny, 1)) ph_matvec_t<true>(x, M, tl, sm);
  else ph_matvec_t<false>(x, M, tl, sm);
}

// ---- the matvec with halos copied by the tensor memory accelerator ---------
// The kernel graph's form of ph_matvec.  Each CTA takes the level-0 tiles
// blockIdx.x, blockIdx.x + gridDim.x, ... and has TMA copy the halo of its next
// tile (z and p_old) into one of two shared-memory stages while it computes the
// current one.  A copy is a 40 x 34 box of binary32 from column i0 - 4 and row
// j0 - 1: the tile's 34 x 34 halo, widened so that the copy starts on a 16-byte
// boundary (i0 is a multiple of 32); cells outside the grid read as zero.  The
// per-cell arithmetic (p = z or z + beta p_old, q = A p), the tile sums and
// their order are those of ph_matvec, so both forms give the same bits.
constexpr int MV_W = BX + 8, MV_H = BY + 2;
constexpr int MV_X0 = 4;                       // column of cell i0 in a stage row
constexpr unsigned MV_BYTES = MV_W * MV_H * sizeof(float);
constexpr int MV_SPIN_LIMIT = 1 << 20;         // polls of a stage's barrier before the kernel gives up
struct alignas(128) MvStage {
  float v[MV_H][MV_W];
};
struct MvSmem {
  MvStage z[2], p[2];
  unsigned long long bar[2];
  RedSmem rsm;
};

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(b)), "r"(parity)
      : "memory");
  return ok != 0u;
}

__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* b, unsigned parity, int limit = MV_SPIN_LIMIT) {
  for (int i = 0; i < limit; ++i)
    if (mbar_try_wait(b, parity)) return true;
  return false;
}

// box at (x, y) of the tensor `map` (a tensor map in global memory) into dst; x * 4 bytes
// is a multiple of 16
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, unsigned long long* b) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(smem_addr(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(smem_addr(b))
      : "memory");
}

// thread 0: the copies of tile tl's halo into stage s (p_old only after the first
// iteration; k is the instance's inner iteration)
__device__ __forceinline__ void mv_issue(const MixDesc& M, const MTile& tl, int k, MvSmem& sm, int s) {
  const int xs = tl.i0 - MV_X0, ys = tl.j0 - 1;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // the stage's earlier reads come first
  mbar_expect_tx(&sm.bar[s], k == 0 ? MV_BYTES : 2u * MV_BYTES);
  tma_load_2d(&sm.z[s], M.tmap + 0, xs, ys, &sm.bar[s]);
  if (k != 0) tma_load_2d(&sm.p[s], M.tmap + ((k & 1) ? 2 : 1), xs, ys, &sm.bar[s]);   // p_old: p1 if k odd
}

template <bool IN>
__device__ __forceinline__ void mv_tile_t(const CtaCtx& x, const MixDesc& M, const MTile& tl, int k, float beta,
                                          const MvStage& zs, const MvStage& ps, RedSmem& rsm) {
  const Lvl L0 = M.lev[0];
  float* pnew = (k & 1) ? M.p0 : M.p1;
  const int i0 = tl.i0, j0 = tl.j0;
  const float din = mg_diag_in(L0);
  // p at halo cell (j, i): formed where it is read, with ph_matvec's operation
  auto at = [&](int j, int i) {
    const int r = j - j0 + 1, c = i - i0 + MV_X0;
    const float zv = zs.v[r][c];
    return k == 0 ? zv : fmaf(beta, ps.v[r][c], zv);
  };
  const int tx = x.tid() & 31;
  const int gi = i0 + tx;
  FF v[1] = {{0.f, 0.f}};
  MX_ROWS_X({
    const int gj = j0 + ty;
    if (IN || (gi < L0.nx && gj < L0.ny)) {
      const float pv = at(gj, gi);
      const float qv = lv_diag<IN>(L0, din, gj, gi) * pv - lv_nsum<IN>(L0, gj, gi, at);
      const long o = (long)gj * L0.ld + gi;
      pnew[o] = pv;
      M.q[o] = qv;
      ff_add_prod(v[0], pv, qv);
    }
  })
  // the tile's partial of p.q, formed as dred_sum_ff forms it and stored without a
  // fence: the CTA publishes its tiles of an instance together (mv_publish)
  const FF a = ff_warp_sum(v[0]);
  if ((x.tid() & 31) == 0) rsm.w[0][x.tid() >> 5] = (double)a.hi + (double)a.lo;
  double d[1] = {0.0};
  dred_warps<1, MT>(x, d, rsm);
  if (x.tid() == 0) M.part[tl.loc] = d[0];
}

// Publish cnt tile partials of instance M (one fence and one arrival for all of
// them); the CTA whose arrival completes the instance's tiles adds the partials in
// tile order exactly as dred_finish does and forms alpha.
__device__ __forceinline__ void mv_publish(const CtaCtx& x, const MixDesc& M, int cnt, RedSmem& rsm) {
  if (x.tid() == 0) {
    __threadfence();
    const unsigned before = atomicAdd(M.ticket, (unsigned)cnt);
    rsm.last = (before + (unsigned)cnt == (unsigned)M.nt0) ? 1 : 0;
  }
  x.sync();
  if (!rsm.last) return;
  __threadfence();
  double sum[1] = {0.0};
  for (int k = x.tid(); k < M.nt0; k += MT) sum[0] += __ldcg(&M.part[k]);
  dred_block<1, MT>(x, sum, rsm);
  if (x.tid() == 0) {
    atomicExch(M.ticket, 0u);
    MixCtrl* ctrl = M.ctrl;
    ctrl->pq = sum[0];
    ctrl->alpha = cget(&ctrl->rho) / sum[0];
  }
}

// e += alpha p; r -= alpha q (from residual buffer k & 1 into buffer (k + 1) & 1);
// ||r||^2 and the inner stopping test; then, for an instance with a level below,
// the fused down-sweep of level 0 on the new residual (its 3-cell halo formed
// from the old residual and q, which no tile of this phase writes).
struct UpdDownSmem {
  float sf[BY + 2 * H3][BX + 2 * H3];
  DownSmem d;
  RedSmem rsm;
};

template <bool IN, class X>
__device__ __forceinline__ void ph_update_down_t(const X& x, const MixDesc& M, const MTile& tl, MixLoop* ml,
                                               cudaGraphConditionalHandle cond_inner, int use_cond, Smooth sw,
                                               UpdDownSmem& sm) {
  RedSmem& rsm = sm.rsm;
  Lvl L0 = M.lev[0];
  MixCtrl* ctrl = M.ctrl;
  const int k = cget(&ctrl->inner);
  const float* fo = (k & 1) ? M.f0b : L0.f;
  float* fn = (k & 1) ? L0.f : M.f0b;
  const float* p = (k & 1) ? M.p0 : M.p1;
  const float alpha = (float)cget(&ctrl->alpha);
  FF v[1] = {{0.f, 0.f}};
  double out[1];
  {
    // four adjacent cells of one row a thread, as 16-byte accesses (rows start on 128-byte
    // boundaries: the pitch is a multiple of 32 cells); a group that crosses the last
    // column goes cell by cell
    const int j = tl.j0 + (x.tid() >> 3), i = tl.i0 + ((x.tid() & 7) << 2);
    if (j < L0.ny && i < L0.nx) {
      const long o = (long)j * L0.ld + i;
      if (i + 3 < L0.nx) {
        const float4 p4 = x.ld(reinterpret_cast<const float4*>(p + o));
        const float4 e4 = x.ld(reinterpret_cast<const float4*>(M.e + o));
        const float4 q4 = x.ld(reinterpret_cast<const float4*>(M.q + o));
        const float4 r4 = x.ld(reinterpret_cast<const float4*>(fo + o));
        const float4 en = make_float4(fmaf(alpha, p4.x, e4.x), fmaf(alpha, p4.y, e4.y), fmaf(alpha, p4.z, e4.z),
                                      fmaf(alpha, p4.w, e4.w));
        const float4 rn = make_float4(fmaf(-alpha, q4.x, r4.x), fmaf(-alpha, q4.y, r4.y), fmaf(-alpha, q4.z, r4.z),
                                      fmaf(-alpha, q4.w, r4.w));
        *reinterpret_cast<float4*>(M.e + o) = en;
        *reinterpret_cast<float4*>(fn + o) = rn;
        ff_add_prod(v[0], rn.x, rn.x);
        ff_add_prod(v[0], rn.y, rn.y);
        ff_add_prod(v[0], rn.z, rn.z);
        ff_add_prod(v[0], rn.w, rn.w);
      } else {
        for (int c = 0; c < 4 && i + c < L0.nx; ++c) {
          const float pv = x.ld(p + o + c), ev = x.ld(M.e + o + c), qv = x.ld(M.q + o + c), rv0 = x.ld(fo + o + c);
          M.e[o + c] = fmaf(alpha, pv, ev);
          const float rv = fmaf(-alpha, qv, rv0);
          fn[o + c] = rv;
          ff_add_prod(v[0], rv, rv);
        }
      }
    }
  }
  if (X_RED_FF(1, v, out) && x.tid() == 0) {
    const double rr = out[0];
    const int it = k + 1;
    ctrl->inner = it;
    ctrl->inner_total = cget(&ctrl->inner_total) + 1;
    ctrl->rr_in = rr;
    if (!(sqrt(rr) > cget(&ctrl->tol_abs_in)) || it >= cget(&ctrl->max_inner)) {
      ctrl->inner_done = 1;
      if (atomicSub(&ml->inner_active, 1) == 1 && use_cond) cudaGraphSetConditional(cond_inner, 0u);
    }
  }
  if (M.nlev < 2) return;
  // the new residual on the tile and a 3-cell halo (every load first, then the
  // stores), then the down-sweep as ph_down
  const int i0 = tl.i0, j0 = tl.j0;
  const float din = mg_diag_in(L0);
  auto inside = [&](int gj, int gi) { return IN || (gj >= 0 && gj < L0.ny && gi >= 0 && gi < L0.nx); };
  // (in two batches of loads: the kernel's register budget holds half the halo)
  constexpr int HW = BX + 2 * H3, HN = (BY + 2 * H3) * HW, NI = (HN + MT - 1) / MT, NB = (NI + 1) / 2;
#pragma unroll
  for (int b = 0; b < NI; b += NB) {
    float hq[NB], hf[NB];
#pragma unroll
    for (int t = 0; t < NB; ++t) {
      const int idx = x.tid() + (b + t) * MT;
      const int gj = j0 + idx / HW - H3, gi = i0 + idx % HW - H3;
      hq[t] = 0.f;
      hf[t] = 0.f;
      if (b + t < NI && (b + t < NI - 1 || idx < HN) && inside(gj, gi)) {
        const long o = (long)gj * L0.ld + gi;
        hq[t] = x.ld(M.q + o);
        hf[t] = x.ld(fo + o);
      }
    }
#pragma unroll
    for (int t = 0; t < NB; ++t) {
      const int idx = x.tid() + (b + t) * MT;
      if (b + t < NI && (b + t < NI - 1 || idx < HN)) {
        const int jj = idx / HW - H3, ii = idx % HW - H3;
        float r = 0.f;
        if (inside(j0 + jj, i0 + ii)) r = fmaf(-alpha, hq[t], hf[t]);
        sm.sf[jj + H3][ii + H3] = r;
      }
    }
  }
  x.sync();
  const Lvl C = M.lev[1];
  DownSmem& d = sm.d;
  auto fval = [&](int gj, int gi) { return sm.sf[gj - j0 + H3][gi - i0 + H3]; };
  for (int idx = x.tid(); idx < (BY + 2 * H3) * (BX + 2 * H3); idx += MT) {
    const int jj = idx / (BX + 2 * H3) - H3, ii = idx % (BX + 2 * H3) - H3;
    const int gj = j0 + jj, gi = i0 + ii;
    float s1 = 0.f;
    if (inside(gj, gi)) s1 = __fdividef(sw.w1 * fval(gj, gi), lv_diag<IN>(L0, din, gj, gi));
    d.s1[jj + H3][ii + H3] = s1;
  }
  x.sync();
  for (int idx = x.tid(); idx < (BY + 4) * (BX + 4); idx += MT) {
    const int jj = idx / (BX + 4) - 2, ii = idx % (BX + 4) - 2;
    const int gj = j0 + jj, gi = i0 + ii;
    float s2 = 0.f;
    if (inside(gj, gi)) {
      auto at = [&](int j, int i) { return d.s1[j - j0 + H3][i - i0 + H3]; };
      s2 = fmaf(1.f - sw.w2, d.s1[jj + H3][ii + H3],
                __fdividef(sw.w2 * (fval(gj, gi) + lv_nsum<IN>(L0, gj, gi, at)), lv_diag<IN>(L0, din, gj, gi)));
    }
    d.s2[jj + 2][ii + 2] = s2;
  }
  x.sync();
  for (int idx = x.tid(); idx < (BY + 2) * (BX + 2); idx += MT) {
    const int jj = idx / (BX + 2) - 1, ii = idx % (BX + 2) - 1;
    const int gj = j0 + jj, gi = i0 + ii;
    float rr = 0.f;
    if (inside(gj, gi)) {
      auto at = [&](int j, int i) { return d.s2[j - j0 + 2][i - i0 + 2]; };
      const float t = d.s2[jj + 2][ii + 2];
      rr = fval(gj, gi) - (lv_diag<IN>(L0, din, gj, gi) * t - lv_nsum<IN>(L0, gj, gi, at));
      if (jj >= 0 && jj < BY && ii >= 0 && ii < BX) L0.t[(long)gj * L0.ld + gi] = t;
    }
    d.rs[jj + 1][ii + 1] = rr;
  }
  x.sync();
  const int cw = BX / L0.kx, chh = BY / L0.ky;
  const int I0 = i0 / L0.kx, J0 = j0 / L0.ky;
  for (int idx = x.tid(); idx < cw * chh; idx += MT) {
    const int jj = idx / cw, ii = idx - jj * cw;
    const int I = I0 + ii, J = J0 + jj;
    if (IN || (I < C.nx && J < C.ny))
      C.f[(long)J * C.ld + I] = restrict_lv<IN>(&d.rs[0][0], BX + 2, j0 - 1, i0 - 1, C.nx, C.ny, L0.kx, L0.ky, J, I);
  }
}

template <class X>
__device__ __forceinline__ void ph_update_down(const X& x, const MixDesc& M, const MTile& tl, MixLoop* ml,
                                               cudaGraphConditionalHandle cond_inner, int use_cond, Smooth sw,
                                               UpdDownSmem& sm) {
  if (M.interior && tile_interior(tl, M.lev[0].nx, M.lev[0].ny, H3)) ph_update_down_t<true>(x, M, tl, ml, cond_inner, use_cond, sw, sm);
  else ph_update_down_t<false>(x, M, tl, ml, cond_inner, use_cond, sw, sm);
}

union TileSmem {
  DownSmem d;
  PostSmem p;
  MatvecSmem m;
  UpdDownSmem u;
  RedSmem r;
};

// x += e - e[0] (binary64)
template <class X>
__device__ __forceinline__ void ph_correct(const X& x, const MixDesc& M, const MTile& tl) {
  const Geo G = M.G;
  const long lde = M.lev[0].ld;
  const int i = tl.i0 + (x.tid() & 31);
  const double e0 = f2d(x.ld(M.e));
  double xv[RPT];
  float ev[RPT];
#pragma unroll
  for (int r_ = 0; r_ < RPT; ++r_) {
    const int j = tl.j0 + (x.tid() >> 5) + r_ * (MT / 32);
    if (i < G.nx && j < G.ny) {
      xv[r_] = x.ld(M.x + (long)j * G.ld + i);
      ev[r_] = x.ld(M.e + (long)j * lde + i);
    }
  }
#pragma unroll
  for (int r_ = 0; r_ < RPT; ++r_) {
    const int j = tl.j0 + (x.tid() >> 5) + r_ * (MT / 32);
    if (i < G.nx && j < G.ny) M.x[(long)j * G.ld + i] = __dadd_rn(xv[r_], __dsub_rn(f2d(ev[r_]), e0));
  }
}

// r64 = b - A x (the pinned operator, row 0 the identity; lap_recip_at elsewhere);
// ||r64||^2, sum(r64); outer test
template <class X>
__device__ __forceinline__ void ph_resid(const X& x, const MixDesc& M, const MTile& tl, MixLoop* ml,
                                         cudaGraphConditionalHandle cond_outer, int use_cond, RedSmem& rsm) {
  const Geo G = M.G;
  MixCtrl* ctrl = M.ctrl;
  const int i = tl.i0 + (x.tid() & 31);
  double v[2] = {0.0, 0.0}, out[2];
  const auto Xv = x.view(M.x, G.ld);
  MX_ROWS_X({
    const int j = tl.j0 + ty;
    if (i < G.nx && j < G.ny) {
      const double ax = (i == 0 && j == 0) ? Xv(0, 0) : -lap_recip_at(Xv, j, i, G);
      const long o = (long)j * G.ld + i;
      const double rv = __dsub_rn(x.ld(M.b + o), ax);
      M.r64[o] = rv;
      v[0] += rv * rv;
      v[1] += rv;
    }
  })
  if (X_RED(2, v, out) && x.tid() == 0) {
    const double rr = out[0];
    ctrl->rr64 = rr;
    ctrl->sum64 = out[1];
    const int outer = cget(&ctrl->outer) + 1;
    ctrl->outer = outer;
    const bool conv = !(sqrt(rr) > cget(&ctrl->tol_abs_out));
    ctrl->converged = conv ? 1 : 0;
    if (outer == 1) {
      // the first pass's outcome steers the next solves' first passes (ph_prep)
      if (cget(&ctrl->reach_tried)) {
        if (!conv) {
          ctrl->reach = 0;
          ctrl->reach_wait = REACH_WAIT;
        }
      } else if (!cget(&ctrl->reach)) {
        const int w = cget(&ctrl->reach_wait) - 1;
        ctrl->reach_wait = w;
        if (w <= 0) ctrl->reach = 1;
      }
    }
    if (conv || outer >= cget(&ctrl->max_outer)) {
      ctrl->outer_done = 1;
      if (atomicSub(&ml->outer_active, 1) == 1 && use_cond) cudaGraphSetConditional(cond_outer, 0u);
    }
  }
}

// Levels of at most 4096 cells run inside one CTA per instance: all of them
// live in shared memory and one V-cycle (the same smoother, restriction and
// prolongation as the global levels; the bottom level, at most 64 cells, by its
// pseudo-inverse, else eight Jacobi sweeps) forms the coarse "solve" -- a fixed
// linear, symmetric operator, as PCG requires.  The CTA has NT threads (1024, or
// 512 for batches of more instances than SMs, two CTAs to an SM); every cell is
// computed with the same operations whatever NT is, and every sum is taken in an
// order that does not depend on NT, so both give the same bits.
constexpr int CT = 1024;                     // threads of the coarse CTA (and of the persistent CTAs)
constexpr int CT2 = 512;                     // the batch form
constexpr int CMAX = 4096;                   // cells of its finest level
constexpr int BMAX = 64;                     // bottom levels up to this size are solved exactly

// A shared-memory level, stored with a one-cell ring around it: interior cell
// (j, i) at off + (j + 1) * pw + i + 1, pw = nx + 2.  The ring makes every
// stencil branch-free.  It holds zeros while the array is the source of a
// smoothing sweep or of a residual (a Neumann level has no neighbour across a
// wall; the diagonal counts only the faces that exist), and the mirror image of
// the edge cells while the array is read by the restriction or the prolongation
// (a wall cell then takes all of its parent's weight, 3/4 + 1/4 of the same value,
// as the global levels' wall rules give it).
struct CLvl {
  int nx, ny, off, pw;
  float cx, cy;
  int kx, ky;                                // coarsening factors to the next level
};


// cx (a_W + a_E) + cy (a_S + a_N) at padded index c (the ring supplies the walls' zeros)
__device__ __forceinline__ float c_nsum(const CLvl& L, const float* a, int c) {
  return fmaf(L.cy, a[c + L.pw], fmaf(L.cy, a[c - L.pw], fmaf(L.cx, a[c + 1], L.cx * a[c - 1])));
}

// v into the ring cells next to edge cell (j, i) at padded index c (corners included)
__device__ __forceinline__ void c_ring(float* a, const CLvl& L, int c, int j, int i, float v) {
  const bool w0 = i == 0, w1 = i == L.nx - 1;
  if (w0) a[c - 1] = v;
  if (w1) a[c + 1] = v;
  if (j == 0) {
    a[c - L.pw] = v;
    if (w0) a[c - L.pw - 1] = v;
    if (w1) a[c - L.pw + 1] = v;
  }
  if (j == L.ny - 1) {
    a[c + L.pw] = v;
    if (w0) a[c + L.pw - 1] = v;
    if (w1) a[c + L.pw + 1] = v;
  }
}

// Cells of a shared-memory level, visited by the CTA's NT / 32 warps, a row of 32
// cells to a warp; c is the padded index of cell (j, i).  The column is the outer
// loop, so that what depends on i alone (the x faces of the diagonal, the left and
// right rings) is computed once for the thread's rows.
#define C_FOR(Lv, ...)                                               \
  for (int i = threadIdx.x & 31; i < (Lv).nx; i += 32)               \
    for (int j = threadIdx.x >> 5; j < (Lv).ny; j += NT / 32) {      \
      const int c = (Lv).off + (j + 1) * (Lv).pw + i + 1;            \
      __VA_ARGS__                                                    \
    }

// C_FOR with v = tab[3 fx + fy], the cell's entry in a level's nine-entry diagonal
// table (fx, fy: the faces it has in x, in y).  The column's two candidates (rows
// inside, rows on a y edge) are read once per column; the row picks one of them.
#define C_FORD(Lv, tab, v, ...)                                                \
  for (int i = threadIdx.x & 31; i < (Lv).nx; i += 32) {                       \
    const int kx_ = 3 * ((i > 0) + (i < (Lv).nx - 1));                         \
    const float vin_ = (tab)[kx_ + 2], ved_ = (tab)[kx_ + ((Lv).ny > 1)];      \
    for (int j = threadIdx.x >> 5; j < (Lv).ny; j += NT / 32) {                \
      const int c = (Lv).off + (j + 1) * (Lv).pw + i + 1;                      \
      const float v = (j > 0 && j < (Lv).ny - 1) ? vin_ : ved_;                \
      __VA_ARGS__                                                              \
    }                                                                          \
  }

// one weighted-Jacobi sweep src -> dst on level L (zero ring on src); rd: the level's
// reciprocal diagonals; all threads, ends with a barrier
template <int NT>
__device__ __forceinline__ void c_sweep(const CLvl& L, const float* rd, const float* f, const float* src, float* dst,
                                        float omega) {
  C_FORD(L, rd, r, { dst[c] = fmaf(1.f - omega, src[c], omega * (f[c] + c_nsum(L, src, c)) * r); })
  __syncthreads();
}

// Shared tables of the coarse V-cycle: the level table and each level's nine
// diagonals and their reciprocals.
struct CoarseSmem {
  CLvl L[8];
  float d[8][9], rd[8][9];
  int tot;
};

constexpr int NSL = 16;   // slices of the exact bottom solve's sums (held in w: at least NSL * BMAX floats)

// The part of the coarse V-cycle that reads only static data: the level table and
// diagonals and the zeros of e and w (rings included).  It may run before the wait
// on the kernels that write the cycle's right-hand side.  sm: rh, e and w, tot
// floats each (w at least NSL * BMAX when the bottom level is solved exactly).  No
// closing barrier: coarse_run starts with one.
template <int NT>
__device__ void coarse_prep(const MixDesc& M, CoarseSmem& cs, float* sm) {
  const Lvl& C = M.lev[M.nlev - 1];
  const int nl = M.coarse_levels;
  if (threadIdx.x == 0) {
    int nx = C.nx, ny = C.ny, t = 0;
    for (int l = 0; l < nl; ++l) {
      cs.L[l] = CLvl{nx, ny, t, nx + 2, M.ccx[l], M.ccy[l], M.ckx[l], M.cky[l]};
      t += (nx + 2) * (ny + 2);
      nx /= M.ckx[l];
      ny /= M.cky[l];
    }
    cs.tot = t;
  }
  if (threadIdx.x < 8 * 9) {
    const int l = threadIdx.x / 9, k = threadIdx.x - 9 * l, fx = k / 3, fy = k - 3 * fx;
    if (l < nl) {
      float d = 0.f;
      if (fx >= 1) d += M.ccx[l];
      if (fx == 2) d += M.ccx[l];
      if (fy >= 1) d += M.ccy[l];
      if (fy == 2) d += M.ccy[l];
      cs.d[l][k] = d;
      cs.rd[l][k] = d > 0.f ? 1.f / d : 0.f;
    }
  }
  __syncthreads();
  const int tot = cs.tot;
  for (int k = threadIdx.x; k < 2 * tot; k += NT) sm[tot + k] = 0.f;   // e and w with their rings
}

// The coarse V-cycle of instance M by the whole NT-thread CTA, after coarse_prep.
template <int NT>
__device__ void coarse_run(const MixDesc& M, int bottom_sweeps, Smooth sw, const CoarseSmem& cs, float* sm) {
  __syncthreads();
  Lvl C = M.lev[M.nlev - 1];
  if (M.nlev == 1) C.f = f_cur(M);
  const int nl = M.coarse_levels;
  const CLvl* L = cs.L;
  const int tot = cs.tot;
  float* rh = sm;            // right-hand side of every level (level 0: the entry level's f)
  float* e = sm + tot;       // pre-smoothed iterate on the way down; the bottom solution
  float* w = sm + 2 * tot;   // residual on the way down; each level's result on the way up
  const CLvl Le = L[0];   // register copies of the level descriptors (the level arrays are written
                          // through pointers the compiler cannot tell from the shared table)
  // the loop state that the closing r.z of a single-level instance updates, read now
  // so that its latency overlaps the cycle (only this CTA writes them meanwhile)
  int inner0 = 0;
  double rho0 = 0.0;
  if (M.nlev == 1 && threadIdx.x == 0) {
    inner0 = cget(&M.ctrl->inner);
    rho0 = cget(&M.ctrl->rho);
  }
  {
    // the entry level's right-hand side, eight loads in flight a thread: cells
    // threadIdx.x + k NT in row-major order, (j, i) stepped by (NT / nx, NT % nx)
    const int dj = NT / Le.nx, di = NT - dj * Le.nx;
    int j = threadIdx.x / Le.nx, i = threadIdx.x - j * Le.nx;
    while (j < Le.ny) {
      float t[8];
      int c[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const bool in = j < Le.ny;
        t[u] = in ? __ldcg(C.f + (long)j * C.ld + i) : 0.f;
        c[u] = in ? Le.off + (j + 1) * Le.pw + i + 1 : -1;
        i += di;
        j += dj;
        if (i >= Le.nx) {
          i -= Le.nx;
          ++j;
        }
      }
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (c[u] >= 0) rh[c[u]] = t[u];
    }
  }
  __syncthreads();
  for (int l = 0; l + 1 < nl; ++l) {
    const CLvl Lv = L[l];
    const float* d = cs.d[l];
    const float* rd = cs.rd[l];
    // e = S(S(0)): the first sweep from zero is pointwise, w = w1 D^-1 rh (zero ring), then the second
    C_FORD(Lv, rd, r, { w[c] = sw.w1 * rh[c] * r; })
    __syncthreads();
    C_FORD(Lv, rd, r, { e[c] = fmaf(1.f - sw.w2, w[c], sw.w2 * (rh[c] + c_nsum(Lv, w, c)) * r); })
    __syncthreads();
    // residual rh - A e into w, its ring the mirror of its edges; then rh_{l+1} = P^T w
    C_FORD(Lv, d, dv, {
      const float v = rh[c] - (dv * e[c] - c_nsum(Lv, e, c));
      w[c] = v;
      c_ring(w, Lv, c, j, i, v);
    })
    __syncthreads();
    const CLvl Cv = L[l + 1];
    const float* wf = w + Lv.off + Lv.pw + 1;
    C_FOR(Cv, { rh[c] = restrict_lv<true>(wf, Lv.pw, 0, 0, Cv.nx, Cv.ny, Lv.kx, Lv.ky, j, i); })
    __syncthreads();
  }
  {
    const CLvl Lv = L[nl - 1];
    const int nb = Lv.nx * Lv.ny;
    auto cell = [&Lv](int q) {            // padded index of bottom cell q (row-major)
      const int qj = q / Lv.nx;
      return Lv.off + (qj + 1) * Lv.pw + (q - qj * Lv.nx) + 1;
    };
    if (M.binv) {
      // exact bottom solve: e = A+ rh (at most BMAX cells).  A+ is exactly symmetric, so
      // column q0 is read for row q0 (consecutive threads, consecutive addresses); the
      // sum over q is split into NSL slices of qs <= 4 terms, added in slice order
      // through w (dead past the restrictions; the up-sweep rewrites it, rings included).
      const int qs = (nb + NSL - 1) / NSL;
      for (int v = threadIdx.x; v < NSL * nb; v += NT) {
        const int h = v / nb, q0 = v - h * nb, qa = h * qs;
        float b[4], r[4];
        int qj = qa / Lv.nx, qi = qa - qj * Lv.nx;   // cell qa + k, stepped along its row
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const bool in = k < qs && qa + k < nb;
          b[k] = in ? __ldg(M.binv + (long)(qa + k) * nb + q0) : 0.f;
          r[k] = in ? rh[Lv.off + (qj + 1) * Lv.pw + qi + 1] : 0.f;
          if (++qi == Lv.nx) {
            qi = 0;
            ++qj;
          }
        }
        float acc = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (k < qs && qa + k < nb) acc = fmaf(b[k], r[k], acc);
        w[v] = acc;
      }
      __syncthreads();
      for (int q0 = threadIdx.x; q0 < nb; q0 += NT) {
        float sacc = w[q0];
        for (int k = 1; k < NSL; ++k) sacc += w[k * nb + q0];
        const int qj = q0 / Lv.nx, c = cell(q0);
        e[c] = sacc;
        c_ring(e, Lv, c, qj, q0 - qj * Lv.nx, sacc);
      }
      __syncthreads();
    } else {
      // Jacobi sweeps from e = 0 between e and w (both zero, rings included), then the
      // result into e with its mirror ring
      for (int q = 0; q < bottom_sweeps; ++q) c_sweep<NT>(Lv, cs.rd[nl - 1], rh, (q & 1) ? w : e, (q & 1) ? e : w, sw.wb);
      const float* res = (bottom_sweeps & 1) ? w : e;
      C_FOR(Lv, {
        const float v = res[c];
        e[c] = v;
        c_ring(e, Lv, c, j, i, v);
      })
      __syncthreads();
    }
  }
  // up: w_l = S(S(e_l + P result_{l+1})); the bottom's result is in e, every other level's in w
  for (int l = nl - 2; l >= 0; --l) {
    const CLvl Lv = L[l];
    const CLvl Cv = L[l + 1];
    const float* rd = cs.rd[l];
    const float* zc = ((l + 1 == nl - 1) ? e : w) + Cv.off + Cv.pw + 1;   // mirror ring
    const int cpw = Cv.pw;
    auto catc = [zc, cpw](int J, int I) { return zc[J * cpw + I]; };
    C_FOR(Lv, {
      w[c] = e[c] + prolong_lv<true>(catc, Cv.nx, Cv.ny, Lv.kx, Lv.ky, j, i);
      c_ring(w, Lv, c, j, i, 0.f);         // zero ring: w is the next sweep's source
    })
    __syncthreads();
    c_sweep<NT>(Lv, rd, rh, w, e, sw.w2);
    C_FORD(Lv, rd, r, {
      const float v = fmaf(1.f - sw.w1, e[c], sw.w1 * (rh[c] + c_nsum(Lv, e, c)) * r);
      w[c] = v;
      if (l > 0) c_ring(w, Lv, c, j, i, v);   // mirror ring for the next prolongation
    })
    __syncthreads();
  }
  const float* z = (nl == 1) ? e : w;
  C_FOR(Le, { C.u[(long)j * C.ld + i] = z[c]; })
  if (M.nlev == 1) {
    // the V-cycle ran entirely here: rho = r.z over level 0, summed as the tile phases do,
    // as 1024 lanes (row j to lane-row j mod 32) whatever NT is
    __shared__ double wsum[CT / 32];
    const CLvl L0 = L[0];
#pragma unroll
    for (int m = 0; m < CT / NT; ++m) {
      const int vw = (threadIdx.x >> 5) + m * (NT / 32);
      FF acc = {0.f, 0.f};
      for (int j = vw; j < L0.ny; j += CT / 32)
        for (int i = threadIdx.x & 31; i < L0.nx; i += 32) {
          const int c = (j + 1) * L0.pw + i + 1;
          ff_add_prod(acc, rh[c], z[c]);
        }
      acc = ff_warp_sum(acc);
      if ((threadIdx.x & 31) == 0) wsum[vw] = (double)acc.hi + (double)acc.lo;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      // the CT / 32 row sums by a fixed shuffle tree (every lane ends with the same bits)
      double rz = wsum[threadIdx.x];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) rz += __shfl_xor_sync(0xffffffffu, rz, o);
      if (threadIdx.x == 0) {
        if (inner0 > 0) M.ctrl->beta = rz / rho0;
        M.ctrl->rho = rz;
      }
    }
  }
  __syncthreads();
}

// ---- kernels: one tile per 256-thread CTA -----------------------------------

// The CTA's tile; its instance's descriptor staged in shared memory before the
// wait on the predecessor, and the liveness test after it.
#define CTA_TILE(gate)                          \
  pdl_launch();                                 \
  __shared__ MixDesc smd_;                      \
  const MTile tl = TL[blockIdx.x];              \
  stage_desc(MD + tl.inst, &smd_);              \
  pdl_wait();                                   \
  __syncthreads();                              \
  const MixDesc& M = smd_;                      \
  if (!mx_live(M, gate)) return;                \
  const CtaCtx x{};

__global__ void __launch_bounds__(MT, 6) k_mg_down(const MixDesc* __restrict__ MD, const MTile* __restrict__ TL, int l,
                                                 int gate, Smooth sw) {
  CTA_TILE(gate)
  __shared__ DownSmem sm;
  ph_down(x, M, tl, l, sw, sm);
}

__global__ void __launch_bounds__(MT, 5) k_mg_post(const MixDesc* __restrict__ MD, const MTile* __restrict__ TL, int l,
                                                 int gate, Smooth sw) {
  CTA_TILE(gate)
  __shared__ PostSmem sm;
  ph_post(x, M, tl, l, sw, sm);
}

// one CTA per instance
template <int NT>
__global__ void __launch_bounds__(NT, CT / NT) k_mg_coarse(const MixDesc* __restrict__ MD, const int* __restrict__ order,
                                                            int gate, int bottom_sweeps, Smooth sw) {
  pdl_launch();
  __shared__ MixDesc smd;
  __shared__ CoarseSmem cs;
  extern __shared__ float csm[];
  stage_desc(MD + order[blockIdx.x], &smd);
  __syncthreads();
  const MixDesc& M = smd;
  coarse_prep<NT>(M, cs, csm);      // static data only: overlaps the predecessor
  pdl_wait();
  if (!mx_live(M, gate)) return;
  coarse_run<NT>(M, bottom_sweeps, sw, cs, csm);
}

__global__ void __launch_bounds__(MT) k_mx_init(const MixDesc* __restrict__ MD, const MTile* __restrict__ TL,
                                                 MixLoop* ml) {
  pdl_launch();
  __shared__ MixDesc smd;
  const MTile tl = TL[blockIdx.x];
  stage_desc(MD + tl.inst, &smd);
  pdl_wait();
  __syncthreads();
  const MixDesc& M = smd;
  if (!*M.active) return;
  __shared__ RedSmem rsm;
  ph_init(CtaCtx{}, M, tl, ml, rsm);
}

__global__ void k_ml_reset(MixLoop* ml, int which) {
  pdl_enter();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (which == 0) {
    ml->outer_active = 0;
    ml->guard_o = 0;
    ml->tripped = 0;
    ml->gb.count = 0u;
    ml->gb.err = 0;
    __threadfence();
  } else {
    ml->inner_active = 0;
    ml->guard_i = 0;
  }
}

// condition of a loop = some instance still in it
__global__ void k_ml_arm(MixLoop* ml, int which, cudaGraphConditionalHandle cond, int use_cond) {
  pdl_enter();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int a = which == 0 ? ml->outer_active : ml->inner_active;
  if (use_cond) cudaGraphSetConditional(cond, a > 0 ? 1u : 0u);
}

__global__ void __launch_bounds__(MT) k_mx_prep(const MixDesc* __restrict__ MD, const MTile* __restrict__ TL,
                                                 MixLoop* ml) {
  CTA_TILE(0)
  __shared__ RedSmem rsm;
  ph_prep(x, M, tl, ml, rsm);
}

__global__ void __launch_bounds__(MT, 6) k_mx_matvec(const MixDesc* __restrict__ MD, const MTile* __restrict__ TL) {
  CTA_TILE(1)
  __shared__ MatvecSmem sm;
  ph_matvec(x, M, tl, sm);
}

// The TMA form (see mv_tile_t).  A stage's barrier that is not complete after
// MV_SPIN_LIMIT polls stops the kernel: the CTA records it in the loop control's
// error flag (the step then reports a failed solve), waits -- again bounded --
// for the copy it has in flight into the other stage, and returns.
__global__ void __launch_bounds__(MT, 4) k_mx_matvec_tma(const MixDesc* __restrict__ MD, const MTile* __restrict__ TL,
                                                          int ntiles, MixLoop* ml) {
  pdl_launch();
  __shared__ MvSmem sm;
  const CtaCtx x{};
  if (x.tid() == 0) {
    mbar_init(&sm.bar[0], 1u);
    mbar_init(&sm.bar[1], 1u);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  const int g = gridDim.x;
  int t = blockIdx.x;
  // the tile table is read one tile ahead of its use (the next tile's entry is at hand
  // when its copies are issued), and what a tile needs of its instance (live or not, the
  // inner iteration, beta) is read once per run of tiles of one instance: none of it
  // changes during the launch, so the chain of dependent loads is paid per instance
  MTile tl = t < ntiles ? TL[t] : MTile{0, 0, 0, 0};
  MTile tln = t + g < ntiles ? TL[t + g] : MTile{0, 0, 0, 0};
  pdl_wait();                       // the barriers and the tile table need no predecessor
  __syncthreads();
  int ii = -1, ilive = 0, ik = 0;   // thread 0's instance of the copies
  auto issue = [&](const MTile& u, int stage) -> bool {
    if (u.inst != ii) {
      ii = u.inst;
      ilive = mx_live(MD[ii], 1) ? 1 : 0;
      ik = ilive ? cget(&MD[ii].ctrl->inner) : 0;
    }
    if (ilive) mv_issue(MD[ii], u, ik, sm, stage);
    return ilive != 0;
  };
  if (t < ntiles && x.tid() == 0) issue(tl, 0);
  unsigned phase = 0u;
  int cur = -1, cnt = 0;        // the instance of the partials not yet published, and their number
  bool live = false;
  int k = 0;
  float beta = 0.f;
  for (int n = 0; t < ntiles; ++n) {
    const int s = n & 1;
    const int tn = t + g;
    const MTile tlnn = tn + g < ntiles ? TL[tn + g] : MTile{0, 0, 0, 0};
    // the next tile's copies go into the other stage, whose last reader (the tile before)
    // finished with the barriers of its reduction
    bool next = false;
    if (tn < ntiles && x.tid() == 0) next = issue(tln, s ^ 1);
    if (tl.inst != cur) {
      if (cnt) mv_publish(x, MD[cur], cnt, sm.rsm);
      cur = tl.inst;
      cnt = 0;
      const MixDesc& Mc = MD[cur];
      live = mx_live(Mc, 1);
      k = live ? cget(&Mc.ctrl->inner) : 0;
      beta = live ? (float)cget(&Mc.ctrl->beta) : 0.f;
    }
    if (live) {
      const unsigned par = (phase >> s) & 1u;
      const bool ok = mbar_wait_bounded(&sm.bar[s], par);
      phase ^= 1u << s;
      if (__syncthreads_or(!ok)) {
        // a copy did not land in time: flag the error, and before the CTA (and its
        // shared memory) goes, wait -- longer, still bounded -- for each copy it may
        // have in flight: this tile's (stage s) unless thread 0 saw it land, and the
        // next tile's (stage s ^ 1) if thread 0 issued it.  A copy still outstanding
        // after that is abandoned; the step reports the failed wait to the host.
        if (x.tid() == 0) {
          atomicExch(&ml->gb.err, 1);
          if (!ok) mbar_wait_bounded(&sm.bar[s], par, 16 * MV_SPIN_LIMIT);
          if (next) mbar_wait_bounded(&sm.bar[s ^ 1], (phase >> (s ^ 1)) & 1u, 16 * MV_SPIN_LIMIT);
        }
        return;
      }
      const MixDesc& M = MD[cur];
      if (M.interior && tile_interior(tl, M.lev[0].nx, M.lev[0].ny, 1))
        mv_tile_t<true>(x, M, tl, k, beta, sm.z[s], sm.p[s], sm.rsm);
      else
        mv_tile_t<false>(x, M, tl, k, beta, sm.z[s], sm.p[s], sm.rsm);
      ++cnt;
    }
    t = tn;
    tl = tln;
    tln = tlnn;
  }
  if (cnt) mv_publish(x, MD[cur], cnt, sm.rsm);
}

// The guard of a loop body, run by the last CTA of the body's last kernel to
// finish (an arrival ticket over the launch): it counts the body's trips and stops
// the loop at its trip bound whatever the instances report (the host then reports
// an error instead of waiting on a loop that does not end).  Every CTA of the
// launch arrives, whether or not its instance was live.
__device__ __forceinline__ void loop_guard(MixLoop* ml, int which, cudaGraphConditionalHandle cond) {
  __shared__ int s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned* t = which == 0 ? &ml->ticket_o : &ml->ticket_i;
    __threadfence();
    s_last = (atomicAdd(t, 1u) == gridDim.x - 1) ? 1 : 0;
    if (s_last) {
      __threadfence();
      atomicExch(t, 0u);
      const int g = which == 0 ? ++ml->guard_o : ++ml->guard_i;
      const int gmax = which == 0 ? ml->gmax_o : ml->gmax_i;
      const int a = atomicAdd(which == 0 ? &ml->outer_active : &ml->inner_active, 0);
      if (g >= gmax && a > 0) {
        ml->tripped = 1;
        cudaGraphSetConditional(cond, 0u);
      }
    }
  }
}

__global__ void __launch_bounds__(MT, 5) k_mx_update_down(const MixDesc* __restrict__ MD, const MTile* __restrict__ TL,
                                                        MixLoop* ml, cudaGraphConditionalHandle cond_inner, int use_cond,
                                                        Smooth sw) {
  pdl_launch();
  __shared__ MixDesc smd;
  const MTile tl = TL[blockIdx.x];
  stage_desc(MD + tl.inst, &smd);
  pdl_wait();
  __syncthreads();
  const MixDesc& M = smd;
  __shared__ UpdDownSmem sm;
  if (mx_live(M, 1)) ph_update_down(CtaCtx{}, M, tl, ml, cond_inner, use_cond, sw, sm);
  if (use_cond) loop_guard(ml, 1, cond_inner);
}

__global__ void __launch_bounds__(MT) k_mx_correct(const MixDesc* __restrict__ MD, const MTile* __restrict__ TL) {
  CTA_TILE(0)
  ph_correct(x, M, tl);
}

__global__ void __launch_bounds__(MT) k_mx_resid(const MixDesc* __restrict__ MD, const MTile* __restrict__ TL,
                                                  MixLoop* ml, cudaGraphConditionalHandle cond_outer, int use_cond) {
  pdl_launch();
  __shared__ MixDesc smd;
  const MTile tl = TL[blockIdx.x];
  stage_desc(MD + tl.inst, &smd);
  pdl_wait();
  __syncthreads();
  const MixDesc& M = smd;
  __shared__ RedSmem rsm;
  if (mx_live(M, 0)) ph_resid(CtaCtx{}, M, tl, ml, cond_outer, use_cond, rsm);
  if (use_cond) loop_guard(ml, 0, cond_outer);
}

// summary of the mixed solve for the step record
// ---- the persistent solve ------------------------------------------------------
//
// The whole refinement of every instance in one cooperative launch: one
// 1024-thread CTA per SM, each CTA four 256-thread groups that take the tiles of
// a phase in turn, and a grid barrier between phases.  The loop decisions
// (instances still refining, still in the inner solve) are read after a
// barrier, so every CTA takes the same branch.  A group that takes several
// tiles of a phase passes its barrier between them (a phase's first loop may
// write shared arrays its last loop still reads).  The phases are the functions
// the ordinary kernels run, on the same tiles in the same order, so the
// results are the same bits.  Loop trip bounds stop a solve whose instances do
// not report; a barrier that waits too long sets the error flag, and every CTA
// returns at its next barrier.

struct PersistArgs {
  const MixDesc* dd;
  int n, maxlev;
  const MTile* tl0;
  int nt0;
  const MTile* tpre[MAX_LEVELS];
  int ntpre[MAX_LEVELS];
  MixLoop* ml;
  Smooth sw;
  int bottom_sweeps;
};

__global__ void __launch_bounds__(CT, 1) k_mx_persist(PersistArgs A) {
  extern __shared__ __align__(16) unsigned char psm[];
  __shared__ CoarseSmem pcs;
  const GroupCtx x{(int)(threadIdx.x >> 8)};
  TileSmem& ts = reinterpret_cast<TileSmem*>(psm)[x.g];
  const int ngroups = gridDim.x * 4;
  const int gid = blockIdx.x * 4 + x.g;
  MixLoop* ml = A.ml;
  GridBar* gb = &ml->gb;
  auto vcycle = [&](int l0) -> bool {
    for (int l = l0; l + 1 < A.maxlev; ++l) {
      for (int t = gid; t < A.ntpre[l]; t += ngroups) {
        const MTile tl = A.tpre[l][t];
        const MixDesc& M = A.dd[tl.inst];
        if (mx_live(M, 1)) ph_down(x, M, tl, l, A.sw, ts.d);
        x.sync();
      }
      if (!grid_sync(gb)) return false;
    }
    for (int k = blockIdx.x; k < A.n; k += gridDim.x) {
      const MixDesc& M = A.dd[k];
      if (mx_live(M, 1)) {
        coarse_prep<CT>(M, pcs, reinterpret_cast<float*>(psm));
        coarse_run<CT>(M, A.bottom_sweeps, A.sw, pcs, reinterpret_cast<float*>(psm));
      }
    }
    if (!grid_sync(gb)) return false;
    for (int l = A.maxlev - 2; l >= 0; --l) {
      for (int t = gid; t < A.ntpre[l]; t += ngroups) {
        const MTile tl = A.tpre[l][t];
        const MixDesc& M = A.dd[tl.inst];
        if (mx_live(M, 1)) ph_post(x, M, tl, l, A.sw, ts.p);
        x.sync();
      }
      if (!grid_sync(gb)) return false;
    }
    return true;
  };
#define PERSIST_TILES(gate, body)                                  \
  for (int t = gid; t < A.nt0; t += ngroups) {                     \
    const MTile tl = A.tl0[t];                                     \
    const MixDesc& M = A.dd[tl.inst];                              \
    if (mx_live(M, gate)) { body; }                                \
    x.sync();                                                      \
  }
  for (int t = gid; t < A.nt0; t += ngroups) {
    const MTile tl = A.tl0[t];
    const MixDesc& M = A.dd[tl.inst];
    if (*M.active) ph_init(x, M, tl, ml, ts.r);
    x.sync();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) ml->inner_active = 0;
  if (!grid_sync(gb)) return;
  int pass = 0;
  for (; pass < ml->gmax_o; ++pass) {
    if (cget(&ml->outer_active) == 0) break;
    PERSIST_TILES(0, ph_prep(x, M, tl, ml, ts.r))
    if (!grid_sync(gb)) return;
    for (int t = gid; t < A.ntpre[0]; t += ngroups) {
      const MTile tl = A.tpre[0][t];
      const MixDesc& M = A.dd[tl.inst];
      if (mx_live(M, 1)) ph_down(x, M, tl, 0, A.sw, ts.d);
      x.sync();
    }
    if (!grid_sync(gb)) return;
    int it = 0;
    for (; it < ml->gmax_i; ++it) {
      if (cget(&ml->inner_active) == 0) break;
      if (!vcycle(1)) return;
      PERSIST_TILES(1, ph_matvec(x, M, tl, ts.m))
      if (!grid_sync(gb)) return;
      PERSIST_TILES(1, ph_update_down(x, M, tl, ml, 0ull, 0, A.sw, ts.u))
      if (!grid_sync(gb)) return;
    }
    if (it == ml->gmax_i && cget(&ml->inner_active) > 0 && blockIdx.x == 0 && threadIdx.x == 0) ml->tripped = 1;
    PERSIST_TILES(0, ph_correct(x, M, tl))
    if (!grid_sync(gb)) return;
    PERSIST_TILES(0, ph_resid(x, M, tl, ml, 0ull, 0, ts.r))
    if (blockIdx.x == 0 && threadIdx.x == 0) ml->inner_active = 0;
    if (!grid_sync(gb)) return;
  }
  if (pass == ml->gmax_o && cget(&ml->outer_active) > 0 && blockIdx.x == 0 && threadIdx.x == 0) ml->tripped = 1;
#undef PERSIST_TILES
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < A.n; k += gridDim.x * blockDim.x) mx_finish_one(A.dd[k]);
}

// Dependent binary32 FMAs for a few tens of microseconds (no memory waits):
// keeps the stream busy while the host queues the launches behind it.
__global__ void k_pad(float* sink, int n) {
  float x = (float)threadIdx.x;
  for (int i = 0; i < n; ++i) x = fmaf(x, 1.0000001f, 0.5f);
  if (x == -1.f) *sink = x;
}

// ---- host side --------------------------------------------------------------

static long round_up(long a, long m) { return (a + m - 1) / m * m; }

// One level of a multigrid plan: size, face coefficients (binary64 before
// rounding to the level's binary32) and the coarsening factors to the next level.
struct PlanLvl {
  int nx, ny;
  double cx, cy;
  int kx, ky;
};

struct Plan {
  std::vector<PlanLvl> global;   // global levels (kernels over tiles); the last is the CTA's first
  std::vector<PlanLvl> cta;      // levels of the coarse CTA (cta[0] == global.back())
  int cta_tot = 0;               // cells of all CTA levels, each with a one-cell ring
};

// Coarsening from a level: halve both axes when the coupling is balanced, or only
// the strongly coupled axis when one face coefficient exceeds twice the other
// (point smoothers leave errors that are smooth along the strong axis only).
static bool pick_coarsening(const PlanLvl& L, int minside, int& kx, int& ky) {
  const bool fx = L.nx % 2 == 0 && L.nx / 2 >= minside, fy = L.ny % 2 == 0 && L.ny / 2 >= minside;
  int px = 2, py = 2;
  if (L.cx > 2.0 * L.cy) py = 1;
  else if (L.cy > 2.0 * L.cx) px = 1;
  auto ok = [&](int a, int b) { return (a == 1 || fx) && (b == 1 || fy); };
  if (ok(px, py)) {
    kx = px;
    ky = py;
    return true;
  }
  if (fx && fy) { kx = 2; ky = 2; return true; }
  if (fx) { kx = 2; ky = 1; return true; }
  if (fy) { kx = 1; ky = 2; return true; }
  return false;
}

static PlanLvl coarsen(const PlanLvl& L, int kx, int ky) {
  PlanLvl c;
  c.nx = L.nx / kx;
  c.ny = L.ny / ky;
  c.cx = L.cx * ky / kx;
  c.cy = L.cy * kx / ky;
  c.kx = c.ky = 1;
  return c;
}

static Plan make_plan(int nx, int ny, double dx, double dy) {
  Plan P;
  PlanLvl L{nx, ny, (double)(float)(1.0 / (dx * dx)), (double)(float)(1.0 / (dy * dy)), 1, 1};
  P.global.push_back(L);
  while ((int)P.global.size() < MAX_LEVELS && (long)L.nx * L.ny > CMAX) {
    int kx, ky;
    if (!pick_coarsening(L, 8, kx, ky)) break;
    P.global.back().kx = kx;
    P.global.back().ky = ky;
    L = coarsen(L, kx, ky);
    P.global.push_back(L);
  }
  P.cta.push_back(L);
  while ((int)P.cta.size() < 8 && (long)L.nx * L.ny > BMAX) {
    int kx, ky;
    if (!pick_coarsening(L, 2, kx, ky)) break;
    P.cta.back().kx = kx;
    P.cta.back().ky = ky;
    L = coarsen(L, kx, ky);
    P.cta.push_back(L);
  }
  for (const PlanLvl& c : P.cta) P.cta_tot += (c.nx + 2) * (c.ny + 2);   // with their rings
  return P;
}

// Pseudo-inverse of the Neumann operator of an nx x ny level (face coefficients
// cx, cy), as binary32 row-major n x n.  A is symmetric positive semidefinite
// with the constants as its null space, so A+ = (A + J/n)^-1 - J/n with J the
// all-ones matrix; the inverse is Gauss-Jordan elimination in binary64.
static void neumann_pinv(int nx, int ny, double cx, double cy, std::vector<float>& out) {
  const int n = nx * ny;
  std::vector<double> a((size_t)n * 2 * n, 0.0);
  auto A = [&](int r, int c) -> double& { return a[(size_t)r * 2 * n + c]; };
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const int r = j * nx + i;
      double d = 0.0;
      if (i > 0) { d += cx; A(r, r - 1) -= cx; }
      if (i < nx - 1) { d += cx; A(r, r + 1) -= cx; }
      if (j > 0) { d += cy; A(r, r - nx) -= cy; }
      if (j < ny - 1) { d += cy; A(r, r + nx) -= cy; }
      A(r, r) += d;
    }
  for (int r = 0; r < n; ++r) {
    for (int c = 0; c < n; ++c) A(r, c) += 1.0 / n;
    A(r, n + r) = 1.0;
  }
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(A(r, c)) > std::fabs(A(piv, c))) piv = r;
    if (piv != c)
      for (int k = 0; k < 2 * n; ++k) std::swap(A(c, k), A(piv, k));
    const double inv = 1.0 / A(c, c);
    for (int k = 0; k < 2 * n; ++k) A(c, k) *= inv;
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = A(r, c);
      if (f != 0.0)
        for (int k = 0; k < 2 * n; ++k) A(r, k) -= f * A(c, k);
    }
  }
  out.assign((size_t)n * n, 0.f);
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) {
      // symmetrise the binary64 inverse before rounding, so the bottom operator is exactly symmetric
      const double v = 0.5 * (A(r, n + c) + A(c, n + r)) - 1.0 / n;
      out[(size_t)r * n + c] = (float)v;
    }
}

// The smoother: the error of a sweep x += w D^-1 (f - A x) is multiplied by
// (1 - w lambda) on each eigenvalue lambda of D^-1 A, which lies in [0, 2] for these
// operators.  Two sweeps with w = 1 / the roots of the degree-2 Chebyshev polynomial
// of [a, 2] bound that product by 1 / T2((2 + a) / (2 - a)) on [a, 2]: 0.22 on
// [0.5, 2], where the modes that full coarsening cannot represent lie, against 0.36
// for two damped-Jacobi sweeps with w = 0.8.  a = 0.4 (0.29 on [0.4, 2], more damping
// of the modes just below) took the fewest iterations over the 512^2, 2048^2 and
// batched cavities (a from 0.3 to 0.75 measured).  The factors commute, so the sweeps
// after the coarse correction (in reverse order) are the adjoint of those before and
// the V-cycle stays symmetric.  PFGB_MG_SMOOTHER=jacobi selects the damped-Jacobi
// pair, cheb:<a> the Chebyshev pair of [a, 2].
static Smooth make_smoother() {
  Smooth s = {0.8f, 0.8f, 0.8f};
  double a = 0.4;
  if (const char* ev = std::getenv("PFGB_MG_SMOOTHER")) {
    const std::string v(ev);
    if (v == "jacobi") return s;
    if (v.rfind("cheb:", 0) == 0) {
      const double x = std::atof(v.c_str() + 5);
      if (x > 0.0 && x < 2.0) a = x;
    }
  }
  const double b = 2.0, pi = 3.14159265358979323846;
  const double l1 = 0.5 * (b + a) + 0.5 * (b - a) * std::cos(pi / 4.0);
  const double l2 = 0.5 * (b + a) + 0.5 * (b - a) * std::cos(3.0 * pi / 4.0);
  s.w1 = (float)(1.0 / l1);
  s.w2 = (float)(1.0 / l2);
  return s;
}

// cuTensorMapEncodeTiled, fetched once through the runtime (the library does not
// link the driver API); null where the driver does not provide it
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
  static const EncodeTiledFn fn = []() -> EncodeTiledFn {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

// The halo box of the TMA matvec over a level-0 binary32 array of nx x ny cells with
// a pitch of ld floats: 40 x 34 floats, no swizzle, zero fill outside the array.
// The encoder checks the base (16-byte aligned), the pitch (a multiple of 16 bytes)
// and the box's row (160 bytes).
static bool encode_halo_map(CUtensorMap* m, const float* base, int nx, int ny, long ld) {
  const EncodeTiledFn fn = encode_tiled();
  if (!fn || (reinterpret_cast<uintptr_t>(base) & 15u) != 0 || (ld * sizeof(float)) % 16 != 0) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)nx, (cuuint64_t)ny};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)MV_W, (cuuint32_t)MV_H};
  const cuuint32_t es[2] = {1u, 1u};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static void add_mtiles(std::vector<MTile>& v, int k, int nx, int ny) {
  int loc = 0;
  for (int j0 = 0; j0 < ny; j0 += BY)
    for (int i0 = 0; i0 < nx; i0 += BX) v.push_back(MTile{k, i0, j0, loc++});
}

int batch_create(const MixParams* prm, int n, Batch** out) {
  Batch* B = new Batch();
  B->n = n;
  B->hd.resize(n);
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  size_t bytes = 0;
  std::vector<Plan> plan(n);
  size_t smem = 0, smem2 = 0;
  for (int k = 0; k < n; ++k) {
    plan[k] = make_plan(prm[k].nx, prm[k].ny, prm[k].dx, prm[k].dy);
    const PlanLvl& last = plan[k].global.back();
    if ((long)last.nx * last.ny > CMAX) {
      delete B;
      return set_error(PFGB_EINVAL, "mixed solver: the coarse multigrid level would exceed 4096 cells "
                                    "(nx and ny need enough factors of two)");
    }
    const PlanLvl& bot = plan[k].cta.back();
    const size_t cfl = (size_t)2 * plan[k].cta_tot +
                       std::max((size_t)plan[k].cta_tot, (size_t)(bot.nx * bot.ny <= BMAX ? NSL * BMAX : 0));
    smem = std::max(smem, cfl * sizeof(float));
    smem2 = smem;
    if (bot.nx * bot.ny <= BMAX) bytes += up((size_t)bot.nx * bot.ny * bot.nx * bot.ny * sizeof(float));
    B->maxlev = std::max(B->maxlev, (int)plan[k].global.size());
    for (auto& d : plan[k].global) bytes += 3 * up((size_t)round_up(d.nx, 32) * d.ny * sizeof(float));
    const size_t v0 = up((size_t)round_up(prm[k].nx, 32) * prm[k].ny * sizeof(float));
    const size_t nt0 = (size_t)((prm[k].nx + BX - 1) / BX) * ((prm[k].ny + BY - 1) / BY);
    bytes += 5 * v0 + up((size_t)prm[k].ld64 * prm[k].ny * sizeof(double)) + up(MAX_RED * nt0 * sizeof(double)) +
             up(sizeof(unsigned)) + up(sizeof(MixCtrl));
  }
  // tile tables
  std::vector<MTile> tl[MAX_LEVELS], tpre[MAX_LEVELS];
  for (int k = 0; k < n; ++k) {
    const auto& gl = plan[k].global;
    const int nl = (int)gl.size();
    for (int l = 0; l < nl; ++l) {
      add_mtiles(tl[l], k, gl[l].nx, gl[l].ny);
      if (l + 1 < nl) add_mtiles(tpre[l], k, gl[l].nx, gl[l].ny);
    }
  }
  for (int l = 0; l < B->maxlev; ++l)
    bytes += up(tl[l].size() * sizeof(MTile)) + up(tpre[l].size() * sizeof(MTile));
  bytes += up(n * sizeof(MixDesc)) + up(sizeof(MixLoop)) + up(sizeof(float)) + up(3 * n * sizeof(CUtensorMap)) +
           up(n * sizeof(int));
  if (cudaMalloc(&B->ws, bytes) != cudaSuccess) {
    delete B;
    return set_error(PFGB_ENOMEM, "cudaMalloc of the mixed-solver workspace failed");
  }
  cudaMemset(B->ws, 0, bytes);
  B->ws_bytes = bytes;
  char* c = B->ws;
  auto take = [&](size_t b) { char* r = c; c += up(b); return r; };
  int gmax_i = 1, gmax_o = 1;
  // PFGB_TILE_INTERIOR=0 sends every tile through the general phase forms (the
  // interior forms give the same bits; the switch lets that be checked)
  const char* tiv = std::getenv("PFGB_TILE_INTERIOR");
  const int interior = (tiv && std::string(tiv) == "0") ? 0 : 1;
  for (int k = 0; k < n; ++k) {
    MixDesc& M = B->hd[k];
    M.G.nx = prm[k].nx;
    M.G.ny = prm[k].ny;
    M.G.ld = prm[k].ld64;
    M.G.g.nx = prm[k].nx;
    M.G.g.ny = prm[k].ny;
    M.G.g.sx = spacing_for(prm[k].dx);
    M.G.g.sy = spacing_for(prm[k].dy);
    M.G.rdx = 1.0 / prm[k].dx;
    M.G.rdy = 1.0 / prm[k].dy;
    M.G.rdx2 = 1.0 / (prm[k].dx * prm[k].dx);
    M.G.rdy2 = 1.0 / (prm[k].dy * prm[k].dy);
    const Plan& PL = plan[k];
    M.nlev = (int)PL.global.size();
    M.coarse_levels = (int)PL.cta.size();
    for (int l = 0; l < M.coarse_levels; ++l) {
      M.ccx[l] = (float)PL.cta[l].cx;
      M.ccy[l] = (float)PL.cta[l].cy;
      M.ckx[l] = PL.cta[l].kx;
      M.cky[l] = PL.cta[l].ky;
    }
    for (int l = 0; l < M.nlev; ++l) {
      Lvl& v = M.lev[l];
      v.nx = PL.global[l].nx;
      v.ny = PL.global[l].ny;
      v.ld = round_up(v.nx, 32);
      v.cx = (float)PL.global[l].cx;
      v.cy = (float)PL.global[l].cy;
      v.kx = PL.global[l].kx;
      v.ky = PL.global[l].ky;
      const size_t nb = (size_t)v.ld * v.ny * sizeof(float);
      v.u = (float*)take(nb);
      v.t = (float*)take(nb);
      v.f = (float*)take(nb);
    }
    const size_t v0 = (size_t)M.lev[0].ld * prm[k].ny * sizeof(float);
    M.e = (float*)take(v0);
    M.f0b = (float*)take(v0);
    M.p0 = (float*)take(v0);
    M.p1 = (float*)take(v0);
    M.q = (float*)take(v0);
    M.r64 = (double*)take((size_t)prm[k].ld64 * prm[k].ny * sizeof(double));
    M.nt0 = ((prm[k].nx + BX - 1) / BX) * ((prm[k].ny + BY - 1) / BY);
    M.interior = interior;
    M.part = (double*)take(MAX_RED * (size_t)M.nt0 * sizeof(double));
    M.ticket = (unsigned*)take(sizeof(unsigned));
    M.ctrl = (MixCtrl*)take(sizeof(MixCtrl));
    M.binv = nullptr;
    const PlanLvl& bot = PL.cta.back();
    if (bot.nx * bot.ny <= BMAX) {
      std::vector<float> pinv;
      neumann_pinv(bot.nx, bot.ny, (double)(float)bot.cx, (double)(float)bot.cy, pinv);
      float* dst = (float*)take(pinv.size() * sizeof(float));
      cudaMemcpy(dst, pinv.data(), pinv.size() * sizeof(float), cudaMemcpyHostToDevice);
      M.binv = dst;
    }
    M.b = prm[k].b;
    M.bsum = prm[k].bsum;
    M.n_cells = (double)prm[k].nx * (double)prm[k].ny;
    M.res_out = prm[k].res_out;
    M.x = prm[k].x;
    M.pprev = prm[k].pprev;
    M.ldp = prm[k].ldp;
    M.ctrl64 = prm[k].ctrl64;
    M.active = prm[k].active;
    M.maxiter_report = prm[k].maxiter_report;
    MixCtrl hc = {};
    hc.tol_out = prm[k].tol_out;
    hc.tol_in = prm[k].tol_in;
    hc.max_outer = prm[k].max_outer;
    hc.max_inner = prm[k].max_inner;
    hc.warm = prm[k].warm ? 1 : 0;
    hc.reach = 1;
    hc.reach_wait = 0;
    hc.inner_done = 1;
    hc.outer_done = 1;
    cudaMemcpy(M.ctrl, &hc, sizeof(MixCtrl), cudaMemcpyHostToDevice);
    gmax_i = std::max(gmax_i, prm[k].max_inner + 1);
    gmax_o = std::max(gmax_o, prm[k].max_outer + 1);
  }
  for (int l = 0; l < B->maxlev; ++l) {
    auto put = [&](std::vector<MTile>& v, MTile*& dst, int& cnt) {
      cnt = (int)v.size();
      dst = (MTile*)take(v.size() * sizeof(MTile));
      if (cnt) cudaMemcpy(dst, v.data(), v.size() * sizeof(MTile), cudaMemcpyHostToDevice);
    };
    put(tl[l], B->tl[l], B->ntl[l]);
    put(tpre[l], B->tpre[l], B->ntpre[l]);
  }
  B->dd = (MixDesc*)take(n * sizeof(MixDesc));
  B->loop = (MixLoop*)take(sizeof(MixLoop));
  B->pad = (float*)take(sizeof(float));
  {
    // Launch order of the coarse CTAs.  CTAs are handed to SMs roughly in launch order,
    // one to each SM before any SM gets a second, and a coarse CTA sharing its SM with a
    // second one runs slower (both compete for the SM's issue slots); the launch is as
    // long as its slowest SM.  So the CTAs with the most coarse work (cells of the CTA's
    // levels) go first, one to an SM, and the rest follow in increasing order of work, so
    // that the largest instances share their SMs with the smallest.  Every CTA computes
    // the same values wherever it runs.
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    std::vector<int> ord(n);
    for (int k = 0; k < n; ++k) ord[k] = k;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return plan[a].cta_tot > plan[b].cta_tot; });
    if (n > sms) std::reverse(ord.begin() + sms, ord.end());
    B->corder = (int*)take(n * sizeof(int));
    cudaMemcpy(B->corder, ord.data(), n * sizeof(int), cudaMemcpyHostToDevice);
  }
  {
    // tensor maps of the TMA matvec: z, p0, p1 of every instance.  That form pays when
    // a CTA takes several tiles of one instance in turn (each instance's lookups once, the
    // next tile's copies in flight during the current one): measured on GB300, 2048^2
    // 34.8 against 48.5 us a launch; with one tile per CTA (512^2: 14.3 against 12.3 us)
    // or many small instances (the 256-instance batch: 1.668 against 1.585 ms a step) the
    // one-tile-per-CTA matvec is faster.  So by default the TMA form is taken for batches
    // of at least 64 level-0 tiles per instance and at least 2 tiles per CTA (the second
    // test below, once the grid is known); PFGB_MATVEC_TMA=1 or 0 forces it on or off.
    // Both forms give the same bits.
    CUtensorMap* tm = (CUtensorMap*)take(3 * n * sizeof(CUtensorMap));
    const char* tv = std::getenv("PFGB_MATVEC_TMA");
    B->mv_force = (tv && std::string(tv) == "1") ? 1 : ((tv && std::string(tv) == "0") ? -1 : 0);
    // the maps are encoded for any batch (unless the form is forced off), so that the
    // tuner can try the form; the rule above picks it by default
    bool ok = B->mv_force >= 0 && n > 0;
    const bool by_rule = B->mv_force > 0 || (long)B->ntl[0] >= 64L * n;
    std::vector<CUtensorMap> hm(ok ? 3 * n : 0);
    for (int k = 0; ok && k < n; ++k) {
      const MixDesc& M = B->hd[k];
      const float* src[3] = {M.lev[0].u, M.p0, M.p1};
      for (int a = 0; ok && a < 3; ++a) ok = encode_halo_map(&hm[3 * k + a], src[a], M.lev[0].nx, M.lev[0].ny, M.lev[0].ld);
    }
    if (!ok && std::getenv("PFGB_GRAPH_DEBUG"))
      std::fprintf(stderr, "pfgb mixed batch: TMA matvec maps %s\n",
                   B->mv_force < 0 ? "not wanted"
                   : hm.empty()    ? "not used (fewer than 64 level-0 tiles per instance)"
                   : encode_tiled() ? "refused by the encoder"
                                    : "without an encoder");
    if (ok && cudaMemcpy(tm, hm.data(), hm.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice) != cudaSuccess) ok = false;
    for (int k = 0; k < n; ++k) B->hd[k].tmap = ok ? tm + 3 * k : nullptr;
    B->mv_avail = ok ? 1 : 0;
    B->mv_tma = (ok && by_rule) ? 1 : 0;
    cudaGetLastError();
  }
  // PFGB_TEST_LOOP_BOUND lowers both loops' trip bounds (a test of the guards: the
  // instances then need more trips than the guards allow)
  if (const char* tb = std::getenv("PFGB_TEST_LOOP_BOUND")) {
    const int b = std::atoi(tb);
    if (b > 0) {
      gmax_o = std::min(gmax_o, b);
      gmax_i = std::min(gmax_i, b);
    }
  }
  B->gmax_o = gmax_o;
  B->gmax_i = gmax_i;
  B->sw = make_smoother();
  MixLoop ml0 = {0, 0, 0, 0, gmax_o, gmax_i, 0, 0u, 0u, {0u, 0u, 0, 0}};
  cudaMemcpy(B->loop, &ml0, sizeof(MixLoop), cudaMemcpyHostToDevice);
  cudaError_t e = cudaMemcpy(B->dd, B->hd.data(), n * sizeof(MixDesc), cudaMemcpyHostToDevice);
  B->coarse_smem = smem;
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mg_coarse<CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mg_coarse<CT2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2);
  if (e == cudaSuccess) {
    // two CTAs to an SM need most of its shared memory: ask for the largest carveout
    if (cudaFuncSetAttribute(k_mg_coarse<CT2>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
      cudaGetLastError();
  }
  if (e == cudaSuccess) {
    // more coarse CTAs than one wave of 1024-thread CTAs holds: 512-thread CTAs, two to an SM
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_mg_coarse<CT2>, CT2, smem2) == cudaSuccess && occ >= 2)
      B->coarse_avail2 = 1;
    if (n > sms && B->coarse_avail2) {
      B->coarse_nt = CT2;
      B->coarse_smem = smem2;
    }
    if (std::getenv("PFGB_GRAPH_DEBUG"))
      std::fprintf(stderr, "pfgb mixed batch: %d instances, coarse CTA %d threads (%zu B shared, %d per SM at 512)\n", n,
                   B->coarse_nt, B->coarse_smem, occ);
    cudaGetLastError();
  }
  if (e == cudaSuccess && B->mv_avail) {
    // the TMA matvec: as many CTAs as fit on the device at once, at most one per tile
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_mx_matvec_tma, MT, 0) == cudaSuccess && occ >= 1)
      B->mv_grid = std::min(B->ntl[0], sms * occ);
    else
      B->mv_avail = B->mv_tma = 0;
    if (B->mv_tma && B->mv_force == 0 && B->ntl[0] < 2 * B->mv_grid) B->mv_tma = 0;   // under 2 tiles per CTA
    cudaGetLastError();
  }
  if (std::getenv("PFGB_GRAPH_DEBUG"))
    std::fprintf(stderr, "pfgb mixed batch: TMA matvec %s, %d CTAs\n", B->mv_tma ? "on" : "off", B->mv_grid);
  if (e == cudaSuccess) {
    // the persistent solve: one 1024-thread CTA per SM, if the device co-schedules them
    const size_t psmem = std::max(4 * sizeof(TileSmem), smem);
    int dev = 0, sms = 0, coop = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (coop && cudaFuncSetAttribute(k_mx_persist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_mx_persist, CT, psmem) == cudaSuccess && occ >= 1) {
      B->persist_ok = 1;
      B->persist = 0;      // opt-in (pfgb_set_persistent): the kernel graph is faster on GB300
      B->pgrid = sms;
      B->psmem = psmem;
    }
    cudaGetLastError();   // a refused attribute or query only disables the persistent form
  }
  if (e != cudaSuccess) {
    batch_destroy(B);
    return set_error(PFGB_ECUDA, std::string("mixed batch set-up: ") + cudaGetErrorString(e));
  }
  *out = B;
  return PFGB_OK;
}

int set_tolerances(Batch* B, int k, double tol_out, double tol_in, int max_outer, int max_inner, int warm,
                   int maxiter_report) {
  if (k < 0 || k >= B->n) return set_error(PFGB_EINVAL, "instance index out of range");
  if (max_outer < 1 || max_outer + 1 > B->gmax_o || max_inner < 1 || max_inner + 1 > B->gmax_i)
    return set_error(PFGB_EINVAL, "mixed iteration limits above the batch's largest");
  MixCtrl head = {};
  head.tol_out = tol_out;
  head.tol_in = tol_in;
  head.max_outer = max_outer;
  head.max_inner = max_inner;
  head.warm = warm ? 1 : 0;
  head.reach = 1;
  head.reach_wait = 0;
  // the leading fields up to bnorm; the rest of the control block is rewritten by every solve
  cudaError_t e = cudaMemcpy(B->hd[k].ctrl, &head, offsetof(MixCtrl, bnorm), cudaMemcpyHostToDevice);
  B->hd[k].maxiter_report = maxiter_report;
  if (e == cudaSuccess)
    e = cudaMemcpy(reinterpret_cast<char*>(B->dd + k) + offsetof(MixDesc, maxiter_report), &maxiter_report,
                   sizeof(int), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("mixed tolerances: ") + cudaGetErrorString(e));
  return PFGB_OK;
}

void batch_destroy(Batch* B) {
  if (!B) return;
  if (B->ws) cudaFree(B->ws);
  delete B;
}

// the V-cycle from down-sweep level l0 on (l0 = 1: level 0's down-sweep is fused into the update)
static void add_vcycle(GraphChain& c, Batch* B, int gate, Smooth sw, int l0 = 0) {
  const MixDesc* dd = B->dd;
  for (int l = l0; l + 1 < B->maxlev; ++l) {
    if (B->ntpre[l]) c.kernel(k_mg_down, dim3(B->ntpre[l]), dim3(MT), dd, (const MTile*)B->tpre[l], l, gate, sw);
  }
  if (B->coarse_nt == CT2)
    c.kernel_smem(k_mg_coarse<CT2>, dim3(B->n), dim3(CT2), B->coarse_smem, dd, (const int*)B->corder, gate, 8, sw);
  else
    c.kernel_smem(k_mg_coarse<CT>, dim3(B->n), dim3(CT), B->coarse_smem, dd, (const int*)B->corder, gate, 8, sw);
  for (int l = B->maxlev - 2; l >= 0; --l)
    if (B->ntpre[l]) c.kernel(k_mg_post, dim3(B->ntpre[l]), dim3(MT), dd, (const MTile*)B->tpre[l], l, gate, sw);
}

static PersistArgs persist_args(const Batch* B, Smooth sw) {
  PersistArgs a = {};
  a.dd = B->dd;
  a.n = B->n;
  a.maxlev = B->maxlev;
  a.tl0 = B->tl[0];
  a.nt0 = B->ntl[0];
  for (int l = 0; l < MAX_LEVELS; ++l) {
    a.tpre[l] = B->tpre[l];
    a.ntpre[l] = B->ntpre[l];
  }
  a.ml = B->loop;
  a.sw = sw;
  a.bottom_sweeps = 8;
  return a;
}

int set_persistent(Batch* B, int on) {
  B->persist = (on && B->persist_ok) ? 1 : 0;
  return PFGB_OK;
}

int append_solve(GraphChain& c, Batch* B) {
  const Smooth sw = B->sw;
  if (B->persist) {
    c.kernel(k_ml_reset, dim3(1), dim3(32), B->loop, 0);
    c.kernel_coop(k_mx_persist, dim3(B->pgrid), dim3(CT), B->psmem, persist_args(B, sw));
    if (c.status() != cudaSuccess)
      return set_error(PFGB_ECUDA, std::string("building the persistent solve: ") + cudaGetErrorString(c.status()));
    return PFGB_OK;
  }
  const MixDesc* dd = B->dd;
  const dim3 g0(B->ntl[0]);
  cudaGraphConditionalHandle cond_outer = 0, cond_inner = 0;
  cudaError_t e = cudaGraphConditionalHandleCreate(&cond_outer, c.graph(), 0u, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("outer conditional: ") + cudaGetErrorString(e));
  c.kernel(k_ml_reset, dim3(1), dim3(32), B->loop, 0);
  c.kernel(k_mx_init, g0, dim3(MT), dd, (const MTile*)B->tl[0], B->loop);
  c.kernel(k_ml_arm, dim3(1), dim3(32), B->loop, 0, cond_outer, 1);
  GraphChain outer = c.while_loop_with(cond_outer);
  if (outer.status() != cudaSuccess) return set_error(PFGB_ECUDA, "outer loop node");
  e = cudaGraphConditionalHandleCreate(&cond_inner, outer.graph(), 0u, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("inner conditional: ") + cudaGetErrorString(e));
  outer.kernel(k_ml_reset, dim3(1), dim3(32), B->loop, 1);
  outer.kernel(k_mx_prep, g0, dim3(MT), dd, (const MTile*)B->tl[0], B->loop);
  if (B->ntpre[0]) outer.kernel(k_mg_down, dim3(B->ntpre[0]), dim3(MT), dd, (const MTile*)B->tpre[0], 0, 1, sw);
  outer.kernel(k_ml_arm, dim3(1), dim3(32), B->loop, 1, cond_inner, 1);
  // one PCG iteration per trip, ending with its stopping test: the V-cycle on r_k (its
  // level-0 down-sweep done by the phase before), p and q = A p, then x, r and the fused
  // level-0 down-sweep of r_{k+1}; no V-cycle runs after the last test
  GraphChain inner = outer.while_loop_with(cond_inner);
  add_vcycle(inner, B, 1, sw, 1);
  if (B->mv_tma)
    inner.kernel(k_mx_matvec_tma, dim3(B->mv_grid), dim3(MT), dd, (const MTile*)B->tl[0], B->ntl[0], B->loop);
  else
    inner.kernel(k_mx_matvec, g0, dim3(MT), dd, (const MTile*)B->tl[0]);
  inner.kernel(k_mx_update_down, g0, dim3(MT), dd, (const MTile*)B->tl[0], B->loop, cond_inner, 1, sw);
  outer.kernel(k_mx_correct, g0, dim3(MT), dd, (const MTile*)B->tl[0]);
  outer.kernel(k_mx_resid, g0, dim3(MT), dd, (const MTile*)B->tl[0], B->loop, cond_outer, 1);
  if (std::getenv("PFGB_GRAPH_DEBUG"))
    std::fprintf(stderr, "pfgb mixed graph: programmatic edges outer %d inner %d; last refusal: %s\n", outer.n_prog_,
                 inner.n_prog_, cudaGetErrorString(inner.last_prog_err_));
  cudaError_t st = c.status() != cudaSuccess ? c.status() : (outer.status() != cudaSuccess ? outer.status() : inner.status());
  if (st != cudaSuccess) return set_error(PFGB_ECUDA, std::string("building the mixed solve: ") + cudaGetErrorString(st));
  return PFGB_OK;
}

// Host-driven form of append_solve with direct launches: the loop decisions
// are read back from the loop control after each stopping test.  Used for
// profiling (ncu does not profile kernels of graphs with conditional nodes, and
// with B->kp set every launch is timed with events).
static void launch_vcycle(Batch* B, int gate, Smooth sw, cudaStream_t s, int l0 = 0) {
  KProf* kp = B->kp;
  for (int l = l0; l + 1 < B->maxlev; ++l) {
    if (B->ntpre[l]) PFGB_TIMED(kp, "k_mg_down", l, s, k_mg_down<<<B->ntpre[l], MT, 0, s>>>(B->dd, B->tpre[l], l, gate, sw));
  }
  // (each instance's coarse CTA starts from that instance's last global level)
  if (B->coarse_nt == CT2)
    PFGB_TIMED(kp, "k_mg_coarse", -1, s, k_mg_coarse<CT2><<<B->n, CT2, B->coarse_smem, s>>>(B->dd, B->corder, gate, 8, sw));
  else
    PFGB_TIMED(kp, "k_mg_coarse", -1, s, k_mg_coarse<CT><<<B->n, CT, B->coarse_smem, s>>>(B->dd, B->corder, gate, 8, sw));
  for (int l = B->maxlev - 2; l >= 0; --l)
    if (B->ntpre[l]) PFGB_TIMED(kp, "k_mg_post", l, s, k_mg_post<<<B->ntpre[l], MT, 0, s>>>(B->dd, B->tpre[l], l, gate, sw));
}

// A few tens of microseconds of device work ahead of the next launches (profiling only).
static void pad_stream(Batch* B, cudaStream_t s) {
  if (B->kp) k_pad<<<1, 32, 0, s>>>(B->pad, 20000);
}

int run_direct(Batch* B, cudaStream_t s) {
  const Smooth sw = B->sw;
  KProf* kp = B->kp;
  if (B->persist) {
    k_ml_reset<<<1, 32, 0, s>>>(B->loop, 0);
    PersistArgs a = persist_args(B, sw);
    void* args[] = {&a};
    cudaError_t e = cudaSuccess;
    pad_stream(B, s);
    PFGB_TIMED(kp, "k_mx_persist", -1, s,
               e = cudaLaunchCooperativeKernel((const void*)k_mx_persist, dim3(B->pgrid), dim3(CT), args, B->psmem, s));
    if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("persistent solve launch: ") + cudaGetErrorString(e));
    return PFGB_OK;
  }
  const int g0 = B->ntl[0];
  MixLoop h;
  auto read = [&]() -> bool {
    const bool ok = cudaMemcpyAsync(&h, B->loop, sizeof(MixLoop), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
                    cudaStreamSynchronize(s) == cudaSuccess;
    pad_stream(B, s);
    return ok;
  };
  k_ml_reset<<<1, 32, 0, s>>>(B->loop, 0);
  PFGB_TIMED(kp, "k_mx_init", -1, s, k_mx_init<<<g0, MT, 0, s>>>(B->dd, B->tl[0], B->loop));
  if (!read()) return set_error(PFGB_ECUDA, "mixed solve: control read failed");
  for (int po = 0; h.outer_active > 0 && po < h.gmax_o; ++po) {
    k_ml_reset<<<1, 32, 0, s>>>(B->loop, 1);
    PFGB_TIMED(kp, "k_mx_prep", -1, s, k_mx_prep<<<g0, MT, 0, s>>>(B->dd, B->tl[0], B->loop));
    if (B->ntpre[0]) PFGB_TIMED(kp, "k_mg_down", 0, s, k_mg_down<<<B->ntpre[0], MT, 0, s>>>(B->dd, B->tpre[0], 0, 1, sw));
    if (!read()) return set_error(PFGB_ECUDA, "mixed solve: control read failed");
    for (int pi = 0; h.inner_active > 0 && pi < h.gmax_i; ++pi) {
      launch_vcycle(B, 1, sw, s, 1);
      if (B->mv_tma)
        PFGB_TIMED(kp, "k_mx_matvec_tma", -1, s,
                   k_mx_matvec_tma<<<B->mv_grid, MT, 0, s>>>(B->dd, B->tl[0], B->ntl[0], B->loop));
      else
        PFGB_TIMED(kp, "k_mx_matvec", -1, s, k_mx_matvec<<<g0, MT, 0, s>>>(B->dd, B->tl[0]));
      PFGB_TIMED(kp, "k_mx_update_down", -1, s, k_mx_update_down<<<g0, MT, 0, s>>>(B->dd, B->tl[0], B->loop, 0ull, 0, sw));
      if (!read()) return set_error(PFGB_ECUDA, "mixed solve: control read failed");
    }
    PFGB_TIMED(kp, "k_mx_correct", -1, s, k_mx_correct<<<g0, MT, 0, s>>>(B->dd, B->tl[0]));
    PFGB_TIMED(kp, "k_mx_resid", -1, s, k_mx_resid<<<g0, MT, 0, s>>>(B->dd, B->tl[0], B->loop, 0ull, 0));
    if (!read()) return set_error(PFGB_ECUDA, "mixed solve: control read failed");
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("mixed solve launch: ") + cudaGetErrorString(e));
  return PFGB_OK;
}

// ---- launch-shape tuner --------------------------------------------------------

int variant_of(const Batch* B) { return 2 * (B->mv_tma ? 1 : 0) + (B->coarse_nt == CT2 ? 1 : 0); }

int set_variant(Batch* B, int variant) {
  if (variant < 0 || variant > 3) return set_error(PFGB_EINVAL, "mixed launch variant must be 0..3");
  const int tma = variant >> 1, narrow = variant & 1;
  if (tma && !B->mv_avail) return set_error(PFGB_EINVAL, "this batch cannot run the TMA matvec");
  if (narrow && !B->coarse_avail2) return set_error(PFGB_EINVAL, "two 512-thread coarse CTAs do not fit on an SM");
  B->mv_tma = tma;
  B->coarse_nt = narrow ? CT2 : CT;
  return PFGB_OK;
}

// A fixed pseudo-random pattern in [-1, 1) in both level-0 residual buffers and a zero
// correction: a PCG run from it keeps every quantity finite for the timed iterations.
__global__ void k_tune_fill_m(const MixDesc* __restrict__ MD, const MTile* __restrict__ TL) {
  const MTile tl = TL[blockIdx.x];
  const MixDesc& M = MD[tl.inst];
  const Lvl L0 = M.lev[0];
  for (int c = threadIdx.x; c < BX * BY; c += blockDim.x) {
    const int i = tl.i0 + c % BX, j = tl.j0 + c / BX;
    if (i >= L0.nx || j >= L0.ny) continue;
    unsigned h = (unsigned)(j * 73856093) ^ (unsigned)(i * 19349663) ^ (unsigned)(tl.inst * 83492791);
    h ^= h >> 13;
    h *= 0x5bd1e995u;
    h ^= h >> 15;
    const float v = (float)(h & 0xffffu) * (1.f / 32768.f) - 1.f;
    const long o = (long)j * L0.ld + i;
    L0.f[o] = v;
    M.f0b[o] = v;
    M.e[o] = 0.f;
  }
}

// Every instance in the inner loop, with a stopping test that never passes.
__global__ void k_tune_arm_m(const MixDesc* __restrict__ MD, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n || !*MD[k].active) return;
  MixCtrl* c = MD[k].ctrl;
  c->outer_done = 0;
  c->inner_done = 0;
  c->inner = 0;
  c->inner_total = 0;
  c->max_inner = 1 << 30;
  c->tol_abs_in = -1.0;
  c->rho = 1.0;
  c->beta = 0.0;
}

int tune(Batch* B, cudaStream_t s, int* chosen, double* us) {
  if (B->persist) {                     // one cooperative launch: no launch shapes to choose
    if (chosen) *chosen = variant_of(B);
    return PFGB_OK;
  }
  const int orig = variant_of(B);
  std::vector<MixCtrl> ctrl(B->n);
  MixLoop loop;
  cudaError_t err = cudaStreamSynchronize(s);
  for (int k = 0; k < B->n && err == cudaSuccess; ++k)
    err = cudaMemcpy(&ctrl[k], B->hd[k].ctrl, sizeof(MixCtrl), cudaMemcpyDeviceToHost);
  if (err == cudaSuccess) err = cudaMemcpy(&loop, B->loop, sizeof(MixLoop), cudaMemcpyDeviceToHost);
  if (err != cudaSuccess) return set_error(PFGB_ECUDA, std::string("tune: saving the solver state: ") + cudaGetErrorString(err));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  KProf* kp = B->kp;
  B->kp = nullptr;
  const Smooth sw = B->sw;
  float best = 1e30f;
  int best_v = orig;
  const int g0 = B->ntl[0];
  for (int v = 0; v < 4 && err == cudaSuccess; ++v) {
    if (us) us[v] = -1.0;
    if (set_variant(B, v) != PFGB_OK) continue;
    k_tune_fill_m<<<g0, MT, 0, s>>>(B->dd, B->tl[0]);
    k_tune_arm_m<<<(B->n + 127) / 128, 128, 0, s>>>(B->dd, B->n);
    k_ml_reset<<<1, 32, 0, s>>>(B->loop, 0);
    k_ml_reset<<<1, 32, 0, s>>>(B->loop, 1);
    if (B->ntpre[0]) k_mg_down<<<B->ntpre[0], MT, 0, s>>>(B->dd, B->tpre[0], 0, 1, sw);
    constexpr int WARM = 2, REPS = 10;
    for (int it = 0; it < WARM + REPS; ++it) {
      if (it == WARM) cudaEventRecord(e0, s);
      launch_vcycle(B, 1, sw, s, 1);
      if (B->mv_tma)
        k_mx_matvec_tma<<<B->mv_grid, MT, 0, s>>>(B->dd, B->tl[0], B->ntl[0], B->loop);
      else
        k_mx_matvec<<<g0, MT, 0, s>>>(B->dd, B->tl[0]);
      k_mx_update_down<<<g0, MT, 0, s>>>(B->dd, B->tl[0], B->loop, 0ull, 0, sw);
    }
    cudaEventRecord(e1, s);
    err = cudaEventSynchronize(e1);
    if (err != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const float per = 1e3f * ms / REPS;
    if (us) us[v] = per;
    if (per < best) {
      best = per;
      best_v = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  B->kp = kp;
  if (err == cudaSuccess) err = cudaGetLastError();
  // the instances' solver state (the refinement's per-instance history among it) as it was
  for (int k = 0; k < B->n && err == cudaSuccess; ++k)
    err = cudaMemcpy(B->hd[k].ctrl, &ctrl[k], sizeof(MixCtrl), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(B->loop, &loop, sizeof(MixLoop), cudaMemcpyHostToDevice);
  if (err != cudaSuccess) {
    set_variant(B, orig);
    return set_error(PFGB_ECUDA, std::string("tune: ") + cudaGetErrorString(err));
  }
  set_variant(B, best_v);
  if (chosen) *chosen = best_v;
  return PFGB_OK;
}

}  // namespace mixed
}  // namespace pfgb
