// Mixed-precision pressure solve (FP64 refinement around FP32 multigrid-PCG):
// device structures and the host interface used by the step graph.
#pragma once
#include <cuda.h>           // CUtensorMap (the encoder is fetched through the runtime; no libcuda link)
#include <cuda_runtime.h>

#include <vector>

#include "graph.cuh"
#include "kprof.cuh"
#include "persist.cuh"
#include "stencil.cuh"
#include "step64.cuh"

namespace pfgb {
namespace mixed {

constexpr int MAX_LEVELS = 16;
constexpr int MAX_RED = 4;     // most sums one tile reduction carries

// One multigrid level: binary32 arrays of (ny, ld); cx, cy are the face
// coefficients.  The coarse operators are rediscretised consistently with
// R = P^T, which sums kx * ky children: cx' = cx ky / kx, cy' = cy kx / ky
// (halving both axes keeps the coefficients).
struct Lvl {
  int nx, ny;
  long ld;
  float cx, cy;
  int kx, ky;   // coarsening factors (1 or 2) to the next level
  float* u;   // V-cycle result
  float* t;   // pre-smoothed iterate
  float* f;   // right-hand side (on level 0: the PCG residual)
};

// Relaxation weights of the multigrid smoother: the two sweeps before and after
// each coarse correction are x += w D^-1 (f - A x) with w1 and w2 (the two roots of
// the degree-2 Chebyshev polynomial on the upper part of the spectrum of D^-1 A);
// wb is the weight of the damped-Jacobi sweeps of a bottom level without a
// pseudo-inverse.
struct Smooth {
  float w1, w2, wb;
};

// binary64 geometry of the refinement
struct Geo {
  int nx, ny;
  long ld;
  Grid2 g;
  double rdx, rdy;             // 1/dx, 1/dy
  double rdx2, rdy2;           // 1/dx^2, 1/dy^2
};

struct MixCtrl {
  double tol_out, tol_in;
  int max_outer, max_inner;
  int warm;                    // start from the previous pressure (else from zero)
  int reach;                   // the first pass aims at the outer target (see ph_prep)
  int reach_wait;              // steps until that is tried again after a miss
  double bnorm, tol_abs_out, rr64, sum64;
  double rt_norm, tol_abs_in;
  double rho, beta, pq, alpha, rr_in;
  int outer, inner, inner_total, converged;
  int inner_done, outer_done;
  int cold;                    // this solve's first pass starts from zero (the warm guess was worse)
  int reach_tried;             // this solve's first pass aimed at the outer target
};

// One tile of work of a mixed batch: instance and the tile's first cell.
struct MTile {
  int inst, i0, j0, loc;       // loc: index of the tile among its instance's tiles of the level
};

// Everything the mixed-precision kernels need about one instance.
struct MixDesc {
  Geo G;                       // binary64 geometry of the refinement
  int nlev;                    // global levels; the last one is solved by the coarse CTA
  int coarse_levels;           // levels resolved inside the coarse CTA
  const float* binv;           // pseudo-inverse of the bottom level (null: Jacobi sweeps instead)
  float ccx[8], ccy[8];        // face coefficients of the coarse CTA's levels
  int ckx[8], cky[8];          // their coarsening factors to the next level
  Lvl lev[MAX_LEVELS];
  float *e, *p0, *p1, *q;      // binary32 PCG vectors (pitch lev[0].ld)
  float* f0b;                  // the second level-0 residual buffer: iteration k reads r from
                               // buffer k & 1 (lev[0].f is buffer 0) and writes buffer (k + 1) & 1
  double* r64;                 // binary64 refinement residual (pitch G.ld)
  double* b;                   // the step's right-hand side (binary64, pitch G.ld); mean removed here
  const double* bsum;          // exactly rounded sum of the right-hand side (from the RHS kernel)
  double n_cells;
  double* res_out;             // where the final ||b - A x||^2 goes (the step's residual record)
  double* x;                   // the step's pressure solution
  const double* const* pprev;  // where the step's pressure field pointer lives (interior, pitch ldp)
  long ldp;
  double* part;                // per-tile partial sums of the reductions (MAX_RED x nt0)
  unsigned* ticket;            // arrival counter of the reductions
  MixCtrl* ctrl;
  Ctrl64* ctrl64;              // the step's control block (iteration summary)
  const int* active;           // the step's per-instance activity flag
  int maxiter_report;
  int nt0;                     // tiles of level 0 (= tiles of the binary64 grid)
  int interior;                // tiles away from the walls take the interior forms of the phases
  const CUtensorMap* tmap;     // level-0 halo copies of z (= lev[0].u), p0, p1 (null: no TMA form)
};

// Batch-wide control of the two WHILE loops.
struct MixLoop {
  int outer_active, inner_active;
  int guard_o, guard_i;
  int gmax_o, gmax_i;
  int tripped;
  unsigned ticket_o, ticket_i;   // CTAs done in the current launch of a loop's last kernel
  GridBar gb;     // barrier of the persistent solve; its err also records a TMA matvec copy that never landed
};

struct Batch {
  int n = 0;
  std::vector<MixDesc> hd;
  MixDesc* dd = nullptr;
  int maxlev = 0;                              // most global levels of any instance
  MTile* tl[MAX_LEVELS] = {};                  // tiles of level l of the instances that have it
  int ntl[MAX_LEVELS] = {};
  MTile* tpre[MAX_LEVELS] = {};                // tiles of level l of the instances that smooth on it (l < nlev-1)
  int ntpre[MAX_LEVELS] = {};
  size_t coarse_smem = 0;                      // dynamic shared memory of the coarse CTA (largest instance)
  int coarse_nt = 1024;                        // threads of the coarse CTA (512: two to an SM)
  MixLoop* loop = nullptr;
  int gmax_o = 1, gmax_i = 1;                  // trip bounds of the loop guards
  Smooth sw = {0.8f, 0.8f, 0.8f};              // smoother weights
  // profiling (direct launches): per-kernel events, owned by the step's instance
  KProf* kp = nullptr;
  float* pad = nullptr;                        // sink of the profiling pad kernel
  int* corder = nullptr;                       // instance of each coarse CTA, in launch order
  // the persistent form of the solve (one cooperative launch)
  int persist_ok = 0;                          // the device co-schedules its CTAs
  int persist = 0;                             // in use
  int pgrid = 0;
  size_t psmem = 0;
  // the matvec of the kernel graph with TMA-copied halos (persistent over the level-0 tiles)
  int mv_tma = 0;                              // in use (every instance has its tensor maps)
  int mv_avail = 0;                            // the TMA form can run (maps encoded, a grid that fits)
  int coarse_avail2 = 0;                       // two 512-thread coarse CTAs fit on an SM
  int mv_force = 0;                            // PFGB_MATVEC_TMA: 1 on, -1 off, 0 chosen by the batch's shape
  int mv_grid = 0;                             // its CTAs
  char* ws = nullptr;
  size_t ws_bytes = 0;
};

struct MixParams {
  int nx, ny;
  double dx, dy;
  long ld64;
  double tol_out, tol_in;
  int max_outer, max_inner;
  double* b;
  const double* bsum;
  double* res_out;
  double* x;
  const double* const* pprev;
  long ldp;
  int warm;
  Ctrl64* ctrl64;
  const int* active;
  int maxiter_report;
};

// The summary of instance M's solve for the step record (iterations, passes,
// convergence, ||b||, the final ||b - A x||^2); run once the solve has ended.
__device__ __forceinline__ void mx_finish_one(const MixDesc& M) {
  if (!*M.active) return;
  const MixCtrl* m = M.ctrl;
  Ctrl64* c = M.ctrl64;
  c->iter = __ldcg(&m->inner_total);
  c->refine_passes = __ldcg(&m->outer);
  c->info = __ldcg(&m->converged) ? 0 : M.maxiter_report;
  const double bn = __ldcg(&m->bnorm);
  c->zero_rhs = (bn == 0.0) ? 1 : 0;
  c->bnrm2 = bn;
  *M.res_out = __ldcg(&m->rr64);      // ||b - A x||^2 of the final x (the refinement's own residual)
}

int batch_create(const MixParams* prm, int n, Batch** out);
void batch_destroy(Batch* B);
// Append the refinement of every instance (x = A^{-1} b) to a graph chain.
int append_solve(GraphChain& c, Batch* B);
// The same with direct launches and host loop control (for profiling).
int run_direct(Batch* B, cudaStream_t s);
// Use the persistent cooperative solve (on, where the device allows it) or the kernel graph.
int set_persistent(Batch* B, int on);
// 1 when the kernel graph's matvec is the TMA form (persistent over the level-0 tiles)
inline int matvec_form(const Batch* B) { return B->mv_tma; }
// Launch shapes of the solve that give the same bits: variant = 2 * (TMA matvec) + (512-thread
// coarse CTAs).  set_variant refuses one the batch cannot run; tune times every runnable one
// on the batch's own instances (us[4] receives microseconds per PCG iteration, -1 where not
// runnable) and keeps the fastest.  The instances' solver state is kept across tuning.
int variant_of(const Batch* B);
int set_variant(Batch* B, int variant);
int tune(Batch* B, cudaStream_t s, int* chosen, double* us);
// New tolerances and iteration limits for instance k (limits within the loop guards).
int set_tolerances(Batch* B, int k, double tol_out, double tol_in, int max_outer, int max_inner, int warm,
                   int maxiter_report);

}  // namespace mixed
}  // namespace pfgb
