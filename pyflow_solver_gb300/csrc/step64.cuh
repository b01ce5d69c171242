// Binary64 projection step: device structures shared by the kernels and the
// host driver.  Kernels work on a *batch* of independent cavity instances:
// every CTA reads its tile (instance, origin) from a tile table and that
// instance's descriptor from an instance table; a single cavity is a batch of
// one.
#pragma once
#include "common.cuh"
#include "stencil.cuh"
#include "xacc.cuh"

namespace pfgb {

// Reduction sites of one step (each an XASlot).
enum Slot64 {
  S_DIVC_BEFORE = 0,   // ||div_central(u,v;1,1)||^2 before the step      (solver.py:45)
  S_DIVSTAR,           // ||div_c(u*,v*)||^2   -> divergence_norm_initial (pressure_solver.py:121)
  S_BSUM,              // sum of the raw RHS     -> np.mean              (pressure_solver.py:126)
  S_BB,                // ||b||^2                -> bnrm2 of scipy cg
  S_RZ0,               // r.z at iteration 0
  S_PQ,                // p.q                     (one per CG iteration)
  S_RR,                // r.r                     (one per CG iteration)
  S_RZ,                // r.z                     (one per CG iteration)
  S_RES,               // ||b - A x||^2           (interface.py:48-49)
  S_RU,                // sum (u - u_old)^2       (solver.py:106-109)
  S_RV,
  S_DIVAFTER,          // ||div_c(u,v)||^2 after correction (pressure_solver.py:165-170)
  S_LINRES,            // ||A p - b||^2           (pressure_solver.py:174-178)
  S_CONT,              // ||div_central(u,v;1,1)||^2 after the step (solver.py:111)
  S_COUNT
};

// Host-written inputs of one step.
struct StepIn {
  double dt_prev;
  double hist[5];
  int hist_len;
  int iteration;
};

// Device control block of one instance (written by finalisers / tiny kernels).
struct Ctrl64 {
  unsigned long long umax_bits, vmax_bits;  // running maxima (prestep)
  double umax, vmax;                         // + 1e-12 applied
  double div_before;
  double dt, dtm, cfl;
  double rdtm;          // 1 / dtm (the mixed form multiplies by it)
  int safeguard;
  // CG
  int iter, done, info, zero_rhs;
  double mean, bnrm2, atol, rho, rho_prev, pq, rr;
  double alpha, beta;    // rho/pq and rho/rho_prev, formed once by the finalisers
  unsigned nan_flag;
  int refine_passes;     // mixed precision: outer refinement passes
};

// Everything the host reads back after a step (one copy).
struct StepOut64 {
  double umax, vmax, div_before, dt, cfl;
  int safeguard, cg_iters, cg_info, nan_flag;
  double divstar2, bnrm2, res2, ru2, rv2, divafter2, linres2, cont2;
  unsigned flags_or;    // OR of the result flags of all slots (inexact / overflow diagnostics)
  int refine_passes;
  int loop_status;      // bit 0: a loop guard stopped the step; bit 1: the persistent solve's barrier timed out
  int steady;           // the steady-state test passed at this step (SteadyRing)
  double steady_slope;  // its least-squares slope of log10(Ru); NaN when not formed
};

// The steady-state test of the steady driver (src/pyflow/driver/simulation_driver.py:135-149),
// kept per instance on the device: the residual tracker's Ru series -- its seed 1.0, then
// each full step's Ru -- as log10 values in a ring, and after every step the least-squares
// slope of the last `window` entries against 0 .. window - 1.  The test passes when every
// entry of the window is positive and |slope| < tol.  window 0 turns it off.
constexpr int STEADY_MAX_WINDOW = 1024;
struct SteadyRing {
  int window;
  int count;            // entries of the series so far (the seed included)
  double tol;
  double y[STEADY_MAX_WINDOW];   // entry k at y[k % STEADY_MAX_WINDOW]; NaN where Ru <= 0
};

struct Geo64 {
  int nx, ny;
  long ld;            // pitch of the work vectors (doubles)
  long lds;           // pitch of the state arrays (nx + 2)
  Grid2 g;
  double invd;        // interior Jacobi entry 1/(2/dx^2 + 2/dy^2)
  int jacobi;
  double rdx, rdy;    // 1/dx, 1/dy (the mixed form multiplies by them)
};

struct CGArgs {
  double rtol;
  int maxiter;
  double n_cells;     // N as a double (exact)
};

struct DtArgs {
  double dx, dy, cfl_target, growth, nu;
};

struct LidArgs {
  int has_lid;
  double lid;
};

// One tile of work: instance index and the tile's first cell.
struct Tile {
  int inst, i0, j0, loc;       // loc: index of the tile among its instance's tiles of the table
};

// Everything the kernels need about one instance.
struct InstDesc {
  Geo64 G;
  CGArgs A;
  DtArgs D;
  LidArgs L;
  int scheme;          // advection scheme of the predictor
  int adjust;          // 1: projection RHS (mean removal, b[0] = 0); 0: b as given
  int mode;            // correction: 0 full step (lid, residuals), 1 projection only
  int active;          // 0: the instance sits out this launch (all its kernels return)
  double *ui, *vi, *pi;        // state interiors (pitch G.lds)
  double *us, *vs;             // u*, v* (pitch usld)
  long usld;
  double *b, *x, *r, *p0, *p1, *q;
  double* z;                   // M r of the Jacobi-preconditioned CG, written by the kernels that form r
                               // (null: the matvec forms M r itself)
  XASlot* slots;
  Ctrl64* ctrl;
  const StepIn* in;
  StepOut64* out;
  int nt_pc, nt_cg;            // this instance's tiles in the per-cell / CG tile tables
  int nt_m;                    // this instance's tiles in the mixed-form per-cell table (32 x 32)
  double* part;                // per-tile partial sums of the deterministic reductions
  unsigned* ticket;            // their arrival counter
  SteadyRing* steady;          // the device-side steady-state test of this instance
};

// Batch-wide loop control of a WHILE node: the number of instances still
// iterating, and a guard that stops the loop after guard_max trips whatever
// the instances report.
struct LoopCtl {
  int active;
  int guard;
  int guard_max;
  int tripped;
};

}  // namespace pfgb
