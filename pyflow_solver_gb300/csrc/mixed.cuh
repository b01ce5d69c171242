// Mixed-precision pressure solve (FP64 refinement around FP32 multigrid-PCG):
// device structures and the host interface used by the step graph.
#pragma once
#include <cuda_runtime.h>

#include "graph.cuh"
#include "stencil.cuh"
#include "step64.cuh"
#include "xacc.cuh"

namespace pfgb {
namespace mixed {

constexpr int MAX_LEVELS = 16;

// One multigrid level: binary32 arrays of (ny, ld); cx, cy are the face
// coefficients (1/dx^2, 1/dy^2 on every level: with R = P^T summing about four
// children, the rediscretised coarse operator keeps the fine coefficients).
struct Lvl {
  int nx, ny;
  long ld;
  float cx, cy;
  float* u;   // V-cycle result
  float* t;   // pre-smoothed iterate
  float* f;   // right-hand side (on level 0: the PCG residual)
  float* r;   // residual f - A t after pre-smoothing
};

// binary64 geometry of the refinement
struct Geo {
  int nx, ny;
  long ld;
  Grid2 g;
};

enum MixSlot { M_RR64 = 0, M_SUM64, M_RT, M_RZ, M_PQ, M_RR, M_COUNT };

struct MixCtrl {
  double tol_out, tol_in;
  int max_outer, max_inner;
  double bnorm, tol_abs_out, rr64, sum64;
  double rt_norm, tol_abs_in;
  double rho, beta, pq, alpha, rr_in;
  int outer, inner, inner_total, converged;
  int inner_done, outer_done;
};

struct Solver {
  Geo G;
  double tol_out, tol_in;
  int max_outer, max_inner;
  int nlev = 0;
  Lvl lev[MAX_LEVELS];
  int coarse_levels = 1;       // levels resolved inside the coarse CTA
  size_t coarse_smem = 0;      // its dynamic shared memory
  char* ws = nullptr;
  size_t ws_bytes = 0;
  float *e, *p0, *p1, *q;
  double* r64;
  XASlot* slots;
  MixCtrl* ctrl;
};

int solver_create(int nx, int ny, double dx, double dy, long ld64, double tol_out, double tol_in, int max_outer,
                  int max_inner, Solver** out);
void solver_destroy(Solver* S);
// Append x = A^{-1} b (refinement loop) to a graph chain, then record the
// total inner iterations / convergence in the step's control block.
int append_solve(GraphChain& c, Solver* S, const double* b, double* x, Ctrl64* ctrl64, int maxiter_report);
// The same solve with direct launches and host loop control (for profiling).
int run_direct(Solver* S, const double* b, double* x, Ctrl64* ctrl64, int maxiter_report, cudaStream_t s);

}  // namespace mixed
}  // namespace pfgb
