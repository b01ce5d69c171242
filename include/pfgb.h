/*
 * pfgb.h - C ABI of libpfgb.so, the GB300 (sm_103a) projection step of PyFlow's
 * 2-D lid-driven cavity solver.
 *
 * Every entry point returns an int status: 0 on success, a negative PFGB_E*
 * code on error (never an exception).  pfgb_last_error() returns the message of
 * the last error of the calling thread.  Pointers named "device" must point to
 * device memory of the current CUDA device; `stream` is a cudaStream_t (NULL =
 * the legacy default stream).  Arrays are row-major with row index = y; `ld` is
 * the row pitch in elements.
 *
 * Reference citations are paths inside the PyFlow-Solver project.
 */
#ifndef PFGB_H
#define PFGB_H

#include <stddef.h>

#if defined(__GNUC__)
#define PFGB_API __attribute__((visibility("default")))
#else
#define PFGB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define PFGB_OK 0
#define PFGB_EINVAL (-1)   /* invalid argument */
#define PFGB_ECUDA (-2)    /* a CUDA runtime call failed */
#define PFGB_ENOMEM (-3)   /* allocation failed */
#define PFGB_ESTATE (-4)   /* handle used in the wrong state */

/* Advection schemes (config.advection_scheme / disable_advection). */
#define PFGB_SCHEME_UPWIND 0
#define PFGB_SCHEME_QUICK 1
#define PFGB_SCHEME_NONE 2

/* Operators of the pressure solve. */
#define PFGB_OP_NEG_LAPLACIAN_PINNED 0  /* _NegLaplacianPinned, src/pyflow/solvers/pressure_solver.py:97-105 */
#define PFGB_OP_LAPLACIAN_DIRICHLET 1   /* _PosLaplacianDirichlet, src/pyflow/solvers/pressure_solver.py:69-77 */

/* Parameters of one cavity instance; the fields are the attributes that
 * step() reads from its config (src/pyflow/solvers/solver.py:15-99,
 * src/pyflow/solvers/pressure_solver.py:130-146).  Host code computes the
 * derived values exactly as the reference rounds them:
 *   dx = lx / max(nx-1, 1),  nu = 1.0 / Re,
 *   jacobi_interior = 1.0 / (2.0/dx**2 + 2.0/dy**2). */
typedef struct pfgb_params {
  int nx, ny;                /* interior cells */
  double dx, dy;
  double nu;                 /* 1/Re */
  double cfl_target, cfl_growth;
  double lin_tol;            /* rtol of the CG */
  int lin_maxiter;
  int scheme;                /* PFGB_SCHEME_* */
  int enable_jacobi;         /* enable_jacobi_pc */
  double jacobi_interior;
  int has_lid;               /* lid_velocity is not None */
  double lid_velocity;
  int precision;             /* 0: binary64 throughout (the reference's CG); 1: mixed */
  /* precision 1 only: FP64 iterative refinement of the pressure solve to
   * ||b - A x|| <= mixed_tol_outer*||b|| (lin_tol when 0) around a binary32
   * multigrid-preconditioned CG with relative tolerance mixed_tol_inner (1e-5
   * when 0); at most mixed_max_outer passes (8 when 0) of mixed_max_inner
   * inner iterations (50 when 0).  nx and ny must halve down to at most 1024
   * cells on the coarsest multigrid level.  The refinement starts from the
   * pressure the state holds (shifted so that its cell 0 is 0) when that leaves a
   * residual no larger than ||b||, else from zero; mixed_cold_start = 1 starts
   * every solve from zero, as the reference's CG does.  Each inner solve also
   * stops once its residual is below a quarter of the outer target. */
  double mixed_tol_outer, mixed_tol_inner;
  int mixed_max_outer, mixed_max_inner;
  int mixed_cold_start;
  int reserved[3];
} pfgb_params;

/* Host-side state.meta carried into a step (solver.py:32,46-50). */
typedef struct pfgb_step_in {
  double dt_prev;            /* state.meta['dt_prev'] (default 1e-2) */
  double hist[5];            /* state.meta['divergence_history'] (at most 5) */
  int hist_len;
  int iteration;
} pfgb_step_in;

/* Raw step results.  Norms are returned squared (exactly rounded sums); the
 * host applies sqrt and the divisions of the reference. */
typedef struct pfgb_step_out {
  double umax, vmax;         /* max|u| + 1e-12, max|v| + 1e-12 */
  double div_before;         /* ||div_central(u,v;1,1)|| before the step */
  double dt, cfl;
  int safeguard;             /* dt halved by the divergence-trend safeguard */
  int cg_iterations;         /* true number of CG iterations executed */
  int cg_info;               /* scipy info: 0 converged, maxiter otherwise */
  int nan_detected;
  double divstar_sq;         /* ||div_c(u*,v*)||^2 */
  double bnorm;              /* ||b|| of the pressure system */
  double res_sq;             /* ||b - A x||^2 */
  double ru_sq, rv_sq;       /* sum (u-u_old)^2, sum (v-v_old)^2 */
  double divafter_sq;        /* ||div_c(u,v)||^2 after the correction */
  double linres_sq;          /* ||A p - b||^2 */
  double cont_sq;            /* ||div_central(u,v;1,1)||^2 after the step */
  unsigned reduction_flags;  /* bit 3: a term fell below 2^-1184, bit 4: overflow */
  int refine_passes;         /* precision 1: FP64 refinement passes of the pressure solve */
  double steady_slope;       /* pfgb_set_steady: least-squares slope of log10(Ru) over the window (NaN if none) */
  int steady;                /* pfgb_set_steady: the steady-state test passed at this step */
} pfgb_step_out;

typedef struct pfgb_solve_out {
  int info;                  /* scipy info: 0 converged, maxiter otherwise */
  int iterations;            /* true iteration count */
  double bnorm;              /* ||b|| */
  double res_sq;             /* ||b - A x||^2 */
} pfgb_solve_out;

typedef struct pfgb_handle pfgb_handle;

/* Library version (major*10000 + minor*100 + patch). */
PFGB_API int pfgb_version(void);

/* Copy the last error message of this thread into buf (NUL terminated). */
PFGB_API int pfgb_last_error(char* buf, size_t len);

/* ---- one cavity instance ------------------------------------------------ */

/* Replaces the per-step setup of step() (src/pyflow/solvers/solver.py:15-99)
 * and the Jacobi assembly of solve_pressure_poisson
 * (src/pyflow/solvers/pressure_solver.py:15-40,139-145).  Allocates the
 * instance workspace on the current device. */
PFGB_API int pfgb_create(const pfgb_params* params, pfgb_handle** handle);
PFGB_API int pfgb_destroy(pfgb_handle* handle);
/* Bytes of device workspace held by the handle. */
PFGB_API size_t pfgb_workspace_bytes(const pfgb_handle* handle);

/* One projection step, in place on the ghosted state arrays u, v, p (device,
 * shape (ny+2, nx+2), ld = nx+2, interior [1:-1,1:-1]).  Replaces step()
 * (src/pyflow/solvers/solver.py:15-121) including solve_pressure_poisson
 * (src/pyflow/solvers/pressure_solver.py:95-219) and the CG of
 * src/pyflow/linear_solvers/interface.py:23-53.  Synchronises `stream`. */
PFGB_API int pfgb_step(pfgb_handle* handle, double* u, double* v, double* p, long ld,
              const pfgb_step_in* in, void* stream, pfgb_step_out* out);

/* ---- batches of independent cavities ----------------------------------- */

/* n instances (params[k] each; all with the same precision) advanced together: every
 * kernel of a step covers the tiles of all instances (one CUDA graph launch
 * per step, CG loop as one WHILE node with per-instance convergence masks).
 * Same per-instance semantics as pfgb_step (src/pyflow/solvers/solver.py:15-121
 * for each cavity). */
PFGB_API int pfgb_batch_create(const pfgb_params* params, int n, pfgb_handle** handle);
/* One step of every instance k with u[k], v[k], p[k] non-null (the others sit
 * the step out): state arrays as in pfgb_step, in[k] / out[k] per instance.
 * Synchronises `stream`. */
PFGB_API int pfgb_batch_step(pfgb_handle* handle, double* const* u, double* const* v, double* const* p,
                             const pfgb_step_in* in, void* stream, pfgb_step_out* out);
PFGB_API int pfgb_batch_size(const pfgb_handle* handle);
/* New physical parameters (Re, lid velocity, CFL, tolerance, scheme, ...) for
 * instance k, e.g. when a serving slot takes a new request.  Grid, spacing,
 * precision and preconditioner stay those of the slot. */
PFGB_API int pfgb_batch_set_params(pfgb_handle* handle, int k, const pfgb_params* params);

/* Stand-alone projection of the state's current u, v with a given dt:
 * solve_pressure_poisson in normal mode
 * (src/pyflow/solvers/pressure_solver.py:95-219 with rhs_override None).
 * u, v are corrected in place and p receives the pinned pressure.  Fills the
 * projection fields of `out` (divstar_sq, bnorm, res_sq, divafter_sq,
 * linres_sq, cg_iterations, cg_info, nan_detected).  Synchronises `stream`. */
PFGB_API int pfgb_project(pfgb_handle* handle, double* u, double* v, double* p, long ld, double dt,
                          void* stream, pfgb_step_out* out);

/* Run pfgb_step as one CUDA graph (on = 1, the default) or as individual
 * launches (0).  The graph is built on the first step and rebuilt when the
 * state arrays move; the CG loop is a WHILE conditional node, so the device
 * decides when it stops.  With on = 1 consecutive kernels are joined by
 * programmatic dependent-launch edges (the next kernel is launched while the
 * previous one runs and waits for it on the device); on = 2 builds the graph
 * with ordinary edges.  All modes give identical results.  No reference
 * counterpart. */
PFGB_API int pfgb_set_graph(pfgb_handle* handle, int on);

/* ---- array operators (device arrays, no synchronisation) --------------- */

/* gradient_coherent, src/pyflow/numerics/core_ops_coherent.py:45-61 */
PFGB_API int pfgb_gradient_coherent(const double* p, long ldp, double* gx, double* gy, long ldo,
                           int nx, int ny, double dx, double dy, void* stream);
/* divergence_coherent, src/pyflow/numerics/core_ops_coherent.py:63-79 */
PFGB_API int pfgb_divergence_coherent(const double* u, const double* v, long ldi, double* div, long ldo,
                             int nx, int ny, double dx, double dy, void* stream);
/* laplacian_coherent, src/pyflow/numerics/core_ops_coherent.py:81-84 */
PFGB_API int pfgb_laplacian_coherent(const double* p, long ldp, double* lap, long ldo,
                            int nx, int ny, double dx, double dy, void* stream);
/* divergence (central), src/pyflow/numerics/fluid_ops.py:8-41 */
PFGB_API int pfgb_divergence_central(const double* u, const double* v, long ldi, double* div, long ldo,
                            int nx, int ny, double dx, double dy, void* stream);
/* advect_upwind / advect_quick, src/pyflow/numerics/operators/advection.py:17-84 */
PFGB_API int pfgb_advect(int scheme, const double* u, const double* v, const double* f, long ldi,
                double* conv, long ldo, int nx, int ny, double dx, double dy, void* stream);
/* y = A x for the pressure operators (PFGB_OP_*); x, y contiguous (ny*nx) */
PFGB_API int pfgb_apply_operator(int op, const double* x, double* y, int nx, int ny, double dx, double dy,
                        void* stream);

/* out[i] = a[i] / d with the division the stencils use for a grid spacing d > 0
 * (method 0: exact reciprocal product for powers of two, else the integer-pipe
 * division by an invariant divisor) or the hardware IEEE division (method 1).
 * Both return the correctly rounded quotient of NumPy's `a / d`, the form of
 * every `/ dx`, `/ dy` of src/pyflow/numerics/core_ops_coherent.py:57-77. */
PFGB_API int pfgb_div_by_constant(const double* a, double* out, long n, double d, int method, void* stream);

/* ---- exactly rounded reductions ------------------------------------------ */

/* result = RN(sum a[i]*b[i]) with exact products (order independent); the
 * twin of np.dot.  Synchronises `stream`; result is a host pointer. */
PFGB_API int pfgb_xdot(const double* a, const double* b, long n, double* result, void* stream);
/* result = RN(sum a[i]) (order independent). */
PFGB_API int pfgb_xsum(const double* a, long n, double* result, void* stream);

/* ---- linear-solver operator interface ------------------------------------ */

/* PCG of scipy.sparse.linalg.cg as called by solve()
 * (src/pyflow/linear_solvers/interface.py:23-53): x0 = 0, rtol = tol,
 * M = Jacobi (jacobi_preconditioner, src/pyflow/linear_solvers/preconditioners.py:8-25)
 * when precond = 1, identity when 0.  b and x are contiguous device vectors of
 * nx*ny doubles (row-major, k = j*nx + i).  Synchronises `stream`. */
PFGB_API int pfgb_cg_solve(int op, const double* b, double* x, int nx, int ny, double dx, double dy,
                  int precond, double jacobi_interior, double tol, int maxiter,
                  void* stream, pfgb_solve_out* out);

/* ---- operator interface: an assembled sparse matrix ------------------------- */

/* y = A x for an n x n CSR matrix in device memory (row pointers int64, n + 1 of
 * them; column indices int32; values binary64): each row's terms summed in
 * storage order, one rounded product and one rounded addition per term, as
 * scipy's CSR product.  Replaces `A @ x` of the reference's solve
 * (src/pyflow/linear_solvers/interface.py:48). */
PFGB_API int pfgb_csr_matvec(long n, const long* rowptr, const int* colind, const double* vals, const double* x,
                             double* y, void* stream);
/* solve(A, b, method, tol, maxiter, M) of the reference for an assembled sparse
 * matrix (src/pyflow/linear_solvers/interface.py:23-53): method 0 runs
 * scipy.sparse.linalg.cg, method 1 scipy.sparse.linalg.bicgstab (SciPy 1.13.1 as
 * the reference pins it), from x0 = 0 with rtol = tol; inv_diag (may be NULL:
 * no preconditioner) is the Jacobi preconditioner's vector of 1/diag(A)
 * (src/pyflow/linear_solvers/preconditioners.py:8-25).  Dot products and norms
 * are exactly rounded.  out: info (0 converged, maxiter when the loop ran out,
 * -10 / -11 for BiCGSTAB's breakdowns), the iterations executed, ||b||, and
 * ||b - A x||^2.  x (n doubles) is overwritten.  Allocates its work vectors
 * stream-ordered and synchronises `stream` at every scalar the iteration
 * tests. */
PFGB_API int pfgb_csr_solve(int method, long n, const long* rowptr, const int* colind, const double* vals,
                            const double* inv_diag, const double* b, double* x, double tol, int maxiter,
                            void* stream, pfgb_solve_out* out);

/* Same solve as pfgb_cg_solve, but it allocates nothing: no cudaMalloc,
 * cudaMallocAsync, cudaFree or other allocating call.  It has no counterpart in
 * the reference; it exists for callers that cannot allocate device memory when
 * they solve: a real-time loop that must not stall on cudaMalloc/cudaFree (they
 * can synchronise the whole device), or a host application that has reserved
 * the device memory for its own pool and admits no third-party allocation.
 * The CG work vectors live in one fixed device array compiled into the library
 * (about 8.5 MiB), reserved on a device when the library's module is loaded
 * there -- with CUDA's lazy module loading, the default, that can be this
 * function's first call on the device -- and held until the process exits, so
 * nx*ny must not exceed 262,144 cells (512 x 512); larger grids return
 * PFGB_EINVAL without launching anything.
 * The first call on a device looks up that array's device address (once per
 * device, with the device current); make that first call before any stream
 * capture.  Every call reuses the same array: two calls that overlap on the GPU
 * (different streams or host threads without ordering) race and corrupt each
 * other's results, so serialise them.  Synchronises `stream`. */
PFGB_API int pfgb_cg_solve_noalloc(int op, const double* b, double* x, int nx, int ny, double dx, double dy,
                                   int precond, double jacobi_interior, double tol, int maxiter,
                                   void* stream, pfgb_solve_out* out);

/* Page-lock the host range [ptr, ptr + bytes) (cudaHostRegister, portable) so
 * that copies between it and device memory are direct DMA transfers, without a
 * staging copy through a driver buffer.  For callers that keep their fields in
 * host arrays and step them in place: the arrays are registered once and every
 * step's transfers go straight into and out of them.  Fails (PFGB_ECUDA, nothing
 * registered) when the range overlaps a registered one.  pfgb_host_unregister
 * releases a range by its start address; an array must be unregistered before
 * its memory is freed.  No reference counterpart. */
PFGB_API int pfgb_host_register(void* ptr, size_t bytes);
PFGB_API int pfgb_host_unregister(void* ptr);

/* With precision 1: run each step's pressure solve as one persistent cooperative
 * launch (on; available where the device co-schedules one 1024-thread CTA per
 * SM) or as a graph of per-phase kernels with WHILE loop nodes (off, the
 * default).  Both give the same bits.  No reference counterpart. */
PFGB_API int pfgb_set_persistent(pfgb_handle* handle, int on);

/* With precision 1: *tma = 1 when the kernel graph's PCG matvec is the TMA form
 * (persistent over the level-0 tiles, halos copied by the tensor memory
 * accelerator; chosen for instances of at least 64 tiles and at least 2 tiles per
 * CTA, or forced by PFGB_MATVEC_TMA=1 / 0 when the instance is created), 0 when it
 * is one tile per CTA.  Both give the same bits.  No reference counterpart. */
PFGB_API int pfgb_matvec_form(pfgb_handle* handle, int* tma);

/* Device-side steady-state test of instance k of a handle (k = 0 for a single
 * cavity): the residual tracker's Ru series -- seed 1.0, then the Ru of every
 * following full step -- is kept on the device, and each step record reports
 * the least-squares slope of log10(Ru) over the last `window` entries
 * (steady_slope) and whether every entry was positive and |slope| < slope_tol
 * (steady).  window 0 turns the test off; otherwise 2 <= window <= 1024.
 * Each call restarts the series from its seed.  Replaces the host-side test of
 * the steady driver (src/pyflow/driver/simulation_driver.py:135-149); lets a
 * batch retire instances on it without reading their Ru series back. */
PFGB_API int pfgb_set_steady(pfgb_handle* handle, int k, int window, double slope_tol);

/* ---- tile autotuner ---------------------------------------------------------- */

/* Time the launch shapes of this handle's pressure solve on its own instances
 * and keep the fastest for its following steps; every shape gives identical
 * results.  Precision 0: the three tile shapes of the binary64 CG kernel pair
 * (32 x 8, 32 x 16, 32 x 32 cells per CTA; the exactly rounded reductions make
 * the shape invisible in the results), variant 0..2.  Precision 1: the four
 * launch variants of the binary32 PCG iteration, variant = 2 * (TMA matvec:
 * persistent over the level-0 tiles with halos copied by the tensor memory
 * accelerator) + (512-thread coarse CTAs, two to an SM, instead of 1024),
 * those the batch cannot run skipped; the tile shape there is fixed at 32 x 32
 * because it fixes the summation order of the tile sums.  `variant` (may be
 * NULL) receives the choice, `us_per_iteration` (may be NULL, else room for 4
 * doubles) the measured microseconds per iteration of each shape (-1 where not
 * run).  Synchronises `stream`; the handle's work vectors are overwritten
 * (every step rewrites them) and its solver state is kept.  A no-op for the
 * persistent form of the mixed solve.  No reference counterpart: the reference
 * has no device kernels to tune. */
PFGB_API int pfgb_autotune(pfgb_handle* handle, void* stream, int* variant, double* us_per_iteration);
/* Select a CG tile shape directly (a choice cached from an earlier autotune). */
PFGB_API int pfgb_set_cg_variant(pfgb_handle* handle, int variant);
/* Select a launch variant of the mixed solve directly (0..3 as pfgb_autotune
 * numbers them; PFGB_EINVAL for one the batch cannot run). */
PFGB_API int pfgb_set_mixed_variant(pfgb_handle* handle, int variant);

/* ---- measurement ----------------------------------------------------------- */

/* Record CUDA events around every kernel launch of the following steps of this
 * handle.  Steps then run as individual launches (no graph); after each host
 * read-back inside a step a short spin kernel keeps the stream busy, so the
 * events bracket kernel execution rather than host launch latency.  No
 * reference counterpart: benchmark instrumentation. */
PFGB_API int pfgb_set_profiling(pfgb_handle* handle, int on);
/* Total device time (ms) and number of the pressure-matvec launches (p = z +
 * beta p; q = A p; p.q) of the last profiled step: the binary64 CG matvec, or
 * with precision 1 the binary32 PCG matvec of the inner solves (or the
 * persistent solve as one launch where that form runs). */
PFGB_API int pfgb_profile_result(pfgb_handle* handle, double* ms, int* launches);

/* Device time of one kernel over the last profiled step. */
typedef struct pfgb_kernel_time {
  char name[48];     /* kernel name; multigrid kernels carry their level ("k_mg_down@1") */
  int launches;
  double total_ms;
} pfgb_kernel_time;
/* Per-kernel sums of the last profiled step, in order of first launch: writes up
 * to `capacity` entries and sets *count to the number of kernels (which may
 * exceed capacity).  Call after the step returned (its stream is synchronised).
 * No reference counterpart: benchmark instrumentation. */
PFGB_API int pfgb_profile_kernels(pfgb_handle* handle, pfgb_kernel_time* out, int capacity, int* count);
/* Self-test of the integer-pipe number conversions the kernels use in place of
 * the hardware ones (binary64 -> binary32 round to nearest even, binary32 ->
 * binary64, exact halving of a binary64 value): `samples` pseudo-random bit
 * patterns (exponents concentrated around the binary32 range and its
 * boundaries, with ties and specials) are converted both ways on the device;
 * mismatches[0..2] receive the number of differing results of each conversion
 * (NaN against NaN counts as equal).  No reference counterpart. */
PFGB_API int pfgb_selftest_conversions(long samples, void* stream, long long* mismatches);
/* Measured FP64 FMA issue rate of the current device, in 1e12 instructions/s.
 * No reference counterpart: the denominator of the FP64 roofline. */
PFGB_API int pfgb_probe_fp64(void* stream, double* tops);

#ifdef __cplusplus
}
#endif

#endif /* PFGB_H */
