// Internal declarations shared by the translation units of libpfgb.so.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/pfgb.h"

namespace pfgb {

// Record the message of the last error of this thread and return `code`.
int set_error(int code, const std::string& msg);
int check_cuda(cudaError_t e, const char* what);

struct StepIn;
struct Instance64;
int instance64_create(const pfgb_params* prm, Instance64** out);
int instance64_create_batch(const pfgb_params* prms, int n, Instance64** out);
int instance64_count(const Instance64* I);
int instance64_batch_step(Instance64* I, double* const* u, double* const* v, double* const* p, const StepIn* in,
                          cudaStream_t s, pfgb_step_out* out);
void instance64_destroy(Instance64* I);
size_t instance64_workspace_bytes(const Instance64* I);
int instance64_project(Instance64* I, double* u, double* v, double* p, long lds, double dt, cudaStream_t s,
                       pfgb_step_out* out);
int instance64_set_graph(Instance64* I, int on);
int instance64_set_persistent(Instance64* I, int on);
int instance64_matvec_form(const Instance64* I, int* tma);
int instance64_autotune(Instance64* I, cudaStream_t s, int* chosen, double* us);
int instance64_set_cg_variant(Instance64* I, int v);
int instance64_set_mixed_variant(Instance64* I, int variant);
int instance64_set_params(Instance64* I, int k, const pfgb_params* prm);
int instance64_set_steady(Instance64* I, int k, int window, double tol);
int instance64_set_profiling(Instance64* I, int on);
int instance64_profile_result(Instance64* I, double* ms, int* launches);
struct KTime;
int instance64_profile_kernels(Instance64* I, std::vector<KTime>& out);
int probe_fp64(cudaStream_t s, double* tops);
int exact_reduce(const double* a, const double* b, long n, int mode, double* result, cudaStream_t s);
int icvt_selftest(long n, cudaStream_t s, long long* mismatches);
int csr_matvec_run(long n, const long* rp, const int* ci, const double* va, const double* x, double* y,
                   cudaStream_t s);
int csr_solve_run(int method, long n, const long* rp, const int* ci, const double* va, const double* invd,
                  const double* b, double* x, double tol, int maxiter, cudaStream_t s, pfgb_solve_out* out);
int cg_solve_noalloc_run(int op, const double* b, double* x, int nx, int ny, double dx, double dy, int precond,
                         double invd, double tol, int maxiter, cudaStream_t s, pfgb_solve_out* out);
int cg_solve_run(int op, const double* b, double* x, int nx, int ny, double dx, double dy, int precond,
                 double invd, double tol, int maxiter, cudaStream_t s, pfgb_solve_out* out);
int instance64_step(Instance64* I, double* u, double* v, double* p, long lds, const StepIn& in,
                    cudaStream_t s, pfgb_step_out* out);

}  // namespace pfgb
