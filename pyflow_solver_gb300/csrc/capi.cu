// C ABI entry points of libpfgb.so (declared in include/pfgb.h): handles,
// error reporting, the projection step and the operator-interface CG.
#include <cstring>
#include <string>
#include <vector>

#include "kprof.cuh"
#include "pfgb_internal.h"
#include "step64.cuh"

namespace pfgb {

static thread_local std::string g_last_error;

int set_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return PFGB_OK;
  return set_error(PFGB_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace pfgb

struct pfgb_handle {
  pfgb::Instance64* inst;
};

using namespace pfgb;

extern "C" int pfgb_version(void) { return 100; }

extern "C" int pfgb_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return PFGB_EINVAL;
  size_t n = g_last_error.size() < len - 1 ? g_last_error.size() : len - 1;
  memcpy(buf, g_last_error.data(), n);
  buf[n] = '\0';
  return PFGB_OK;
}

extern "C" int pfgb_create(const pfgb_params* params, pfgb_handle** handle) {
  if (!params || !handle) return set_error(PFGB_EINVAL, "null argument");
  if (params->precision != 0 && params->precision != 1) return set_error(PFGB_EINVAL, "precision must be 0 or 1");
  if (params->scheme < 0 || params->scheme > 2) return set_error(PFGB_EINVAL, "unknown advection scheme");
  if (params->lin_maxiter < 0) return set_error(PFGB_EINVAL, "lin_maxiter must be >= 0");
  Instance64* inst = nullptr;
  int rc = instance64_create(params, &inst);
  if (rc) return rc;
  pfgb_handle* h = new pfgb_handle;
  h->inst = inst;
  *handle = h;
  return PFGB_OK;
}

extern "C" int pfgb_destroy(pfgb_handle* handle) {
  if (!handle) return PFGB_OK;
  instance64_destroy(handle->inst);
  delete handle;
  return PFGB_OK;
}

extern "C" size_t pfgb_workspace_bytes(const pfgb_handle* handle) {
  return handle ? instance64_workspace_bytes(handle->inst) : 0;
}

extern "C" int pfgb_step(pfgb_handle* handle, double* u, double* v, double* p, long ld, const pfgb_step_in* in,
                         void* stream, pfgb_step_out* out) {
  if (!handle || !u || !v || !p || !in || !out) return set_error(PFGB_EINVAL, "null argument");
  if (in->hist_len < 0 || in->hist_len > 5) return set_error(PFGB_EINVAL, "hist_len must be in [0, 5]");
  StepIn si;
  si.dt_prev = in->dt_prev;
  for (int k = 0; k < 5; ++k) si.hist[k] = in->hist[k];
  si.hist_len = in->hist_len;
  si.iteration = in->iteration;
  return instance64_step(handle->inst, u, v, p, ld, si, (cudaStream_t)stream, out);
}

extern "C" int pfgb_project(pfgb_handle* handle, double* u, double* v, double* p, long ld, double dt, void* stream,
                            pfgb_step_out* out) {
  if (!handle || !u || !v || !p || !out) return set_error(PFGB_EINVAL, "null argument");
  return instance64_project(handle->inst, u, v, p, ld, dt, (cudaStream_t)stream, out);
}

extern "C" int pfgb_cg_solve(int op, const double* b, double* x, int nx, int ny, double dx, double dy, int precond,
                             double jacobi_interior, double tol, int maxiter, void* stream, pfgb_solve_out* out) {
  if (!b || !x || !out) return set_error(PFGB_EINVAL, "null argument");
  return cg_solve_run(op, b, x, nx, ny, dx, dy, precond, jacobi_interior, tol, maxiter, (cudaStream_t)stream, out);
}

extern "C" int pfgb_set_profiling(pfgb_handle* handle, int on) {
  if (!handle) return set_error(PFGB_EINVAL, "null handle");
  return instance64_set_profiling(handle->inst, on);
}

extern "C" int pfgb_profile_result(pfgb_handle* handle, double* ms, int* launches) {
  if (!handle || !ms || !launches) return set_error(PFGB_EINVAL, "null argument");
  return instance64_profile_result(handle->inst, ms, launches);
}

extern "C" int pfgb_profile_kernels(pfgb_handle* handle, pfgb_kernel_time* out, int capacity, int* count) {
  if (!handle || !count || (capacity > 0 && !out)) return set_error(PFGB_EINVAL, "null argument");
  std::vector<KTime> kt;
  if (int rc = instance64_profile_kernels(handle->inst, kt)) return rc;
  *count = (int)kt.size();
  for (int k = 0; k < capacity && k < (int)kt.size(); ++k) {
    std::memset(out[k].name, 0, sizeof(out[k].name));
    std::strncpy(out[k].name, kt[k].name.c_str(), sizeof(out[k].name) - 1);
    out[k].launches = kt[k].launches;
    out[k].total_ms = kt[k].ms;
  }
  return PFGB_OK;
}

extern "C" int pfgb_probe_fp64(void* stream, double* tops) {
  if (!tops) return set_error(PFGB_EINVAL, "null argument");
  return probe_fp64((cudaStream_t)stream, tops);
}

extern "C" int pfgb_cg_solve_noalloc(int op, const double* b, double* x, int nx, int ny, double dx, double dy,
                                     int precond, double jacobi_interior, double tol, int maxiter, void* stream,
                                     pfgb_solve_out* out) {
  if (!b || !x || !out) return set_error(PFGB_EINVAL, "null argument");
  return cg_solve_noalloc_run(op, b, x, nx, ny, dx, dy, precond, jacobi_interior, tol, maxiter, (cudaStream_t)stream,
                              out);
}

extern "C" int pfgb_autotune(pfgb_handle* handle, void* stream, int* variant, double* us_per_iteration) {
  if (!handle) return set_error(PFGB_EINVAL, "null handle");
  return instance64_autotune(handle->inst, (cudaStream_t)stream, variant, us_per_iteration);
}

extern "C" int pfgb_set_mixed_variant(pfgb_handle* handle, int variant) {
  if (!handle) return set_error(PFGB_EINVAL, "null handle");
  return instance64_set_mixed_variant(handle->inst, variant);
}

extern "C" int pfgb_set_cg_variant(pfgb_handle* handle, int variant) {
  if (!handle) return set_error(PFGB_EINVAL, "null handle");
  return instance64_set_cg_variant(handle->inst, variant);
}

extern "C" int pfgb_host_register(void* ptr, size_t bytes) {
  if (!ptr || bytes == 0) return set_error(PFGB_EINVAL, "empty host range");
  const cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterPortable);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(PFGB_ECUDA, std::string("cudaHostRegister: ") + cudaGetErrorString(e));
  }
  return PFGB_OK;
}

extern "C" int pfgb_host_unregister(void* ptr) {
  if (!ptr) return set_error(PFGB_EINVAL, "null host pointer");
  const cudaError_t e = cudaHostUnregister(ptr);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(PFGB_ECUDA, std::string("cudaHostUnregister: ") + cudaGetErrorString(e));
  }
  return PFGB_OK;
}

extern "C" int pfgb_set_persistent(pfgb_handle* handle, int on) {
  if (!handle) return set_error(PFGB_EINVAL, "null handle");
  return instance64_set_persistent(handle->inst, on);
}

extern "C" int pfgb_matvec_form(pfgb_handle* handle, int* tma) {
  if (!handle || !tma) return set_error(PFGB_EINVAL, "null argument");
  return instance64_matvec_form(handle->inst, tma);
}

extern "C" int pfgb_set_graph(pfgb_handle* handle, int on) {
  if (!handle) return set_error(PFGB_EINVAL, "null handle");
  return instance64_set_graph(handle->inst, on);
}

extern "C" int pfgb_batch_create(const pfgb_params* params, int n, pfgb_handle** handle) {
  if (!params || !handle || n < 1) return set_error(PFGB_EINVAL, "invalid batch arguments");
  for (int k = 0; k < n; ++k) {
    if (params[k].precision != 0 && params[k].precision != 1) return set_error(PFGB_EINVAL, "precision must be 0 or 1");
    if (params[k].scheme < 0 || params[k].scheme > 2) return set_error(PFGB_EINVAL, "unknown advection scheme");
  }
  Instance64* inst = nullptr;
  int rc = instance64_create_batch(params, n, &inst);
  if (rc) return rc;
  pfgb_handle* h = new pfgb_handle;
  h->inst = inst;
  *handle = h;
  return PFGB_OK;
}

extern "C" int pfgb_batch_step(pfgb_handle* handle, double* const* u, double* const* v, double* const* p,
                               const pfgb_step_in* in, void* stream, pfgb_step_out* out) {
  if (!handle || !u || !v || !p || !in || !out) return set_error(PFGB_EINVAL, "null argument");
  const int n = instance64_count(handle->inst);
  std::vector<StepIn> si(n);
  for (int k = 0; k < n; ++k) {
    if (in[k].hist_len < 0 || in[k].hist_len > 5) return set_error(PFGB_EINVAL, "hist_len must be in [0, 5]");
    si[k].dt_prev = in[k].dt_prev;
    for (int q = 0; q < 5; ++q) si[k].hist[q] = in[k].hist[q];
    si[k].hist_len = in[k].hist_len;
    si[k].iteration = in[k].iteration;
  }
  return instance64_batch_step(handle->inst, u, v, p, si.data(), (cudaStream_t)stream, out);
}

extern "C" int pfgb_batch_size(const pfgb_handle* handle) { return handle ? instance64_count(handle->inst) : 0; }

extern "C" int pfgb_batch_set_params(pfgb_handle* handle, int k, const pfgb_params* params) {
  if (!handle || !params) return set_error(PFGB_EINVAL, "null argument");
  return instance64_set_params(handle->inst, k, params);
}

extern "C" int pfgb_set_steady(pfgb_handle* handle, int k, int window, double slope_tol) {
  if (!handle) return set_error(PFGB_EINVAL, "null handle");
  return instance64_set_steady(handle->inst, k, window, slope_tol);
}

extern "C" int pfgb_csr_matvec(long n, const long* rowptr, const int* colind, const double* vals, const double* x,
                               double* y, void* stream) {
  if (n > 0 && (!rowptr || !colind || !vals || !x || !y)) return set_error(PFGB_EINVAL, "null argument");
  return csr_matvec_run(n, rowptr, colind, vals, x, y, (cudaStream_t)stream);
}

extern "C" int pfgb_csr_solve(int method, long n, const long* rowptr, const int* colind, const double* vals,
                              const double* inv_diag, const double* b, double* x, double tol, int maxiter, void* stream,
                              pfgb_solve_out* out) {
  if (!rowptr || !colind || !vals || !b || !x || !out) return set_error(PFGB_EINVAL, "null argument");
  return csr_solve_run(method, n, rowptr, colind, vals, inv_diag, b, x, tol, maxiter, (cudaStream_t)stream, out);
}
