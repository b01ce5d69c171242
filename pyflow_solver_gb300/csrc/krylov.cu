// Krylov solves of a general sparse matrix on the GPU: the operator interface's
// solve(A, b, method='cg' | 'bicgstab', tol, maxiter, M) for an assembled matrix
// (src/pyflow/linear_solvers/interface.py:23-53, which calls scipy.sparse.linalg.cg or
// .bicgstab; SciPy 1.13.1 as pinned by the reference), with the Jacobi preconditioner
// of such a matrix (src/pyflow/linear_solvers/preconditioners.py:8-25) as a vector of
// reciprocal diagonal entries.
//
// The matrix is CSR (row pointers int64, column indices int32, values binary64) in
// device memory.  The product sums each row's terms in storage order, one rounded
// product and one rounded addition per term (as scipy's CSR product does); vector
// updates round each product before the sum (as NumPy's in-place ufuncs do); every
// dot product and norm is exactly rounded (xacc.cuh), so the iteration is the oracle
// twin's bit for bit.  The iteration runs on the host over device vectors, reading
// each scalar back as SciPy's loop uses it: this is the general interface, not the
// time step, whose pressure solve is the fused stencil CG of step64.cu.
#include <cmath>
#include <string>
#include <vector>

#include "pfgb_internal.h"

namespace pfgb {

namespace {

constexpr int KT = 256;

__global__ void k_csr_matvec(long n, const long* __restrict__ rp, const int* __restrict__ ci,
                             const double* __restrict__ va, const double* __restrict__ x, double* __restrict__ y) {
  const long i = (long)blockIdx.x * KT + threadIdx.x;
  if (i >= n) return;
  double acc = 0.0;
  for (long jj = rp[i]; jj < rp[i + 1]; ++jj) acc = __dadd_rn(acc, __dmul_rn(va[jj], x[ci[jj]]));
  y[i] = acc;
}

// y = y + a * x (the product rounded first)
__global__ void k_axpy(long n, double a, const double* __restrict__ x, double* __restrict__ y) {
  const long i = (long)blockIdx.x * KT + threadIdx.x;
  if (i < n) y[i] = __dadd_rn(y[i], __dmul_rn(a, x[i]));
}

// p = p * beta + z (two roundings)
__global__ void k_scale_add(long n, double beta, const double* __restrict__ z, double* __restrict__ p) {
  const long i = (long)blockIdx.x * KT + threadIdx.x;
  if (i < n) p[i] = __dadd_rn(__dmul_rn(p[i], beta), z[i]);
}

// p = p * beta
__global__ void k_scale(long n, double beta, double* __restrict__ p) {
  const long i = (long)blockIdx.x * KT + threadIdx.x;
  if (i < n) p[i] = __dmul_rn(p[i], beta);
}

// z = d * r (Jacobi) or z = r (d null)
__global__ void k_precond(long n, const double* __restrict__ d, const double* __restrict__ r, double* __restrict__ z) {
  const long i = (long)blockIdx.x * KT + threadIdx.x;
  if (i < n) z[i] = d ? __dmul_rn(d[i], r[i]) : r[i];
}

// r = b - y
__global__ void k_sub(long n, const double* __restrict__ b, const double* __restrict__ y, double* __restrict__ r) {
  const long i = (long)blockIdx.x * KT + threadIdx.x;
  if (i < n) r[i] = __dsub_rn(b[i], y[i]);
}

struct Csr {
  long n;
  const long* rp;
  const int* ci;
  const double* va;
};

class Run {
 public:
  Run(const Csr& A, const double* invd, cudaStream_t s) : A_(A), d_(invd), s_(s), blocks_((unsigned)((A.n + KT - 1) / KT)) {}
  ~Run() {
    for (double* v : vecs_) cudaFreeAsync(v, s_);
  }
  double* vec() {
    double* v = nullptr;
    if (cudaMallocAsync(&v, A_.n * sizeof(double), s_) != cudaSuccess) {
      err_ = set_error(PFGB_ENOMEM, "cudaMallocAsync of a Krylov work vector failed");
      return nullptr;
    }
    vecs_.push_back(v);
    return v;
  }
  void matvec(const double* x, double* y) { k_csr_matvec<<<blocks_, KT, 0, s_>>>(A_.n, A_.rp, A_.ci, A_.va, x, y); }
  void axpy(double a, const double* x, double* y) { k_axpy<<<blocks_, KT, 0, s_>>>(A_.n, a, x, y); }
  void scale_add(double beta, const double* z, double* p) { k_scale_add<<<blocks_, KT, 0, s_>>>(A_.n, beta, z, p); }
  void scale(double beta, double* p) { k_scale<<<blocks_, KT, 0, s_>>>(A_.n, beta, p); }
  void psolve(const double* r, double* z) { k_precond<<<blocks_, KT, 0, s_>>>(A_.n, d_, r, z); }
  void copy(const double* src, double* dst) { cudaMemcpyAsync(dst, src, A_.n * sizeof(double), cudaMemcpyDeviceToDevice, s_); }
  void sub(const double* b, const double* y, double* r) { k_sub<<<blocks_, KT, 0, s_>>>(A_.n, b, y, r); }
  double dot(const double* a, const double* b) {
    double r = 0.0;
    if (!err_) err_ = exact_reduce(a, b, A_.n, 0, &r, s_);
    return r;
  }
  double norm(const double* a) { return std::sqrt(dot(a, a)); }
  int err() const { return err_; }
  int launch_err() {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess && !err_) err_ = set_error(PFGB_ECUDA, std::string("krylov kernel: ") + cudaGetErrorString(e));
    return err_;
  }

 private:
  Csr A_;
  const double* d_;
  cudaStream_t s_;
  unsigned blocks_;
  std::vector<double*> vecs_;
  int err_ = PFGB_OK;
};

// scipy.sparse.linalg.cg with x0 = 0 (the sequence oracle/cg.py restates)
int cg(Run& R, const double* b, double* x, double tol, int maxiter, int* info, int* iters) {
  double *r = R.vec(), *z = R.vec(), *p = R.vec(), *q = R.vec();
  if (R.err()) return R.err();
  const double bnrm2 = R.norm(b);
  const double atol = std::fmax(0.0, tol * bnrm2);
  *iters = 0;
  if (bnrm2 == 0.0) {
    R.copy(b, x);
    *info = 0;
    return R.launch_err();
  }
  R.copy(b, r);
  double rho_prev = 0.0;
  for (int it = 0; it < maxiter; ++it) {
    if (R.norm(r) < atol) {
      *info = 0;
      *iters = it;
      return R.launch_err();
    }
    R.psolve(r, z);
    const double rho = R.dot(r, z);
    if (it > 0) R.scale_add(rho / rho_prev, z, p);
    else R.copy(z, p);
    R.matvec(p, q);
    const double alpha = rho / R.dot(p, q);
    R.axpy(alpha, p, x);
    R.axpy(-alpha, q, r);
    rho_prev = rho;
    if (R.err()) return R.err();
  }
  *info = maxiter;
  *iters = maxiter;
  return R.launch_err();
}

// scipy.sparse.linalg.bicgstab with x0 = 0: rho and omega breakdown tests at eps^2
// (info -10, -11), rv == 0 (info -11), the early exit on ||s|| < atol
int bicgstab(Run& R, const double* b, double* x, double tol, int maxiter, int* info, int* iters) {
  double *r = R.vec(), *rt = R.vec(), *p = R.vec(), *v = R.vec(), *s = R.vec(), *ph = R.vec(), *sh = R.vec(),
         *t = R.vec();
  if (R.err()) return R.err();
  const double bnrm2 = R.norm(b);
  const double atol = std::fmax(0.0, tol * bnrm2);
  *iters = 0;
  if (bnrm2 == 0.0) {
    R.copy(b, x);
    *info = 0;
    return R.launch_err();
  }
  const double eps = 2.220446049250313e-16, rhotol = eps * eps, omegatol = rhotol;
  R.copy(b, r);
  R.copy(r, rt);
  double rho_prev = 0.0, omega = 0.0, alpha = 0.0;
  for (int it = 0; it < maxiter; ++it) {
    *iters = it;
    if (R.norm(r) < atol) {
      *info = 0;
      return R.launch_err();
    }
    const double rho = R.dot(rt, r);
    if (std::fabs(rho) < rhotol) {
      *info = -10;
      return R.launch_err();
    }
    if (it > 0) {
      if (std::fabs(omega) < omegatol) {
        *info = -11;
        return R.launch_err();
      }
      const double beta = (rho / rho_prev) * (alpha / omega);
      R.axpy(-omega, v, p);            // p -= omega v
      R.scale(beta, p);                // p *= beta
      R.axpy(1.0, r, p);               // p += r
    } else {
      R.copy(r, p);
    }
    R.psolve(p, ph);
    R.matvec(ph, v);
    const double rv = R.dot(rt, v);
    if (rv == 0.0) {
      *info = -11;
      return R.launch_err();
    }
    alpha = rho / rv;
    R.axpy(-alpha, v, r);              // r -= alpha v
    R.copy(r, s);
    if (R.norm(s) < atol) {
      R.axpy(alpha, ph, x);
      *info = 0;
      *iters = it + 1;
      return R.launch_err();
    }
    R.psolve(s, sh);
    R.matvec(sh, t);
    omega = R.dot(t, s) / R.dot(t, t);
    R.axpy(alpha, ph, x);
    R.axpy(omega, sh, x);
    R.axpy(-omega, t, r);
    rho_prev = rho;
    if (R.err()) return R.err();
  }
  *info = maxiter;
  *iters = maxiter;
  return R.launch_err();
}

}  // namespace

int csr_matvec_run(long n, const long* rp, const int* ci, const double* va, const double* x, double* y,
                   cudaStream_t s) {
  if (n < 0) return set_error(PFGB_EINVAL, "negative size");
  if (n == 0) return PFGB_OK;
  k_csr_matvec<<<(unsigned)((n + KT - 1) / KT), KT, 0, s>>>(n, rp, ci, va, x, y);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(PFGB_ECUDA, std::string("csr matvec: ") + cudaGetErrorString(e));
  return PFGB_OK;
}

int csr_solve_run(int method, long n, const long* rp, const int* ci, const double* va, const double* invd,
                  const double* b, double* x, double tol, int maxiter, cudaStream_t s, pfgb_solve_out* out) {
  if (n <= 0) return set_error(PFGB_EINVAL, "the system must have at least one row");
  if (n > (1L << 31) - 1) return set_error(PFGB_EINVAL, "more rows than the kernels index");
  if (maxiter < 0) return set_error(PFGB_EINVAL, "maxiter must be >= 0");
  if (method != 0 && method != 1) return set_error(PFGB_EINVAL, "method must be 0 (cg) or 1 (bicgstab)");
  if (cudaMemsetAsync(x, 0, n * sizeof(double), s) != cudaSuccess)
    return set_error(PFGB_ECUDA, "clearing x failed");
  Run R(Csr{n, rp, ci, va}, invd, s);
  int info = 0, iters = 0;
  int rc = method == 0 ? cg(R, b, x, tol, maxiter, &info, &iters) : bicgstab(R, b, x, tol, maxiter, &info, &iters);
  if (rc) return rc;
  // the reference's residual: r = b - A x, ||r|| (interface.py:48-49)
  double* y = R.vec();
  double* r = R.vec();
  if (R.err()) return R.err();
  R.matvec(x, y);
  R.sub(b, y, r);
  const double rr = R.dot(r, r);
  const double bb = R.dot(b, b);
  if ((rc = R.launch_err())) return rc;
  out->info = info;
  out->iterations = iters;
  out->bnorm = std::sqrt(bb);
  out->res_sq = rr;
  return PFGB_OK;
}

}  // namespace pfgb
