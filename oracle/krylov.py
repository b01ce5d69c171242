"""Restated Krylov solves over an assembled sparse matrix (test infrastructure only).

The reference's ``solve`` (src/pyflow/linear_solvers/interface.py:23-53) calls
``scipy.sparse.linalg.cg`` for method 'cg' and ``scipy.sparse.linalg.bicgstab``
otherwise (SciPy 1.13.1 pinned by the reference's pyproject.toml:20; SciPy is
not vendored), with x0 = 0 and rtol = tol, on a SciPy sparse matrix (dense
inputs converted to CSR).  Restated here:

* ``csr_matvec``: scipy's CSR product -- per row, the terms in storage order,
  ``acc = acc + a_jj * x[c_jj]`` with the product rounded before the sum;
* ``jacobi_inv``: preconditioners.py:18-21, ``invD = 1/diag(A)`` where non-zero;
* CG: ``oracle.cg.pcg``;
* ``bicgstab``: SciPy's published BiCGSTAB sequence, with a pluggable dot and
  norm (np.dot / np.linalg.norm as SciPy calls them, or exactly rounded):

      bnrm2 = ||b||;  atol = max(0, rtol*bnrm2);  if bnrm2 == 0: return b, 0
      rhotol = omegatol = eps**2;  r = b (copy);  rtilde = r (copy)
      for it in range(maxiter):
          if ||r|| < atol: return x, 0
          rho = rtilde.r;  if |rho| < rhotol: return x, -10
          if it > 0:
              if |omega| < omegatol: return x, -11
              beta = (rho/rho_prev)*(alpha/omega);  p -= omega*v;  p *= beta;  p += r
          else: p = r (copy)
          phat = M p;  v = A phat;  rv = rtilde.v;  if rv == 0: return x, -11
          alpha = rho/rv;  r -= alpha*v;  s = r (copy)
          if ||s|| < atol: x += alpha*phat; return x, 0
          shat = M s;  t = A shat;  omega = (t.s)/(t.t)
          x += alpha*phat;  x += omega*shat;  r -= omega*t;  rho_prev = rho
      return x, maxiter

  ``iterations`` counts the loop passes begun and not left at their first test
  (an exit on ||s|| inside a pass counts that pass).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def csr_matvec(indptr, indices, data, x):
    indptr = np.asarray(indptr, dtype=np.int64)
    n = indptr.size - 1
    lens = np.diff(indptr)
    acc = np.zeros(n)
    for k in range(int(lens.max()) if n else 0):
        rows = np.nonzero(lens > k)[0]
        jj = indptr[rows] + k
        acc[rows] = acc[rows] + data[jj] * x[indices[jj]]
    return acc


def jacobi_inv(diag):
    d = np.asarray(diag, dtype=np.float64)
    with np.errstate(divide="ignore"):
        return np.where(d != 0, 1.0 / d, 0.0)


@dataclass
class KrylovResult:
    x: np.ndarray
    info: int
    iterations: int


def bicgstab(matvec, psolve, b, rtol, maxiter, dot, norm) -> KrylovResult:
    b = np.asarray(b, dtype=np.float64)
    x = np.zeros_like(b)
    bnrm2 = norm(b)
    atol = max(0.0, float(rtol) * float(bnrm2))
    if bnrm2 == 0:
        return KrylovResult(b.copy(), 0, 0)
    eps = np.finfo(np.float64).eps
    rhotol = omegatol = eps ** 2
    r = b.copy()
    rtilde = r.copy()
    rho_prev = omega = alpha = None
    p = v = s = None
    for it in range(maxiter):
        if norm(r) < atol:
            return KrylovResult(x, 0, it)
        rho = np.float64(dot(rtilde, r))
        if np.abs(rho) < rhotol:
            return KrylovResult(x, -10, it)
        if it > 0:
            if np.abs(omega) < omegatol:
                return KrylovResult(x, -11, it)
            beta = (rho / rho_prev) * (alpha / omega)
            p -= omega * v
            p *= beta
            p += r
        else:
            s = np.empty_like(r)
            p = r.copy()
        phat = psolve(p)
        v = matvec(phat)
        rv = np.float64(dot(rtilde, v))
        if rv == 0:
            return KrylovResult(x, -11, it)
        alpha = rho / rv
        r -= alpha * v
        s[:] = r[:]
        if norm(s) < atol:
            x += alpha * phat
            return KrylovResult(x, 0, it + 1)
        shat = psolve(s)
        t = matvec(shat)
        omega = np.float64(dot(t, s)) / np.float64(dot(t, t))
        x += alpha * phat
        x += omega * shat
        r -= omega * t
        rho_prev = rho
    return KrylovResult(x, maxiter, maxiter)


def solve_csr(indptr, indices, data, b, method, tol, maxiter, inv_diag=None, red="exact"):
    """(x, info, true iterations, ||b - A x||) of the reference's solve on a CSR matrix."""
    from .cg import pcg
    from .step import _red
    R = _red(red)
    mv = lambda v: csr_matvec(indptr, indices, data, v)  # noqa: E731
    ps = (lambda v: inv_diag * v) if inv_diag is not None else (lambda v: v.copy())  # noqa: E731
    if method == "cg":
        res = pcg(mv, ps, b, tol, maxiter, R.dot, R.norm)
        x, info, its = res.x, res.info, res.iterations
    else:
        res = bicgstab(mv, ps, b, tol, maxiter, R.dot, R.norm)
        x, info, its = res.x, res.info, res.iterations
    r = np.asarray(b, dtype=np.float64) - mv(x)
    return x, info, its, R.norm(r)
