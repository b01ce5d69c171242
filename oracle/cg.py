"""Restated preconditioned CG (test infrastructure only).

The reference calls ``scipy.sparse.linalg.cg`` (SciPy, pinned 1.13.1 in the
reference's pyproject.toml:20; SciPy is not vendored) through
``solve`` (src/pyflow/linear_solvers/interface.py:23-53) with ``x0 = 0``,
``rtol = lin_tol`` and ``M`` = the Jacobi operator.  SciPy's published
sequence, restated here with a pluggable dot product:

    bnrm2 = ||b||;  atol = max(0, rtol*bnrm2);  if bnrm2 == 0: return b, 0
    r = b (copy);  for it in range(maxiter):
        if ||r|| < atol: return x, 0
        z = M r;  rho = r.z
        p = z (first)  or  p = p*beta + z,  beta = rho/rho_prev
        q = A p;  alpha = rho / (p.q)
        x += alpha*p;  r -= alpha*q;  rho_prev = rho
    return x, maxiter

``x += alpha*p`` rounds ``alpha*p`` first and then the sum (NumPy in-place
ufuncs, no contraction); ``p *= beta; p += z`` likewise.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class CGResult:
    x: np.ndarray
    info: int          # 0 converged, maxiter when the loop ran out
    iterations: int    # true number of iterations executed
    rr_history: list   # ||r||^2 seen at each convergence check


def pcg(matvec, psolve, b, rtol, maxiter, dot, norm, callback=None) -> CGResult:
    b = np.asarray(b, dtype=np.float64)
    x = np.zeros_like(b)
    bnrm2 = norm(b)
    atol = max(0.0, float(rtol) * float(bnrm2))
    if bnrm2 == 0:
        return CGResult(b, 0, 0, [])
    r = b.copy()
    rho_prev = None
    p = None
    hist = []
    for it in range(maxiter):
        rn = norm(r)
        hist.append(rn)
        if rn < atol:
            return CGResult(x, 0, it, hist)
        z = psolve(r)
        rho = np.float64(dot(r, z))
        if it > 0:
            beta = rho / rho_prev
            p *= beta
            p += z
        else:
            p = np.empty_like(r)
            p[:] = z[:]
        q = matvec(p)
        alpha = rho / np.float64(dot(p, q))
        x += alpha * p
        r -= alpha * q
        rho_prev = rho
        if callback is not None:
            callback(x)
    return CGResult(x, maxiter, maxiter, hist)
