"""Linear-solve wrapper on the GPU.

Same API as src/pyflow/linear_solvers/interface.py:9-53:
``solve(A, b, method, tol, maxiter, **kwargs) -> LinearSolveResult``, x0 = 0,
``rtol = tol``, result fields (x, converged, iterations, residual_norm, method)
with the reference's semantics: ``iterations`` is scipy's ``info`` (0 when
converged, maxiter otherwise), ``residual_norm = ||b - A x||`` and
``converged = info == 0 and residual_norm <= tol*||b||``.  ``true_iterations``
adds the executed iteration count.

``A`` is either the matrix-free ``PressureOperator`` (with ``M`` its
``JacobiPreconditioner`` or none; method 'cg': the fused stencil kernels of the
time step's pressure solve) or an assembled matrix -- a SciPy sparse matrix, a
dense array (converted to CSR, as the reference converts it) or a ``CsrMatrix``
-- with ``M`` its ``jacobi_preconditioner`` or none, solved by CG or BiCGSTAB on
the device over the CSR matrix (``pfgb_csr_solve``).  scipy.sparse.linalg.cg and
.bicgstab (SciPy 1.13.1, as pinned by the reference) are restated in the CUDA
code with exactly rounded dot products.  A ``LinearOperator`` whose ``matvec`` is
Python code has no device form and is refused.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Literal

import numpy as np
import torch

from .. import _capi
from .._device import ptr, require_cuda, stream_handle, to_device
from .operators import PressureOperator
from .preconditioners import JacobiPreconditioner


@dataclass(slots=True)
class LinearSolveResult:
    x: object
    converged: bool
    iterations: int
    residual_norm: float
    method: str
    true_iterations: int = 0


def _is_matrix(A) -> bool:
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    from .sparse import CsrMatrix
    if isinstance(A, CsrMatrix) or sp.issparse(A):
        return True
    if isinstance(A, (spla.LinearOperator, PressureOperator)):
        return False
    return isinstance(A, (np.ndarray, list, tuple))


def _solve_matrix(A, b, method, tol, maxiter, M) -> LinearSolveResult:
    from .sparse import CsrMatrix, DiagonalPreconditioner, jacobi_of_matrix
    Acsr = CsrMatrix.from_any(A)
    bt, host = to_device(b)
    bt = bt.reshape(-1).contiguous()
    if bt.numel() != Acsr.shape[0]:
        raise ValueError("dimension mismatch")
    if M is not None and not isinstance(M, DiagonalPreconditioner):
        if _is_matrix(M):
            M = jacobi_of_matrix(M)
        else:
            raise TypeError("M must be the jacobi_preconditioner of an assembled matrix")
    if M is not None and M.inv_diag.numel() != Acsr.shape[0]:
        raise ValueError("preconditioner dimension mismatch")
    x = torch.empty_like(bt)
    out = _capi.SolveOut()
    # the reference runs CG for 'cg' and BiCGSTAB for any other name
    _capi.check(_capi.load().pfgb_csr_solve(0 if method == "cg" else 1, Acsr.shape[0], ptr(Acsr.indptr),
                                            ptr(Acsr.indices), ptr(Acsr.data),
                                            ptr(M.inv_diag) if M is not None else None, ptr(bt), ptr(x),
                                            float(tol), int(maxiter), stream_handle(), out), "csr_solve")
    info = out.info
    rnorm = math.sqrt(out.res_sq)
    bnorm = out.bnorm or 1.0
    converged = (info == 0) and (rnorm <= tol * bnorm)
    iterations = info if info > 0 else 0
    xo = x.cpu().numpy() if host else x
    return LinearSolveResult(x=xo, converged=converged, iterations=iterations, residual_norm=rnorm,
                             method=method, true_iterations=out.iterations)


def solve(A, b, method: Literal["cg", "bicgstab"] = "bicgstab", tol: float = 1e-8, maxiter: int = 500,
          **kwargs) -> LinearSolveResult:
    M = kwargs.pop("M", None)
    if kwargs:
        raise TypeError(f"unexpected arguments {sorted(kwargs)}")
    require_cuda()
    if _is_matrix(A):
        return _solve_matrix(A, b, method, tol, maxiter, M)
    if not isinstance(A, PressureOperator):
        raise TypeError("the GPU solve takes an assembled matrix (SciPy sparse, dense or CsrMatrix) or a "
                        "PressureOperator; a LinearOperator's Python matvec has no device form")
    if method != "cg":
        raise NotImplementedError("BiCGSTAB runs on assembled matrices: pass the operator's matrix "
                                  "(e.g. assemble_negative_laplacian) instead of the matrix-free operator")
    bt, host = to_device(b)
    bt = bt.reshape(-1).contiguous()
    if bt.numel() != A.shape[0]:
        raise ValueError("dimension mismatch")
    precond, interior = 0, 0.0
    if M is not None:
        if not isinstance(M, JacobiPreconditioner) or (M.nx, M.ny) != (A.nx, A.ny):
            raise TypeError("M must be the JacobiPreconditioner of A")
        precond, interior = 1, M.interior
    x = torch.empty_like(bt)
    out = _capi.SolveOut()
    _capi.check(_capi.load().pfgb_cg_solve(A.op, ptr(bt), ptr(x), A.nx, A.ny, A.dx, A.dy, precond, interior,
                                           float(tol), int(maxiter), stream_handle(), out), "cg_solve")
    info = out.info
    rnorm = math.sqrt(out.res_sq)
    bnorm = out.bnorm or 1.0
    converged = (info == 0) and (rnorm <= tol * bnorm)
    iterations = info if info > 0 else 0
    xo = x.cpu().numpy() if host else x
    return LinearSolveResult(x=xo, converged=converged, iterations=iterations, residual_norm=rnorm,
                             method=method, true_iterations=out.iterations)
