"""Linear-solve wrapper on the GPU.

Same API as src/pyflow/linear_solvers/interface.py:9-53:
``solve(A, b, method, tol, maxiter, **kwargs) -> LinearSolveResult``, x0 = 0,
``rtol = tol``, result fields (x, converged, iterations, residual_norm, method)
with the reference's semantics: ``iterations`` is scipy's ``info`` (0 when
converged, maxiter otherwise), ``residual_norm = ||b - A x||`` and
``converged = info == 0 and residual_norm <= tol*||b||``.  ``true_iterations``
adds the executed iteration count.

``A`` is a ``PressureOperator``; ``M`` (optional) a ``JacobiPreconditioner``.
The CG of scipy.sparse.linalg.cg (SciPy 1.13.1, as pinned by the reference) is
restated in the CUDA kernels with exactly rounded dot products.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Literal

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


def solve(A, b, method: Literal["cg", "bicgstab"] = "bicgstab", tol: float = 1e-8, maxiter: int = 500,
          **kwargs) -> LinearSolveResult:
    if not isinstance(A, PressureOperator):
        raise TypeError("the GPU solve takes a PressureOperator (matrix-free pressure operator)")
    if method != "cg":
        raise NotImplementedError("only method='cg' (the pressure solve's method) runs on the GPU")
    M = kwargs.pop("M", None)
    if kwargs:
        raise TypeError(f"unexpected arguments {sorted(kwargs)}")
    require_cuda()
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
