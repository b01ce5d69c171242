"""Jacobi preconditioners of the pressure solve and of assembled matrices.

Same contract as src/pyflow/linear_solvers/preconditioners.py:8-25
(``invD = 1/diag(A)`` where the diagonal is non-zero).  The reference builds it
from ``assemble_negative_laplacian`` (src/pyflow/solvers/pressure_solver.py:15-40),
whose diagonal is 1.0 on the boundary ring and 2/dx**2 + 2/dy**2 inside; the
GPU kernels apply that diagonal analytically, so this object only carries the
interior value, rounded exactly as the reference rounds it.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class JacobiPreconditioner:
    nx: int
    ny: int
    interior: float        # 1.0 / (2.0/dx**2 + 2.0/dy**2)

    @property
    def shape(self):
        n = self.nx * self.ny
        return (n, n)


def jacobi_interior(dx: float, dy: float) -> float:
    return 1.0 / (2.0 / dx**2 + 2.0 / dy**2)


def jacobi_preconditioner(A):
    """Jacobi preconditioner (src/pyflow/linear_solvers/preconditioners.py:8-25).

    For the pinned pressure operator: the diagonal of assemble_negative_laplacian,
    applied analytically by the stencil kernels (``JacobiPreconditioner``).  For an
    assembled matrix (SciPy sparse, dense, or ``CsrMatrix``): invD = 1/diag(A) where
    the diagonal is non-zero, 0 elsewhere, as a device vector
    (``DiagonalPreconditioner``) for the CSR solves."""
    from .operators import PressureOperator
    if isinstance(A, PressureOperator):
        if A.kind != "neg_laplacian_pinned":
            raise NotImplementedError("the stencil Jacobi applies the diagonal of assemble_negative_laplacian; "
                                      "assemble the operator's matrix for another diagonal")
        return JacobiPreconditioner(A.nx, A.ny, jacobi_interior(A.dx, A.dy))
    from .sparse import jacobi_of_matrix
    return jacobi_of_matrix(A)


def diag_matches_assembled(D: np.ndarray, nx: int, ny: int, dx: float, dy: float) -> bool:
    """True when a diagonal equals the one of assemble_negative_laplacian."""
    ref = np.ones((ny, nx))
    if nx > 2 and ny > 2:
        ref[1:-1, 1:-1] = 2.0 / dx**2 + 2.0 / dy**2
    return np.array_equal(np.asarray(D).reshape(ny, nx), ref)
