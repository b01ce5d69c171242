"""GPU linear operators of the pressure solve (matrix-free, binary64).

``PressureOperator(kind, nx, ny, dx, dy)`` is the device counterpart of the
reference's ``scipy.sparse.linalg.LinearOperator`` subclasses:

* ``"neg_laplacian_pinned"``  _NegLaplacianPinned, src/pyflow/solvers/pressure_solver.py:97-105
  (A x = -lap_c(x) with row 0 replaced by the identity: non-symmetric)
* ``"laplacian_dirichlet"``   _PosLaplacianDirichlet, src/pyflow/solvers/pressure_solver.py:69-77
  (A x = lap_c(x) with identity rows on the boundary ring)

Vectors are flattened row-major (k = j*nx + i) float64 CUDA tensors.
"""
from __future__ import annotations

import torch

from .. import _capi
from .._device import ptr, require_cuda, stream_handle, to_device

KINDS = {"neg_laplacian_pinned": _capi.OP_NEG_LAPLACIAN_PINNED,
         "laplacian_dirichlet": _capi.OP_LAPLACIAN_DIRICHLET}


class PressureOperator:
    def __init__(self, kind: str, nx: int, ny: int, dx: float, dy: float):
        if kind not in KINDS:
            raise ValueError(f"unknown operator kind {kind!r}")
        if nx < 2 or ny < 2:
            raise ValueError("nx and ny must be >= 2")
        self.kind, self.op = kind, KINDS[kind]
        self.nx, self.ny, self.dx, self.dy = int(nx), int(ny), float(dx), float(dy)
        self.shape = (self.nx * self.ny, self.nx * self.ny)
        self.dtype = torch.float64

    def matvec(self, x):
        require_cuda()
        xt, host = to_device(x)
        xt = xt.reshape(-1).contiguous()
        if xt.numel() != self.shape[1]:
            raise ValueError("dimension mismatch")
        y = torch.empty_like(xt)
        _capi.check(_capi.load().pfgb_apply_operator(self.op, ptr(xt), ptr(y), self.nx, self.ny, self.dx, self.dy,
                                                      stream_handle()), "apply_operator")
        return y.cpu().numpy() if host else y

    def __matmul__(self, x):
        return self.matvec(x)
