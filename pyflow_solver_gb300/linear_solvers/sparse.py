"""Assembled sparse matrices and their Jacobi preconditioner on the GPU.

``CsrMatrix`` holds an n x n CSR matrix in device memory (row pointers int64,
column indices int32, values float64) -- the device form of the SciPy sparse
matrices that the reference passes to ``solve`` (src/pyflow/linear_solvers/
interface.py:23-53, converting dense inputs to CSR the same way).  Its product
(``matvec``, ``@``) sums each row's terms in storage order, as scipy's CSR
product does.  ``DiagonalPreconditioner`` is ``jacobi_preconditioner`` of such
a matrix (src/pyflow/linear_solvers/preconditioners.py:8-25): the vector
``invD = 1/diag(A)`` where the diagonal is non-zero, 0 elsewhere, formed from
the matrix's diagonal exactly as the reference forms it.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from .. import _capi
from .._device import ptr, require_cuda, stream_handle, to_device


class CsrMatrix:
    def __init__(self, indptr, indices, data, shape):
        require_cuda()
        n, m = int(shape[0]), int(shape[1])
        if n != m:
            raise ValueError("the Krylov solves take a square matrix")
        self.shape = (n, m)
        self.dtype = torch.float64
        self.indptr = torch.as_tensor(np.asarray(indptr, dtype=np.int64)).to("cuda")
        self.indices = torch.as_tensor(np.asarray(indices, dtype=np.int32)).to("cuda")
        self.data = torch.as_tensor(np.asarray(data, dtype=np.float64)).to("cuda")
        if self.indptr.numel() != n + 1:
            raise ValueError("indptr must have n + 1 entries")
        self._diag = None

    @classmethod
    def from_any(cls, A) -> CsrMatrix:
        """A SciPy sparse matrix (any format), a dense array, or a CsrMatrix."""
        if isinstance(A, CsrMatrix):
            return A
        import scipy.sparse as sp
        M = A.tocsr() if sp.issparse(A) else sp.csr_matrix(np.asarray(A, dtype=np.float64))
        M = M.astype(np.float64)
        obj = cls(M.indptr, M.indices, M.data, M.shape)
        obj._diag = np.asarray(M.diagonal(), dtype=np.float64).ravel()
        return obj

    def diagonal(self) -> np.ndarray:
        if self._diag is None:
            ip = self.indptr.cpu().numpy()
            ix = self.indices.cpu().numpy()
            va = self.data.cpu().numpy()
            d = np.zeros(self.shape[0])
            rows = np.repeat(np.arange(self.shape[0]), np.diff(ip))
            on = rows == ix
            np.add.at(d, rows[on], va[on])
            self._diag = d
        return self._diag

    def matvec(self, x):
        xt, host = to_device(x)
        xt = xt.reshape(-1).contiguous()
        if xt.numel() != self.shape[1]:
            raise ValueError("dimension mismatch")
        y = torch.empty_like(xt)
        _capi.check(_capi.load().pfgb_csr_matvec(self.shape[0], ptr(self.indptr), ptr(self.indices), ptr(self.data),
                                                  ptr(xt), ptr(y), stream_handle()), "csr_matvec")
        return y.cpu().numpy() if host else y

    def __matmul__(self, x):
        return self.matvec(x)


@dataclass
class DiagonalPreconditioner:
    inv_diag: torch.Tensor      # 1/diag(A) where non-zero, 0 elsewhere (device, float64)

    @property
    def shape(self):
        n = self.inv_diag.numel()
        return (n, n)

    def matvec(self, x):
        xt, host = to_device(x)
        y = self.inv_diag * xt.reshape(-1)
        return y.cpu().numpy() if host else y


def jacobi_of_matrix(A) -> DiagonalPreconditioner:
    D = CsrMatrix.from_any(A).diagonal() if not hasattr(A, "diagonal") or isinstance(A, CsrMatrix) \
        else np.asarray(A.diagonal(), dtype=np.float64).ravel()
    with np.errstate(divide="ignore"):
        inv = np.where(D != 0, 1.0 / D, 0.0)
    return DiagonalPreconditioner(torch.from_numpy(np.ascontiguousarray(inv)).to("cuda"))


__all__ = ["CsrMatrix", "DiagonalPreconditioner", "jacobi_of_matrix"]
