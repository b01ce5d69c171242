"""Pressure projection on the GPU.

Same API and diagnostics as src/pyflow/solvers/pressure_solver.py:42-219:
``solve_pressure_poisson(state, dt, dx, dy, cfg, preconditioner=None,
rhs_override=None) -> (p, diagnostics)``.

* normal mode: RHS ``-div_c(u*)/max(dt,1e-14)`` made mean-free with ``b[0] = 0``,
  Jacobi-PCG on the pinned operator, ``p -= p[0]``, ``u -= dt grad_c p`` in
  place -- all in the fused kernels of ``pfgb_project``;
* manufactured mode (``rhs_override``): Dirichlet Laplacian with identity ring
  rows, CG without preconditioner, p written to the state, no correction.

``assemble_negative_laplacian`` builds the reference's sparse matrix (the same
CSR entries and values, src/pyflow/solvers/pressure_solver.py:15-40) for callers
of the operator interface; the time step itself only needs its diagonal
(through ``jacobi_preconditioner``), which the kernels apply analytically.
"""
from __future__ import annotations

import ctypes
import math

import torch

from .. import _capi
from .._device import ptr, require_cuda, stream_handle, to_device
from ..core.ghost_fields import interior_view
from ..linear_solvers.interface import solve
from ..linear_solvers.operators import PressureOperator
from ..linear_solvers.preconditioners import JacobiPreconditioner, jacobi_interior
from ._handle import instance_for
from .fields import device_fields


def assemble_negative_laplacian(nx: int, ny: int, dx: float, dy: float):
    """The reference's assembled matrix (pressure_solver.py:15-40) as SciPy CSR: an
    identity row on every boundary cell (the reference cell 0 included), and inside the
    5-point -Laplacian (centre 2/dx**2 + 2/dy**2, neighbours -1/dx**2 and -1/dy**2),
    columns sorted within each row as the reference's LIL-to-CSR conversion leaves them."""
    import numpy as np
    import scipy.sparse as sp
    N = nx * ny
    idx = np.arange(N).reshape(ny, nx)
    interior = np.zeros((ny, nx), dtype=bool)
    interior[1:-1, 1:-1] = True
    inner = idx[interior]
    ring = idx[~interior]
    cx, cy, cc = -1.0 / dx**2, -1.0 / dy**2, 2.0 / dx**2 + 2.0 / dy**2
    # per interior row the five columns in increasing order: -nx, -1, 0, +1, +nx
    cols = np.stack([inner - nx, inner - 1, inner, inner + 1, inner + nx], axis=1)
    vals = np.broadcast_to(np.array([cy, cx, cc, cx, cy]), cols.shape)
    rows = np.concatenate([np.repeat(inner, 5), ring])
    cols = np.concatenate([cols.ravel(), ring])
    vals = np.concatenate([vals.ravel(), np.ones(ring.size)])
    return sp.csr_matrix((vals, (rows, cols)), shape=(N, N))


def _xnorm(t: torch.Tensor) -> float:
    r = ctypes.c_double()
    t = t.reshape(-1).contiguous()
    _capi.check(_capi.load().pfgb_xdot(ptr(t), ptr(t), t.numel(), ctypes.byref(r), stream_handle()), "xdot")
    return math.sqrt(r.value)


def projection_params(nx, ny, dx, dy, lin_tol, lin_maxiter, jacobi: bool, interior: float) -> _capi.Params:
    P = _capi.Params()
    P.nx, P.ny, P.dx, P.dy = nx, ny, float(dx), float(dy)
    P.nu, P.cfl_target, P.cfl_growth = 0.0, 0.5, 1.05
    P.lin_tol, P.lin_maxiter = float(lin_tol), int(lin_maxiter)
    P.scheme = _capi.SCHEME_NONE
    P.enable_jacobi = 1 if jacobi else 0
    P.jacobi_interior = float(interior)
    P.has_lid, P.lid_velocity, P.precision = 0, 0.0, 0
    return P


def solve_pressure_poisson(state, dt, dx, dy, cfg, preconditioner=None, rhs_override=None):
    require_cuda()
    nx, ny = int(state.nx), int(state.ny)
    if rhs_override is not None:
        return _manufactured(state, dt, dx, dy, cfg, preconditioner, rhs_override)
    lin_tol = getattr(cfg, "lin_tol", 1e-10)
    lin_maxiter = getattr(cfg, "lin_maxiter", 400)
    if preconditioner is not None:
        if not isinstance(preconditioner, JacobiPreconditioner):
            raise TypeError("preconditioner must be a JacobiPreconditioner")
        jacobi, interior = True, preconditioner.interior
    elif getattr(cfg, "enable_jacobi_pc", True):
        jacobi, interior = True, jacobi_interior(dx, dy)
    else:
        jacobi, interior = False, 0.0
    P = projection_params(nx, ny, dx, dy, lin_tol, lin_maxiter, jacobi, interior)
    inst = instance_for(state, P, slot="_pfgb_project")
    out = _capi.StepOut()
    with device_fields(state) as (u, v, p):
        _capi.check(_capi.load().pfgb_project(inst.handle, ptr(u), ptr(v), ptr(p), nx + 2, float(dt),
                                              stream_handle(), out), "pfgb_project")
    diag = projection_diagnostics(out, lin_tol)
    p_int = interior_view(state.fields["p"])
    return (p_int.clone() if isinstance(p_int, torch.Tensor) else p_int.copy()), diag


def projection_diagnostics(out, lin_tol: float) -> dict:
    """The diagnostics dict of pressure_solver.py:190-218 from the raw sums."""
    info = int(out.cg_info)
    rnorm = math.sqrt(out.res_sq)
    bnorm = out.bnorm or 1.0
    converged = bool((info == 0) and (rnorm <= lin_tol * bnorm))
    rp_iters = info if info > 0 else 0
    if rp_iters == 0 and rnorm > lin_tol:
        rp_iters = 1
    div_before = math.sqrt(out.divstar_sq)
    div_norm = math.sqrt(out.divafter_sq)
    lin_res = math.sqrt(out.linres_sq)
    red = div_before / div_norm if div_norm not in (None, 0.0) else None
    return {
        "Rp_iterations": rp_iters,
        "Rp_residual": rnorm,
        "Rp_converged": converged,
        "Rp_method": "cg",
        "divergence_norm": div_norm,
        "lin_residual_norm": lin_res,
        "lin_residual_rel": lin_res / bnorm,
        "divergence_reduction_factor": red,
        "divergence_norm_initial": div_before,
        "divergence_norm_after_raw": div_norm,
        "divergence_norm_final": div_norm,
        "cg_true_iterations": int(out.cg_iterations),
    }


def _manufactured(state, dt, dx, dy, cfg, preconditioner, rhs_override):
    nx, ny = int(state.nx), int(state.ny)
    A = PressureOperator("laplacian_dirichlet", nx, ny, dx, dy)
    rhs, _ = to_device(rhs_override)
    rhs = rhs.reshape(-1).contiguous().clone()
    lin_tol = getattr(cfg, "lin_tol", 1e-10)
    lin_maxiter = getattr(cfg, "lin_maxiter", 500)
    kw = {"M": preconditioner} if preconditioner is not None else {}
    res = solve(A, rhs, method="cg", tol=lin_tol, maxiter=lin_maxiter, **kw)
    p = res.x.reshape(ny, nx)
    with device_fields(state) as (_, _, pf):
        interior_view(pf).copy_(p)
    # ||A p - rhs|| equals the solver's ||b - A x|| (p is x unshifted here)
    div_norm = res.residual_norm
    rhs_norm = _xnorm(rhs) or 1.0
    rp_iters = res.iterations
    if rp_iters == 0 and res.residual_norm > lin_tol:
        rp_iters = 1
    diag = {
        "Rp_iterations": rp_iters,
        "Rp_residual": res.residual_norm,
        "Rp_converged": res.converged,
        "Rp_method": "cg",
        "divergence_norm": div_norm,
        "lin_residual_norm": div_norm,
        "lin_residual_rel": div_norm / rhs_norm,
        "divergence_reduction_factor": None,
        "divergence_norm_initial": None,
        "divergence_norm_after_raw": None,
        "divergence_norm_final": div_norm,
        "cg_true_iterations": res.true_iterations,
    }
    return p.clone(), diag
