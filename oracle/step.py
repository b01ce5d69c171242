"""Restated projection step of the reference (test infrastructure only).

Follows, in order and with the same rounding:

* ``step``                   src/pyflow/solvers/solver.py:15-193
* ``solve_pressure_poisson`` src/pyflow/solvers/pressure_solver.py:42-219
* ``solve``                  src/pyflow/linear_solvers/interface.py:23-53
* ``SimulationDriver.run``   src/pyflow/drivers/simulation_driver.py:58-110
* ``ResidualManager``        src/pyflow/residuals/manager.py:2-16

``red`` selects the reductions (``oracle.xsum.Reductions``): ``"numpy"`` is
the reference's own (np.dot / np.linalg.norm / np.mean / np.sum) and
``"exact"`` the exactly rounded twin reproduced by the CUDA path.

Printing, JSONL logging and emergency checkpoints of the reference are host
side effects outside the array path and are not restated.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Any

import numpy as np

from . import ops
from .cg import pcg
from .xsum import Reductions


@dataclass
class State:
    nx: int
    ny: int
    fields: dict
    meta: dict = field(default_factory=dict)


def allocate_state(nx, ny):
    shape = (ny + 2, nx + 2)
    return State(nx, ny, {k: np.zeros(shape) for k in ("u", "v", "p")})


def interior(a):
    return a[1:-1, 1:-1]


class ResidualManager:
    """Stub tracker of the reference: the Ru series seeded with 1.0."""

    def __init__(self):
        self.ru = [1.0]

    def add(self, name, value):
        if name == "Ru":
            self.ru.append(value)


def _red(red):
    return red if isinstance(red, Reductions) else Reductions(red)


def neg_laplacian_matrix(nx, ny, dx, dy):
    """Sparse -lap_c (Neumann, coherent 5-point): the matrix of the reference's operator rows k != 0."""
    import scipy.sparse as sp
    N = nx * ny
    idx = np.arange(N).reshape(ny, nx)
    cx, cy = 1.0 / dx**2, 1.0 / dy**2
    rows, cols, vals = [], [], []
    diag = np.zeros((ny, nx))
    for (a, b, c) in ((idx[:, :-1], idx[:, 1:], cx), (idx[:-1, :], idx[1:, :], cy)):
        a, b = a.ravel(), b.ravel()
        rows += [a, b]
        cols += [b, a]
        vals += [np.full(a.size, -c), np.full(a.size, -c)]
        np.add.at(diag.reshape(-1), a, c)
        np.add.at(diag.reshape(-1), b, c)
    rows.append(idx.ravel())
    cols.append(idx.ravel())
    vals.append(diag.reshape(-1))
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))


def converged_pressure(b, nx, ny, dx, dy):
    """The exact solution of the reference's pinned system A x = b (x[0] = b[0] = 0).

    Rows k != 0 of A restricted to the unknowns k != 0 are SPD; a sparse direct
    solve gives x to binary64 accuracy.  This is the converged FP64 oracle of the
    mixed-precision path (the reference's own CG stops at lin_maxiter unconverged).
    """
    L, lu = _pinned_factor(nx, ny, float(dx), float(dy))
    x = np.zeros(nx * ny)
    x[0] = b[0]
    rhs = b[1:] - L[1:, :1].toarray().ravel() * x[0]
    x[1:] = lu.solve(rhs)
    return x


_FACTORS = {}


def _pinned_factor(nx, ny, dx, dy):
    """Sparse LU of -lap_c restricted to the unknowns k != 0, kept per grid and
    spacing (the matrix is the same at every step of a cavity; at 1024 x 1024
    the factorisation takes seconds and each solve a fraction of one)."""
    key = (nx, ny, dx, dy)
    if key not in _FACTORS:
        import scipy.sparse.linalg as spla
        L = neg_laplacian_matrix(nx, ny, dx, dy).tocsc()
        if len(_FACTORS) >= 4:
            _FACTORS.clear()
        _FACTORS[key] = (L, spla.splu(L[1:, 1:].tocsc()))
    return _FACTORS[key]


def solve_pressure_poisson(state, dt, dx, dy, cfg, red="exact", rhs_override=None, extra=None):
    """Restatement of pressure_solver.py:42-219 (normal and manufactured modes).

    ``cfg.oracle_pressure == "converged"`` replaces the CG by the exact solution
    of the same system (the converged FP64 oracle of the mixed-precision path).
    """
    red = _red(red)
    ui = interior(state.fields["u"])
    vi = interior(state.fields["v"])
    ny, nx = ui.shape
    N = nx * ny
    if rhs_override is not None:
        bmask = np.zeros((ny, nx), dtype=bool)
        bmask[0, :] = bmask[-1, :] = True
        bmask[:, 0] = bmask[:, -1] = True
        b_idx = np.flatnonzero(bmask.reshape(-1))

        def matvec(x):
            out = ops.laplacian_coherent(x.reshape(ny, nx), dx, dy).reshape(-1)
            out[b_idx] = x[b_idx]
            return out

        rhs = np.copy(rhs_override).reshape(-1).astype(np.float64)
        lin_tol = getattr(cfg, "lin_tol", 1e-10)
        lin_maxiter = getattr(cfg, "lin_maxiter", 500)
        res = pcg(matvec, lambda r: r, rhs, lin_tol, lin_maxiter, red.dot, red.norm)
        info, x = res.info, res.x
        r = rhs - matvec(x)
        rnorm = red.norm(r)
        bnorm = red.norm(rhs) or 1.0
        p = x.reshape(ny, nx)
        interior(state.fields["p"])[:] = p
        div_norm = red.norm(matvec(p.reshape(-1)) - rhs)
        div_before = None
        div_after_raw = None
    else:
        def matvec(x):
            return ops.neg_laplacian_pinned(x, nx, ny, dx, dy)

        div_u = ops.divergence_coherent(ui, vi, dx, dy)
        div_before = red.norm(div_u)
        rhs = (-div_u / max(dt, 1e-14)).reshape(-1)
        rhs_mean = red.mean(rhs)
        rhs -= rhs_mean
        rhs[0] = 0.0
        lin_tol = getattr(cfg, "lin_tol", 1e-10)
        lin_maxiter = getattr(cfg, "lin_maxiter", 400)
        if getattr(cfg, "enable_jacobi_pc", True):
            invd = ops.jacobi_inv_diag(nx, ny, dx, dy)
            psolve = lambda r: invd * r  # noqa: E731
        else:
            psolve = lambda r: r  # noqa: E731
        if getattr(cfg, "oracle_pressure", "cg") == "converged":
            from .cg import CGResult
            res = CGResult(converged_pressure(rhs, nx, ny, dx, dy), 0, 0, [])
        else:
            res = pcg(matvec, psolve, rhs, lin_tol, lin_maxiter, red.dot, red.norm)
        info, x = res.info, res.x
        r = rhs - matvec(x)
        rnorm = red.norm(r)
        bnorm = red.norm(rhs) or 1.0
        p = x.reshape(ny, nx)
        p -= p.flat[0]
        interior(state.fields["p"])[:] = p
        p_field = interior(state.fields["p"])
        gx, gy = ops.gradient_coherent(p_field, dx, dy)
        ui[:] -= dt * gx
        vi[:] -= dt * gy
        div_after = ops.divergence_coherent(ui, vi, dx, dy)
        div_after_raw = red.norm(div_after)
        div_norm = red.norm(div_after)
    converged = bool((info == 0) and (rnorm <= lin_tol * bnorm))
    iterations = info if info > 0 else 0
    pvec = p.reshape(-1)
    lin_residual_norm = red.norm(matvec(pvec) - rhs)
    rhs_norm = red.norm(rhs) or 1.0
    lin_residual_rel = lin_residual_norm / rhs_norm
    rp_iters = iterations
    if rp_iters == 0 and rnorm > lin_tol:
        rp_iters = 1
    red_factor = None
    if div_before is not None and div_norm not in (None, 0.0):
        red_factor = div_before / div_norm
    diag = {
        "Rp_iterations": rp_iters,
        "Rp_residual": rnorm,
        "Rp_converged": converged,
        "Rp_method": "cg",
        "divergence_norm": div_norm,
        "lin_residual_norm": lin_residual_norm,
        "lin_residual_rel": lin_residual_rel,
        "divergence_reduction_factor": red_factor,
        "divergence_norm_initial": div_before,
        "divergence_norm_after_raw": div_after_raw,
        "divergence_norm_final": div_norm,
    }
    if extra is not None:
        extra["cg_true_iterations"] = res.iterations
        extra["cg_info"] = info
    return p, diag


def step(config, state, tracker, iteration, red="exact", extra=None):
    """Restatement of solver.py:15-193 (array path, no printing/logging)."""
    red = _red(red)
    ui_full = interior(state.fields["u"])
    vi_full = interior(state.fields["v"])
    ny, nx = ui_full.shape
    lx = getattr(config, "lx", float(nx - 1))
    ly = getattr(config, "ly", float(ny - 1))
    dx = lx / max(nx - 1, 1)
    dy = ly / max(ny - 1, 1)
    umax = float(np.max(np.abs(ui_full))) + 1e-12
    vmax = float(np.max(np.abs(vi_full))) + 1e-12
    cfl_target = getattr(config, "cfl_target", 0.5)
    cfl_growth = getattr(config, "cfl_growth", 1.05)
    Re = float(getattr(config, "Re", 100.0))
    nu = 1.0 / Re
    dt_prev = float(state.meta.get("dt_prev", 1e-2))
    dt_cfl = min(cfl_target * dx / umax, cfl_target * dy / vmax)
    dt_diff = 0.25 * min(dx * dx, dy * dy) / max(nu, 1e-12)
    dt_candidate = min(dt_cfl, dt_diff)
    dt = dt_prev * cfl_growth if dt_candidate > dt_prev * cfl_growth else dt_candidate
    div_before = red.norm(ops.divergence_central(ui_full, vi_full, 1.0, 1.0))
    hist = state.meta.get("divergence_history", [])
    hist.append(div_before)
    hist = hist[-5:]
    state.meta["divergence_history"] = hist
    safeguard = False
    if len(hist) >= 3:
        a, b, c = hist[-3], hist[-2], hist[-1]
        if a > 0 and b > a * 1.01 and c > b * 1.01:
            dt *= 0.5
            safeguard = True
    state.meta["dt_prev"] = dt
    state.meta["dx"] = dx
    state.meta["dy"] = dy
    state.meta["nu"] = nu
    current_cfl = max(umax * dt / dx, vmax * dt / dy)
    u_old = ui_full.copy()
    v_old = vi_full.copy()
    if getattr(config, "disable_advection", False):
        u_star, v_star = u_old.copy(), v_old.copy()
    else:
        scheme = getattr(config, "advection_scheme", "upwind")
        adv = ops.advect_quick if scheme == "quick" else ops.advect_upwind
        u_star = u_old - dt * adv(u_old, v_old, u_old, dx, dy)
        v_star = v_old - dt * adv(u_old, v_old, v_old, dx, dy)
    ui_full[:, :] = u_star
    vi_full[:, :] = v_star
    lid = getattr(config, "lid_velocity", None)
    sub = {} if extra is not None else None
    _, pdiag = solve_pressure_poisson(state, dt, dx, dy, config, red=red, extra=sub)
    state.meta["prev_div_norm"] = pdiag.get("divergence_norm", 0.0)
    if lid is not None:
        state.fields["u"][-2, 1:-1] = lid

    def l2(delta):
        d = delta.ravel()
        return float(math.sqrt(red.sum(d * d)) / max(1, d.size))

    Ru = l2(ui_full - u_old)
    Rv = l2(vi_full - v_old)
    continuity = float(red.norm(ops.divergence_central(ui_full, vi_full, 1.0, 1.0)) / max(1.0, nx * ny))
    nan_detected = not all(np.isfinite(interior(state.fields[k])).all() for k in ("u", "v", "p"))
    tracker.add("Ru", Ru)
    residuals = {"Ru": Ru, "Rv": Rv, "Rp": 0.0, "continuity": continuity}
    ru0 = tracker.ru[0]
    drop = 0.0
    if tracker.ru and Ru > 0 and ru0 > 0:
        drop = math.log10(ru0) - math.log10(Ru)
    diag = {
        "iteration": iteration,
        "dt": dt,
        "CFL": current_cfl,
        "plateau_Ru": False,
        "max_residual": max(residuals.values()),
        "residual_drop_Ru_orders": max(0.0, drop),
        "nu": nu,
        "Rp_iterations": pdiag.get("Rp_iterations", 0),
        "Rp_residual": pdiag.get("Rp_residual", 0.0),
        "Rp_converged": pdiag.get("Rp_converged", False),
        "Rp_method": pdiag.get("Rp_method", "cg"),
        "divergence_norm": pdiag.get("divergence_norm", 0.0),
        "nan_detected": nan_detected,
    }
    if getattr(config, "seed", None) is not None:
        diag["seed"] = config.seed
    if extra is not None:
        extra.update(sub)
        extra["safeguard"] = safeguard
        extra["div_baseline"] = div_before
        extra["pressure_diag"] = pdiag
    return state, residuals, diag


def run(config, state=None, max_steps=1, start_iteration=0, red="exact", tracker=None, extras=None):
    """Restatement of SimulationDriver.run: yields (state, residuals, diagnostics)."""
    tracker = tracker or ResidualManager()
    it = start_iteration
    if state is None:
        state = allocate_state(config.nx, config.ny)
    while max_steps is None or it < max_steps:
        ex = {} if extras is not None else None
        state, res, diag = step(config, state, tracker, it, red=red, extra=ex)
        ui = interior(state.fields["u"])
        nyi, nxi = ui.shape
        ly = getattr(config, "ly", float(nyi - 1))
        ys = [j * (ly / (nyi - 1)) for j in range(nyi)] if nyi > 1 else [0.0]
        diag["u_centerline"] = [ys, ui[:, nxi // 2].tolist()]
        if extras is not None:
            extras.append(ex)
        yield state, res, diag
        it += 1
