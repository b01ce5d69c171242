"""The projection time step on the GPU.

Same signature, dict keys and ``state.meta`` updates as
src/pyflow/solvers/solver.py:15-193:
``step(config, state, tracker, iteration) -> (state, residuals, diagnostics)``.
The config is read through ``getattr`` with the reference's defaults.  All
array work of the step -- max|u|, the central divergence norm, dt/CFL and the
divergence-trend safeguard, the QUICK/upwind predictor, the pressure RHS, the
Jacobi-PCG pressure solve, the pinned correction, the lid and the residual
reductions -- runs in one enqueued kernel sequence of libpfgb.so; the host
receives one record of scalars and forms the dicts exactly as the reference.

``config.precision = "mixed"`` selects the mixed-precision form: the pressure
system is solved to ``||b - A x|| <= lin_tol ||b||`` by binary64 iterative
refinement around a binary32 multigrid-preconditioned CG (``mixed_tol_inner``,
``mixed_max_outer``, ``mixed_max_inner``); everything else stays binary64.  The
refinement starts from the state's previous pressure (``mixed_warm_start``,
default True; it falls back to zero when that guess is worse than zero), so the
same stopping test is met with fewer multigrid cycles on a slowly changing flow.

Host side effects as in the reference (solver.py:170-192): with
``config.log_path`` or ``config.log_stream``, one JSON-lines step record per
step, and on a NaN an error record and an emergency ``*_FAIL_NAN`` checkpoint
(``logging.structured.log_step``).  The ``print`` output of the diagnostic mode
is limited to its scalar lines.
"""
from __future__ import annotations

import math
from typing import Any

from .. import _capi
from .._device import ptr, require_cuda, stream_handle
from ..linear_solvers.preconditioners import jacobi_interior
from ..logging.structured import log_step
from ._handle import instance_for
from .fields import device_fields


def step_params(config, nx: int, ny: int):
    lx = getattr(config, "lx", float(nx - 1))
    ly = getattr(config, "ly", float(ny - 1))
    dx = lx / max(nx - 1, 1)
    dy = ly / max(ny - 1, 1)
    Re = float(getattr(config, "Re", 100.0))
    nu = 1.0 / Re
    P = _capi.Params()
    P.nx, P.ny, P.dx, P.dy, P.nu = nx, ny, dx, dy, nu
    P.cfl_target = float(getattr(config, "cfl_target", 0.5))
    P.cfl_growth = float(getattr(config, "cfl_growth", 1.05))
    P.lin_tol = float(getattr(config, "lin_tol", 1e-10))
    P.lin_maxiter = int(getattr(config, "lin_maxiter", 400))
    if getattr(config, "disable_advection", False):
        P.scheme = _capi.SCHEME_NONE
    else:
        P.scheme = _capi.SCHEME_QUICK if getattr(config, "advection_scheme", "upwind") == "quick" else _capi.SCHEME_UPWIND
    P.enable_jacobi = 1 if getattr(config, "enable_jacobi_pc", True) else 0
    P.jacobi_interior = jacobi_interior(dx, dy) if (nx > 2 and ny > 2) else 1.0
    lid = getattr(config, "lid_velocity", None)
    P.has_lid = 0 if lid is None else 1
    P.lid_velocity = 0.0 if lid is None else float(lid)
    prec = getattr(config, "precision", "fp64")
    if prec not in ("fp64", "mixed"):
        raise ValueError(f"precision must be 'fp64' or 'mixed', not {prec!r}")
    P.precision = 1 if prec == "mixed" else 0
    if P.precision == 1:
        P.mixed_tol_outer = float(getattr(config, "mixed_tol_outer", 0.0))
        P.mixed_tol_inner = float(getattr(config, "mixed_tol_inner", 1e-5))
        P.mixed_max_outer = int(getattr(config, "mixed_max_outer", 8))
        P.mixed_max_inner = int(getattr(config, "mixed_max_inner", 50))
        P.mixed_cold_start = 0 if getattr(config, "mixed_warm_start", True) else 1
    return P, dx, dy, nu


def prepare(config, state, iteration: int):
    """Parameters and per-step inputs of one instance (reads state.meta, not modified)."""
    nx, ny = int(state.nx), int(state.ny)
    P, dx, dy, nu = step_params(config, nx, ny)
    sin = _capi.StepIn()
    sin.dt_prev = float(state.meta.get("dt_prev", 1e-2))
    tail = [float(h) for h in state.meta.get("divergence_history", [])[-5:]]
    for k, h in enumerate(tail):
        sin.hist[k] = h
    sin.hist_len = len(tail)
    sin.iteration = int(iteration)
    return P, sin, (dx, dy, nu)


def finish(config, state, tracker, iteration: int, P, geo, out):
    """Form the reference's residual / diagnostic dicts and state.meta from a step record."""
    dx, dy, nu = geo
    nx, ny = int(state.nx), int(state.ny)
    diagnostics_enabled = getattr(config, "diagnostics", True)
    dt = out.dt
    hist = state.meta.get("divergence_history", [])
    hist.append(out.div_before)
    hist = hist[-5:]
    state.meta["divergence_history"] = hist
    if out.safeguard and diagnostics_enabled:
        a, b, c = hist[-3], hist[-2], hist[-1]
        print(f"[Step {iteration}] dt safeguard triggered (divergence rising {a:.3g}->{b:.3g}->{c:.3g}); new dt={dt:.3g}")
    state.meta["dt_prev"] = dt
    state.meta["dx"] = dx
    state.meta["dy"] = dy
    state.meta["nu"] = nu
    current_cfl = out.cfl
    if diagnostics_enabled:
        print(f"[Step {iteration}] dt={dt:.3g}, umax={out.umax:.3g}, vmax={out.vmax:.3g}, CFL={current_cfl:.3g}")
        print(f"[Step {iteration}] Initial divergence norm: {out.div_before:.3g}")
    lin_tol = P.lin_tol
    info = int(out.cg_info)
    rnorm = math.sqrt(out.res_sq)
    bnorm = out.bnorm or 1.0
    rp_converged = bool((info == 0) and (rnorm <= lin_tol * bnorm))
    rp_iters = info if info > 0 else 0
    if rp_iters == 0 and rnorm > lin_tol:
        rp_iters = 1
    divergence_norm = math.sqrt(out.divafter_sq)
    state.meta["prev_div_norm"] = divergence_norm
    N = nx * ny
    Ru = float(math.sqrt(out.ru_sq) / max(1, N))
    Rv = float(math.sqrt(out.rv_sq) / max(1, N))
    Rp = 0.0
    continuity = float(math.sqrt(out.cont_sq) / max(1.0, nx * ny))
    nan_detected = bool(out.nan_detected)
    if diagnostics_enabled:
        print(f"[Step {iteration}] Pressure solve: iterations={rp_iters}, residual={rnorm:.3g}, converged={rp_converged}")
        print(f"[Step {iteration}] Residuals: Ru={Ru:.3g}, Rv={Rv:.3g}, continuity={continuity:.3g}")
    tracker.add("Ru", Ru)
    tracker.add("Rv", Rv)
    tracker.add("Rp", Rp)
    tracker.add("continuity", continuity)
    tracker.add("Rp_iterations", rp_iters)
    tracker.add("Rp_residual", rnorm)
    residuals = {"Ru": Ru, "Rv": Rv, "Rp": Rp, "continuity": continuity}
    series = getattr(tracker, "series", {})
    ru_series = series["Ru"].values if "Ru" in series else []
    drop = 0.0
    if "Ru" in series and ru_series and residuals["Ru"] > 0 and ru_series[0] > 0:
        drop = math.log10(ru_series[0]) - math.log10(residuals["Ru"])
    diagnostics = {
        "iteration": iteration,
        "dt": dt,
        "CFL": current_cfl,
        "plateau_Ru": tracker.plateau_detect("Ru", window=10, threshold=-0.005),
        "max_residual": max(residuals.values()),
        "residual_drop_Ru_orders": max(0.0, drop),
        "nu": nu,
        "Rp_iterations": rp_iters,
        "Rp_residual": rnorm,
        "Rp_converged": rp_converged,
        "Rp_method": "cg",
        "divergence_norm": divergence_norm,
        "nan_detected": nan_detected,
        "cg_iterations": int(out.cg_iterations),
    }
    if P.precision == 1:
        diagnostics["refine_passes"] = int(out.refine_passes)
    if getattr(config, "seed", None) is not None:
        diagnostics["seed"] = config.seed
    if getattr(config, "assert_invariants", False):
        assert continuity <= max(1e3, divergence_norm * 10)
        p0 = float(state.fields["p"][1, 1])
        assert abs(p0) < 1e-10, "Invariant failed: reference pressure cell not ~0"
    log_step(config, state, iteration, dt, current_cfl, Ru, Rv, continuity, rp_iters, nan_detected, diagnostics)
    return residuals, diagnostics


def step(config, state, tracker, iteration: int) -> tuple[Any, dict[str, float], dict[str, Any]]:
    require_cuda()
    nx, ny = int(state.nx), int(state.ny)
    P, sin, geo = prepare(config, state, iteration)
    if getattr(config, "diagnostics", True):
        print(f"[Step {iteration}] Grid: nx={nx}, ny={ny}, dx={geo[0]:.4g}, dy={geo[1]:.4g}, "
              f"Re={getattr(config, 'Re', 100.0)}")
    inst = instance_for(state, P)
    out = _capi.StepOut()
    with device_fields(state) as (u, v, p):
        _capi.check(_capi.load().pfgb_step(inst.handle, ptr(u), ptr(v), ptr(p), nx + 2, sin, stream_handle(), out),
                    "pfgb_step")
    residuals, diagnostics = finish(config, state, tracker, iteration, P, geo, out)
    return state, residuals, diagnostics
