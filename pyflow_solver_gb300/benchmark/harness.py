"""Benchmark harness over grid sizes, with the reference's JSON shape.

Mirrors src/pyflow/benchmark/harness.py:33-107 (``make_config``, ``run_case``,
``benchmark``, ``main``; output ``{"benchmark": "lid_driven_cavity",
"steps_requested", "runs": [{nx, ny, steps, total_time_s,
avg_time_per_step_s, avg_cg_iterations}]}``) on the GPU step.

The reference's defaults (lid velocity 0, advection off) give a zero
right-hand side at every step, so its runs measure no pressure solve at all.
Here the defaults are a driven cavity (lid 1, QUICK) on the unit square;
``--reference-defaults`` restores the reference's degenerate configuration.
Each run adds ``cell_updates_per_s``, ``avg_true_cg_iterations`` (the CG count
the reference's ``Rp_iterations`` folds into 0 or maxiter) and the precision;
timing synchronises the device after the last step.

    python -m pyflow_solver_gb300.benchmark.harness --grids 32,64,128,256 --steps 100 [--precision mixed]
"""
from __future__ import annotations

import argparse
import json
import time
from types import SimpleNamespace
from typing import Any

import torch

from ..core.ghost_fields import allocate_state
from ..drivers.simulation_driver import SimulationDriver
from ..residuals.manager import ResidualManager


def make_config(nx: int, ny: int, *, Re: float = 100.0, lid_velocity: float = 1.0, disable_advection: bool = False,
                enable_jacobi_pc: bool = True, precision: str = "fp64", reference_defaults: bool = False):
    if reference_defaults:
        return SimpleNamespace(nx=nx, ny=ny, Re=Re, lid_velocity=0.0, cfl_target=0.5, cfl_growth=1.05,
                               advection_scheme="upwind", disable_advection=True, lin_tol=1e-10, lin_maxiter=400,
                               diagnostics=False, enable_jacobi_pc=enable_jacobi_pc, force_quiet=True,
                               lx=nx - 1, ly=ny - 1, precision=precision)
    return SimpleNamespace(nx=nx, ny=ny, Re=Re, lid_velocity=lid_velocity, cfl_target=0.5, cfl_growth=1.05,
                           advection_scheme="quick", disable_advection=disable_advection, lin_tol=1e-8,
                           lin_maxiter=400, diagnostics=False, enable_jacobi_pc=enable_jacobi_pc, force_quiet=True,
                           lx=1.0, ly=1.0, precision=precision)


def run_case(nx: int, ny: int, steps: int, **kw) -> dict[str, Any]:
    cfg = make_config(nx, ny, **kw)
    state = allocate_state(nx, ny)
    tracker = ResidualManager()
    driver = SimulationDriver(cfg, state, tracker)
    torch.cuda.synchronize()
    t0 = time.time()
    total_cg_iter = 0
    total_true = 0
    step_count = 0
    for _s, _res, diag in driver.run(max_steps=steps):
        total_cg_iter += int(diag.get("Rp_iterations", 0))
        total_true += int(diag.get("cg_iterations", 0))
        step_count += 1
    torch.cuda.synchronize()
    total_time = time.time() - t0
    n = max(step_count, 1)
    return {
        "nx": nx,
        "ny": ny,
        "steps": step_count,
        "total_time_s": total_time,
        "avg_time_per_step_s": total_time / n,
        "avg_cg_iterations": total_cg_iter / n,
        "avg_true_cg_iterations": total_true / n,
        "cell_updates_per_s": nx * ny * step_count / total_time if total_time > 0 else None,
        "precision": cfg.precision,
    }


def benchmark(grids: list[int], steps: int, **kw) -> dict[str, Any]:
    runs = [run_case(n, n, steps, **kw) for n in grids]
    return {"benchmark": "lid_driven_cavity", "steps_requested": steps, "runs": runs}


def main(argv: list[str] | None = None) -> int:
    ap = argparse.ArgumentParser(description="PyFlow benchmark harness (GB300 step)")
    ap.add_argument("--grids", type=str, default="32,64,128,256", help="Comma-separated grid sizes (nx=ny)")
    ap.add_argument("--steps", type=int, default=100, help="Number of steps per grid")
    ap.add_argument("--json-out", type=str, default=None, help="Path to write JSON results")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--reference-defaults", action="store_true",
                    help="lid 0, advection off, dx = 1 (the reference harness's configuration)")
    args = ap.parse_args(argv)
    grids = [int(x) for x in args.grids.split(",") if x.strip()]
    result = benchmark(grids, args.steps, precision=args.precision, reference_defaults=args.reference_defaults)
    payload = json.dumps(result, indent=2)
    if args.json_out:
        with open(args.json_out, "w", encoding="utf-8") as f:
            f.write(payload + "\n")
    print(payload)
    return 0


if __name__ == "__main__":  # pragma: no cover
    raise SystemExit(main())

__all__ = ["benchmark", "make_config", "run_case"]
