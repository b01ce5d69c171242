"""Benchmark harness over grid sizes, emitting the reference harness's JSON.

Output shape of src/pyflow/benchmark/harness.py:33-107:
``{"benchmark": "lid_driven_cavity", "steps_requested": S, "runs": [{"nx", "ny",
"steps", "total_time_s", "avg_time_per_step_s", "avg_cg_iterations"}, ...]}``,
the same functions (``make_config``, ``run_case``, ``benchmark``, ``main``) and
command line (``--grids``, ``--steps``, ``--json-out``).

What is measured differs on purpose.  The reference's defaults (lid velocity
0, advection off) give a zero right-hand side at every step, so it times no
pressure solve at all; here a case is a driven cavity (lid 1, QUICK, unit
square) unless ``reference_defaults`` asks for the reference's configuration.
Each case is one ``Case``: its steps run through the generator driver; the
wall clock brackets the whole run (device synchronised at both ends) and CUDA
events bracket every step on the launching stream, so a run reports both the
host-visible and the device time.  Runs add ``device_time_s``,
``cell_updates_per_s``, ``avg_true_cg_iterations`` (the reference's
``Rp_iterations`` folds the count into 0 or maxiter) and the precision.

    python -m pyflow_solver_gb300.benchmark.harness --grids 32,64,128,256 --steps 100 [--precision mixed]
"""
from __future__ import annotations

import argparse
import json
import time
from dataclasses import dataclass
from types import SimpleNamespace
from typing import Any

import torch

from ..core.ghost_fields import allocate_state
from ..drivers.simulation_driver import SimulationDriver
from ..residuals.manager import ResidualManager


def make_config(nx: int, ny: int, *, Re: float = 100.0, lid_velocity: float = 1.0, disable_advection: bool = False,
                enable_jacobi_pc: bool = True, precision: str = "fp64", reference_defaults: bool = False):
    """The step config of one case.  reference_defaults: lid 0, advection off, upwind,
    dx = dy = 1 and lin_tol 1e-10 -- the reference harness's own configuration."""
    common = dict(nx=nx, ny=ny, Re=Re, cfl_target=0.5, cfl_growth=1.05, lin_maxiter=400, diagnostics=False,
                  enable_jacobi_pc=enable_jacobi_pc, force_quiet=True, precision=precision)
    if reference_defaults:
        return SimpleNamespace(**common, lid_velocity=0.0, advection_scheme="upwind", disable_advection=True,
                               lin_tol=1e-10, lx=nx - 1, ly=ny - 1)
    return SimpleNamespace(**common, lid_velocity=lid_velocity, advection_scheme="quick",
                           disable_advection=disable_advection, lin_tol=1e-8, lx=1.0, ly=1.0)


@dataclass
class Case:
    nx: int
    ny: int
    steps: int
    config: Any

    def run(self) -> dict[str, Any]:
        stream = torch.cuda.current_stream()
        marks = []
        rp_iters = true_iters = 0
        driver = SimulationDriver(self.config, allocate_state(self.nx, self.ny), ResidualManager())
        torch.cuda.synchronize()
        wall0 = time.perf_counter()
        marks.append(torch.cuda.Event(enable_timing=True))
        marks[-1].record(stream)
        done = 0
        for _state, _res, diag in driver.run(max_steps=self.steps):
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(stream)
            marks.append(ev)
            rp_iters += int(diag.get("Rp_iterations", 0))
            true_iters += int(diag.get("cg_iterations", 0))
            done += 1
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
        device_s = sum(a.elapsed_time(b) for a, b in zip(marks, marks[1:])) / 1e3
        per = max(done, 1)
        return {
            "nx": self.nx, "ny": self.ny, "steps": done,
            "total_time_s": wall, "avg_time_per_step_s": wall / per,
            "avg_cg_iterations": rp_iters / per,
            "avg_true_cg_iterations": true_iters / per,
            "device_time_s": device_s,
            "cell_updates_per_s": self.nx * self.ny * done / wall if wall > 0 else None,
            "precision": self.config.precision,
        }


def run_case(nx: int, ny: int, steps: int, **kw) -> dict[str, Any]:
    return Case(nx, ny, steps, make_config(nx, ny, **kw)).run()


def benchmark(grids: list[int], steps: int, **kw) -> dict[str, Any]:
    return {"benchmark": "lid_driven_cavity", "steps_requested": steps,
            "runs": [run_case(n, n, steps, **kw) for n in grids]}


def main(argv: list[str] | None = None) -> int:
    ap = argparse.ArgumentParser(description="PyFlow benchmark harness (GB300 step)")
    ap.add_argument("--grids", type=str, default="32,64,128,256", help="Comma-separated grid sizes (nx=ny)")
    ap.add_argument("--steps", type=int, default=100, help="Number of steps per grid")
    ap.add_argument("--json-out", type=str, default=None, help="Path to write JSON results")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--reference-defaults", action="store_true",
                    help="lid 0, advection off, dx = 1 (the reference harness's configuration)")
    args = ap.parse_args(argv)
    grids = [int(g) for g in args.grids.split(",") if g.strip()]
    text = json.dumps(benchmark(grids, args.steps, precision=args.precision,
                                reference_defaults=args.reference_defaults), indent=2)
    if args.json_out:
        with open(args.json_out, "w", encoding="utf-8") as f:
            f.write(text + "\n")
    print(text)
    return 0


if __name__ == "__main__":  # pragma: no cover
    raise SystemExit(main())

__all__ = ["Case", "benchmark", "make_config", "run_case"]
