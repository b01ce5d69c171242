"""Steady-state simulation driver over the GPU step.

Mirrors src/pyflow/driver/simulation_driver.py:44-195: ``PhysicsConfig`` and
``DriverConfig`` with the same fields and defaults, ``SimulationDriver.run()``
yielding one payload dict per step (``iteration``, ``state``, ``residuals``,
``diagnostics``, ``divergence_mean``, ``divergence_mean_free_norm``, ``steady``,
``steady_slope``, ``elapsed``), pre/post-step hooks, the report line every
``report_interval`` steps, and the steady-state test of :135-149: the
least-squares slope of log10(Ru) over the last ``steady_window`` steps, with
``stop_on_steady`` yielding the detecting step and stopping.

The divergence statistics use the GPU central divergence and exactly rounded
sums (``float(field.mean())`` and ``np.linalg.norm(field - mean)`` in the
reference, whose summation order is NumPy's); the slope is the same NumPy
``polyfit`` on the same host series.
"""
from __future__ import annotations

import ctypes
import math
import time
from collections.abc import Callable, Generator
from dataclasses import dataclass
from typing import Any

import numpy as np
import torch

from .. import _capi
from .._device import ptr, stream_handle
from ..core.ghost_fields import State, allocate_state, interior_view
from ..numerics.fluid_ops import divergence as div_op
from ..residuals.manager import ResidualManager
from ..solvers.solver import step as core_step


@dataclass
class PhysicsConfig:
    Re: float = 100.0
    lid_velocity: float = 1.0
    disable_advection: bool = False
    advection_scheme: str = "quick"
    cfl_target: float = 0.5
    cfl_growth: float = 1.05
    lin_tol: float = 1e-10
    lin_maxiter: int = 800
    diagnostics: bool = False
    lx: float = 1.0
    ly: float = 1.0
    precision: str = "fp64"


@dataclass
class DriverConfig:
    nx: int = 65
    ny: int = 65
    max_steps: int = 10_000
    report_interval: int = 100
    steady_window: int = 100
    steady_slope_tol: float = 2e-3
    stop_on_steady: bool = True
    save_interval: int = 0
    pre_step: Callable[[SimulationDriver, int, State], None] | None = None
    post_step: Callable[[SimulationDriver, int, State], None] | None = None


def _xsum(t: torch.Tensor) -> float:
    r = ctypes.c_double()
    t = t.reshape(-1).contiguous()
    _capi.check(_capi.load().pfgb_xsum(ptr(t), t.numel(), ctypes.byref(r), stream_handle()), "xsum")
    return r.value


def _xsumsq(t: torch.Tensor) -> float:
    r = ctypes.c_double()
    t = t.reshape(-1).contiguous()
    _capi.check(_capi.load().pfgb_xdot(ptr(t), ptr(t), t.numel(), ctypes.byref(r), stream_handle()), "xdot")
    return r.value


def mean_free_stats(field) -> tuple[float, float]:
    """(mean, ||field - mean||_2) of a device field (driver/simulation_driver.py:78-81)."""
    if not isinstance(field, torch.Tensor):
        a = np.asarray(field, dtype=np.float64)
        mean = float(a.mean())
        return mean, float(np.linalg.norm(a - mean))
    n = field.numel()
    mean = _xsum(field) / n
    return mean, math.sqrt(_xsumsq(field - mean))


class SimulationDriver:
    def __init__(self, driver_cfg: DriverConfig, physics_cfg: PhysicsConfig | None = None):
        self.driver_cfg = driver_cfg
        self.physics_cfg = physics_cfg or PhysicsConfig()
        self.state: State = allocate_state(driver_cfg.nx, driver_cfg.ny)
        self.tracker = ResidualManager()
        self._start_wall: float | None = None
        self._steady_detected = False
        self._steady_iteration: int | None = None

    @property
    def steady_detected(self) -> bool:
        return self._steady_detected

    @property
    def steady_iteration(self) -> int | None:
        return self._steady_iteration

    @property
    def elapsed(self) -> float:
        if self._start_wall is None:
            return 0.0
        return time.time() - self._start_wall

    def run(self) -> Generator[dict[str, Any], None, None]:
        self._start_wall = time.time()
        cfg = self.driver_cfg
        physics = self.physics_cfg
        state = self.state
        tracker = self.tracker
        for it in range(cfg.max_steps):
            if cfg.pre_step:
                cfg.pre_step(self, it, state)
            state, residuals, diag = core_step(physics, state, tracker, it)
            ui = interior_view(state.fields["u"])
            vi = interior_view(state.fields["v"])
            div_full = div_op(ui, vi, state.meta["dx"], state.meta["dy"])
            div_mean, div_mf = mean_free_stats(div_full)
            steady = False
            steady_slope = None
            ru = tracker.series["Ru"].values if "Ru" in tracker.series else []
            if len(ru) >= cfg.steady_window:
                recent = np.array(ru[-cfg.steady_window:])
                if np.all(recent > 0):
                    xs = np.arange(recent.size)
                    steady_slope = float(np.polyfit(xs, np.log10(recent), 1)[0])
                    if abs(steady_slope) < cfg.steady_slope_tol:
                        self._steady_detected = True
                        self._steady_iteration = it
                        steady = True
                        if cfg.stop_on_steady:
                            yield self._build_payload(it, residuals, diag, div_mean, div_mf, steady, steady_slope)
                            break
            payload = self._build_payload(it, residuals, diag, div_mean, div_mf, steady, steady_slope)
            if cfg.post_step:
                cfg.post_step(self, it, state)
            if it % cfg.report_interval == 0 or (steady and cfg.stop_on_steady) or it == cfg.max_steps - 1:
                print(f"Iter {it:5d} | dt={diag['dt']:.3e} CFL={diag['CFL']:.2f} "
                      f"Ru={residuals['Ru']:.3e} Rv={residuals['Rv']:.3e} div_mf={div_mf:.3e} div_mean={div_mean:.3e}"
                      + (f" steady|slope={steady_slope:.3e}" if steady else ""))
            yield payload

    def _build_payload(self, iteration, residuals, diag, div_mean, div_mf, steady, steady_slope) -> dict[str, Any]:
        return {
            "iteration": iteration,
            "state": self.state,
            "residuals": residuals,
            "diagnostics": diag,
            "divergence_mean": div_mean,
            "divergence_mean_free_norm": div_mf,
            "steady": steady,
            "steady_slope": steady_slope,
            "elapsed": self.elapsed,
        }


def create_default_driver() -> SimulationDriver:
    return SimulationDriver(DriverConfig(), PhysicsConfig())


__all__ = ["DriverConfig", "PhysicsConfig", "SimulationDriver", "create_default_driver", "mean_free_stats"]
