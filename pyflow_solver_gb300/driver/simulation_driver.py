"""Steady-state driver over the GPU step.

Public surface of src/pyflow/driver/simulation_driver.py:44-195: the
``PhysicsConfig`` and ``DriverConfig`` dataclasses (same fields and defaults,
plus ``precision``), ``SimulationDriver(driver_cfg, physics_cfg)`` with
``run()`` yielding one payload dict per step (``iteration``, ``state``,
``residuals``, ``diagnostics``, ``divergence_mean``,
``divergence_mean_free_norm``, ``steady``, ``steady_slope``, ``elapsed``), the
``steady_detected`` / ``steady_iteration`` / ``elapsed`` properties, the
pre/post-step hooks, the report line every ``report_interval`` steps and
``create_default_driver``.

How it runs here: the cavity is a one-instance ``BatchedCavities`` whose
device-side steady-state test is armed (``pfgb_set_steady``).  The test of the
reference (:135-149) -- the least-squares slope of log10(Ru) over the last
``steady_window`` entries of the residual tracker's Ru series, steady when every
entry is positive and |slope| < ``steady_slope_tol`` -- is evaluated by the
step's last kernel on a ring of the series kept on the GPU, and arrives in the
step record with the rest of the step's scalars.  The host keeps no window and
fits nothing.  The divergence statistics of each step (mean and mean-free norm
of the central divergence, :78-81) come from the GPU operator and exactly
rounded device sums.  As in the reference, the step that detects the steady
state is yielded without the post-step hook or a report line, and the run ends
there when ``stop_on_steady``.
"""
from __future__ import annotations

import ctypes
import math
import time
from collections.abc import Callable, Generator
from dataclasses import dataclass, fields
from types import SimpleNamespace
from typing import Any

import numpy as np
import torch

from .. import _capi
from .._device import ptr, stream_handle
from ..batch import BatchedCavities
from ..core.ghost_fields import State, allocate_state, interior_view
from ..numerics.fluid_ops import divergence as central_divergence


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


def _device_sum(t: torch.Tensor, square: bool) -> float:
    """Exactly rounded sum (or sum of squares) of a device tensor."""
    t = t.reshape(-1).contiguous()
    out = ctypes.c_double()
    lib = _capi.load()
    if square:
        rc = lib.pfgb_xdot(ptr(t), ptr(t), t.numel(), ctypes.byref(out), stream_handle())
    else:
        rc = lib.pfgb_xsum(ptr(t), t.numel(), ctypes.byref(out), stream_handle())
    _capi.check(rc, "exact device sum")
    return out.value


def mean_free_stats(field) -> tuple[float, float]:
    """(mean, ||field - mean||_2) of a divergence field: exactly rounded device sums for a
    CUDA tensor, NumPy's for a host array."""
    if not isinstance(field, torch.Tensor):
        a = np.asarray(field, dtype=np.float64)
        m = float(a.mean())
        return m, float(np.linalg.norm(a - m))
    m = _device_sum(field, square=False) / field.numel()
    return m, math.sqrt(_device_sum(field - m, square=True))


class SimulationDriver:
    """Runs one cavity to a steady state (or max_steps), one payload per step."""

    def __init__(self, driver_cfg: DriverConfig, physics_cfg: PhysicsConfig | None = None):
        self.driver_cfg = driver_cfg
        self.physics_cfg = physics_cfg or PhysicsConfig()
        self.state: State = allocate_state(driver_cfg.nx, driver_cfg.ny)
        self._t0: float | None = None
        self._detected_at: int | None = None
        step_cfg = SimpleNamespace(nx=driver_cfg.nx, ny=driver_cfg.ny,
                                   **{f.name: getattr(self.physics_cfg, f.name) for f in fields(self.physics_cfg)})
        self._batch = BatchedCavities([step_cfg], [self.state])
        if driver_cfg.steady_window >= 2:
            self._batch.set_steady(0, driver_cfg.steady_window, driver_cfg.steady_slope_tol)
        self.tracker = self._batch.trackers[0]

    @property
    def steady_detected(self) -> bool:
        return self._detected_at is not None

    @property
    def steady_iteration(self) -> int | None:
        return self._detected_at

    @property
    def elapsed(self) -> float:
        return 0.0 if self._t0 is None else time.time() - self._t0

    def _divergence_stats(self) -> tuple[float, float]:
        st = self.state
        div = central_divergence(interior_view(st.fields["u"]), interior_view(st.fields["v"]), st.meta["dx"],
                                 st.meta["dy"])
        return mean_free_stats(div)

    def _steady_of(self, record) -> tuple[bool, float | None]:
        """(steady, slope) from the step record; slope None where no fit was formed (fewer
        entries than the window, or a non-positive Ru in it)."""
        if self.driver_cfg.steady_window < 2:
            return False, None
        slope = float(record["steady_slope"])
        return bool(record["steady"]), (None if math.isnan(slope) else slope)

    def run(self) -> Generator[dict[str, Any], None, None]:
        cfg = self.driver_cfg
        self._t0 = time.time()
        for it in range(cfg.max_steps):
            if cfg.pre_step:
                cfg.pre_step(self, it, self.state)
            residuals, diag = self._batch.step()[0]
            steady, slope = self._steady_of(self._batch.last_out[0])
            div_mean, div_mf = self._divergence_stats()
            payload = {
                "iteration": it, "state": self.state, "residuals": residuals, "diagnostics": diag,
                "divergence_mean": div_mean, "divergence_mean_free_norm": div_mf,
                "steady": steady, "steady_slope": slope, "elapsed": self.elapsed,
            }
            if steady:
                self._detected_at = it
                if cfg.stop_on_steady:
                    yield payload
                    return
            if cfg.post_step:
                cfg.post_step(self, it, self.state)
            if it % cfg.report_interval == 0 or it == cfg.max_steps - 1:
                tail = f" steady|slope={slope:.3e}" if steady else ""
                print(f"Iter {it:5d} | dt={diag['dt']:.3e} CFL={diag['CFL']:.2f} Ru={residuals['Ru']:.3e} "
                      f"Rv={residuals['Rv']:.3e} div_mf={div_mf:.3e} div_mean={div_mean:.3e}{tail}")
            yield payload

    def close(self):
        self._batch.close()


def create_default_driver() -> SimulationDriver:
    return SimulationDriver(DriverConfig(), PhysicsConfig())


__all__ = ["DriverConfig", "PhysicsConfig", "SimulationDriver", "create_default_driver", "mean_free_stats"]
