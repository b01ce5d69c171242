"""Generator driver over the GPU step.

Same contract as src/pyflow/drivers/simulation_driver.py:38-110: yields
``(state, residuals, diagnostics)`` after every step, the same State object
mutated in place; ``diagnostics`` gains ``u_centerline`` ([y coords,
u[:, nx//2]]) and ``wall_time``; ``ValueError`` when neither a state nor
``config.nx/ny`` is given; checkpoint errors are reported as
``checkpoint_written = False``.
"""
from __future__ import annotations

import time
from collections.abc import Callable, Generator
from typing import Any

from ..core.ghost_fields import State, allocate_state, interior_view
from ..io.checkpoint import save_checkpoint
from ..residuals.manager import ResidualManager
from ..solvers.solver import step


class SimulationDriver:
    def __init__(self, config: Any, state: State | None = None, tracker: ResidualManager | None = None, *,
                 allocate: Callable[[int, int], State] = allocate_state):
        self.config = config
        self.state = state
        self.tracker = tracker or ResidualManager()
        self.allocate_fn = allocate
        self._t0 = None
        self.iteration = 0

    def ensure_state(self, nx: int, ny: int) -> State:
        if self.state is None:
            self.state = self.allocate_fn(nx, ny)
        return self.state

    def run(self, max_steps: int | None = None, *, start_iteration: int = 0, progress: bool = False,
            checkpoint_path: str | None = None,
            checkpoint_interval: int | None = None) -> Generator[tuple[State, dict[str, float], dict[str, Any]], None, None]:
        self.iteration = start_iteration
        self._t0 = time.time()
        while True:
            if max_steps is not None and self.iteration >= max_steps:
                return
            if self.state is None:
                nx = getattr(self.config, "nx", None)
                ny = getattr(self.config, "ny", None)
                if nx is None or ny is None:
                    raise ValueError("SimulationDriver requires either an initial State or config.nx & config.ny for allocation")
                self.state = self.allocate_fn(nx, ny)
            state, residuals, diagnostics = step(self.config, self.state, self.tracker, self.iteration)
            try:
                ui = interior_view(state.fields["u"])
                nyi, nxi = ui.shape
                cx = nxi // 2
                col = ui[:, cx]
                u_center = col.cpu().tolist() if hasattr(col, "cpu") else col.tolist()
                ly_val = getattr(self.config, "ly", float(nyi - 1))
                y_coords = [j * (ly_val / (nyi - 1)) for j in range(nyi)] if nyi > 1 else [0.0]
                diagnostics["u_centerline"] = [y_coords, u_center]
            except Exception:  # pragma: no cover
                pass
            diagnostics["wall_time"] = time.time() - self._t0
            if progress:
                print(f"iter={self.iteration} dt={diagnostics.get('dt'):.3g} CFL={diagnostics.get('CFL'):.3g} "
                      f"continuity={residuals.get('continuity'):.3e}")
            yield state, residuals, diagnostics
            if checkpoint_path and checkpoint_interval and checkpoint_interval > 0:
                if (self.iteration % checkpoint_interval) == 0:
                    try:
                        save_checkpoint(checkpoint_path, state, self.iteration,
                                        diagnostics.get("time", diagnostics.get("wall_time", 0.0)), self.config)
                        diagnostics["checkpoint_written"] = True
                    except Exception:  # pragma: no cover
                        diagnostics["checkpoint_written"] = False
            self.iteration += 1


__all__ = ["SimulationDriver"]
