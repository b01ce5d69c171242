"""GB300-native (sm_103a) projection step of PyFlow's 2-D lid-driven cavity.

The package mirrors the reference's public path (``pyflow``):

* ``drivers.simulation_driver.SimulationDriver``  (src/pyflow/drivers/simulation_driver.py)
* ``solvers.solver.step``                          (src/pyflow/solvers/solver.py)
* ``solvers.pressure_solver.solve_pressure_poisson`` (src/pyflow/solvers/pressure_solver.py)
* ``linear_solvers.interface.solve / LinearSolveResult``, ``preconditioners.jacobi_preconditioner``
* ``numerics`` operators, ``core.ghost_fields`` state, ``residuals.manager.ResidualManager``

All array work runs in hand-written CUDA kernels of ``libpfgb.so`` through its
C ABI (``include/pfgb.h``); PyTorch only owns device memory and streams.
There is no CPU fallback.
"""
from .core.ghost_fields import State, allocate_state, interior_view  # noqa: F401
from .drivers.simulation_driver import SimulationDriver  # noqa: F401
from .residuals.manager import ResidualManager  # noqa: F401
from .solvers.solver import step  # noqa: F401

__version__ = "0.1.0"
