"""Steady-state driver (src/pyflow/driver/)."""
from .simulation_driver import DriverConfig, PhysicsConfig, SimulationDriver, create_default_driver, mean_free_stats

__all__ = ["DriverConfig", "PhysicsConfig", "SimulationDriver", "create_default_driver", "mean_free_stats"]
