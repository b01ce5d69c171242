"""Seeded synthetic workloads of the benchmark configurations.

* ``batched_instances`` -- 256 lid-driven cavities from seed 0: for each, in
  draw order, nx and ny uniform over {32, 48, 64, 96, 128}, Re log-uniform in
  [100, 5000], lid velocity uniform in [0.5, 2.0]; unit square, zero fields.
* ``serving_trace`` -- Poisson arrivals (rate per second, duration) from seed 1:
  per request, in draw order, the inter-arrival gap, a square side from
  {32, 64, 128, 256, 512, 1024} with probabilities {.3, .25, .2, .15, .07, .03},
  Re log-uniform in [100, 3200], lid velocity uniform in [0.5, 2.0], and a step
  count uniform in [100, 2000].
There is no dataset behind these configurations: the draws stand in for it.
"""
from __future__ import annotations

from dataclasses import dataclass
from types import SimpleNamespace

import numpy as np

SIDES_BATCH = [32, 48, 64, 96, 128]
SIDES_SERVE = [32, 64, 128, 256, 512, 1024]
P_SERVE = [0.3, 0.25, 0.2, 0.15, 0.07, 0.03]


def batched_instances(n: int = 256, seed: int = 0):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nx = int(rng.choice(SIDES_BATCH))
        ny = int(rng.choice(SIDES_BATCH))
        Re = float(np.exp(rng.uniform(np.log(100.0), np.log(5000.0))))
        U = float(rng.uniform(0.5, 2.0))
        out.append((nx, ny, Re, U))
    return out


def cavity_config(nx, ny, Re, U, precision="mixed", scheme="quick", lin_tol=1e-8, lin_maxiter=300):
    """The step config of one benchmark cavity (unit square, CFL 0.5 / growth 1.05)."""
    return SimpleNamespace(nx=nx, ny=ny, lx=1.0, ly=1.0, Re=Re, lid_velocity=U, advection_scheme=scheme,
                           cfl_target=0.5, cfl_growth=1.05, lin_tol=lin_tol, lin_maxiter=lin_maxiter,
                           enable_jacobi_pc=True, diagnostics=False, precision=precision)


@dataclass
class Request:
    rid: int
    arrival: float        # seconds from the start of the trace
    side: int
    Re: float
    U: float
    steps: int


def serving_trace(rate: float = 200.0, duration: float = 60.0, seed: int = 1):
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t >= duration:
            break
        side = int(rng.choice(SIDES_SERVE, p=P_SERVE))
        Re = float(np.exp(rng.uniform(np.log(100.0), np.log(3200.0))))
        U = float(rng.uniform(0.5, 2.0))
        steps = int(rng.integers(100, 2001))
        out.append(Request(len(out), t, side, Re, U, steps))
    return out
