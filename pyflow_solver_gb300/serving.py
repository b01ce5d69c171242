"""Continuous batching of lid-driven-cavity solves on one GPU.

``ServingEngine`` keeps a pool of *slots* -- resident cavity states of fixed
sizes -- inside one native batch (``pfgb_batch_*``): every engine step is one
CUDA graph launch that advances every occupied slot by one projection step
(free slots sit the step out).  Requests wait in a FIFO queue per grid size; a
request is admitted into a free slot of its size as soon as one frees up (the
slot's fields are zeroed and its Re / lid velocity set in place with
``pfgb_batch_set_params``), so requests that arrive while others are on the
GPU join the next step and their work shares its launches.  The slot pool is
sized to a device-memory budget before any request is taken.

A request ends after its step count or, from its second step on, when its
continuity residual falls below the tolerance -- or, with ``steady_window`` set,
when the device-side steady-state test fires for its slot (the steady driver's
least-squares slope of log10(Ru) over the last ``steady_window`` steps below
``steady_slope_tol``; src/pyflow/driver/simulation_driver.py:135-149), read from
the step records without any host-side series.  The reference's CLI breaks on
``continuity < threshold`` after any step (src/pyflow/cli.py:174-178); after
step 0 of a zero initial field the continuity is exactly 0, so the test
starts at step 1 here, or every request would end after one step.

With ``sink`` set, every step of every request is streamed as the CLI's
JSON-line step record (one ``str`` per call, the request id added as
``"request"``); the residual and diagnostic dicts are then formed for every
slot and step, which costs host time.

Every slot computes exactly what the same request computes alone: the batch
shares launches, not arithmetic.
"""
from __future__ import annotations

import json
import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from .batch import BatchedCavities
from .cli import step_payload
from .core.ghost_fields import allocate_state
from .residuals.manager import ResidualManager
from .workloads import cavity_config


@dataclass
class Served:
    rid: int
    side: int
    arrival: float
    steps: int
    start: float = math.nan
    finish: float = math.nan
    steps_done: int = 0
    stop: str = ""                       # "steps" | "continuity" | "steady"
    last_continuity: float = math.nan
    fields: dict | None = None           # final u, v, p (kept with keep_fields=True)


@dataclass
class ServeReport:
    completed: list = field(default_factory=list)
    in_flight: int = 0
    queued: int = 0
    cell_updates: int = 0
    wall_s: float = 0.0
    engine_steps: int = 0
    slots: int = 0
    device_bytes: int = 0

    def latency_percentiles(self):
        lat = sorted(r.finish - r.arrival for r in self.completed)
        if not lat:
            return {}
        pick = lambda q: lat[min(len(lat) - 1, int(q * (len(lat) - 1) + 0.5))]  # noqa: E731
        return {"p50": pick(0.50), "p95": pick(0.95), "p99": pick(0.99)}


def slot_plan(sides, budget_bytes: float, probe_bytes, weights=None):
    """Slots per side within the budget: the budget is shared in proportion to
    `weights` (default: equal) and each share divided by the side's measured
    slot bytes (``probe_bytes(side)``)."""
    sides = list(sides)
    w = np.ones(len(sides)) if weights is None else np.asarray(weights, dtype=np.float64)
    w = w / w.sum()
    plan = {}
    for s, ws in zip(sides, w):
        b = probe_bytes(s)
        plan[s] = max(1, int(budget_bytes * ws // b))
    return plan


class ServingEngine:
    def __init__(self, slots: dict, precision: str = "mixed", continuity_tol: float = 1e-6,
                 memory_budget_bytes: float = 60e9, lin_tol: float = 1e-8, lin_maxiter: int = 300,
                 steady_window: int = 0, steady_slope_tol: float = 2e-3):
        self.precision = precision
        self.tol = continuity_tol
        self.steady_window = int(steady_window)
        self.steady_tol = float(steady_slope_tol)
        self.lin_tol = lin_tol
        self.lin_maxiter = lin_maxiter
        self.sides = []
        configs, states = [], []
        state_bytes = 0
        for side in sorted(slots):
            for _ in range(slots[side]):
                self.sides.append(side)
                configs.append(self._config(side, 100.0, 1.0))
                states.append(allocate_state(side, side))
                state_bytes += 3 * (side + 2) ** 2 * 8
        self.batch = BatchedCavities(configs, states)
        self.device_bytes = state_bytes + self.batch.workspace_bytes()
        if self.device_bytes > memory_budget_bytes:
            self.batch.close()
            raise ValueError(f"the slot plan needs {self.device_bytes / 1e9:.2f} GB of device memory, above the "
                             f"{memory_budget_bytes / 1e9:.2f} GB budget")
        n = len(self.sides)
        self.side_arr = np.array(self.sides, dtype=np.int64)
        self.owner: list[Served | None] = [None] * n
        self.busy = np.zeros(n, dtype=bool)
        self.target = np.zeros(n, dtype=np.int64)
        self.done = np.zeros(n, dtype=np.int64)

    def _config(self, side, Re, U):
        return cavity_config(side, side, Re, U, self.precision, lin_tol=self.lin_tol, lin_maxiter=self.lin_maxiter)

    def _assign(self, k: int, req, now: float):
        self.batch.set_params(k, self._config(req.side, req.Re, req.U), reset=True)
        if self.steady_window:
            self.batch.set_steady(k, self.steady_window, self.steady_tol)
        self.owner[k] = Served(req.rid, req.side, req.arrival, req.steps, start=now)
        self.busy[k] = True
        self.target[k] = req.steps
        self.done[k] = 0

    def run(self, trace, max_wall: float | None = None, realtime: bool = True, sink=None, keep_fields=False,
            clock=time.perf_counter):
        """Serve `trace` (requests ordered by arrival).  With realtime=False the
        arrival times are ignored and every request is queued at once.  Stops
        when every request is done or, with max_wall, at that many seconds."""
        B = self.batch
        rep = ServeReport(slots=len(self.sides), device_bytes=self.device_bytes)
        queues: dict[int, deque] = {}
        free: dict[int, deque] = {}
        for k, s in enumerate(self.sides):
            free.setdefault(s, deque()).append(k)
            queues.setdefault(s, deque())
        pending = deque(trace)
        t0 = clock()
        while True:
            now = clock() - t0
            while pending and (not realtime or pending[0].arrival <= now):
                r = pending.popleft()
                if r.side not in queues:
                    raise ValueError(f"no slot of side {r.side}")
                queues[r.side].append(r)
            for side, q in queues.items():
                fr = free[side]
                while q and fr:
                    self._assign(fr.popleft(), q.popleft(), now)
            if not self.busy.any():
                if not pending:
                    break
                if realtime:
                    time.sleep(max(0.0, min(0.005, pending[0].arrival - now)))
                continue
            if max_wall is not None and now >= max_wall:
                break
            busy = self.busy.copy()
            its = B.iterations.copy()
            if sink is None:
                out = B.step_arrays(busy)
                cont = B.continuity(out)
            else:
                res_list = B.step(busy)
                out = B.last_out
                cont = np.array([r[0]["continuity"] if r is not None else 0.0 for r in res_list])
                for k in np.nonzero(busy)[0]:
                    res, diag = res_list[k]
                    payload = step_payload(diag, res)
                    payload["request"] = self.owner[k].rid
                    sink(json.dumps(payload, separators=(",", ":")))
            rep.engine_steps += 1
            t_done = clock() - t0
            self.done[busy] += 1
            rep.cell_updates += int((self.side_arr[busy] ** 2).sum())
            by_steps = busy & (self.done >= self.target)
            by_cont = busy & ~by_steps & (its >= 1) & (cont < self.tol)
            by_steady = busy & ~by_steps & ~by_cont & (out["steady"] != 0)
            for k in np.nonzero(by_steps | by_cont | by_steady)[0]:
                s = self.owner[k]
                s.steps_done = int(self.done[k])
                s.last_continuity = float(cont[k])
                s.stop = "steps" if by_steps[k] else ("continuity" if by_cont[k] else "steady")
                s.finish = t_done
                if keep_fields:
                    s.fields = {f: a.clone() for f, a in B.states[k].fields.items()}
                rep.completed.append(s)
                self.owner[k] = None
                self.busy[k] = False
                free[self.sides[k]].append(int(k))
        torch.cuda.synchronize()
        rep.wall_s = clock() - t0
        rep.in_flight = int(self.busy.sum())
        rep.queued = sum(len(q) for q in queues.values()) + len(pending)
        return rep

    def state_of(self, k):
        return self.batch.states[k]

    def close(self):
        self.batch.close()


def run_alone(req, precision="mixed", continuity_tol=1e-6, lin_tol=1e-8, lin_maxiter=300, steady_window=0,
              steady_slope_tol=2e-3):
    """The same request by itself through the single-instance step: (state, steps run).
    The steady-state stop here is the reference's host-side test (NumPy polyfit on the
    tracker's Ru series), against which the engine's device-side test is checked."""
    from .solvers.solver import step
    cfg = cavity_config(req.side, req.side, req.Re, req.U, precision, lin_tol=lin_tol, lin_maxiter=lin_maxiter)
    st = allocate_state(req.side, req.side)
    tr = ResidualManager()
    n = 0
    for it in range(req.steps):
        _, res, _ = step(cfg, st, tr, it)
        n += 1
        if it >= 1 and res["continuity"] < continuity_tol:
            break
        ru = tr.series["Ru"].values
        if steady_window and len(ru) >= steady_window:
            recent = np.array(ru[-steady_window:])
            if np.all(recent > 0):
                slope = float(np.polyfit(np.arange(recent.size), np.log10(recent), 1)[0])
                if abs(slope) < steady_slope_tol:
                    break
    return st, n
