"""Continuous batching of lid-driven-cavity solves on one GPU.

``ServingEngine`` keeps a pool of *slots* -- resident cavity states of fixed
sizes -- inside one native batch (``pfgb_batch_*``): every engine step is one
CUDA graph launch that advances every occupied slot by one projection step
(per-instance masks leave free slots out).  Requests wait in a FIFO queue per
grid size; a request is admitted into a free slot of its size as soon as one
frees up (the slot's fields are zeroed and its Re / lid velocity set with
``pfgb_batch_set_params``), so requests that arrive while others are on the GPU
join the next step.  The slot pool itself is sized to a device-memory budget.
A request ends after its step count or, from its second step on, when its
continuity residual falls below the tolerance (at step 0 the continuity of the
zero initial field is exactly 0, see the reference's CLI early stop,
src/pyflow/cli.py:175-178).

Every slot computes exactly what the same request computes alone: the batch
shares launches, not arithmetic (the tests check this bit for bit).
"""
from __future__ import annotations

import ctypes
import math
import time
from collections import deque
from dataclasses import dataclass, field

import torch

from . import _capi
from .batch import BatchedCavities
from .core.ghost_fields import allocate_state
from .residuals.manager import ResidualManager
from .solvers.solver import prepare
from .workloads import cavity_config


def slot_bytes(side: int, precision: str = "mixed") -> int:
    """Device bytes of one slot: state, binary64 work vectors, mixed-precision levels."""
    ld = (side + 31) // 32 * 32
    state = 3 * (side + 2) ** 2 * 8
    work = 8 * ld * side * 8
    mixed = 0
    if precision == "mixed":
        mixed = int(4 * ld * side * 4 * 4 / 3) + 4 * ld * side * 4 + ld * side * 8
    return state + work + mixed + 64 * 1024


@dataclass
class Served:
    rid: int
    side: int
    arrival: float
    start: float = math.nan
    finish: float = math.nan
    steps_done: int = 0
    stop: str = ""                       # "steps" | "continuity"
    last_continuity: float = math.nan


@dataclass
class ServeReport:
    completed: list = field(default_factory=list)
    in_flight: int = 0
    queued: int = 0
    cell_updates: int = 0
    wall_s: float = 0.0
    engine_steps: int = 0

    def latency_percentiles(self):
        lat = sorted(r.finish - r.arrival for r in self.completed)
        if not lat:
            return {}
        pick = lambda q: lat[min(len(lat) - 1, int(q * (len(lat) - 1) + 0.5))]  # noqa: E731
        return {"p50": pick(0.50), "p95": pick(0.95), "p99": pick(0.99)}


class ServingEngine:
    def __init__(self, slots: dict, precision: str = "mixed", continuity_tol: float = 1e-6,
                 memory_budget_bytes: float = 60e9, lin_tol: float = 1e-8, lin_maxiter: int = 300):
        need = sum(n * slot_bytes(s, precision) for s, n in slots.items())
        if need > memory_budget_bytes:
            raise ValueError(f"slot plan needs {need / 1e9:.1f} GB, above the {memory_budget_bytes / 1e9:.1f} GB budget")
        self.precision = precision
        self.tol = continuity_tol
        self.lin_tol = lin_tol
        self.lin_maxiter = lin_maxiter
        self.sides = []
        configs, states = [], []
        for side in sorted(slots):
            for _ in range(slots[side]):
                self.sides.append(side)
                configs.append(cavity_config(side, side, 100.0, 1.0, precision, lin_tol=lin_tol,
                                             lin_maxiter=lin_maxiter))
                states.append(allocate_state(side, side))
        self.batch = BatchedCavities(configs, states)
        self.bytes = need
        self.owner = [None] * len(self.sides)          # slot -> Served

    def _assign(self, k: int, req, now: float):
        B = self.batch
        cfg = cavity_config(req.side, req.side, req.Re, req.U, self.precision, lin_tol=self.lin_tol,
                            lin_maxiter=self.lin_maxiter)
        st = B.states[k]
        for f in st.fields.values():
            f.zero_()
        st.meta.clear()
        B.configs[k] = cfg
        B.trackers[k] = ResidualManager()
        B.iterations[k] = 0
        P, _, geo = prepare(cfg, st, 0)
        B._params[k] = P
        B._geo[k] = geo
        _capi.check(_capi.load().pfgb_batch_set_params(B._h, k, ctypes.byref(P)), "pfgb_batch_set_params")
        s = Served(req.rid, req.side, req.arrival, start=now)
        self.owner[k] = (s, req.steps)

    def run(self, trace, max_wall: float | None = None, clock=time.perf_counter, realtime: bool = True):
        """Serve `trace` (arrival-ordered requests).  With realtime=False the
        arrival times are ignored and every request is queued at once."""
        rep = ServeReport()
        queues = {}
        free = {}
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
                while q and free[side]:
                    self._assign(free[side].popleft(), q.popleft(), now)
            active = [o is not None for o in self.owner]
            if not any(active):
                if not pending:
                    break
                if realtime:
                    time.sleep(max(0.0, min(0.01, pending[0].arrival - now)))
                continue
            if max_wall is not None and now >= max_wall:
                break
            out = self.batch.step(active=active)
            rep.engine_steps += 1
            done_t = clock() - t0
            for k, o in enumerate(out):
                if o is None:
                    continue
                res, diag = o
                s, nsteps = self.owner[k]
                s.steps_done += 1
                s.last_continuity = res["continuity"]
                rep.cell_updates += self.sides[k] ** 2
                stop = ""
                if s.steps_done >= nsteps:
                    stop = "steps"
                elif diag["iteration"] >= 1 and res["continuity"] < self.tol:
                    stop = "continuity"
                if stop:
                    s.stop = stop
                    s.finish = done_t
                    rep.completed.append(s)
                    self.owner[k] = None
                    free[self.sides[k]].append(k)
        rep.wall_s = clock() - t0
        rep.in_flight = sum(o is not None for o in self.owner)
        rep.queued = sum(len(q) for q in queues.values()) + len(pending)
        torch.cuda.synchronize()
        return rep


def run_alone(req, precision="mixed", continuity_tol=1e-6, lin_tol=1e-8, lin_maxiter=300):
    """The same request by itself (single-instance step loop): fields and step count."""
    from .solvers.solver import step
    cfg = cavity_config(req.side, req.side, req.Re, req.U, precision, lin_tol=lin_tol, lin_maxiter=lin_maxiter)
    st = allocate_state(req.side, req.side)
    tr = ResidualManager()
    n = 0
    for it in range(req.steps):
        _, res, diag = step(cfg, st, tr, it)
        n += 1
        if it >= 1 and res["continuity"] < continuity_tol:
            break
    return st, n
