"""Many independent cavities advanced together on one GPU.

``BatchedCavities(configs, states)`` binds one State per config (uneven nx, ny,
Re, lid velocity, scheme, ...) to a single native batch: every step is one CUDA
graph launch whose kernels cover the tiles of all instances, with per-instance
convergence masks in the CG loop.  Each instance gets exactly the dicts and
``state.meta`` updates that ``step`` gives it alone (same per-instance
arithmetic: the batch changes nothing but the launch), so a result is the same
alone and in the mix.  ``step(active=...)`` lets instances sit a step out
(continuous batching admits and retires instances without rebuilding).
"""
from __future__ import annotations

import ctypes

from . import _capi
from ._device import ptr, require_cuda, stream_handle
from .residuals.manager import ResidualManager
from .solvers.fields import device_fields
from .solvers.solver import finish, prepare


class BatchedCavities:
    def __init__(self, configs, states, trackers=None):
        require_cuda()
        if len(configs) != len(states) or not configs:
            raise ValueError("one state per config, at least one")
        self.configs = list(configs)
        self.states = list(states)
        self.trackers = list(trackers) if trackers is not None else [ResidualManager() for _ in configs]
        self.iterations = [0] * len(configs)
        n = len(configs)
        params = (_capi.Params * n)()
        self._geo = []
        for k, (cfg, st) in enumerate(zip(self.configs, self.states)):
            P, _, geo = prepare(cfg, st, 0)
            params[k] = P
            if P.precision != params[0].precision:
                raise ValueError("all instances of a batch share one precision")
            self._geo.append(geo)
        self._params = params
        h = ctypes.c_void_p()
        _capi.check(_capi.load().pfgb_batch_create(params, n, ctypes.byref(h)), "pfgb_batch_create")
        self._h = h

    def __len__(self):
        return len(self.configs)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _capi.load().pfgb_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, active=None):
        """One step of every active instance; returns [(residuals, diagnostics) or None]."""
        n = len(self.configs)
        active = [True] * n if active is None else list(active)
        ins = (_capi.StepIn * n)()
        outs = (_capi.StepOut * n)()
        U = (ctypes.c_void_p * n)()
        V = (ctypes.c_void_p * n)()
        Pp = (ctypes.c_void_p * n)()
        ctxs = []
        try:
            for k in range(n):
                if not active[k]:
                    continue
                _, sin, _ = prepare(self.configs[k], self.states[k], self.iterations[k])
                ins[k] = sin
                cm = device_fields(self.states[k])
                u, v, p = cm.__enter__()
                ctxs.append(cm)
                U[k], V[k], Pp[k] = ptr(u), ptr(v), ptr(p)
            _capi.check(_capi.load().pfgb_batch_step(self._h, U, V, Pp, ins, stream_handle(), outs), "pfgb_batch_step")
        finally:
            for cm in reversed(ctxs):
                cm.__exit__(None, None, None)
        results = []
        for k in range(n):
            if not active[k]:
                results.append(None)
                continue
            res, diag = finish(self.configs[k], self.states[k], self.trackers[k], self.iterations[k], self._params[k],
                               self._geo[k], outs[k])
            self.iterations[k] += 1
            results.append((res, diag))
        return results
