"""Many independent cavities advanced together on one GPU.

``BatchedCavities(configs, states)`` binds one State per config (uneven nx, ny,
Re, lid velocity, scheme, ...) to a single native batch: every step is one CUDA
graph launch whose kernels cover the tiles of all instances, with per-instance
convergence masks in the CG loop.

Two host paths share the same launch:

* ``step(active=None)`` gives every active instance exactly the residual and
  diagnostic dicts, tracker entries and ``state.meta`` updates that
  ``solvers.solver.step`` gives it alone (same per-instance arithmetic: the
  batch changes nothing but the launch), so a result is the same alone and in
  the mix;
* ``step_arrays(active=None)`` returns the raw step records as a NumPy
  structured array and keeps the per-instance step bookkeeping (previous dt,
  the last five divergence norms, the iteration) in arrays -- O(1) Python work
  per step whatever the batch size; ``sync_meta()`` writes that bookkeeping
  back into each ``state.meta``.

The state arrays must stay the same CUDA tensors (they are updated in place);
``rebind(k)`` re-reads instance k's arrays after they were replaced.
``set_params(k, config)`` gives slot k new physical parameters (continuous
batching reuses slots for new requests).  ``set_steady(k, window, tol)`` arms
the device-side steady-state test of instance k (the steady driver's slope test
on its Ru series); the step records then carry ``steady`` and
``steady_slope``.  ``graph=False`` launches the kernels one by one instead of
one CUDA graph per step (for kernel profilers).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _capi
from ._device import require_cuda, stream_handle
from .residuals.manager import ResidualManager
from .solvers.solver import finish, prepare

_VP = ctypes.POINTER(ctypes.c_void_p)


class BatchedCavities:
    def __init__(self, configs, states, trackers=None, graph=None):
        require_cuda()
        if len(configs) != len(states) or not configs:
            raise ValueError("one state per config, at least one")
        self.configs = list(configs)
        self.states = list(states)
        self.trackers = list(trackers) if trackers is not None else [ResidualManager() for _ in configs]
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
        self.cells = np.array([int(s.nx) * int(s.ny) for s in self.states], dtype=np.int64)
        # per-instance step bookkeeping (the array form of state.meta's dt_prev / divergence_history)
        self.iterations = np.zeros(n, dtype=np.int64)
        self._dt_prev = np.zeros(n)
        self._hist = np.zeros((n, 5))
        self._hist_len = np.zeros(n, dtype=np.int64)
        for k in range(n):
            self._load_meta(k)
        self._ins = (_capi.StepIn * n)()
        self._outs = (_capi.StepOut * n)()
        self._in_np = np.ctypeslib.as_array(self._ins)
        self._out_np = np.ctypeslib.as_array(self._outs)
        self._ptr = np.zeros((3, n), dtype=np.uint64)
        for k in range(n):
            self.rebind(k)
        h = ctypes.c_void_p()
        _capi.check(_capi.load().pfgb_batch_create(params, n, ctypes.byref(h)), "pfgb_batch_create")
        self._h = h
        if graph is None:
            from .solvers import _handle
            graph = _handle.GRAPH_MODE
        _capi.check(_capi.load().pfgb_set_graph(h, int(graph)), "pfgb_set_graph")
        from .solvers import _handle
        _capi.check(_capi.load().pfgb_set_persistent(h, 1 if _handle.PERSISTENT else 0), "pfgb_set_persistent")
        self._steady = {}
        self.last_out = None
        self.cg_variant = None
        if _handle.AUTOTUNE and not (params[0].precision == 1 and _handle.PERSISTENT):
            key = ("batch",) + tuple(sorted((int(s.nx), int(s.ny)) for s in self.states))
            self.cg_variant = _handle.autotune(h, key, int(params[0].precision))

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

    def workspace_bytes(self) -> int:
        return int(_capi.load().pfgb_workspace_bytes(self._h))

    # ---- bookkeeping -------------------------------------------------------
    def _load_meta(self, k):
        meta = self.states[k].meta
        self._dt_prev[k] = float(meta.get("dt_prev", 1e-2))
        tail = [float(h) for h in meta.get("divergence_history", [])[-5:]]
        self._hist[k] = 0.0
        self._hist[k, :len(tail)] = tail
        self._hist_len[k] = len(tail)

    def reload_meta(self, k=None):
        """Read state.meta of instance k (all if None) into the array bookkeeping, after
        the caller replaced that state's fields and meta (e.g. restored a snapshot)."""
        for j in (range(len(self)) if k is None else [k]):
            self._load_meta(j)

    def sync_meta(self, k=None):
        """Write the array bookkeeping of instance k (all if None) into state.meta."""
        for j in (range(len(self)) if k is None else [k]):
            meta = self.states[j].meta
            meta["dt_prev"] = float(self._dt_prev[j])
            meta["divergence_history"] = [float(h) for h in self._hist[j, :self._hist_len[j]]]
            dx, dy, nu = self._geo[j]
            meta["dx"], meta["dy"], meta["nu"] = dx, dy, nu

    def rebind(self, k):
        """Validate and cache the device pointers of instance k's u, v, p."""
        st = self.states[k]
        shape = (int(st.ny) + 2, int(st.nx) + 2)
        for r, name in enumerate(("u", "v", "p")):
            a = st.fields[name]
            if not (isinstance(a, torch.Tensor) and a.dtype == torch.float64 and a.device.type == "cuda"
                    and tuple(a.shape) == shape and a.is_contiguous()):
                raise ValueError(f"instance {k}: field {name!r} must be a contiguous float64 CUDA tensor of shape {shape}")
            self._ptr[r, k] = a.data_ptr()

    def set_steady(self, k, window, tol=2e-3):
        """Arm (window >= 2) or disarm (window 0) the device-side steady-state test of
        instance k: least-squares slope of log10(Ru) over the last `window` entries of
        its Ru series (seed 1.0, then every step), passed when |slope| < tol.  The
        series restarts from its seed."""
        _capi.check(_capi.load().pfgb_set_steady(self._h, int(k), int(window), float(tol)), "pfgb_set_steady")
        if window:
            self._steady[int(k)] = (int(window), float(tol))
        else:
            self._steady.pop(int(k), None)

    def set_params(self, k, config, reset=True):
        """New physical parameters for slot k (same grid, spacing and precision).

        With reset, the state's fields are zeroed and its bookkeeping, tracker
        and iteration count start afresh (a new request in the slot)."""
        st = self.states[k]
        P, _, geo = prepare(config, st, 0)
        if P.precision != self._params[k].precision:
            raise ValueError("a slot keeps its precision")
        _capi.check(_capi.load().pfgb_batch_set_params(self._h, k, ctypes.byref(P)), "pfgb_batch_set_params")
        self.configs[k] = config
        self._params[k] = P
        self._geo[k] = geo
        if reset:
            for f in st.fields.values():
                f.zero_()
            st.meta.clear()
            self.trackers[k] = ResidualManager()
            self.iterations[k] = 0
            self._load_meta(k)
            if k in self._steady:
                self.set_steady(k, *self._steady[k])

    # ---- stepping ----------------------------------------------------------
    def step_arrays(self, active=None):
        """One step of every active instance; returns a copy of the step records
        (NumPy structured array, field names of pfgb_step_out; rows of inactive
        instances are zero)."""
        n = len(self)
        act = np.ones(n, dtype=bool) if active is None else np.asarray(active, dtype=bool)
        if act.shape != (n,):
            raise ValueError(f"active must have {n} entries")
        ins = self._in_np
        ins["dt_prev"] = self._dt_prev
        ins["hist"] = self._hist
        ins["hist_len"] = self._hist_len
        ins["iteration"] = self.iterations
        ptr = np.where(act, self._ptr, np.uint64(0))
        self._out_np[...] = 0
        _capi.check(_capi.load().pfgb_batch_step(
            self._h, ptr[0].ctypes.data_as(_VP), ptr[1].ctypes.data_as(_VP), ptr[2].ctypes.data_as(_VP),
            self._ins, stream_handle(), self._outs), "pfgb_batch_step")
        out = self._out_np.copy()
        self.last_out = out
        idx = np.nonzero(act)[0]
        self._dt_prev[idx] = out["dt"][idx]
        full = idx[self._hist_len[idx] >= 5]
        part = idx[self._hist_len[idx] < 5]
        self._hist[full, :4] = self._hist[full, 1:]
        self._hist[full, 4] = out["div_before"][full]
        self._hist[part, self._hist_len[part]] = out["div_before"][part]
        self._hist_len[part] += 1
        self.iterations[idx] += 1
        return out

    def continuity(self, out):
        """The reference's continuity residual of each record: ||div||_2 / max(1, nx ny)."""
        return np.sqrt(out["cont_sq"]) / np.maximum(1.0, self.cells.astype(np.float64))

    def step(self, active=None):
        """One step of every active instance; returns [(residuals, diagnostics) or None]."""
        n = len(self)
        act = np.ones(n, dtype=bool) if active is None else np.asarray(active, dtype=bool)
        its = self.iterations.copy()
        self.step_arrays(act)
        results = []
        for k in range(n):
            if not act[k]:
                results.append(None)
                continue
            res, diag = finish(self.configs[k], self.states[k], self.trackers[k], int(its[k]), self._params[k],
                               self._geo[k], self._outs[k])
            results.append((res, diag))
        return results

