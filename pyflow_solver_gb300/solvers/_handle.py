"""Per-state cache of the native instance handle (libpfgb.so ``pfgb_handle``)."""
from __future__ import annotations

import ctypes

from .. import _capi


# Run each step as one CUDA graph (True) or as individual kernel launches.
GRAPH_MODE = True


class Instance:
    """Owns one ``pfgb_handle`` (device workspace of one cavity)."""

    def __init__(self, params: _capi.Params):
        lib = _capi.load()
        h = ctypes.c_void_p()
        _capi.check(lib.pfgb_create(ctypes.byref(params), ctypes.byref(h)), "pfgb_create")
        self._h = h
        self.params = params
        _capi.check(lib.pfgb_set_graph(h, 1 if GRAPH_MODE else 0), "pfgb_set_graph")

    @property
    def handle(self):
        return self._h

    def workspace_bytes(self) -> int:
        return int(_capi.load().pfgb_workspace_bytes(self._h))

    def close(self):
        if self._h is not None and self._h.value:
            _capi.load().pfgb_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def params_key(p: _capi.Params):
    return (p.nx, p.ny, p.dx, p.dy, p.nu, p.cfl_target, p.cfl_growth, p.lin_tol, p.lin_maxiter, p.scheme,
            p.enable_jacobi, p.jacobi_interior, p.has_lid, p.lid_velocity, p.precision, p.mixed_tol_outer,
            p.mixed_tol_inner, p.mixed_max_outer, p.mixed_max_inner)


def instance_for(state, params: _capi.Params, slot: str = "_pfgb_step") -> Instance:
    key = params_key(params)
    cached = getattr(state, slot, None)
    if cached is not None and cached[0] == key:
        return cached[1]
    if cached is not None:
        cached[1].close()
    inst = Instance(params)
    object.__setattr__(state, slot, (key, inst))
    return inst
