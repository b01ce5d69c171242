"""Per-state cache of the native instance handle (libpfgb.so ``pfgb_handle``)."""
from __future__ import annotations

import ctypes

from .. import _capi


# Run each step as one CUDA graph (True; 2: without programmatic dependent-launch
# edges) or as individual kernel launches (False).
GRAPH_MODE = True
# Mixed form: the pressure solve as one persistent cooperative launch (True) or
# as a graph of per-phase kernels (False, the faster on GB300); both give the same bits.
PERSISTENT = False
# Pick the binary64 CG tile shape by timing (pfgb_autotune) once per grid size.
AUTOTUNE = True
_TUNED: dict = {}


def autotune(handle, key) -> int:
    """Tile variant of the binary64 CG kernels for this handle: timed once per key, then reused."""
    lib = _capi.load()
    if key in _TUNED:
        _capi.check(lib.pfgb_set_cg_variant(handle, _TUNED[key]), "pfgb_set_cg_variant")
        return _TUNED[key]
    from .._device import stream_handle
    v = ctypes.c_int()
    _capi.check(lib.pfgb_autotune(handle, stream_handle(), ctypes.byref(v), None), "pfgb_autotune")
    _TUNED[key] = v.value
    return v.value


class Instance:
    """Owns one ``pfgb_handle`` (device workspace of one cavity)."""

    def __init__(self, params: _capi.Params):
        lib = _capi.load()
        h = ctypes.c_void_p()
        _capi.check(lib.pfgb_create(ctypes.byref(params), ctypes.byref(h)), "pfgb_create")
        self._h = h
        self.params = params
        _capi.check(lib.pfgb_set_graph(h, int(GRAPH_MODE)), "pfgb_set_graph")
        _capi.check(lib.pfgb_set_persistent(h, 1 if PERSISTENT else 0), "pfgb_set_persistent")
        self.cg_variant = None
        if AUTOTUNE and params.precision == 0:
            self.cg_variant = autotune(h, ("single", params.nx, params.ny))

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
            p.mixed_tol_inner, p.mixed_max_outer, p.mixed_max_inner, p.mixed_cold_start)


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
