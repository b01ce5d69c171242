"""Per-state cache of the native instance handle (libpfgb.so ``pfgb_handle``)."""
from __future__ import annotations

import ctypes
import json
import os

from .. import _capi


# Run each step as one CUDA graph (True; 2: without programmatic dependent-launch
# edges) or as individual kernel launches (False).
GRAPH_MODE = True
# Mixed form: the pressure solve as one persistent cooperative launch (True) or
# as a graph of per-phase kernels (False, the faster on GB300); both give the same bits.
PERSISTENT = False
# Pick the launch shape of the pressure solve by timing (pfgb_autotune) once per grid
# size or batch composition: the binary64 CG tile shape, or the mixed solve's matvec
# form and coarse CTA width.  Every shape gives the same bits.
AUTOTUNE = True
_TUNED: dict = {}
_CACHE_LOADED = False


def tune_cache_path() -> str:
    """The JSON file that keeps the tuner's choices between processes (PFGB_TUNE_CACHE,
    default ~/.cache/pyflow_solver_gb300/tune.json; "" turns the file off)."""
    p = os.environ.get("PFGB_TUNE_CACHE")
    if p is not None:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "pyflow_solver_gb300", "tune.json")


def _cache_key(precision: int, key) -> str:
    """Device, precision and the grid (or the batch's sorted grids, as a digest)."""
    import hashlib

    import torch
    text = json.dumps(list(key))
    if len(text) > 64:
        text = f"{key[0]}:{len(key) - 1}:" + hashlib.sha1(text.encode()).hexdigest()[:16]
    return f"{torch.cuda.get_device_name()}|p{precision}|{text}"


def _load_cache():
    global _CACHE_LOADED
    if _CACHE_LOADED:
        return
    _CACHE_LOADED = True
    path = tune_cache_path()
    try:
        with open(path) as f:
            data = json.load(f)
        _TUNED.update({k: int(v) for k, v in data.get("choices", {}).items()})
    except (OSError, ValueError, AttributeError):
        pass


def _save_cache():
    path = tune_cache_path()
    if not path:
        return
    try:
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        tmp = f"{path}.{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump({"choices": _TUNED}, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def autotune(handle, key, precision: int = 0) -> int:
    """Launch variant of this handle's pressure solve: timed once per key (and device),
    then reused from memory or the JSON cache."""
    lib = _capi.load()
    _load_cache()
    ck = _cache_key(precision, key)
    setter = lib.pfgb_set_cg_variant if precision == 0 else lib.pfgb_set_mixed_variant
    if ck in _TUNED and setter(handle, _TUNED[ck]) == 0:
        return _TUNED[ck]
    from .._device import stream_handle
    v = ctypes.c_int()
    _capi.check(lib.pfgb_autotune(handle, stream_handle(), ctypes.byref(v), None), "pfgb_autotune")
    _TUNED[ck] = v.value
    _save_cache()
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
        if AUTOTUNE and not (params.precision == 1 and PERSISTENT):
            self.cg_variant = autotune(h, ("single", params.nx, params.ny), params.precision)

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
