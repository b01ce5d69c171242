"""ctypes binding of libpfgb.so (the C ABI declared in include/pfgb.h).

The library is built in-tree by ``pyflow_solver_gb300._build``.  There is no
CPU fallback: if the library is missing or a CUDA device is absent, the calls
raise.
"""
from __future__ import annotations

import ctypes
import os

from ._build import LIB

c_double_p = ctypes.POINTER(ctypes.c_double)


class Params(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double),
        ("nu", ctypes.c_double),
        ("cfl_target", ctypes.c_double), ("cfl_growth", ctypes.c_double),
        ("lin_tol", ctypes.c_double), ("lin_maxiter", ctypes.c_int),
        ("scheme", ctypes.c_int), ("enable_jacobi", ctypes.c_int),
        ("jacobi_interior", ctypes.c_double),
        ("has_lid", ctypes.c_int), ("lid_velocity", ctypes.c_double),
        ("precision", ctypes.c_int),
        ("mixed_tol_outer", ctypes.c_double), ("mixed_tol_inner", ctypes.c_double),
        ("mixed_max_outer", ctypes.c_int), ("mixed_max_inner", ctypes.c_int),
        ("mixed_cold_start", ctypes.c_int),
        ("reserved", ctypes.c_int * 3),
    ]


class StepIn(ctypes.Structure):
    _fields_ = [
        ("dt_prev", ctypes.c_double), ("hist", ctypes.c_double * 5),
        ("hist_len", ctypes.c_int), ("iteration", ctypes.c_int),
    ]


class StepOut(ctypes.Structure):
    _fields_ = [
        ("umax", ctypes.c_double), ("vmax", ctypes.c_double),
        ("div_before", ctypes.c_double), ("dt", ctypes.c_double), ("cfl", ctypes.c_double),
        ("safeguard", ctypes.c_int), ("cg_iterations", ctypes.c_int),
        ("cg_info", ctypes.c_int), ("nan_detected", ctypes.c_int),
        ("divstar_sq", ctypes.c_double), ("bnorm", ctypes.c_double),
        ("res_sq", ctypes.c_double), ("ru_sq", ctypes.c_double), ("rv_sq", ctypes.c_double),
        ("divafter_sq", ctypes.c_double), ("linres_sq", ctypes.c_double),
        ("cont_sq", ctypes.c_double),
        ("reduction_flags", ctypes.c_uint), ("refine_passes", ctypes.c_int),
        ("steady_slope", ctypes.c_double), ("steady", ctypes.c_int),
    ]


class SolveOut(ctypes.Structure):
    _fields_ = [
        ("info", ctypes.c_int), ("iterations", ctypes.c_int),
        ("bnorm", ctypes.c_double), ("res_sq", ctypes.c_double),
    ]


class KernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 48), ("launches", ctypes.c_int), ("total_ms", ctypes.c_double)]


# name -> (restype, argtypes)
_P = ctypes.c_void_p
_L = ctypes.c_long
_I = ctypes.c_int
_D = ctypes.c_double
SIGNATURES = {
    "pfgb_version": (_I, []),
    "pfgb_last_error": (_I, [ctypes.c_char_p, ctypes.c_size_t]),
    "pfgb_create": (_I, [ctypes.POINTER(Params), ctypes.POINTER(_P)]),
    "pfgb_destroy": (_I, [_P]),
    "pfgb_workspace_bytes": (ctypes.c_size_t, [_P]),
    "pfgb_step": (_I, [_P, _P, _P, _P, _L, ctypes.POINTER(StepIn), _P, ctypes.POINTER(StepOut)]),
    "pfgb_project": (_I, [_P, _P, _P, _P, _L, _D, _P, ctypes.POINTER(StepOut)]),
    "pfgb_batch_create": (_I, [ctypes.POINTER(Params), _I, ctypes.POINTER(_P)]),
    "pfgb_batch_step": (_I, [_P, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(StepIn), _P,
                             ctypes.POINTER(StepOut)]),
    "pfgb_batch_size": (_I, [_P]),
    "pfgb_batch_set_params": (_I, [_P, _I, ctypes.POINTER(Params)]),
    "pfgb_gradient_coherent": (_I, [_P, _L, _P, _P, _L, _I, _I, _D, _D, _P]),
    "pfgb_divergence_coherent": (_I, [_P, _P, _L, _P, _L, _I, _I, _D, _D, _P]),
    "pfgb_laplacian_coherent": (_I, [_P, _L, _P, _L, _I, _I, _D, _D, _P]),
    "pfgb_divergence_central": (_I, [_P, _P, _L, _P, _L, _I, _I, _D, _D, _P]),
    "pfgb_advect": (_I, [_I, _P, _P, _P, _L, _P, _L, _I, _I, _D, _D, _P]),
    "pfgb_apply_operator": (_I, [_I, _P, _P, _I, _I, _D, _D, _P]),
    "pfgb_div_by_constant": (_I, [_P, _P, _L, _D, _I, _P]),
    "pfgb_xdot": (_I, [_P, _P, _L, c_double_p, _P]),
    "pfgb_xsum": (_I, [_P, _L, c_double_p, _P]),
    "pfgb_cg_solve": (_I, [_I, _P, _P, _I, _I, _D, _D, _I, _D, _D, _I, _P, ctypes.POINTER(SolveOut)]),
    "pfgb_cg_solve_noalloc": (_I, [_I, _P, _P, _I, _I, _D, _D, _I, _D, _D, _I, _P, ctypes.POINTER(SolveOut)]),
    "pfgb_csr_matvec": (_I, [_L, _P, _P, _P, _P, _P, _P]),
    "pfgb_csr_solve": (_I, [_I, _L, _P, _P, _P, _P, _P, _P, _D, _I, _P, ctypes.POINTER(SolveOut)]),
    "pfgb_set_graph": (_I, [_P, _I]),
    "pfgb_set_persistent": (_I, [_P, _I]),
    "pfgb_matvec_form": (_I, [_P, ctypes.POINTER(_I)]),
    "pfgb_host_register": (_I, [_P, ctypes.c_size_t]),
    "pfgb_host_unregister": (_I, [_P]),
    "pfgb_autotune": (_I, [_P, _P, ctypes.POINTER(_I), c_double_p]),
    "pfgb_set_cg_variant": (_I, [_P, _I]),
    "pfgb_set_mixed_variant": (_I, [_P, _I]),
    "pfgb_set_profiling": (_I, [_P, _I]),
    "pfgb_profile_result": (_I, [_P, c_double_p, ctypes.POINTER(_I)]),
    "pfgb_profile_kernels": (_I, [_P, ctypes.POINTER(KernelTime), _I, ctypes.POINTER(_I)]),
    "pfgb_set_steady": (_I, [_P, _I, _I, _D]),
    "pfgb_probe_fp64": (_I, [_P, c_double_p]),
    "pfgb_selftest_conversions": (_I, [_L, _P, ctypes.POINTER(ctypes.c_longlong)]),
}

SCHEME_UPWIND, SCHEME_QUICK, SCHEME_NONE = 0, 1, 2
OP_NEG_LAPLACIAN_PINNED, OP_LAPLACIAN_DIRICHLET = 0, 1

_lib = None


class PFGBError(RuntimeError):
    pass


def load(path: str | None = None):
    """Load libpfgb.so (once) and declare its signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB
    if not os.path.exists(path):
        raise PFGBError(
            f"{path} is missing: build it with `python -m pyflow_solver_gb300._build` "
            "(there is no CPU fallback)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    load().pfgb_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, what: str):
    if rc != 0:
        raise PFGBError(f"{what} failed ({rc}): {last_error()}")


def profile_kernels(handle) -> list:
    """Per-kernel device time of the last profiled step of a handle:
    [(name, launches, total_ms)] in order of first launch."""
    lib = load()
    cap = 64
    while True:
        buf = (KernelTime * cap)()
        n = ctypes.c_int()
        check(lib.pfgb_profile_kernels(handle, buf, cap, ctypes.byref(n)), "pfgb_profile_kernels")
        if n.value <= cap:
            return [(buf[k].name.decode(), int(buf[k].launches), float(buf[k].total_ms)) for k in range(n.value)]
        cap = n.value
