"""QUICK and first-order upwind convective derivatives on the GPU.

Same values as src/pyflow/numerics/operators/advection.py:17-84 (the reference's
per-cell Python loops): QUICK with edge padding by two cells and the sign test
``u >= 0``; upwind with the sign test ``u > 0`` and clamped one-sided edges.
"""
from __future__ import annotations

from ... import _capi
from .._launch import call, empty_like, finish, prepare, ptr, stream_handle

__all__ = ["advect_quick", "advect_upwind"]


def _advect(scheme, u, v, field, dx, dy):
    (ut, vt, ft), ld, host = prepare(u, v, field)
    ny, nx = ft.shape
    if nx < 2 or ny < 2:
        raise ValueError("advection kernels need nx, ny >= 2")
    out = empty_like(ft)
    call("pfgb_advect", scheme, ptr(ut), ptr(vt), ptr(ft), ld, ptr(out), nx, nx, ny, float(dx), float(dy),
         stream_handle())
    return finish(out, host)


def advect_upwind(u, v, field, dx, dy):
    return _advect(_capi.SCHEME_UPWIND, u, v, field, dx, dy)


def advect_quick(u, v, field, dx, dy):
    return _advect(_capi.SCHEME_QUICK, u, v, field, dx, dy)
