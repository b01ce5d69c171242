"""Central-difference divergence on the GPU (src/pyflow/numerics/fluid_ops.py:8-41).

One-sided differences on the edges and corners; the last column of rows
1..ny-2 is left at zero exactly as the reference leaves it.
"""
from __future__ import annotations

from ._launch import call, empty_like, finish, prepare, ptr, stream_handle

__all__ = ["divergence"]


def divergence(u, v, dx: float, dy: float):
    (ut, vt), ld, host = prepare(u, v)
    ny, nx = ut.shape
    if nx < 2 or ny < 2:
        raise IndexError("divergence needs at least two rows and two columns (as the reference indexes them)")
    d = empty_like(ut)
    call("pfgb_divergence_central", ptr(ut), ptr(vt), ld, ptr(d), nx, nx, ny, float(dx), float(dy), stream_handle())
    return finish(d, host)
