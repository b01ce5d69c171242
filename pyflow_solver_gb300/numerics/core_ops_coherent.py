"""Coherent forward-gradient / backward-divergence pair on the GPU.

Same contract as src/pyflow/numerics/core_ops_coherent.py:45-84:
``laplacian_coherent(p) == divergence_coherent(*gradient_coherent(p))`` bit for
bit.  Inputs are (ny, nx) float64 arrays (CUDA tensors, or host arrays that are
copied and returned as NumPy arrays).
"""
from __future__ import annotations

import torch

from ._launch import call, empty_like, finish, prepare, ptr, stream_handle

__all__ = ["divergence_coherent", "gradient_coherent", "laplacian_coherent"]


def _degenerate(t):
    return t.shape[0] < 2 or t.shape[1] < 2


def gradient_coherent(p, dx: float, dy: float):
    (pt,), ld, host = prepare(p)
    ny, nx = pt.shape
    if _degenerate(pt):
        z = torch.zeros_like(pt)
        return finish(z, host), finish(z.clone(), host)
    gx, gy = empty_like(pt), empty_like(pt)
    call("pfgb_gradient_coherent", ptr(pt), ld, ptr(gx), ptr(gy), nx, nx, ny, float(dx), float(dy), stream_handle())
    return finish(gx, host), finish(gy, host)


def divergence_coherent(u, v, dx: float, dy: float):
    (ut, vt), ld, host = prepare(u, v)
    ny, nx = ut.shape
    if _degenerate(ut):
        return finish(torch.zeros_like(ut), host)
    d = empty_like(ut)
    call("pfgb_divergence_coherent", ptr(ut), ptr(vt), ld, ptr(d), nx, nx, ny, float(dx), float(dy), stream_handle())
    return finish(d, host)


def laplacian_coherent(p, dx: float, dy: float):
    (pt,), ld, host = prepare(p)
    ny, nx = pt.shape
    if _degenerate(pt):
        return finish(torch.zeros_like(pt), host)
    out = empty_like(pt)
    call("pfgb_laplacian_coherent", ptr(pt), ld, ptr(out), nx, nx, ny, float(dx), float(dy), stream_handle())
    return finish(out, host)
