"""Call helpers for the array operators of libpfgb.so."""
from __future__ import annotations

import numpy as np
import torch

from .. import _capi
from .._device import ptr, require_cuda, row_pitch, stream_handle, to_device


def prepare(*arrays):
    """Device tensors with unit column stride, their pitches, and whether any input was on the host."""
    require_cuda()
    outs, host = [], False
    for a in arrays:
        t, h = to_device(a)
        t, _ = row_pitch(t)
        outs.append(t)
        host = host or h
    shape = tuple(outs[0].shape)
    for t in outs[1:]:
        if tuple(t.shape) != shape:
            raise ValueError("operand shapes differ")
    # one common pitch: make everything contiguous when pitches differ
    pitches = {t.stride(0) for t in outs}
    if len(pitches) > 1:
        outs = [t.contiguous() for t in outs]
    return outs, outs[0].stride(0), host


def finish(out: torch.Tensor, host: bool):
    if host:
        return out.cpu().numpy()
    return out


def empty_like(t: torch.Tensor) -> torch.Tensor:
    return torch.empty(t.shape, dtype=torch.float64, device=t.device)


def call(name: str, *args):
    fn = getattr(_capi.load(), name)
    _capi.check(fn(*args), name)


__all__ = ["prepare", "finish", "empty_like", "call", "ptr", "stream_handle", "np"]
