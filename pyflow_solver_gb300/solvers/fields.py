"""Device views of a state's fields (host NumPy fields are staged through the GPU)."""
from __future__ import annotations

import contextlib
import weakref

import numpy as np
import torch

from .._device import require_cuda

# Host arrays of at least this many bytes are page-locked in place
# (pfgb_host_register) the first time they are stepped, so that every later
# transfer into and out of them is a direct DMA; smaller arrays, which may share
# pages with other allocations, are copied through torch's pinned buffers.
REGISTER_MIN_BYTES = 1 << 20
_registered: dict[int, weakref.finalize] = {}


def _unregister(ptr: int) -> None:
    _registered.pop(ptr, None)
    try:
        from .. import _capi
        _capi.load().pfgb_host_unregister(ptr)
    except Exception:   # interpreter shutdown: the CUDA context may be gone already
        pass


def _memory_owner(arr):
    o = arr
    while isinstance(o.base, np.ndarray):
        o = o.base
    return o if o.base is None else o.base


def host_registered(arr: np.ndarray) -> bool:
    """Page-lock arr's memory once (unregistered when its owner is freed); False if not possible."""
    if arr.nbytes < REGISTER_MIN_BYTES or not arr.flags.c_contiguous or not arr.flags.writeable:
        return False
    ptr = arr.__array_interface__["data"][0]
    if ptr in _registered:
        return True
    try:
        owner = _memory_owner(arr)
        weakref.ref(owner)
    except TypeError:   # memory owned by an object that takes no weak reference
        return False
    from .. import _capi
    if _capi.load().pfgb_host_register(ptr, arr.nbytes) != 0:
        return False
    _registered[ptr] = weakref.finalize(owner, _unregister, ptr)
    return True


def _mirrors(state, shape):
    """The state's persistent device copies of host fields (stable pointers across steps)."""
    m = getattr(state, "_pfgb_mirror", None)
    if m is None or m[0] != shape:
        m = (shape, {})
        object.__setattr__(state, "_pfgb_mirror", m)
    return m[1]


@contextlib.contextmanager
def device_fields(state):
    """Yield (u, v, p) as contiguous float64 CUDA tensors of shape (ny+2, nx+2).

    CUDA tensors are used in place.  NumPy fields are copied into device copies
    that the state keeps from step to step, and the results are copied back into
    the same arrays on exit (the State keeps its identity and its arrays, as the
    reference's in-place contract requires).  Large host arrays are page-locked
    on first use, so both copies are direct DMA transfers on the current stream.
    """
    require_cuda()
    names = ("u", "v", "p")
    shape = (state.ny + 2, state.nx + 2)
    dev, back = [], []
    mirrors = None
    for k in names:
        a = state.fields[k]
        if isinstance(a, torch.Tensor):
            if a.dtype != torch.float64 or a.device.type != "cuda" or tuple(a.shape) != shape or not a.is_contiguous():
                raise ValueError(f"field {k!r} must be a contiguous float64 CUDA tensor of shape {shape}")
            dev.append(a)
            continue
        arr = np.asarray(a)
        if arr.dtype != np.float64 or arr.shape != shape:
            raise ValueError(f"field {k!r} must be float64 of shape {shape}")
        if mirrors is None:
            mirrors = _mirrors(state, shape)
        t = mirrors.get(k)
        if t is None:
            t = mirrors[k] = torch.empty(shape, dtype=torch.float64, device="cuda")
        if host_registered(arr):
            t.copy_(torch.from_numpy(arr), non_blocking=True)
        else:
            t.copy_(torch.from_numpy(np.ascontiguousarray(arr)).pin_memory(), non_blocking=True)
        dev.append(t)
        back.append((arr, t))
    try:
        yield tuple(dev)
    finally:
        if back:
            for arr, t in back:
                if host_registered(arr):
                    torch.from_numpy(arr).copy_(t, non_blocking=True)
                else:
                    arr[...] = t.cpu().numpy()
            torch.cuda.current_stream().synchronize()
