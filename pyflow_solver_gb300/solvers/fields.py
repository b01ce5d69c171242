"""Device views of a state's fields (host NumPy fields are staged through the GPU)."""
from __future__ import annotations

import contextlib

import numpy as np
import torch

from .._device import require_cuda


@contextlib.contextmanager
def device_fields(state):
    """Yield (u, v, p) as contiguous float64 CUDA tensors of shape (ny+2, nx+2).

    CUDA tensors are used in place.  NumPy fields are copied to the device and
    the results copied back into the same arrays on exit (the State keeps its
    identity and its arrays, as the reference's in-place contract requires).
    """
    require_cuda()
    names = ("u", "v", "p")
    shape = (state.ny + 2, state.nx + 2)
    dev, back = [], []
    for k in names:
        a = state.fields[k]
        if isinstance(a, torch.Tensor):
            if a.dtype != torch.float64 or a.device.type != "cuda" or tuple(a.shape) != shape or not a.is_contiguous():
                raise ValueError(f"field {k!r} must be a contiguous float64 CUDA tensor of shape {shape}")
            dev.append(a)
        else:
            arr = np.asarray(a)
            if arr.dtype != np.float64 or arr.shape != shape:
                raise ValueError(f"field {k!r} must be float64 of shape {shape}")
            t = torch.from_numpy(np.ascontiguousarray(arr)).pin_memory().to("cuda", non_blocking=True)
            dev.append(t)
            back.append((arr, t))
    try:
        yield tuple(dev)
    finally:
        for arr, t in back:
            arr[...] = t.cpu().numpy()
