"""Device plumbing shared by the host modules (torch owns memory and streams)."""
from __future__ import annotations

import numpy as np
import torch

from . import _capi


def require_cuda():
    if not torch.cuda.is_available():
        raise _capi.PFGBError("a CUDA device is required (there is no CPU fallback)")
    _capi.load()


def stream_handle() -> int:
    return torch.cuda.current_stream().cuda_stream


def to_device(a):
    """Return (float64 CUDA tensor, was_host). Host arrays are copied."""
    require_cuda()
    if isinstance(a, torch.Tensor):
        if a.dtype != torch.float64:
            raise TypeError("arrays must be float64")
        if a.device.type != "cuda":
            return a.to("cuda"), True
        return a, False
    arr = np.asarray(a, dtype=np.float64)
    return torch.from_numpy(np.ascontiguousarray(arr)).to("cuda"), True


def row_pitch(t: torch.Tensor) -> tuple[torch.Tensor, int]:
    """A 2-D tensor with unit column stride and its row pitch (in elements)."""
    if t.dim() != 2:
        raise ValueError("expected a 2-D array")
    if t.stride(1) != 1:
        t = t.contiguous()
    return t, t.stride(0) if t.shape[0] > 1 else t.shape[1]


def ptr(t: torch.Tensor) -> int:
    return t.data_ptr()
