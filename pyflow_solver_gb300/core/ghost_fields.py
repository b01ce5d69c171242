"""Simulation state with ghosted device fields.

Mirrors src/pyflow/core/ghost_fields.py:8-60: ``State{nx, ny, fields, meta}``,
fields of shape (ny+2, nx+2) float64 whose ghost ring is never read or written
by the step (the lid lives on the top interior row), ``interior_view(a) ==
a[1:-1, 1:-1]``.  Fields here are CUDA tensors owned by PyTorch.
"""
from __future__ import annotations

from collections.abc import Mapping
from dataclasses import dataclass, field
from typing import Any

import torch


@dataclass
class State:
    nx: int
    ny: int
    fields: dict[str, Any]
    meta: dict[str, Any] = field(default_factory=dict)

    def arr(self, name: str):
        return self.fields[name]

    def __getitem__(self, key: str):
        return self.fields[key]

    def __setitem__(self, key: str, value) -> None:
        self.fields[key] = value

    def get(self, key: str, default=None):
        if key in self.fields:
            return self.fields[key]
        return self.meta.get(key, default)

    def set_meta(self, key: str, value: Any) -> None:
        self.meta[key] = value

    def keys(self):
        return self.fields.keys()

    def items(self):
        return self.fields.items()

    def values(self):
        return self.fields.values()


def allocate_state(nx: int, ny: int, fields: tuple[str, ...] = ("u", "v", "p"), device="cuda") -> State:
    """Zero float64 fields of shape (ny+2, nx+2) on the GPU."""
    shape = (ny + 2, nx + 2)
    arrs = {k: torch.zeros(shape, dtype=torch.float64, device=device) for k in fields}
    return State(nx=nx, ny=ny, fields=arrs)


def interior_view(arr):
    return arr[1:-1, 1:-1]


def ghost_shapes(state: Mapping | State) -> dict[str, tuple[int, int]]:
    items = state.fields.items() if isinstance(state, State) else state.items()
    return {k: tuple(v.shape) for k, v in items if hasattr(v, "shape")}
