"""Checkpoint files in the reference's format (src/pyflow/io/checkpoint.py:51-127).

``.npz`` with a JSON ``meta`` entry (iteration, time, nx, ny, config_hash,
structured_config_hash, field_hashes, seed, schema_version) and one
``field_<name>`` array per field including ghosts; written atomically
(temporary file, fsync, replace).  Device fields are copied to the host.

One addition: ``meta["state_meta"]`` keeps the step bookkeeping of
``state.meta`` (``dt_prev`` and the last five divergence norms, which set the
next dt and the safeguard), and ``load_checkpoint`` puts it back, so that a run
restarted from a checkpoint continues exactly as the uninterrupted run would.
The reference writes no such entry and restarts with fresh bookkeeping (dt_prev
1e-2); files without it load the same way here.  Readers that do not know the
key ignore it.
"""
from __future__ import annotations

import hashlib
import io
import json
import os
import tempfile
from typing import Any

import numpy as np

from ..core.ghost_fields import State


def _host(a) -> np.ndarray:
    return a.detach().cpu().numpy() if hasattr(a, "detach") else np.asarray(a)


def _hash_config(cfg: Any) -> str:
    try:
        if hasattr(cfg, "__dict__"):
            data = {k: v for k, v in vars(cfg).items() if not k.startswith("_")}
        else:
            data = {k: getattr(cfg, k) for k in dir(cfg) if not k.startswith("_")}
        blob = json.dumps(data, sort_keys=True, default=str).encode()
        return hashlib.sha1(blob).hexdigest()[:10]
    except Exception:
        return "unknown"


def _hash_array(arr: np.ndarray) -> str:
    return hashlib.sha1(arr.tobytes()).hexdigest()[:16]


def _structured_hash(cfg):
    """The SimulationConfig hash, only for a SimulationConfig (as the reference does)."""
    from ..config.model import SimulationConfig
    if isinstance(cfg, SimulationConfig):
        try:
            return cfg.config_hash
        except Exception:
            return None
    return None


def _state_meta(state):
    meta = getattr(state, "meta", None) or {}
    if "dt_prev" not in meta:
        return None
    return {"dt_prev": float(meta["dt_prev"]),
            "divergence_history": [float(h) for h in meta.get("divergence_history", [])][-5:]}


def _meta(state, iteration, sim_time, cfg, arrays, structured=True):
    m = {
        "iteration": iteration, "time": sim_time, "nx": state.nx, "ny": state.ny,
        "config_hash": _hash_config(cfg),
    }
    if structured:
        m["structured_config_hash"] = _structured_hash(cfg)
    m.update({"field_hashes": {k: _hash_array(v) for k, v in arrays.items()},
              "seed": getattr(cfg, "seed", None), "schema_version": 1})
    sm = _state_meta(state)
    if sm is not None:
        m["state_meta"] = sm
    return m


def _state_from(meta, fields, device):
    if device is not None:
        import torch
        fields = {k: torch.from_numpy(v).to(device) for k, v in fields.items()}
    st = State(nx=meta.get("nx"), ny=meta.get("ny"), fields=fields)
    sm = meta.get("state_meta")
    if isinstance(sm, dict) and "dt_prev" in sm:
        st.meta = {"dt_prev": float(sm["dt_prev"]),
                   "divergence_history": [float(h) for h in sm.get("divergence_history", [])]}
    return st


def save_checkpoint(path: str, state: State, iteration: int, sim_time: float, cfg: Any) -> str:
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    arrays = {k: _host(v) for k, v in state.fields.items()}
    meta = _meta(state, iteration, sim_time, cfg, arrays)
    fd, tmp = tempfile.mkstemp(suffix=".tmp", dir=os.path.dirname(path) or ".")
    try:
        with os.fdopen(fd, "wb") as f:
            np.savez_compressed(f, meta=json.dumps(meta), **{f"field_{k}": v for k, v in arrays.items()})
            f.flush()
            try:
                os.fsync(f.fileno())
            except OSError:
                pass
        os.replace(tmp, path)
    finally:
        if os.path.exists(tmp):
            try:
                os.remove(tmp)
            except Exception:
                pass
    return path


def load_checkpoint(path: str, device: str | None = None) -> tuple[State, dict[str, Any]]:
    """The state (NumPy fields, as the reference returns them; or tensors on
    `device`) and the meta entry of a checkpoint file."""
    with np.load(path) as data:
        meta = json.loads(str(data["meta"]))
        fields = {k.removeprefix("field_"): data[k].copy() for k in data.files if k.startswith("field_")}
    return _state_from(meta, fields, device), meta


def save_checkpoint_bytes(state: State, iteration: int, sim_time: float, cfg: Any) -> bytes:
    arrays = {k: _host(v) for k, v in state.fields.items()}
    meta = _meta(state, iteration, sim_time, cfg, arrays, structured=False)
    bio = io.BytesIO()
    np.savez_compressed(bio, meta=json.dumps(meta), **{f"field_{k}": v for k, v in arrays.items()})
    return bio.getvalue()


def load_checkpoint_bytes(buf: bytes, device: str | None = None) -> tuple[State, dict[str, Any]]:
    with np.load(io.BytesIO(buf)) as data:
        meta = json.loads(str(data["meta"]))
        fields = {k.removeprefix("field_"): data[k].copy() for k in data.files if k.startswith("field_")}
    return _state_from(meta, fields, device), meta


__all__ = ["save_checkpoint", "load_checkpoint", "save_checkpoint_bytes", "load_checkpoint_bytes"]
