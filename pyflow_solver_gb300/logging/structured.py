"""JSON-lines step log of the projection step (src/pyflow/logging/structured.py).

``JsonlLogger(path=..., stream=...)`` appends one compact JSON object per
``log(record)`` call, stamped with ``ts`` (seconds since the epoch) unless the
record has one, to a line-buffered file (directories created) or to a caller's
text stream; writes from several threads do not interleave.
``close_all_jsonl_logs()`` closes every logger still open.

``log_step(config, state, iteration, ...)`` is the step's side effect that the
reference writes at the end of ``step`` (src/pyflow/solvers/solver.py:170-192):
with ``config.log_path`` or ``config.log_stream`` set, one ``{"type": "step",
"it", "dt", "CFL", "Ru", "Rv", "continuity", "Rp_it", "nan"}`` record per step
through a logger kept on the config (``config._logger_instance``); when the
step produced a NaN, an ``{"type": "error", "reason": "nan_detected"}`` record
and an emergency checkpoint -- ``<base>_FAIL_NAN.<ext>`` beside
``config.emergency_checkpoint_path``, or ``emergency_FAIL_NAN_it<N>.npz`` --
followed by an ``emergency_checkpoint`` record with its path (or
``"status": "failed"``).
"""
from __future__ import annotations

import json
import os
import threading
import time
import weakref
from typing import IO, Any

_write_lock = threading.Lock()
_open_loggers: weakref.WeakSet = weakref.WeakSet()


class JsonlLogger:
    def __init__(self, path: str | None = None, stream: IO[str] | None = None):
        if path is None and stream is None:
            raise ValueError("JsonlLogger needs a path or a stream")
        self._stream = stream
        self._file = None
        if stream is None:
            os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
            self._file = open(path, "a", encoding="utf-8", buffering=1)
        _open_loggers.add(self)

    def log(self, record: dict[str, Any]) -> None:
        sink = self._stream if self._stream is not None else self._file
        if sink is None:
            return
        record.setdefault("ts", time.time())
        line = json.dumps(record, separators=(",", ":")) + "\n"
        with _write_lock:
            sink.write(line)
            try:
                sink.flush()
            except Exception:
                pass

    def close(self) -> None:
        f, self._file = self._file, None
        if f is not None:
            try:
                f.close()
            except Exception:
                pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def close_all_jsonl_logs() -> None:
    for lg in list(_open_loggers):
        lg.close()


def _logger_for(config):
    lg = getattr(config, "_logger_instance", None)
    if lg is None:
        lg = JsonlLogger(path=getattr(config, "log_path", None), stream=getattr(config, "log_stream", None))
        try:
            config._logger_instance = lg
        except Exception:
            pass
    return lg


def _fail_path(config, iteration: int) -> str:
    ck = getattr(config, "emergency_checkpoint_path", None)
    if not ck:
        return f"emergency_FAIL_NAN_it{iteration}.npz"
    base, _, ext = ck.rpartition(".")
    if not base:
        base, ext = ck, "npz"
    return f"{base}_FAIL_NAN.{ext}"


def log_step(config, state, iteration: int, dt: float, cfl: float, Ru: float, Rv: float, continuity: float,
             rp_iterations: int, nan_detected: bool, diagnostics: dict) -> None:
    """The step's JSON-lines record and, on a NaN, the emergency checkpoint (no-op
    unless the config names a log path or stream)."""
    if not (getattr(config, "log_path", None) or getattr(config, "log_stream", None)):
        return
    lg = _logger_for(config)
    lg.log({"type": "step", "it": iteration, "dt": dt, "CFL": cfl, "Ru": Ru, "Rv": Rv, "continuity": continuity,
            "Rp_it": rp_iterations, "nan": nan_detected})
    if not nan_detected:
        return
    lg.log({"type": "error", "it": iteration, "reason": "nan_detected"})
    path = _fail_path(config, iteration)
    try:
        from ..io.checkpoint import save_checkpoint
        save_checkpoint(path, state, iteration, diagnostics.get("time", diagnostics.get("wall_time", 0.0)), config)
        lg.log({"type": "emergency_checkpoint", "path": path, "it": iteration})
    except Exception:
        lg.log({"type": "emergency_checkpoint", "status": "failed", "it": iteration})


__all__ = ["JsonlLogger", "close_all_jsonl_logs", "log_step"]
