"""Simulation config with the reference's fields, ranges and hash.

Mirrors ``SimulationConfig`` of src/pyflow/config/model.py:15-99 without
pydantic: the same field names and defaults, the same range checks (raising
``ConfigError``, a ValueError), and the same ``config_hash`` (sha1 of the
canonical JSON of every field except ``log_stream`` and ``force_quiet``, first
12 hex digits), so checkpoints written by either side carry comparable hashes.
``precision`` is this package's addition ("fp64" or "mixed"); it joins the
hash only when it is not the default, so binary64 configs hash as in the
reference.
"""
from __future__ import annotations

import hashlib
import json
from dataclasses import asdict, dataclass, fields
from typing import Any


class ConfigError(ValueError):
    pass


@dataclass
class SimulationConfig:
    nx: int
    ny: int
    Re: float = 100.0
    lid_velocity: float = 1.0
    cfl_target: float = 0.5
    cfl_growth: float = 1.05
    lin_tol: float = 1e-10
    lin_maxiter: int = 200
    advection_scheme: str = "upwind"
    disable_advection: bool = False
    diagnostics: bool = True
    log_path: str | None = None
    log_stream: Any | None = None
    force_quiet: bool = False
    checkpoint_interval: int | None = None
    emergency_checkpoint_path: str | None = None
    seed: int | None = None
    schema_version: int = 1
    turbulence_model: str | None = None
    precision: str = "fp64"

    def __post_init__(self):
        issues = []

        def check(cond, msg):
            if not cond:
                issues.append(msg)

        check(isinstance(self.nx, int) and self.nx >= 3, "nx: must be an integer >= 3")
        check(isinstance(self.ny, int) and self.ny >= 3, "ny: must be an integer >= 3")
        check(self.Re > 0.0, "Re: must be > 0")
        check(0.0 < self.cfl_target <= 1.0, "cfl_target: must be in (0, 1]")
        check(1.0 < self.cfl_growth <= 1.2, "cfl_growth: must be in (1, 1.2]")
        check(1e-14 <= self.lin_tol <= 1e-2, "lin_tol: must be in [1e-14, 1e-2]")
        check(isinstance(self.lin_maxiter, int) and 1 <= self.lin_maxiter <= 10000, "lin_maxiter: must be in [1, 10000]")
        check(self.advection_scheme in ("upwind", "quick"), "advection_scheme: must be 'upwind' or 'quick'")
        check(self.checkpoint_interval is None or self.checkpoint_interval >= 1, "checkpoint_interval: must be >= 1")
        check(self.seed is None or 0 <= self.seed <= 2**32 - 1, "seed: must be in [0, 2**32-1]")
        check(self.precision in ("fp64", "mixed"), "precision: must be 'fp64' or 'mixed'")
        if self.log_path and self.log_stream is not None:
            issues.append("log_path and log_stream are mutually exclusive")
        if issues:
            raise ConfigError("; ".join(issues))

    def hash_payload(self) -> dict:
        data = {f.name: getattr(self, f.name) for f in fields(self)}
        for k in ("log_stream", "force_quiet"):
            data.pop(k, None)
        if data.get("precision") == "fp64":
            data.pop("precision")
        return data

    @property
    def config_hash(self) -> str:
        blob = json.dumps(self.hash_payload(), sort_keys=True, separators=(",", ":")).encode()
        return hashlib.sha1(blob).hexdigest()[:12]

    def model_dump(self) -> dict:
        d = asdict(self)
        d.pop("log_stream", None)
        return d

    def brief(self) -> dict:
        return {"nx": self.nx, "ny": self.ny, "Re": self.Re,
                "scheme": (None if self.disable_advection else self.advection_scheme),
                "lin_tol": self.lin_tol, "lin_maxiter": self.lin_maxiter, "cfl_target": self.cfl_target,
                "cfl_growth": self.cfl_growth, "hash": self.config_hash}
