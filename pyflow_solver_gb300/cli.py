"""Command line front-end: ``python -m pyflow_solver_gb300 run|validate|show-config``.

Same arguments, JSON-line stream and exit codes as src/pyflow/cli.py:35-194:
``run --json-stream`` prints one ``{"type": "step", "iteration", "dt", "CFL",
"continuity", "wall_time", "residuals": {...}, "diagnostics": {...}}`` line per
step; exit 2 on an invalid config, 3 when a restart checkpoint's config hash
differs (unless --allow-hash-mismatch), 130 after Ctrl-C (with a final
checkpoint).  ``--precision mixed`` selects the mixed-precision pressure solve.
"""
from __future__ import annotations

import argparse
import json
import sys

from .config.model import ConfigError, SimulationConfig


def build_parser() -> argparse.ArgumentParser:
    p = argparse.ArgumentParser(description="PyFlow projection step on GB300")
    sub = p.add_subparsers(dest="command", required=True)

    def add_common(sp):
        sp.add_argument("--nx", type=int, default=64)
        sp.add_argument("--ny", type=int, default=64)
        sp.add_argument("--re", type=float, default=100.0)
        sp.add_argument("--lid-velocity", type=float, default=1.0)
        sp.add_argument("--scheme", choices=["quick", "upwind"], default="quick")
        sp.add_argument("--disable-advection", action="store_true")
        sp.add_argument("--cfl", type=float, default=0.5)
        sp.add_argument("--cfl-growth", type=float, default=1.05)
        sp.add_argument("--lin-tol", type=float, default=1e-10)
        sp.add_argument("--lin-maxiter", type=int, default=300)
        sp.add_argument("--checkpoint-interval", type=int, default=0)
        sp.add_argument("--log-jsonl", type=str, default=None)
        sp.add_argument("--seed", type=int, default=None)
        sp.add_argument("--diagnostics", action="store_true")
        sp.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")

    run_p = sub.add_parser("run", help="Run a simulation")
    add_common(run_p)
    run_p.add_argument("--steps", type=int, default=100)
    run_p.add_argument("--checkpoint", type=str, default=None)
    run_p.add_argument("--restart", type=str, default=None)
    run_p.add_argument("--allow-hash-mismatch", action="store_true")
    run_p.add_argument("--json-stream", action="store_true")
    run_p.add_argument("--continuity-threshold", type=float, default=None)
    run_p.add_argument("--progress", action="store_true")
    run_p.add_argument("--assert-invariants", action="store_true")
    add_common(sub.add_parser("validate", help="Validate and display normalized config"))
    add_common(sub.add_parser("show-config", help="Show normalized config (hash only)"))
    return p


def step_payload(diag: dict, residuals: dict, seed=None) -> dict:
    """One JSON line of the stream (cli.py:153-173 schema)."""
    payload = {
        "type": "step",
        "iteration": diag.get("iteration"),
        "dt": diag.get("dt"),
        "CFL": diag.get("CFL"),
        "continuity": residuals.get("continuity"),
        "wall_time": diag.get("wall_time"),
        "residuals": {k: residuals.get(k) for k in ("Ru", "Rv", "Rp", "continuity")},
        "diagnostics": {k: v for k, v in diag.items() if k not in ("iteration", "dt", "CFL", "wall_time")},
    }
    if seed is not None:
        payload.setdefault("run_meta", {})["seed"] = seed
    return payload


def make_config(args) -> SimulationConfig:
    ck = args.checkpoint_interval if args.checkpoint_interval not in (None, 0) else None
    return SimulationConfig(nx=args.nx, ny=args.ny, Re=args.re, lid_velocity=args.lid_velocity, cfl_target=args.cfl,
                            cfl_growth=args.cfl_growth, advection_scheme=args.scheme,
                            disable_advection=args.disable_advection, lin_tol=args.lin_tol,
                            lin_maxiter=args.lin_maxiter, diagnostics=args.diagnostics, checkpoint_interval=ck,
                            log_path=args.log_jsonl, seed=args.seed, precision=args.precision)


def main(argv: list[str] | None = None) -> int:
    args = build_parser().parse_args(argv)
    try:
        cfg = make_config(args)
    except ConfigError as e:
        print("Configuration invalid:\n" + str(e))
        return 2
    if args.command == "validate":
        out = cfg.model_dump()
        out["config_hash"] = cfg.config_hash
        print(json.dumps(out, indent=2, sort_keys=True))
        return 0
    if args.command == "show-config":
        print(json.dumps({"hash": cfg.config_hash, "brief": cfg.brief()}, indent=2))
        return 0

    from .core.ghost_fields import allocate_state
    from .drivers.simulation_driver import SimulationDriver
    from .io.checkpoint import load_checkpoint, save_checkpoint
    from .residuals.manager import ResidualManager

    tracker = ResidualManager()
    if args.restart:
        try:
            state, meta = load_checkpoint(args.restart, device="cuda")
            ck_hash = meta.get("structured_config_hash")
            if ck_hash and ck_hash != cfg.config_hash and not args.allow_hash_mismatch:
                print(f"Refusing restart: checkpoint hash {ck_hash} != current {cfg.config_hash} "
                      "(use --allow-hash-mismatch to override)")
                return 3
            start_it = int(meta.get("iteration", 0)) + 1
        except Exception as e:
            print(f"Failed to load checkpoint {args.restart}: {e}")
            state = allocate_state(cfg.nx, cfg.ny)
            start_it = 0
    else:
        state = allocate_state(cfg.nx, cfg.ny)
        start_it = 0
    driver = SimulationDriver(cfg, state, tracker)
    json_mode = args.json_stream
    if json_mode:
        cfg.force_quiet = True
        cfg.diagnostics = False
    if args.assert_invariants:
        cfg.assert_invariants = True
    last = None
    try:
        ck_int = None if args.checkpoint_interval in (None, 0) else args.checkpoint_interval
        for st, residuals, diag in driver.run(max_steps=args.steps, start_iteration=start_it,
                                              progress=(args.progress and not json_mode),
                                              checkpoint_path=args.checkpoint, checkpoint_interval=ck_int):
            last = (st, diag)
            if json_mode:
                sys.stdout.write(json.dumps(step_payload(diag, residuals, cfg.seed), separators=(",", ":")) + "\n")
                sys.stdout.flush()
            if args.continuity_threshold is not None and residuals.get("continuity", 1.0) < args.continuity_threshold:
                if not json_mode:
                    print(f"Stopping early: continuity {residuals['continuity']:.3e} < threshold "
                          f"{args.continuity_threshold:.3e}")
                break
    except KeyboardInterrupt:
        ck_path = args.checkpoint or "interrupt_final_checkpoint.npz"
        if last is not None:
            try:
                save_checkpoint(ck_path, last[0], last[1].get("iteration", 0), last[1].get("wall_time", 0.0), cfg)
            except Exception:  # pragma: no cover
                pass
        return 130
    return 0


if __name__ == "__main__":  # pragma: no cover
    raise SystemExit(main())
