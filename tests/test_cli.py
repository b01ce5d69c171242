"""CLI front-end: arguments, exit codes and the reference's config hash."""
import json
import os
import subprocess
import sys

import pytest

from pyflow_solver_gb300.cli import main, step_payload
from pyflow_solver_gb300.config.model import ConfigError, SimulationConfig

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_config_hash_equals_reference():
    with open(os.path.join(ROOT, "tests", "golden", "config_hashes.json")) as f:
        cases = json.load(f)["cases"]
    for c in cases:
        assert SimulationConfig(**c["kwargs"]).config_hash == c["hash"], c


def test_config_ranges_raise():
    for bad in (dict(nx=2, ny=8), dict(nx=8, ny=8, cfl_target=1.5), dict(nx=8, ny=8, lin_maxiter=0),
                dict(nx=8, ny=8, advection_scheme="central"), dict(nx=8, ny=8, precision="fp16")):
        with pytest.raises(ConfigError):
            SimulationConfig(**bad)


def test_validate_and_invalid_exit_codes(capsys):
    assert main(["validate", "--nx", "16", "--ny", "12"]) == 0
    out = json.loads(capsys.readouterr().out)
    assert out["nx"] == 16 and out["config_hash"] == SimulationConfig(nx=16, ny=12, advection_scheme="quick",
                                                                      lin_tol=1e-10, lin_maxiter=300,
                                                                      diagnostics=False).config_hash
    assert main(["show-config", "--nx", "16"]) == 0
    assert main(["validate", "--nx", "1"]) == 2


def test_step_payload_schema():
    diag = {"iteration": 3, "dt": 0.1, "CFL": 0.5, "wall_time": 1.0, "Rp_iterations": 300, "nan_detected": False}
    res = {"Ru": 1e-3, "Rv": 2e-3, "Rp": 0.0, "continuity": 1e-6}
    p = step_payload(diag, res, seed=5)
    assert p["type"] == "step" and p["iteration"] == 3 and p["continuity"] == 1e-6
    assert set(p["residuals"]) == {"Ru", "Rv", "Rp", "continuity"}
    assert "dt" not in p["diagnostics"] and p["diagnostics"]["Rp_iterations"] == 300
    assert p["run_meta"] == {"seed": 5}


@pytest.mark.gpu
def test_run_json_stream_matches_oracle(tmp_path):
    """`run --json-stream` through a subprocess, checked against the oracle twin."""
    from types import SimpleNamespace

    from oracle import step as ost
    cmd = [sys.executable, "-m", "pyflow_solver_gb300", "run", "--nx", "20", "--ny", "16", "--steps", "4",
           "--lin-tol", "1e-8", "--json-stream", "--checkpoint", str(tmp_path / "ck.npz"),
           "--checkpoint-interval", "2"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.strip().splitlines()]
    assert [x["iteration"] for x in lines] == [0, 1, 2, 3]
    cfg = SimpleNamespace(nx=20, ny=16, Re=100.0, lid_velocity=1.0, advection_scheme="quick", cfl_target=0.5,
                          cfl_growth=1.05, lin_tol=1e-8, lin_maxiter=300)
    tw = ost.allocate_state(20, 16)
    for line, (_, res, diag) in zip(lines, ost.run(cfg, tw, max_steps=4, red="exact")):
        assert line["dt"] == diag["dt"] and line["residuals"]["Ru"] == res["Ru"]
        assert line["continuity"] == res["continuity"]
    assert (tmp_path / "ck.npz").exists()
    # restart from the checkpoint: a different config hash is refused with exit code 3
    r2 = subprocess.run([sys.executable, "-m", "pyflow_solver_gb300", "run", "--nx", "20", "--ny", "16", "--re", "50",
                         "--steps", "5", "--restart", str(tmp_path / "ck.npz")], cwd=ROOT, capture_output=True,
                        text=True, timeout=600)
    assert r2.returncode == 3, r2.stdout
