"""Restart from a checkpoint and the CLI's Ctrl-C path.

The reference restarts through ``load_checkpoint`` -> ``driver.run(start_iteration
= it + 1)`` (src/pyflow/cli.py:116-131, io/checkpoint.py:51-127) and, on Ctrl-C,
writes a final checkpoint and exits 130 (cli.py:179-193).  Its checkpoints hold
the fields only, so a restarted run starts with fresh step bookkeeping (dt_prev
1e-2) and does not continue the uninterrupted run exactly; the checkpoints here
also keep ``state.meta`` (meta["state_meta"]), and then it does:

* plain binary64: N steps -> checkpoint -> load -> M steps equals N + M steps
  bit for bit; without the bookkeeping (a reference-style file) the restarted
  run equals the oracle twin restarted the same way, bit for bit;
* mixed precision: equal within the 1e-6 bar (a restarted state gets a new
  solver handle, whose refinement history starts afresh).
"""
import json
import os
import signal
import subprocess
import sys
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import step as ost

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def cavity(precision):
    return SimpleNamespace(nx=48, ny=40, lx=1.0, ly=1.0, Re=400.0, lid_velocity=1.0, advection_scheme="quick",
                           cfl_target=0.5, cfl_growth=1.05, lin_tol=1e-8, lin_maxiter=200, diagnostics=False,
                           precision=precision)


def fields(st):
    from pyflow_solver_gb300 import interior_view
    out = []
    for k in "uvp":
        a = interior_view(st.fields[k])
        out.append(a.cpu().numpy().copy() if hasattr(a, "cpu") else np.array(a))
    return out


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_restart_continues_the_run(tmp_path, precision):
    from pyflow_solver_gb300 import ResidualManager, SimulationDriver, allocate_state
    from pyflow_solver_gb300.io.checkpoint import load_checkpoint, save_checkpoint
    cfg = cavity(precision)
    N, M = 6, 5
    whole = allocate_state(cfg.nx, cfg.ny)
    for _ in SimulationDriver(cfg, whole, ResidualManager()).run(max_steps=N + M):
        pass
    first = allocate_state(cfg.nx, cfg.ny)
    for _, _, diag in SimulationDriver(cfg, first, ResidualManager()).run(max_steps=N):
        pass
    path = save_checkpoint(str(tmp_path / "ck.npz"), first, N - 1, diag["wall_time"], cfg)
    state, meta = load_checkpoint(path, device="cuda")
    assert meta["state_meta"]["dt_prev"] == first.meta["dt_prev"]
    start = int(meta["iteration"]) + 1
    for _ in SimulationDriver(cfg, state, ResidualManager()).run(max_steps=N + M, start_iteration=start):
        pass
    for a, b, k in zip(fields(state), fields(whole), "uvp"):
        if precision == "fp64":
            np.testing.assert_array_equal(a, b, err_msg=k)
        else:
            assert rel(a, b) <= 1e-6, (k, rel(a, b))


def test_reference_style_restart_matches_the_twin(tmp_path):
    """A checkpoint without the bookkeeping restarts as the reference's does: dt_prev
    falls back to 1e-2 and the divergence history starts empty; the GPU run from it
    equals the oracle twin run from the same fields, bit for bit."""
    from pyflow_solver_gb300 import ResidualManager, SimulationDriver, allocate_state
    from pyflow_solver_gb300.io.checkpoint import load_checkpoint, save_checkpoint
    cfg = cavity("fp64")
    first = allocate_state(cfg.nx, cfg.ny)
    for _ in SimulationDriver(cfg, first, ResidualManager()).run(max_steps=4):
        pass
    first.meta = {}
    path = save_checkpoint(str(tmp_path / "ref_style.npz"), first, 3, 0.0, cfg)
    state, meta = load_checkpoint(path, device="cuda")
    assert "state_meta" not in meta and state.meta == {}
    for _ in SimulationDriver(cfg, state, ResidualManager()).run(max_steps=8, start_iteration=4):
        pass
    tw = ost.allocate_state(cfg.nx, cfg.ny)
    host, _ = load_checkpoint(path)
    for k in "uvp":
        tw.fields[k][:] = host.fields[k]
    for _ in ost.run(cfg, tw, max_steps=8, start_iteration=4, red="exact"):
        pass
    for a, k in zip(fields(state), "uvp"):
        np.testing.assert_array_equal(a, ost.interior(tw.fields[k]), err_msg=k)


def test_ctrl_c_writes_a_final_checkpoint_and_exits_130(tmp_path):
    ck = tmp_path / "final.npz"
    cmd = [sys.executable, "-m", "pyflow_solver_gb300", "run", "--nx", "64", "--ny", "64", "--steps", "1000000",
           "--lin-tol", "1e-8", "--json-stream", "--checkpoint", str(ck)]
    p = subprocess.Popen(cmd, cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    try:
        seen = [json.loads(p.stdout.readline()) for _ in range(3)]
        p.send_signal(signal.SIGINT)
        out, err = p.communicate(timeout=300)
    finally:
        if p.poll() is None:
            p.kill()
            p.wait()
    assert p.returncode == 130, err
    assert ck.exists()
    from pyflow_solver_gb300.io.checkpoint import load_checkpoint
    st, meta = load_checkpoint(str(ck))
    last = [json.loads(x) for x in out.strip().splitlines() if x.startswith("{")]
    last_it = (last or seen)[-1]["iteration"]
    # the last step streamed (or the one after it, if the signal came between the step's
    # bookkeeping and its line)
    assert meta["iteration"] in (last_it, last_it + 1) and meta["iteration"] >= seen[-1]["iteration"]
    assert st.fields["u"].shape == (66, 66) and "state_meta" in meta
