"""Host-side logic of the GPU package that needs no GPU."""
import json
from types import SimpleNamespace

import numpy as np
import pytest

from pyflow_solver_gb300 import _capi
from pyflow_solver_gb300.io import checkpoint as ck
from pyflow_solver_gb300.linear_solvers.preconditioners import diag_matches_assembled, jacobi_interior
from pyflow_solver_gb300.solvers.solver import step_params


def test_step_params_follow_reference_getattr_defaults():
    cfg = SimpleNamespace(nx=64, ny=32)
    P, dx, dy, nu = step_params(cfg, 64, 32)
    assert dx == 63.0 / 63 and dy == 31.0 / 31           # CLI path: lx = nx - 1 -> dx = 1
    assert nu == 1.0 / 100.0
    assert P.lin_maxiter == 400 and P.lin_tol == 1e-10   # pressure_solver.py:133-135 defaults
    assert P.scheme == _capi.SCHEME_UPWIND                # solver.py:80 fallback
    assert P.has_lid == 0 and P.enable_jacobi == 1
    cfg = SimpleNamespace(lx=1.0, ly=1.0, advection_scheme="quick", lid_velocity=1.0, Re=1000.0,
                          disable_advection=False, enable_jacobi_pc=False)
    P, dx, dy, nu = step_params(cfg, 512, 512)
    assert dx == 1.0 / 511 and P.scheme == _capi.SCHEME_QUICK and P.has_lid == 1 and P.enable_jacobi == 0
    assert P.jacobi_interior == 1.0 / (2.0 / dx**2 + 2.0 / dy**2)
    P, *_ = step_params(SimpleNamespace(disable_advection=True, advection_scheme="quick"), 8, 8)
    assert P.scheme == _capi.SCHEME_NONE


def test_jacobi_diagonal_equals_assembled():
    from oracle.ops import jacobi_inv_diag
    for nx, ny, dx, dy in [(8, 8, 1 / 7, 1 / 7), (5, 9, 1.0, 1.0), (2, 3, 0.5, 0.25)]:
        inv = jacobi_inv_diag(nx, ny, dx, dy).reshape(ny, nx)
        if nx > 2 and ny > 2:
            assert inv[1, 1] == jacobi_interior(dx, dy)
        D = np.ones((ny, nx))
        if nx > 2 and ny > 2:
            D[1:-1, 1:-1] = 2.0 / dx**2 + 2.0 / dy**2
        assert diag_matches_assembled(D, nx, ny, dx, dy)


def test_checkpoint_format_round_trip(tmp_path):
    from pyflow_solver_gb300.core.ghost_fields import State
    rng = np.random.default_rng(0)
    st = State(4, 3, {k: rng.standard_normal((5, 6)) for k in "uvp"})
    cfg = SimpleNamespace(nx=4, ny=3, seed=7)
    path = ck.save_checkpoint(str(tmp_path / "c.npz"), st, 12, 0.5, cfg)
    with np.load(path) as d:
        assert set(d.files) == {"meta", "field_u", "field_v", "field_p"}
    st2, meta = ck.load_checkpoint(path, device=None)
    assert meta["iteration"] == 12 and meta["nx"] == 4 and meta["seed"] == 7 and meta["schema_version"] == 1
    for k in "uvp":
        np.testing.assert_array_equal(st2.fields[k], st.fields[k])
    assert meta["field_hashes"]["u"] == ck._hash_array(st.fields["u"])
    st3, meta3 = ck.load_checkpoint_bytes(ck.save_checkpoint_bytes(st, 3, 0.0, cfg), device=None)
    assert meta3["iteration"] == 3
    # the reference returns NumPy fields; so does load_checkpoint by default
    st4, _ = ck.load_checkpoint(path)
    assert isinstance(st4.fields["u"], np.ndarray)
    # no step bookkeeping yet: no state_meta entry, and a loaded state starts with empty meta
    assert "state_meta" not in meta and st2.meta == {}
    # the structured hash only for a SimulationConfig (any other object with a string
    # config_hash attribute gets None, as in the reference)
    assert meta["structured_config_hash"] is None
    cfg.config_hash = "abcdef0123"
    assert json.loads(str(np.load(ck.save_checkpoint(str(tmp_path / "d.npz"), st, 1, 0.0, cfg))["meta"]))[
        "structured_config_hash"] is None
    from pyflow_solver_gb300.config.model import SimulationConfig
    sc = SimulationConfig(nx=4, ny=3)
    m5 = json.loads(str(np.load(ck.save_checkpoint(str(tmp_path / "e.npz"), st, 1, 0.0, sc))["meta"]))
    assert m5["structured_config_hash"] == sc.config_hash


def test_checkpoint_keeps_step_bookkeeping(tmp_path):
    """dt_prev and the last five divergence norms go into meta["state_meta"] and come back
    into state.meta (a restart then continues exactly); the reference's own keys stay."""
    from pyflow_solver_gb300.core.ghost_fields import State
    st = State(4, 3, {k: np.zeros((5, 6)) for k in "uvp"})
    st.meta = {"dt_prev": 0.0123, "divergence_history": [1.0, 2.0, 3.0, 4.0, 5.0, 6.0], "dx": 0.3, "nu": 0.01}
    path = ck.save_checkpoint(str(tmp_path / "c.npz"), st, 5, 0.1, SimpleNamespace(nx=4, ny=3))
    st2, meta = ck.load_checkpoint(path)
    assert meta["state_meta"] == {"dt_prev": 0.0123, "divergence_history": [2.0, 3.0, 4.0, 5.0, 6.0]}
    assert st2.meta == {"dt_prev": 0.0123, "divergence_history": [2.0, 3.0, 4.0, 5.0, 6.0]}
    for key in ("iteration", "time", "nx", "ny", "config_hash", "structured_config_hash", "field_hashes", "seed",
                "schema_version"):
        assert key in meta


def test_driver_requires_state_or_grid():
    from pyflow_solver_gb300.drivers.simulation_driver import SimulationDriver
    d = SimulationDriver(SimpleNamespace())
    with pytest.raises(ValueError):
        next(d.run(max_steps=1))


def test_batched_workload_matches_fixture_draws():
    from pyflow_solver_gb300.workloads import batched_instances, serving_trace
    from tests import _golden as G
    g = G.load("batched16")
    inst = batched_instances()
    np.testing.assert_array_equal(np.asarray(inst), g["instances"])
    tr = serving_trace(duration=2.0)
    assert 300 < len(tr) < 500 and all(a.arrival < b.arrival for a, b in zip(tr, tr[1:]))
    assert {r.side for r in tr} <= {32, 64, 128, 256, 512, 1024}


def test_serving_slot_plan_and_latency_percentiles():
    from pyflow_solver_gb300.serving import Served, ServeReport, slot_plan
    plan = slot_plan([32, 64, 128], 1e9, lambda s: s * s * 100, weights=[1, 1, 2])
    assert plan == {32: int(0.25e9 // (32 * 32 * 100)), 64: int(0.25e9 // (64 * 64 * 100)),
                    128: int(0.5e9 // (128 * 128 * 100))}
    rep = ServeReport(completed=[Served(k, 32, 0.0, 10, finish=float(k + 1)) for k in range(100)])
    pct = rep.latency_percentiles()
    assert pct["p50"] == 51.0 and pct["p95"] == 95.0 and pct["p99"] == 99.0


def test_bench_accounting_helpers():
    import bench
    assert bench.mg_levels(512, 512) == 4 and bench.mg_levels(2048, 2048) == 6 and bench.mg_levels(64, 64) == 1
    # elongated cells coarsen the strongly coupled axis only: 256 x 64 -> 128 x 64 -> 64 x 64
    assert bench.mg_levels(128, 32) == 1 and bench.mg_levels(256, 64) == 3
    assert bench.launches_per_step("fp64", 300, 0, 1) == 11 + 900
    assert bench.launches_per_step("mixed", 10, 2, 4, persistent=True) == 7
    # 4 levels: an iteration is 2 down-sweeps, the coarse CTA, 3 up-sweeps, matvec, update
    assert bench.launches_per_step("mixed", 10, 2, 4, persistent=False) == 8 + 2 * 6 + 10 * 8
    # one level (the whole V-cycle in the coarse CTA): coarse, matvec, update; no level-0 down-sweep
    assert bench.launches_per_step("mixed", 10, 2, 1, persistent=False) == 8 + 2 * 5 + 10 * 3
    assert bench.pct([3.0, 1.0, 2.0]) == {"p50": 2.0, "p95": 3.0, "p99": 3.0}
    assert bench.mg_shapes(512, 512) == [(512, 512), (256, 256), (128, 128), (64, 64)]


def test_bench_kernel_table():
    """Per-kernel rows of a profiled step: bytes from the per-cell table times the cells of
    each kernel's level, shares of the profiled time, the largest share first."""
    import bench
    shapes = [bench.mg_shapes(512, 512)]
    prof = [("k_mx_matvec", 6, 0.060), ("k_mg_down@1", 6, 0.030), ("k_mg_coarse", 6, 0.090),
            ("k_mx_update_down", 6, 0.060)]
    rows, step = bench.kernel_table(prof, 512 * 512, shapes, step_ms=0.5, hbm=1000.0)
    assert [r["kernel"] for r in rows][0] == "k_mg_coarse"
    by = {r["kernel"]: r for r in rows}
    assert by["k_mx_matvec"]["bytes_per_launch"] == 16 * 512 * 512
    assert by["k_mg_down@1"]["bytes_per_launch"] == 9 * 256 * 256
    assert by["k_mg_coarse"]["bytes_per_launch"] == 8 * 64 * 64
    assert abs(by["k_mx_matvec"]["us_per_launch"] - 10.0) < 1e-9
    assert abs(by["k_mx_matvec"]["gbs"] - 16 * 512 * 512 / 10e-6 / 1e9) < 1e-6
    assert abs(sum(r["share"] for r in rows) - 1.0) < 1e-12
    total = sum(r["bytes_per_launch"] * r["launches"] for r in rows)
    assert step["bytes"] == total and abs(step["achieved"] - total / 0.5e-3 / 1e9) < 1e-6
    roof = bench.roofline_of(rows, step, "cavity512", 1000.0, "measured")
    assert roof["kernel"] == "k_mg_coarse" and roof["share_of_step"] == rows[0]["share"]
    # a batch: the coarse CTA of each instance starts from its own last global level
    pre, coarse = bench.level_cells([bench.mg_shapes(128, 128), bench.mg_shapes(64, 32)])
    assert pre == {0: 128 * 128} and coarse == 64 * 64 + 64 * 32


def test_step_log_and_nan_emergency_checkpoint(tmp_path):
    """The step's JSON-lines record (src/pyflow/solvers/solver.py:170-192) and, on a NaN,
    the error record and the emergency *_FAIL_NAN checkpoint -- formed from a step record
    on the host, no GPU needed."""
    from pyflow_solver_gb300.core.ghost_fields import State
    from pyflow_solver_gb300.residuals.manager import ResidualManager
    from pyflow_solver_gb300.solvers.solver import finish
    log = tmp_path / "logs" / "run.jsonl"
    cfg = SimpleNamespace(nx=4, ny=3, lx=1.0, ly=1.0, diagnostics=False, log_path=str(log),
                          emergency_checkpoint_path=str(tmp_path / "ck" / "state.npz"))
    st = State(4, 3, {k: np.zeros((5, 6)) for k in "uvp"})
    P, dx, dy, nu = step_params(cfg, 4, 3)
    tr = ResidualManager()
    for it, nan in ((0, 0), (1, 1)):
        out = _capi.StepOut()
        out.dt, out.cfl, out.ru_sq, out.rv_sq, out.cont_sq, out.nan_detected = 0.01, 0.5, 4.0, 9.0, 1.0, nan
        finish(cfg, st, tr, it, P, (dx, dy, nu), out)
    recs = [json.loads(x) for x in log.read_text().splitlines()]
    assert [r["type"] for r in recs] == ["step", "step", "error", "emergency_checkpoint"]
    assert recs[0]["it"] == 0 and recs[0]["Ru"] == 2.0 / 12 and recs[0]["nan"] is False and "ts" in recs[0]
    assert recs[1]["nan"] is True and recs[2]["reason"] == "nan_detected"
    assert recs[3]["path"] == str(tmp_path / "ck" / "state_FAIL_NAN.npz")
    st2, meta = ck.load_checkpoint(recs[3]["path"])
    assert meta["iteration"] == 1
    cfg._logger_instance.close()
