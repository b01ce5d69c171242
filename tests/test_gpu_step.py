"""Parity of the GPU projection step.

P1 (bit for bit): the GPU step against the oracle twin with exactly rounded
reductions -- every field value, every scalar of the residual/diagnostic dicts,
the state.meta updates and the true CG iteration count, at every step.

P2 (against the untouched reference): the GPU error against the reference's
own trajectory (golden fixtures) stays within 2x the summation-order floor,
i.e. the distance between the exact twin and the reference, which here is the
same number because P1 holds bit for bit.
"""
import numpy as np
import pytest

from tests import _golden as G
from tests._gpu_run import SCALARS, gpu_trajectory, rel_err, same, twin_trajectory

pytestmark = pytest.mark.gpu


def check_bitwise(got, ref, name):
    assert len(got) == len(ref)
    for it, (a, b) in enumerate(zip(got, ref)):
        for k in SCALARS:
            assert same(a[k], b[k]), f"{name} step {it} {k}: gpu {a[k]!r} twin {b[k]!r}"
        assert a["cg_iterations"] == b["cg_iterations"], f"{name} step {it} CG iterations"
        assert a["meta"]["dt_prev"] == b["meta"]["dt_prev"]
        assert a["meta"]["hist"] == b["meta"]["hist"]
        np.testing.assert_array_equal(a["centerline"], b["centerline"])
        if "fields" in a and "fields" in b:
            for k in "uvp":
                np.testing.assert_array_equal(a["fields"][k], b["fields"][k], err_msg=f"{name} step {it} {k}")


@pytest.mark.parametrize("name", G.SMALL)
def test_p1_small_fixtures_bitwise(name):
    g = G.load(name)
    cfg = G.config_of(g)
    u0, v0 = G.initial_interior(name, cfg.nx, cfg.ny)
    steps = len(g["dt"])
    got = gpu_trajectory(cfg, cfg.nx, cfg.ny, steps, u0, v0)
    ref = twin_trajectory(cfg, cfg.nx, cfg.ny, steps, u0, v0)
    check_bitwise(got, ref, name)


def test_p1_cavity64_unit_square_50_steps_bitwise():
    g = G.load("cavity64_unit")
    cfg = G.config_of(g)
    keep = set(int(s) for s in g["saved_steps"])
    got = gpu_trajectory(cfg, 64, 64, 50, keep=keep)
    ref = twin_trajectory(cfg, 64, 64, 50, keep=keep)
    check_bitwise(got, ref, "cavity64_unit")
    assert all(r["cg_iterations"] == 300 for r in got[1:])   # the reference never converges at maxiter 300


def test_direct_launches_equal_graph_replay():
    """The step as individual launches and as one CUDA graph give the same bits."""
    from pyflow_solver_gb300.solvers import _handle
    g = G.load("s16x12_quick")
    cfg = G.config_of(g)
    graph = gpu_trajectory(cfg, cfg.nx, cfg.ny, 12)
    _handle.GRAPH_MODE = False
    try:
        direct = gpu_trajectory(cfg, cfg.nx, cfg.ny, 12)
        _handle.GRAPH_MODE = 2
        plain_graph = gpu_trajectory(cfg, cfg.nx, cfg.ny, 12)
    finally:
        _handle.GRAPH_MODE = True
    check_bitwise(direct, graph, "graph vs direct")
    check_bitwise(plain_graph, graph, "graph with and without programmatic edges")


def test_p1_cavity64_cli_spacing_bitwise():
    g = G.load("cavity64_cli")
    cfg = G.config_of(g)
    got = gpu_trajectory(cfg, 64, 64, 20, keep={0, 1, 19})
    ref = twin_trajectory(cfg, 64, 64, 20, keep={0, 1, 19})
    check_bitwise(got, ref, "cavity64_cli")


@pytest.mark.parametrize("name", ["cavity64_unit", "cavity64_cli", "s16x12_quick", "s16_patch"])
def test_p2_against_reference_within_reorder_floor(name):
    g = G.load(name)
    cfg = G.config_of(g)
    steps = len(g["dt"])
    saved = [int(s) for s in g["saved_steps"]]
    u0, v0 = G.initial_interior(name, cfg.nx, cfg.ny)
    got = gpu_trajectory(cfg, cfg.nx, cfg.ny, steps, u0, v0, keep=set(saved))
    twin = twin_trajectory(cfg, cfg.nx, cfg.ny, steps, u0, v0, keep=set(saved))
    for it in saved:
        for k in "uvp":
            ref = g[f"{k}_{it}"]
            floor = rel_err(twin[it]["fields"][k], ref)
            err = rel_err(got[it]["fields"][k], ref)
            assert err <= 2.0 * floor + 1e-15, f"{name} step {it} {k}: gpu {err:.3e} floor {floor:.3e}"


def test_driver_contract_same_state_and_dt_growth():
    from types import SimpleNamespace

    from pyflow_solver_gb300 import ResidualManager, SimulationDriver, allocate_state
    cfg = SimpleNamespace(disable_advection=True, advection_scheme="upwind", cfl_target=0.5, cfl_growth=1.05,
                          Re=100.0, lid_velocity=0.0, lin_tol=1e-10, lin_maxiter=50, nx=8, ny=8, lx=7, ly=7,
                          diagnostics=False)
    state = allocate_state(8, 8)
    last = None
    n = 0
    for st, res, diag in SimulationDriver(cfg, state, ResidualManager()).run(max_steps=5):
        assert st is state
        assert "dt" in diag and "u_centerline" in diag and "wall_time" in diag
        if last is not None:
            assert diag["dt"] <= last * 1.5
        last = diag["dt"]
        n += 1
    assert n == 5


def test_host_numpy_fields_are_updated_in_place():
    """A State with NumPy fields (the reference's own allocate_state) runs through the GPU."""
    from types import SimpleNamespace

    from oracle import step as ost
    from pyflow_solver_gb300.core.ghost_fields import State
    from pyflow_solver_gb300.residuals.manager import ResidualManager
    from pyflow_solver_gb300.solvers.solver import step
    cfg = SimpleNamespace(nx=12, ny=10, lx=1.0, ly=1.0, Re=100.0, lid_velocity=1.0, advection_scheme="quick",
                          lin_tol=1e-8, lin_maxiter=80, diagnostics=False)
    host = State(12, 10, {k: np.zeros((12, 14)) for k in "uvp"})
    u_arr = host.fields["u"]
    twin = ost.allocate_state(12, 10)
    tr = ost.ResidualManager()
    for it in range(3):
        _, res, diag = step(cfg, host, ResidualManager(), it)
        _, rres, rdiag = ost.step(cfg, twin, tr, it, red="exact")
        assert res == rres
    assert host.fields["u"] is u_arr
    for k in "uvp":
        np.testing.assert_array_equal(host.fields[k], twin.fields[k])


def test_host_fields_page_locked_in_place():
    """Host NumPy fields of at least 1 MiB are page-locked in place and stepped through the
    state's persistent device copies: same bits as a device-resident state, the same arrays
    updated in place, and the registration released when the arrays are freed."""
    import gc
    from types import SimpleNamespace

    from pyflow_solver_gb300 import ResidualManager, allocate_state
    from pyflow_solver_gb300.core.ghost_fields import State
    from pyflow_solver_gb300.solvers import fields as F
    from pyflow_solver_gb300.solvers.solver import step
    n = 384
    cfg = SimpleNamespace(nx=n, ny=n, lx=1.0, ly=1.0, Re=400.0, lid_velocity=1.0, advection_scheme="quick",
                          lin_tol=1e-8, lin_maxiter=300, diagnostics=False, precision="mixed")
    host = State(n, n, {k: np.zeros((n + 2, n + 2)) for k in "uvp"})
    arrs = dict(host.fields)
    dev = allocate_state(n, n)
    tr_h, tr_d = ResidualManager(), ResidualManager()
    for it in range(3):
        _, rh, dh = step(cfg, host, tr_h, it)
        _, rd, dd = step(cfg, dev, tr_d, it)
        assert rh == rd and dh == dd
    ptrs = [a.__array_interface__["data"][0] for a in arrs.values()]
    assert all(p in F._registered for p in ptrs)
    for k in "uvp":
        assert host.fields[k] is arrs[k]
        np.testing.assert_array_equal(host.fields[k], dev.fields[k].cpu().numpy())
    del host, arrs
    gc.collect()
    assert not any(p in F._registered for p in ptrs)


def test_pressure_solver_standalone_matches_twin():
    from types import SimpleNamespace

    import torch

    from oracle import step as ost
    from pyflow_solver_gb300 import allocate_state, interior_view
    from pyflow_solver_gb300.solvers.pressure_solver import solve_pressure_poisson
    nx, ny = 24, 20
    for pc in (True, False):
        cfg = SimpleNamespace(lin_tol=1e-10, lin_maxiter=300, enable_jacobi_pc=pc)
        st = allocate_state(nx, ny)
        interior_view(st.fields["u"])[ny // 3, nx // 3] = 1.0
        tw = ost.allocate_state(nx, ny)
        ost.interior(tw.fields["u"])[ny // 3, nx // 3] = 1.0
        _, d = solve_pressure_poisson(st, 0.01, 1.0, 1.0, cfg)
        ex = {}
        _, rd = ost.solve_pressure_poisson(tw, 0.01, 1.0, 1.0, cfg, red="exact", extra=ex)
        for k in "uvp":
            np.testing.assert_array_equal(interior_view(st.fields[k]).cpu().numpy(), ost.interior(tw.fields[k]))
        for k in ("Rp_iterations", "Rp_residual", "Rp_converged", "divergence_norm", "lin_residual_norm",
                  "lin_residual_rel", "divergence_reduction_factor", "divergence_norm_initial"):
            assert d[k] == rd[k], (pc, k)
        assert d["cg_true_iterations"] == ex["cg_true_iterations"]


def test_manufactured_dirichlet_solve_matches_twin():
    from types import SimpleNamespace

    from oracle import step as ost
    from pyflow_solver_gb300 import allocate_state, interior_view
    from pyflow_solver_gb300.solvers.pressure_solver import solve_pressure_poisson
    g = G.load("manufactured")
    cfg = SimpleNamespace(lin_tol=1e-10, lin_maxiter=500)
    st = allocate_state(8, 8)
    _, d = solve_pressure_poisson(st, 1.0, 1.0 / 7, 1.0 / 7, cfg, rhs_override=g["rhs"].copy())
    tw = ost.allocate_state(8, 8)
    ex = {}
    _, rd = ost.solve_pressure_poisson(tw, 1.0, 1.0 / 7, 1.0 / 7, cfg, red="exact", rhs_override=g["rhs"].copy(),
                                       extra=ex)
    np.testing.assert_array_equal(interior_view(st.fields["p"]).cpu().numpy(), ost.interior(tw.fields["p"]))
    assert d["Rp_residual"] == rd["Rp_residual"] and d["divergence_norm"] == rd["divergence_norm"]
    assert d["cg_true_iterations"] == ex["cg_true_iterations"]
    # and the manufactured solution is recovered as in the reference test
    x = np.linspace(0, 1, 8)
    X, Y = np.meshgrid(x, x)
    pa = np.sin(np.pi * X) * np.sin(np.pi * Y)
    assert np.allclose(interior_view(st.fields["p"]).cpu().numpy()[1:-1, 1:-1], pa[1:-1, 1:-1], atol=5e-2)


def test_linear_solve_interface_matches_oracle_cg():
    from oracle import ops
    from oracle.cg import pcg
    from oracle.xsum import xdot, xnorm
    from pyflow_solver_gb300.linear_solvers.interface import solve
    from pyflow_solver_gb300.linear_solvers.operators import PressureOperator
    from pyflow_solver_gb300.linear_solvers.preconditioners import jacobi_preconditioner
    nx, ny, dx, dy = 40, 30, 1.0 / 39, 1.0 / 29
    rng = np.random.default_rng(4)
    b = rng.standard_normal(nx * ny)
    b -= b.mean()
    b[0] = 0.0
    A = PressureOperator("neg_laplacian_pinned", nx, ny, dx, dy)
    M = jacobi_preconditioner(A)
    res = solve(A, b, method="cg", tol=1e-8, maxiter=250, M=M)
    invd = ops.jacobi_inv_diag(nx, ny, dx, dy)
    ref = pcg(lambda x: ops.neg_laplacian_pinned(x, nx, ny, dx, dy), lambda r: invd * r, b, 1e-8, 250, xdot, xnorm)
    np.testing.assert_array_equal(res.x, ref.x)
    assert res.true_iterations == ref.iterations
    assert res.iterations == (ref.info if ref.info > 0 else 0)
    r = b - ops.neg_laplacian_pinned(ref.x, nx, ny, dx, dy)
    assert res.residual_norm == xnorm(r)
