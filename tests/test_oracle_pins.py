"""The oracle is pinned to the reference itself.

In ``numpy`` reduction mode the oracle reproduces the reference's trajectory
bit for bit (u, v, p at the saved steps, every scalar, and the true CG
iteration counts) on the fixtures that ``tests/golden/make_golden.py`` made by
running the reference.  The reference's dot products round in an order chosen
by the BLAS of the machine, so this holds on the machine that made them; on
other machines the test is skipped (the exact twin below is portable).
"""
import platform

import numpy as np
import pytest

from oracle import ops
from oracle import step as ost
from tests import _golden as G

SCALARS = ("dt", "CFL", "Ru", "Rv", "continuity", "Rp_residual", "divergence_norm", "Rp_iterations",
           "max_residual", "residual_drop_Ru_orders", "nu")


def _same_platform(g):
    return G.fixture_platform(g)["machine"] == platform.machine()


def replay(name, mode, steps=None):
    g = G.load(name)
    cfg = G.config_of(g)
    nx, ny = cfg.nx, cfg.ny
    st = ost.allocate_state(nx, ny)
    u0, v0 = G.initial_interior(name, nx, ny)
    ost.interior(st.fields["u"])[:] = u0
    ost.interior(st.fields["v"])[:] = v0
    steps = steps or len(g["dt"])
    extras = []
    out = []
    for s, res, diag in ost.run(cfg, st, max_steps=steps, red=mode, extras=extras):
        rec = {k: (res[k] if k in res else diag[k]) for k in SCALARS}
        rec["fields"] = {k: ost.interior(s.fields[k]).copy() for k in "uvp"}
        rec["centerline"] = np.asarray(diag["u_centerline"][1])
        out.append(rec)
    return g, out, extras


@pytest.mark.parametrize("name", G.SMALL + ["cavity64_cli"])
def test_numpy_mode_is_bit_identical_to_reference(name):
    g = G.load(name)
    if not _same_platform(g):
        pytest.skip("fixture made on another machine (BLAS summation order differs)")
    steps = len(g["dt"])
    g, out, extras = replay(name, "numpy", steps)
    for it, rec in enumerate(out):
        for k in SCALARS:
            assert rec[k] == g[k][it] or (np.isnan(rec[k]) and np.isnan(g[k][it])), (name, it, k)
        for k in "uvp":
            key = f"{k}_{it}"
            if key in g:
                np.testing.assert_array_equal(rec["fields"][k], g[key], err_msg=f"{name} step {it} {k}")
        np.testing.assert_array_equal(rec["centerline"], g["centerline"][it])
    assert [e["cg_true_iterations"] for e in extras] == list(g["cg_true_iterations"])


@pytest.mark.slow
def test_numpy_mode_cavity64_unit_square_50_steps():
    g = G.load("cavity64_unit")
    if not _same_platform(g):
        pytest.skip("fixture made on another machine")
    g, out, extras = replay("cavity64_unit", "numpy")
    for it in g["saved_steps"]:
        for k in "uvp":
            np.testing.assert_array_equal(out[it]["fields"][k], g[f"{k}_{it}"])
    for it, rec in enumerate(out):
        assert rec["dt"] == g["dt"][it] and rec["continuity"] == g["continuity"][it]
    assert [e["cg_true_iterations"] for e in extras] == list(g["cg_true_iterations"])


def test_operators_bit_identical_to_reference():
    g = G.load("ops")
    keys = sorted({k.split("_")[0] for k in g.files if "x" in k.split("_")[0] and k[0].isdigit()})
    assert keys
    for key in keys:
        u, v, p = g[f"{key}_u"], g[f"{key}_v"], g[f"{key}_p"]
        dx, dy = g[f"{key}_dxdy"]
        gx, gy = ops.gradient_coherent(p, dx, dy)
        np.testing.assert_array_equal(gx, g[f"{key}_gx"])
        np.testing.assert_array_equal(gy, g[f"{key}_gy"])
        np.testing.assert_array_equal(ops.divergence_coherent(u, v, dx, dy), g[f"{key}_divc"])
        np.testing.assert_array_equal(ops.laplacian_coherent(p, dx, dy), g[f"{key}_lap"])
        np.testing.assert_array_equal(ops.divergence_central(u, v, 1.0, 1.0), g[f"{key}_divcentral"])
        np.testing.assert_array_equal(ops.divergence_central(u, v, dx, dy), g[f"{key}_divcentral_h"])
        np.testing.assert_array_equal(ops.advect_quick(u, v, u, dx, dy), g[f"{key}_quick_u"])
        np.testing.assert_array_equal(ops.advect_quick(u, v, v, dx, dy), g[f"{key}_quick_v"])
        np.testing.assert_array_equal(ops.advect_upwind(u, v, u, dx, dy), g[f"{key}_upwind_u"])
        np.testing.assert_array_equal(ops.advect_upwind(u, v, v, dx, dy), g[f"{key}_upwind_v"])


def test_manufactured_and_bump_projection_match_reference():
    g = G.load("manufactured")
    if not _same_platform(g):
        pytest.skip("fixture made on another machine")

    class Cfg:
        lin_tol = 1e-10
        lin_maxiter = 500

    st = ost.allocate_state(8, 8)
    ex = {}
    ost.solve_pressure_poisson(st, 1.0, 1.0 / 7, 1.0 / 7, Cfg(), red="numpy", rhs_override=g["rhs"].copy(), extra=ex)
    np.testing.assert_array_equal(ost.interior(st.fields["p"]), g["p"])
    assert ex["cg_true_iterations"] == int(g["cg_true_iterations"][0])
    for pc in (True, False):
        tag = "pc" if pc else "nopc"
        st = ost.allocate_state(24, 20)
        ost.interior(st.fields["u"])[20 // 3, 24 // 3] = 1.0

        class C2:
            lin_tol = 1e-10
            lin_maxiter = 300
            enable_jacobi_pc = pc

        ex = {}
        _, diag = ost.solve_pressure_poisson(st, 0.01, 1.0, 1.0, C2(), red="numpy", extra=ex)
        for k in "uvp":
            np.testing.assert_array_equal(ost.interior(st.fields[k]), g[f"bump_{tag}_{k}"])
        assert ex["cg_true_iterations"] == int(g[f"bump_{tag}_iters"][0])
        for k in ("Rp_iterations", "Rp_residual", "divergence_norm", "lin_residual_norm",
                  "lin_residual_rel", "divergence_norm_initial"):
            assert diag[k] == float(g[f"bump_{tag}_{k}"]), (tag, k)


def test_reorder_floor_is_recorded():
    """The exact twin differs from the reference only through dot rounding order."""
    g = G.load("s16x12_quick")
    _, ex_out, _ = replay("s16x12_quick", "exact")
    # the first step with a non-trivial pressure solve already moves the fields
    diffs = [np.max(np.abs(r["fields"]["u"] - g[f"u_{i}"])) for i, r in enumerate(ex_out)]
    assert diffs[0] == 0.0          # step 0: zero RHS, no CG iteration, identical
    assert max(diffs) > 0.0         # later: summation order matters (non-SPD CG cut at maxiter)


def _krylov_cases():
    import scipy.sparse as sp

    from pyflow_solver_gb300.solvers.pressure_solver import assemble_negative_laplacian
    rng = np.random.default_rng(11)
    A1 = assemble_negative_laplacian(12, 9, 1.0 / 11, 1.0 / 8)
    n = 300
    R = sp.random(n, n, density=0.02, random_state=5, format="csr")
    A2 = (R + sp.diags(np.abs(R).sum(axis=1).A1 + 1.0 + rng.random(n))).tocsr()   # non-symmetric, dominant
    return [(A1, rng.standard_normal(A1.shape[0])), (A2, rng.standard_normal(n))]


@pytest.mark.parametrize("method", ["cg", "bicgstab"])
@pytest.mark.parametrize("pc", [False, True])
def test_krylov_oracle_reproduces_scipy(method, pc):
    """The restated CG and BiCGSTAB over a CSR matrix (np.dot / np.linalg.norm
    reductions) give scipy's own iterates bit for bit, as the reference calls them
    (src/pyflow/linear_solvers/interface.py:17-21,43-46; x0 = 0, rtol = tol, M = Jacobi)."""
    import scipy.sparse.linalg as spla

    from oracle.krylov import jacobi_inv, solve_csr
    for A, b in _krylov_cases():
        inv = jacobi_inv(A.diagonal()) if pc else None
        M = spla.LinearOperator(A.shape, lambda v, inv=inv: inv * v) if pc else None
        fn = spla.cg if method == "cg" else spla.bicgstab
        x_ref, info_ref = fn(A, b, x0=np.zeros_like(b), rtol=1e-9, maxiter=60, M=M)
        x, info, _, _ = solve_csr(A.indptr, A.indices, A.data, b, method, 1e-9, 60, inv, red="numpy")
        np.testing.assert_array_equal(x, x_ref)
        assert info == info_ref
