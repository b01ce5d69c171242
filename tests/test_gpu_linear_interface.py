"""The operator interface on an assembled sparse matrix.

``solve(A, b, method, tol, maxiter, M)`` of src/pyflow/linear_solvers/interface.py
accepts SciPy sparse matrices (dense inputs converted to CSR) and runs
scipy.sparse.linalg.cg for 'cg', .bicgstab otherwise; ``jacobi_preconditioner``
takes the matrix; ``assemble_negative_laplacian`` builds it.  On the GPU the
CSR product, both iterations and the Jacobi vector must give the oracle twin's
(exactly rounded reductions) iterates bit for bit, with the same info, true
iteration count and residual norm.  The reference's own checks on these pieces
(the manufactured Laplacian of tests/test_projection_method_contract.py, the
preconditioned and plain solves agreeing) hold too.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def cases():
    import scipy.sparse as sp

    from pyflow_solver_gb300.solvers.pressure_solver import assemble_negative_laplacian
    rng = np.random.default_rng(21)
    A1 = assemble_negative_laplacian(40, 30, 1.0 / 39, 1.0 / 29)
    n = 2000
    R = sp.random(n, n, density=0.003, random_state=9, format="csr")
    A2 = (R + sp.diags(np.abs(R).sum(axis=1).A1 + 0.5 + rng.random(n))).tocsr()   # non-symmetric
    dense = rng.standard_normal((60, 60)) + 80.0 * np.eye(60)                       # a dense input
    return [("laplacian", A1, rng.standard_normal(A1.shape[0])), ("nonsymmetric", A2, rng.standard_normal(n)),
            ("dense", dense, rng.standard_normal(60))]


def test_csr_product_matches_the_oracle():
    import scipy.sparse as sp

    from oracle.krylov import csr_matvec
    from pyflow_solver_gb300.linear_solvers.sparse import CsrMatrix
    for name, A, b in cases():
        S = sp.csr_matrix(A)
        got = CsrMatrix.from_any(A) @ b
        np.testing.assert_array_equal(got, csr_matvec(S.indptr, S.indices, S.data, b), err_msg=name)


@pytest.mark.parametrize("method", ["cg", "bicgstab"])
@pytest.mark.parametrize("pc", [False, True])
def test_solve_matches_the_twin(method, pc):
    import scipy.sparse as sp

    from oracle.krylov import jacobi_inv, solve_csr
    from pyflow_solver_gb300.linear_solvers.interface import solve
    from pyflow_solver_gb300.linear_solvers.preconditioners import jacobi_preconditioner
    for name, A, b in cases():
        if method == "cg" and name == "nonsymmetric":
            continue                      # CG needs a symmetric system
        S = sp.csr_matrix(A)
        kw = {"M": jacobi_preconditioner(A)} if pc else {}
        res = solve(A, b, method=method, tol=1e-10, maxiter=400, **kw)
        inv = jacobi_inv(S.diagonal()) if pc else None
        x, info, its, rnorm = solve_csr(S.indptr, S.indices, S.data, b, method, 1e-10, 400, inv, red="exact")
        np.testing.assert_array_equal(res.x, x, err_msg=f"{name} {method} pc={pc}")
        assert res.true_iterations == its, (name, res.true_iterations, its)
        assert res.iterations == (info if info > 0 else 0)
        assert res.residual_norm == rnorm
        assert res.method == method
        assert res.converged == ((info == 0) and (rnorm <= 1e-10 * np.linalg.norm(b)))


def test_reference_checks_on_the_assembled_matrix():
    """tests/test_projection_method_contract.py's manufactured Laplacian, through the
    device product, and the preconditioned and plain BiCGSTAB solves agreeing."""
    from pyflow_solver_gb300.linear_solvers.interface import solve
    from pyflow_solver_gb300.linear_solvers.preconditioners import jacobi_preconditioner
    from pyflow_solver_gb300.linear_solvers.sparse import CsrMatrix
    from pyflow_solver_gb300.solvers.pressure_solver import assemble_negative_laplacian
    nx = ny = 8
    X, Y = np.meshgrid(np.arange(1, nx + 1) * 1.0, np.arange(1, ny + 1) * 1.0)
    A = assemble_negative_laplacian(nx, ny, 1.0, 1.0)
    lap = (CsrMatrix.from_any(A) @ ((X**2 + Y**2) / 4.0).ravel()).reshape(ny, nx)
    assert np.allclose(np.abs(lap[2:-2, 2:-2]), 1.0, atol=1e-10)
    A = assemble_negative_laplacian(24, 20, 1.0, 1.0)
    b = np.random.default_rng(3).standard_normal(A.shape[0])
    r_pc = solve(A, b, tol=1e-12, maxiter=2000, M=jacobi_preconditioner(A))
    r_no = solve(A, b, tol=1e-12, maxiter=2000)
    assert r_pc.converged and r_no.converged
    assert np.max(np.abs(r_pc.x - r_no.x)) / np.max(np.abs(r_pc.x)) < 1e-9


def test_python_linear_operators_are_refused():
    import scipy.sparse.linalg as spla

    from pyflow_solver_gb300.linear_solvers.interface import solve
    op = spla.LinearOperator((4, 4), matvec=lambda v: 2.0 * v)
    with pytest.raises(TypeError):
        solve(op, np.ones(4), method="cg")
