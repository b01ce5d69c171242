"""The allocation-free CG entry point against the allocating one.

``pfgb_cg_solve_noalloc`` serves callers that may not allocate device memory
when they solve: a real-time loop that must not stall on cudaMalloc/cudaFree
(both can synchronise the whole device), or an application that reserved the
device memory for its own pool.  It must return exactly what ``pfgb_cg_solve`` returns.  Two calls in a
row with different right-hand sides, then calls on smaller grids of other shapes,
check that the shared scratch array, which keeps the previous call's contents
(vectors and tile tables of a larger grid), does not leak into the next result;
the device's free memory is the same before and after each call once the
library's module is loaded.  This file is collected last on purpose: it passes
alone in a fresh process and after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _rhs(seed, nx, ny):
    rng = np.random.default_rng(seed)
    b = rng.standard_normal(nx * ny)
    b -= b.mean()
    b[0] = 0.0
    return torch.from_numpy(b).cuda()


def _solve(fn, op, b, nx, ny, dx, dy, precond, interior, tol, maxiter, free=None):
    """One solve through the C ABI; with `free` (a list), the device's free bytes just
    before and just after the call are appended to it."""
    from pyflow_solver_gb300 import _capi
    from pyflow_solver_gb300._device import stream_handle
    x = torch.full_like(b, float("nan"))
    out = _capi.SolveOut()
    torch.cuda.synchronize()
    if free is not None:
        free.append(torch.cuda.mem_get_info()[0])
    rc = fn(op, b.data_ptr(), x.data_ptr(), nx, ny, dx, dy, precond, interior, tol, maxiter, stream_handle(),
            ctypes.byref(out))
    if free is not None:
        free.append(torch.cuda.mem_get_info()[0])
    _capi.check(rc, fn.__name__)
    return x.cpu().numpy(), (out.info, out.iterations, out.bnorm, out.res_sq)


@pytest.mark.parametrize("op", [0, 1])
def test_noalloc_cg_matches_allocating_cg_on_two_calls(op):
    from pyflow_solver_gb300 import _capi
    lib = _capi.load()
    precond = 1 if op == 0 else 0
    # two calls on one grid, then smaller grids of other shapes over the scratch that
    # the larger grid left behind (a 2 x N strip included)
    calls = [(96, 80, 1), (96, 80, 2), (40, 70, 3), (2, 301, 4)]
    free = []
    for call, (nx, ny, seed) in enumerate(calls):
        dx, dy = 1.0 / (nx - 1), 1.0 / (ny - 1)
        interior = 1.0 / (2.0 / dx**2 + 2.0 / dy**2)
        b = _rhs(seed, nx, ny)
        x_ref, o_ref = _solve(lib.pfgb_cg_solve, op, b, nx, ny, dx, dy, precond, interior, 1e-8, 120)
        x_new, o_new = _solve(lib.pfgb_cg_solve_noalloc, op, b, nx, ny, dx, dy, precond, interior, 1e-8, 120,
                              free=free if call > 0 else None)
        # the tests of this suite compare CUDA results bit for bit: tolerance 0
        np.testing.assert_array_equal(x_new, x_ref, err_msg=f"call {call} ({nx} x {ny})")
        assert o_new == o_ref, (call, o_new, o_ref)
    # after the first call (which may load the library's module, and with it the
    # array, on this device) no call changes the device's free memory
    assert all(a == b for a, b in zip(free[0::2], free[1::2])), free


def test_noalloc_cg_rejects_grids_beyond_its_scratch():
    from pyflow_solver_gb300 import _capi
    from pyflow_solver_gb300._device import stream_handle
    lib = _capi.load()
    nx, ny = 600, 600                      # 360,000 cells > 262,144
    b = torch.zeros(nx * ny, dtype=torch.float64, device="cuda")
    x = torch.zeros_like(b)
    out = _capi.SolveOut()
    rc = lib.pfgb_cg_solve_noalloc(0, b.data_ptr(), x.data_ptr(), nx, ny, 1.0, 1.0, 0, 0.25, 1e-8, 10,
                                   stream_handle(), ctypes.byref(out))
    assert rc == -1
    assert "262144-cell limit" in _capi.last_error()
