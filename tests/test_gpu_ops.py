"""Array operators and exact reductions of libpfgb.so against the oracle (bit for bit)."""
import numpy as np
import pytest

from oracle import ops, xsum
from tests import _golden as G

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def ghosted(a):
    """A (ny, nx) array placed in the interior of a zero (ny+2, nx+2) device array (pitched view)."""
    ny, nx = a.shape
    g = torch.zeros((ny + 2, nx + 2), dtype=torch.float64, device="cuda")
    g[1:-1, 1:-1] = dev(a)
    return g[1:-1, 1:-1]


def test_operators_match_golden_fixtures():
    from pyflow_solver_gb300.numerics import core_ops_coherent as coh, fluid_ops
    from pyflow_solver_gb300.numerics.operators import advection as adv
    g = G.load("ops")
    keys = sorted({k.split("_")[0] for k in g.files if k[0].isdigit()})
    for key in keys:
        u, v, p = g[f"{key}_u"], g[f"{key}_v"], g[f"{key}_p"]
        dx, dy = (float(x) for x in g[f"{key}_dxdy"])
        for wrap in (dev, ghosted):
            U, V, P = wrap(u), wrap(v), wrap(p)
            gx, gy = coh.gradient_coherent(P, dx, dy)
            np.testing.assert_array_equal(gx.cpu().numpy(), g[f"{key}_gx"])
            np.testing.assert_array_equal(gy.cpu().numpy(), g[f"{key}_gy"])
            np.testing.assert_array_equal(coh.divergence_coherent(U, V, dx, dy).cpu().numpy(), g[f"{key}_divc"])
            np.testing.assert_array_equal(coh.laplacian_coherent(P, dx, dy).cpu().numpy(), g[f"{key}_lap"])
            np.testing.assert_array_equal(fluid_ops.divergence(U, V, 1.0, 1.0).cpu().numpy(), g[f"{key}_divcentral"])
            np.testing.assert_array_equal(fluid_ops.divergence(U, V, dx, dy).cpu().numpy(), g[f"{key}_divcentral_h"])
            np.testing.assert_array_equal(adv.advect_quick(U, V, U, dx, dy).cpu().numpy(), g[f"{key}_quick_u"])
            np.testing.assert_array_equal(adv.advect_quick(U, V, V, dx, dy).cpu().numpy(), g[f"{key}_quick_v"])
            np.testing.assert_array_equal(adv.advect_upwind(U, V, U, dx, dy).cpu().numpy(), g[f"{key}_upwind_u"])
            np.testing.assert_array_equal(adv.advect_upwind(U, V, V, dx, dy).cpu().numpy(), g[f"{key}_upwind_v"])


@pytest.mark.parametrize("nx,ny", [(64, 64), (97, 33), (2, 7), (300, 257)])
@pytest.mark.parametrize("dx", [1.0, 1.0 / 63, 0.37])
def test_operators_random_fields(nx, ny, dx):
    from pyflow_solver_gb300.numerics import core_ops_coherent as coh, fluid_ops
    from pyflow_solver_gb300.numerics.operators import advection as adv
    rng = np.random.default_rng(nx * 1000 + ny)
    u, v, p = (rng.standard_normal((ny, nx)) * 10.0 ** rng.uniform(-3, 3) for _ in range(3))
    dy = dx * 1.5
    U, V, P = ghosted(u), ghosted(v), ghosted(p)
    np.testing.assert_array_equal(coh.laplacian_coherent(P, dx, dy).cpu().numpy(), ops.laplacian_coherent(p, dx, dy))
    np.testing.assert_array_equal(coh.divergence_coherent(U, V, dx, dy).cpu().numpy(), ops.divergence_coherent(u, v, dx, dy))
    np.testing.assert_array_equal(fluid_ops.divergence(U, V, 1.0, 1.0).cpu().numpy(), ops.divergence_central(u, v, 1.0, 1.0))
    np.testing.assert_array_equal(adv.advect_quick(U, V, V, dx, dy).cpu().numpy(), ops.advect_quick(u, v, v, dx, dy))
    np.testing.assert_array_equal(adv.advect_upwind(U, V, U, dx, dy).cpu().numpy(), ops.advect_upwind(u, v, u, dx, dy))


@pytest.mark.parametrize("kind", ["neg_laplacian_pinned", "laplacian_dirichlet"])
def test_pressure_operators(kind):
    from pyflow_solver_gb300.linear_solvers.operators import PressureOperator
    nx, ny, dx, dy = 45, 38, 1.0 / 44, 1.0 / 37
    x = np.random.default_rng(3).standard_normal(nx * ny)
    A = PressureOperator(kind, nx, ny, dx, dy)
    got = A.matvec(dev(x)).cpu().numpy()
    if kind == "neg_laplacian_pinned":
        ref = ops.neg_laplacian_pinned(x, nx, ny, dx, dy)
    else:
        ref = ops.laplacian_coherent(x.reshape(ny, nx), dx, dy).reshape(-1)
        ring = np.zeros((ny, nx), bool)
        ring[0, :] = ring[-1, :] = ring[:, 0] = ring[:, -1] = True
        ref[ring.reshape(-1)] = x[ring.reshape(-1)]
    np.testing.assert_array_equal(got, ref)


def _xdot_gpu(a, b=None):
    import ctypes

    from pyflow_solver_gb300 import _capi
    from pyflow_solver_gb300._device import stream_handle
    lib = _capi.load()
    A = dev(a)
    r = ctypes.c_double()
    if b is None:
        _capi.check(lib.pfgb_xsum(A.data_ptr(), A.numel(), ctypes.byref(r), stream_handle()), "xsum")
    else:
        B = dev(b)
        _capi.check(lib.pfgb_xdot(A.data_ptr(), B.data_ptr(), A.numel(), ctypes.byref(r), stream_handle()), "xdot")
    return r.value


@pytest.mark.parametrize("seed,n,spread", [(0, 1, 0), (1, 1000, 0), (2, 4096, 30), (3, 100_003, 120),
                                           (4, 3_000_000, 8), (5, 50_000, 470), (6, 2048, 480)])
def test_exact_dot_matches_twin(seed, n, spread):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(n) * np.exp2(rng.integers(-spread, spread + 1, n))
    b = rng.standard_normal(n) * np.exp2(rng.integers(-spread, spread + 1, n))
    a[rng.random(n) < 0.05] = 0.0
    assert _xdot_gpu(a, b) == xsum.xdot(a, b)
    assert _xdot_gpu(a) == xsum.xsum(a)


def test_exact_dot_edge_cases():
    rng = np.random.default_rng(7)
    a = rng.standard_normal(5000)
    b = rng.standard_normal(5000)
    assert _xdot_gpu(np.concatenate([a, a]), np.concatenate([b, -b])) == 0.0
    sub = np.array([5e-324, 1e-310, -3e-320, 1.0, -1.0])
    assert _xdot_gpu(sub) == xsum.xsum(sub)
    assert _xdot_gpu(np.array([2.0**-1000, 2.0**-60]), np.array([2.0**-70, 2.0**-1000])) == xsum.xdot(
        np.array([2.0**-1000, 2.0**-60]), np.array([2.0**-70, 2.0**-1000]))
    big = np.array([1e300, 1e300, -1e300])
    assert _xdot_gpu(big) == 1e300
    assert np.isnan(_xdot_gpu(np.array([1.0, np.nan])))
    assert _xdot_gpu(np.array([np.inf, 1.0])) == np.inf
    assert np.isnan(_xdot_gpu(np.array([np.inf, -np.inf])))
    assert np.isnan(_xdot_gpu(np.array([np.inf, 2.0]), np.array([0.0, 1.0])))
    # ties to even at the last place
    t = np.array([1.0, 2.0**-53, 2.0**-110])
    assert _xdot_gpu(t) == xsum.xsum(t)
    t = np.array([1.0, 2.0**-53])
    assert _xdot_gpu(t) == 1.0


def test_integer_pipe_conversions_equal_the_hardware_ones():
    """The binary64 <-> binary32 conversions and the exact halving done with integer
    operations (icvt.cuh) give the hardware instructions' results bit for bit."""
    import ctypes

    from pyflow_solver_gb300 import _capi
    from pyflow_solver_gb300._device import stream_handle
    bad = (ctypes.c_longlong * 3)()
    _capi.check(_capi.load().pfgb_selftest_conversions(1 << 24, stream_handle(), bad), "selftest_conversions")
    assert list(bad) == [0, 0, 0]
