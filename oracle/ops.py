"""NumPy restatement of the reference's array operators (test infrastructure only).

Every function keeps the reference's floating-point evaluation order, so that
each result is bit-identical to the reference function on the same input
(IEEE binary64, no contraction):

* ``gradient_coherent``   src/pyflow/numerics/core_ops_coherent.py:45-61
* ``divergence_coherent`` src/pyflow/numerics/core_ops_coherent.py:63-79
* ``laplacian_coherent``  src/pyflow/numerics/core_ops_coherent.py:81-84
* ``divergence_central``  src/pyflow/numerics/fluid_ops.py:8-28 (``divergence``)
* ``advect_quick``        src/pyflow/numerics/operators/advection.py:45-84
* ``advect_upwind``       src/pyflow/numerics/operators/advection.py:17-43
* ``neg_laplacian_pinned`` the ``_matvec`` of ``_NegLaplacianPinned``,
  src/pyflow/solvers/pressure_solver.py:97-105
* ``jacobi_inv_diag``     ``assemble_negative_laplacian`` (pressure_solver.py:15-40)
  followed by ``jacobi_preconditioner`` (linear_solvers/preconditioners.py:18-19):
  only the diagonal is used, so it is built analytically here.

Arrays are interior fields of shape (ny, nx), row index = y.
"""
from __future__ import annotations

import numpy as np


def gradient_coherent(p, dx, dy):
    ny, nx = p.shape
    if ny < 2 or nx < 2:
        return np.zeros_like(p), np.zeros_like(p)
    gx = np.zeros_like(p)
    gy = np.zeros_like(p)
    gx[:, :-1] = (p[:, 1:] - p[:, :-1]) / dx
    gy[:-1, :] = (p[1:, :] - p[:-1, :]) / dy
    return gx, gy


def divergence_coherent(u, v, dx, dy):
    ny, nx = u.shape
    if ny < 2 or nx < 2:
        return np.zeros_like(u)
    d = np.zeros_like(u)
    # the x part is added to a zero field first, then the y part
    d[:, 1:] += (u[:, 1:] - u[:, :-1]) / dx
    d[:, 0] += u[:, 0] / dx
    d[1:, :] += (v[1:, :] - v[:-1, :]) / dy
    d[0, :] += v[0, :] / dy
    return d


def laplacian_coherent(p, dx, dy):
    gx, gy = gradient_coherent(p, dx, dy)
    return divergence_coherent(gx, gy, dx, dy)


def neg_laplacian_pinned(x_flat, nx, ny, dx, dy):
    """A x with A = -lap_c and row 0 replaced by the identity (non-symmetric pin)."""
    lap = laplacian_coherent(x_flat.reshape(ny, nx), dx, dy)
    out = (-lap).reshape(-1)
    out[0] = x_flat[0]
    return out


def jacobi_inv_diag(nx, ny, dx, dy):
    """Inverse diagonal of the assembled matrix of ``assemble_negative_laplacian``.

    Ring cells (i in {0,nx-1} or j in {0,ny-1}) carry an identity row (D=1);
    the interior carries 2/dx**2 + 2/dy**2.  ``invD = 1/D`` where D != 0.
    """
    inv = np.ones((ny, nx))
    if nx > 2 and ny > 2:
        d_int = 2.0 / dx**2 + 2.0 / dy**2
        inv[1:-1, 1:-1] = 1.0 / d_int
    return inv.reshape(-1)


def jacobi_interior_value(dx, dy):
    """The interior entry of ``invD`` exactly as the reference rounds it."""
    return 1.0 / (2.0 / dx**2 + 2.0 / dy**2)


def divergence_central(u, v, dx, dy):
    """Central divergence with one-sided edges; the last column (rows 1..ny-2) stays 0."""
    ny, nx = u.shape
    d = np.zeros_like(u)
    d[1:-1, 1:-1] = (u[1:-1, 2:] - u[1:-1, 0:-2]) / (2.0 * dx) + (v[2:, 1:-1] - v[0:-2, 1:-1]) / (2.0 * dy)
    d[1:-1, 0] = (u[1:-1, 1] - u[1:-1, 0]) / dx + (v[2:, 0] - v[0:-2, 0]) / (2.0 * dy)
    d[0, 1:-1] = (u[0, 2:] - u[0, :-2]) / (2.0 * dx) + (v[1, 1:-1] - v[0, 1:-1]) / dy
    d[-1, 1:-1] = (u[-1, 2:] - u[-1, :-2]) / (2.0 * dx) + (v[-1, 1:-1] - v[-2, 1:-1]) / dy
    d[0, 0] = (u[0, 1] - u[0, 0]) / dx + (v[1, 0] - v[0, 0]) / dy
    d[0, -1] = (u[0, -1] - u[0, -2]) / dx + (v[1, -1] - v[0, -1]) / dy
    d[-1, 0] = (u[-1, 1] - u[-1, 0]) / dx + (v[-1, 0] - v[-2, 0]) / dy
    d[-1, -1] = (u[-1, -1] - u[-1, -2]) / dx + (v[-1, -1] - v[-2, -1]) / dy
    return d


def _quick_faces(f, vel, axis):
    """QUICK face values (east/west along x for axis=1, north/south along y for axis=0).

    The reference pads ``f`` by 2 cells with edge values and, per cell, picks the
    upstream-biased three-point stencil by the sign of the cell velocity
    (``>= 0`` counts as positive).  Every face value is evaluated as
    ``((3/8)*a + (6/8)*b) - (1/8)*c`` in that order.
    """
    ph = np.pad(f, 2, mode="edge")
    ny, nx = f.shape
    if axis == 1:
        def s(k):  # shifted view: column offset k relative to the cell
            return ph[2:2 + ny, 2 + k:2 + k + nx]
    else:
        def s(k):
            return ph[2 + k:2 + k + ny, 2:2 + nx]
    pos = vel >= 0
    hi_pos = (3 / 8) * s(1) + (6 / 8) * s(0) - (1 / 8) * s(-1)
    hi_neg = (3 / 8) * s(-1) + (6 / 8) * s(0) - (1 / 8) * s(1)
    lo_pos = (3 / 8) * s(0) + (6 / 8) * s(-1) - (1 / 8) * s(-2)
    lo_neg = (3 / 8) * s(-2) + (6 / 8) * s(-1) - (1 / 8) * s(0)
    return np.where(pos, hi_pos, hi_neg), np.where(pos, lo_pos, lo_neg)


def advect_quick(u, v, f, dx, dy):
    phi_e, phi_w = _quick_faces(f, u, axis=1)
    phi_n, phi_s = _quick_faces(f, v, axis=0)
    return (u * phi_e - u * phi_w) / dx + (v * phi_n - v * phi_s) / dy


def advect_upwind(u, v, f, dx, dy):
    ny, nx = f.shape
    # backward difference where the velocity is > 0 (zero difference f-f at the
    # low edge), forward difference (clamped at the high edge) otherwise
    f_w = np.concatenate([f[:, :1], f[:, :-1]], axis=1)
    f_e = np.concatenate([f[:, 1:], f[:, -1:]], axis=1)
    f_s = np.concatenate([f[:1, :], f[:-1, :]], axis=0)
    f_n = np.concatenate([f[1:, :], f[-1:, :]], axis=0)
    fx = np.where(u > 0, (f - f_w) / dx, (f_e - f) / dx)
    fy = np.where(v > 0, (f - f_s) / dy, (f_n - f) / dy)
    return u * fx + v * fy
