"""Exactly rounded reductions for the oracle twin (test infrastructure only).

The reference reduces with ``np.dot`` (BLAS ``ddot``, summation order chosen by
the BLAS kernel of the machine), ``np.linalg.norm`` (``sqrt(dot(x, x))``),
``np.mean`` / ``np.sum`` (NumPy pairwise summation).  Their rounding depends on
the order, and the pressure CG of the reference is cut off at ``lin_maxiter``
on a non-symmetric operator, so that order changes u, v and p well above
1e-10.  The twin therefore defines every reduction as the *exactly rounded*
value of the exact mathematical result:

* ``xdot(a, b)``  = RN(sum_i a_i * b_i)   (products exact, one rounding)
* ``xsum(t)``     = RN(sum_i t_i)
* ``xnorm(a)``    = RN(sqrt(xdot(a, a)))

Those values do not depend on summation order, so the CUDA kernels (any tile
shape, any grid, batched or not) reproduce them bit for bit.

Non-finite operands follow IEEE summation: NaN if any term is NaN or if both
+inf and -inf occur, else the infinity.  Finite totals beyond the double range
round to +-inf.
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

_SPLIT = 134217729.0  # 2**27 + 1, Dekker's splitting constant for binary64
# Range in which Dekker's TwoProduct is exact without FMA: no overflow in the
# split, and error terms far above the subnormal range.
_LO = 2.0 ** -450
_HI = 2.0 ** 450


def _special_total(terms: np.ndarray) -> float:
    if np.isnan(terms).any():
        return math.nan
    pos = bool((terms == np.inf).any())
    neg = bool((terms == -np.inf).any())
    if pos and neg:
        return math.nan
    return math.inf if pos else -math.inf


def _fraction_to_float(f: Fraction) -> float:
    try:
        return float(f)
    except OverflowError:
        return math.inf if f > 0 else -math.inf


def _exact_sum_fraction(values) -> float:
    tot = Fraction(0)
    for v in values:
        tot += Fraction(float(v))
    return _fraction_to_float(tot)


def xsum(t) -> float:
    """Exactly rounded sum of the float64 values ``t`` (order independent)."""
    t = np.ascontiguousarray(t, dtype=np.float64).ravel()
    if t.size == 0:
        return 0.0
    if not np.isfinite(t).all():
        return _special_total(t)
    try:
        return math.fsum(t.tolist())
    except OverflowError:
        return _exact_sum_fraction(t)


def _two_prod(a: np.ndarray, b: np.ndarray):
    """Dekker's TwoProduct: p + e == a*b exactly (in range, without FMA)."""
    p = a * b
    c = _SPLIT * a
    ah = c - (c - a)
    al = a - ah
    c = _SPLIT * b
    bh = c - (c - b)
    bl = b - bh
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
    return p, e


def xdot(a, b) -> float:
    """Exactly rounded dot product RN(sum a_i*b_i) with exact products."""
    a = np.ascontiguousarray(a, dtype=np.float64).ravel()
    b = np.ascontiguousarray(b, dtype=np.float64).ravel()
    if a.size == 0:
        return 0.0
    prod = a * b
    if not np.isfinite(a).all() or not np.isfinite(b).all() or not np.isfinite(prod).all():
        if not np.isfinite(a).all() or not np.isfinite(b).all():
            return _special_total(prod)
        # finite operands whose rounded product overflows: exact path
        return _fraction_to_float(sum((Fraction(float(x)) * Fraction(float(y)) for x, y in zip(a, b)), Fraction(0)))
    aa = np.abs(a)
    ab = np.abs(b)
    in_range = (((aa >= _LO) & (aa <= _HI)) | (aa == 0.0)) & (((ab >= _LO) & (ab <= _HI)) | (ab == 0.0))
    tiny_prod = (np.abs(prod) < 2.0 ** -900) & (prod != 0.0)
    if in_range.all() and not tiny_prod.any():
        p, e = _two_prod(a, b)
        try:
            return math.fsum(np.concatenate([p, e]).tolist())
        except OverflowError:
            pass
    return _fraction_to_float(sum((Fraction(float(x)) * Fraction(float(y)) for x, y in zip(a, b)), Fraction(0)))


def xnorm(a) -> float:
    """RN(sqrt(xdot(a, a))): the twin of ``np.linalg.norm`` on a real vector."""
    return math.sqrt(xdot(a, a))


# Reference-equivalent reductions (bit-identical to the reference on the
# machine that runs them; their rounding depends on the BLAS build).
def ndot(a, b) -> float:
    return float(np.dot(np.ravel(a), np.ravel(b)))


def nnorm(a) -> float:
    return float(np.linalg.norm(a))


def nsum(t) -> float:
    return float(np.sum(t))


def nmean(t) -> float:
    return float(np.mean(t))


def xmean(t) -> float:
    t = np.asarray(t, dtype=np.float64)
    return xsum(t) / t.size


class Reductions:
    """A named set of reductions used by the restated step."""

    def __init__(self, mode: str):
        if mode not in ("numpy", "exact"):
            raise ValueError(f"unknown reduction mode {mode!r}")
        self.mode = mode
        if mode == "numpy":
            self.dot, self.norm, self.sum, self.mean = ndot, nnorm, nsum, nmean
        else:
            self.dot, self.norm, self.sum, self.mean = xdot, xnorm, xsum, xmean
