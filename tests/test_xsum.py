"""The twin's exactly rounded reductions against exact rational arithmetic."""
from fractions import Fraction

import numpy as np
import pytest

from oracle.xsum import xdot, xnorm, xsum


def exact_dot(a, b):
    t = sum((Fraction(float(x)) * Fraction(float(y)) for x, y in zip(a, b)), Fraction(0))
    return float(t)


def vectors(seed, n, spread):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(n) * np.exp2(rng.integers(-spread, spread + 1, n))
    b = rng.standard_normal(n) * np.exp2(rng.integers(-spread, spread + 1, n))
    a[rng.random(n) < 0.05] = 0.0
    return a, b


@pytest.mark.parametrize("seed,n,spread", [(0, 1000, 0), (1, 4096, 30), (2, 777, 200), (3, 64, 400)])
def test_xdot_exactly_rounded(seed, n, spread):
    a, b = vectors(seed, n, spread)
    assert xdot(a, b) == exact_dot(a, b)


def test_xdot_cancellation_and_order_independence():
    rng = np.random.default_rng(5)
    a = rng.standard_normal(2000)
    b = rng.standard_normal(2000)
    a = np.concatenate([a, a])
    b = np.concatenate([b, -b])          # exact cancellation: the sum is 0
    assert xdot(a, b) == 0.0
    perm = rng.permutation(a.size)
    a2, b2 = vectors(9, 3000, 60)
    p2 = rng.permutation(a2.size)
    assert xdot(a2, b2) == xdot(a2[p2], b2[p2])
    assert xdot(a[perm], b[perm]) == 0.0


def test_xsum_and_specials():
    rng = np.random.default_rng(11)
    t = rng.standard_normal(5000) * 1e10
    assert xsum(t) == float(sum((Fraction(float(x)) for x in t), Fraction(0)))
    assert np.isnan(xsum(np.array([1.0, np.nan])))
    assert xsum(np.array([np.inf, 1.0])) == np.inf
    assert np.isnan(xsum(np.array([np.inf, -np.inf])))
    assert np.isnan(xdot(np.array([np.inf]), np.array([0.0])))
    assert xnorm(np.array([3.0, 4.0])) == 5.0
    assert xsum(np.array([])) == 0.0
