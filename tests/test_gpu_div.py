"""Division by a grid spacing on the integer pipe returns the IEEE quotient.

Every ``/ dx`` and ``/ dy`` of the reference's coherent operators is a NumPy
true division by a Python float.  The kernels form it from the operands'
integer significands (division by an invariant divisor with a remainder
correction and round-to-nearest-even); this checks it against the hardware
IEEE division and against NumPy on every operand class: normals over the whole
exponent range, subnormals, zeros, infinities, NaN, and quotients that
overflow or underflow.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

DIVISORS = [1.0 / 63, 1.0 / 511, 1.0 / 2047, 1.0 / 127, 1.0 / 47, 1.0 / 95, 0.37, 3.0, 7.0, 1.0 / 3,
            np.nextafter(1.0, 2.0), np.nextafter(2.0, 1.0), 1e-300, 1e300, 2.2250738585072014e-308 * 3,
            0.25, 1.0]


def operands(seed, n):
    rng = np.random.default_rng(seed)
    bits = rng.integers(0, 2**64, size=n, dtype=np.uint64)
    a = bits.view(np.float64).copy()                       # every exponent, sign and class
    a[: n // 8] = rng.standard_normal(n // 8) * 10.0 ** rng.uniform(-10, 10, n // 8)
    specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
                         1.7976931348623157e308, -1.7976931348623157e308, 1.0, -1.0, 3.0, 1e-310])
    a[: specials.size] = specials
    return a


def run(a, d, method):
    from pyflow_solver_gb300 import _capi
    from pyflow_solver_gb300._device import stream_handle
    A = torch.from_numpy(a).cuda()
    out = torch.empty_like(A)
    _capi.check(_capi.load().pfgb_div_by_constant(A.data_ptr(), out.data_ptr(), A.numel(), float(d), method,
                                                   stream_handle()), "div_by_constant")
    return out.cpu().numpy()


@pytest.mark.parametrize("d", DIVISORS)
def test_spacing_division_equals_ieee(d):
    a = operands(int(abs(np.log2(d)) * 1000) + 7, 1 << 21)
    got = run(a, d, 0)
    hw = run(a, d, 1)
    with np.errstate(all="ignore"):
        ref = a / d
    same_hw = (got.view(np.uint64) == hw.view(np.uint64)) | (np.isnan(got) & np.isnan(hw))
    same_np = (got.view(np.uint64) == ref.view(np.uint64)) | (np.isnan(got) & np.isnan(ref))
    assert same_hw.all(), a[~same_hw][:5]
    assert same_np.all(), a[~same_np][:5]
