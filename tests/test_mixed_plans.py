"""Host-side decisions of the mixed-precision path, checked on the CPU
through the library's test hooks (no GPU needed):

* inner Chebyshev degrees matched to FP32 accuracy: the smallest d with
  2 sigma^d <= eps, sigma = (sqrt(k) - 1) / (sqrt(k) + 1), k = lmax / lmin,
  never above the reference's degree;
* p(0) of the designed filter, against numpy's Chebyshev series evaluated
  at -cc/dd with the oracle's coefficients;
* the refinement plan: degree cap 2 sqrt(lmax / (b - a)), band start
  max(25 / deg^2, 2 b / lmax), per-block degree deg sqrt(theta_0 / theta)
  clamped to [20, deg].
"""
import ctypes as C
import math

import numpy as np
import pytest

from normalmodes_gb300 import nmgpu
from oracle import oracle as O


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _expected_degree(lmin, lmax, ref, eps):
    k = lmax / lmin
    s = (math.sqrt(k) - 1) / (math.sqrt(k) + 1)
    return max(1, min(ref, math.ceil(math.log(eps / 2) / math.log(s))))


@pytest.mark.parametrize("lmin,lmax,ref", [(0.25, 4.3475, 45), (0.5, 2.5, 25), (0.25, 4.3475, 100), (0.1, 50.0, 30)])
def test_fp32_matched_chebyshev_degree(lmin, lmax, ref):
    eps = 2.0 ** -24
    d = nmgpu.lib().nm_test_cheb_degree(lmin, lmax, ref, eps)
    assert d == _expected_degree(lmin, lmax, ref, eps)
    assert d <= ref
    if (lmin, lmax, ref) == (0.25, 4.3475, 45):
        assert d == 36  # P2 mass matrices: 36 instead of the reference's 45


@pytest.mark.parametrize("xintv", [
    [1.579e-6, 3.9478e-5, -5e-9, 1.475e-3],
    [3.9e-7, 1.58e-4, -1e-8, 0.6],
])
def test_filter_value_at_zero(xintv):
    x = np.array(xintv)
    p0 = nmgpu.lib().nm_test_filter_at_zero(_dp(x), 0.8, 0.7, 1)
    p = O.find_pol(xintv, 0.8, 0.7, 2, 10000, 1)
    ref = np.polynomial.chebyshev.chebval(-p.cc / p.dd, p.mu)
    assert abs(p0 - ref) <= 1e-12 * max(1.0, abs(ref))


def _plan(xintv, req):
    x = np.array(xintv, dtype=np.float64)
    out = (C.c_int * 2)()
    band = np.zeros(2)
    nmgpu.lib().nm_test_polish_plan(_dp(x), req, out, _dp(band))
    return out[0], bool(out[1]), band[0], band[1]


def test_refinement_plan_large_model():
    # 1.2 M-DOF P2 ball, 0.1-2.0 mHz: the default degree 80 is below the cap
    a, b, lmax = 3.9478e-7, 1.5791e-4, 0.6
    deg, refine, cfrac, bfloor = _plan([a, b, -1e-9, lmax], 0)
    cap = math.floor(2 * math.sqrt(lmax / (b - a)))
    assert cap > 80 and deg == 80 and refine
    assert bfloor == pytest.approx(2 * b / lmax)
    assert cfrac == pytest.approx(max(25 / 80 ** 2, 2 * b / lmax))
    x = np.array([a, b, -1e-9, lmax])
    band = np.zeros(1)
    for ratio, want in ((1.0, 80), (4.0, 40), (16.0, 20), (400.0, 20)):
        d = nmgpu.lib().nm_test_polish_block(_dp(x), 0, a, a * ratio, _dp(band))
        assert d == want, (ratio, d)
        assert band[0] == pytest.approx(max(25 / d ** 2, 2 * b / lmax))


def test_refinement_plan_narrow_spectrum_and_off():
    # small P1 ball: lmax / (b - a) ~ 40 caps the degree at 12
    a, b, lmax = 1.579e-6, 3.9478e-5, 1.5e-3
    deg, refine, cfrac, _ = _plan([a, b, 0.0, lmax], 0)
    assert deg == math.floor(2 * math.sqrt(lmax / (b - a))) == 12 and refine
    assert cfrac == pytest.approx(max(25 / 144, 2 * b / lmax))
    # off on request, and when the band would start in the upper half
    assert _plan([a, b, 0.0, lmax], -1)[:2] == (0, False)
    assert _plan([1e-3, 0.4, 0.0, 1.0], 0)[1] is False
