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


def _refine_band(theta, res2, lmax, tol, near_c, low_x=0.0):
    t = np.ascontiguousarray(theta, dtype=np.float64)
    r = np.ascontiguousarray(res2, dtype=np.float64)
    out = np.zeros(4)
    nmgpu.lib().nm_test_refine_band(_dp(t), _dp(r), len(t), lmax, tol, near_c, low_x, _dp(out))
    return out[0], int(out[1]), out[2], out[3]


def _degree(theta, res2, c, lmax, tol):
    need = 0.0
    for t, r in zip(theta, res2):
        if r > tol:
            need = max(need, math.acosh(4.0 * (lmax / t) * r / tol) / math.acosh(1 + 2 * (c - t) / (lmax - c)))
    return 0 if need == 0 else max(8, min(4000, math.ceil(need)))


def _growth(theta, c, lmax, d):
    a0 = math.acosh(1 + 2 * c / (lmax - c))
    return max(d * (a0 - math.acosh(1 + 2 * (c - t) / (lmax - c))) for t in theta)


def _low_growth(theta, c, lmax, d, low_x):
    a = lambda x: math.acosh(1 + 2 * (c - x) / (lmax - c))
    xs = [low_x * 10 ** (-0.25 * k) for k in range(33)]
    return max(math.log(x / t) + d * (a(x) - a(t)) for t in theta if t > low_x for x in xs)


# a block of 32 Ritz values of a 1.2M-DOF-like spectrum (lmax / b ~ 1e3)
_TH = np.linspace(1.0e-4, 1.5e-4, 32)
_LMAX = 0.2


@pytest.mark.parametrize("res2", [1e-3, 1e-6, 3e-8])
def test_refinement_first_pass_band(res2):
    """First pass: the damped band starts at 8 x the block's top Ritz value
    (lmax / 2 at most); the degree is the largest over the block of
    acosh(4 (lmax / theta) res2 / tol) / acosh(1 + 2 (c - theta) / (lmax - c))."""
    r = np.full(32, res2)
    tol = 1e-10 * math.sqrt(1.2e6)
    c, d, g, _ = _refine_band(_TH, r, _LMAX, tol, 0.0)
    assert c == pytest.approx(8 * _TH.max(), rel=1e-15)
    assert d == _degree(_TH, r, c, _LMAX, tol)
    if d:
        assert g == pytest.approx(_growth(_TH, c, _LMAX, d), rel=1e-12)


@pytest.mark.parametrize("res2,near,low_x", [(1e-6, 1.05 * 1.5 * 1.5e-4, 0.0), (1e-3, 1.05 * 1.5 * 1.5e-4, 0.0),
                                            (1e-7, 1.6e-4, 0.0), (1e-6, 1.05 * 1.5 * 1.5e-4, 4e-6),
                                            (1e-6, 1.05 * 1.5 * 1.5e-4, 6e-5)])
def test_refinement_near_pass_band_bounds_growth(res2, near, low_x):
    """Later passes: the band starts at near_c (or 1.05 x the block's top),
    moved up only as far as needed to keep the growth below the Ritz
    values, d (acosh l(0) - acosh l(theta)), under log 1e3, and the gain of
    the modes in (0, low_x] below the refined set, log(x / theta) +
    d (acosh l(x) - acosh l(theta)), under log 2."""
    r = np.full(32, res2)
    tol = 1e-10 * math.sqrt(1.2e6)
    c, d, g, gl = _refine_band(_TH, r, _LMAX, tol, near, low_x)
    lo = max(near, 1.05 * _TH.max())
    assert lo <= c <= 8 * _TH.max()
    assert d == _degree(_TH, r, c, _LMAX, tol)
    assert g == pytest.approx(_growth(_TH, c, _LMAX, d), rel=1e-12)
    lim, lim_low = math.log(1e3), math.log(2.0)
    if low_x > 0:
        assert gl == pytest.approx(_low_growth(_TH, c, _LMAX, d, low_x), rel=1e-12, abs=1e-12)
        assert gl <= lim_low + 1e-9
    assert g <= lim + 1e-9
    if c > lo * (1 + 1e-12):
        c2 = c * (1 - 1e-6)
        d2 = _degree(_TH, r, c2, _LMAX, tol)
        assert (_growth(_TH, c2, _LMAX, d2) > lim - 1e-3 or
                (low_x > 0 and _low_growth(_TH, c2, _LMAX, d2, low_x) > lim_low - 1e-3))


def test_filter_value_matches_chebyshev_series():
    xintv = [3.9e-7, 1.58e-4, -1e-8, 0.6]
    x = np.array(xintv)
    p = O.find_pol(xintv, 0.8, 0.7, 2, 10000, 1)
    for lam in (0.0, 1e-5, 1.58e-4, 1.3 * 1.58e-4, 0.3):
        ref = np.polynomial.chebyshev.chebval((lam - p.cc) / p.dd, p.mu)
        got = nmgpu.lib().nm_test_filter_value(_dp(x), 0.8, 0.7, 1, lam)
        assert abs(got - ref) <= 1e-12 * max(1.0, abs(ref))


def _ritz_first(evals, bar, guard_bar, max_guard=-1):
    e = np.ascontiguousarray(evals, dtype=np.float64)
    return nmgpu.lib().nm_test_ritz_first(_dp(e), len(e), bar, guard_bar, max_guard)


def test_ritz_selection_with_guards():
    """The block Lanczos keeps the Ritz values of T (ascending filter
    values) at or above the bar, and with a guard bar up to a cap more just
    below it, largest filter value first."""
    ev = np.array([0.0, 0.01, 0.05, 0.2, 0.5, 0.79, 0.8, 0.9, 1.0])
    assert _ritz_first(ev, 0.8, -1.0) == 6                 # no guards: the bar alone
    assert _ritz_first(ev, 0.8, 0.9) == 6                  # a guard bar above the bar is ignored
    assert _ritz_first(ev, 0.8, 0.1) == 3                  # 0.79, 0.5, 0.2 join as guards
    assert _ritz_first(ev, 0.8, 0.1, max_guard=2) == 4     # capped at two
    assert _ritz_first(ev, 0.8, 1e-9) == 1                 # default cap (3 / 2 + 64) does not bind
    assert _ritz_first(ev, 1.1, 0.1) == len(ev)            # nothing above the bar: no guards either
    big = np.linspace(0.0, 1.0, 1000)
    first = _ritz_first(big, 0.9, 1e-9)
    above = int(np.sum(big >= 0.9))
    assert len(big) - first == above + above // 2 + 64     # default cap


def test_guard_window():
    """The refinement keeps the ascending Rayleigh quotients within
    [a / g, g b]."""
    th = np.ascontiguousarray([1e-9, 0.5, 0.7, 1.0, 2.0, 2.9, 3.1, 10.0])
    out = (C.c_int * 2)()
    nmgpu.lib().nm_test_window_range(_dp(th), len(th), 1.0 / 1.5, 2.0 * 1.5, out)
    assert (out[0], out[1]) == (2, 6)
    nmgpu.lib().nm_test_window_range(_dp(th), len(th), 20.0, 30.0, out)
    assert out[0] == out[1]
