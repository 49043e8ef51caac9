"""Analytic normal-mode frequencies of a homogeneous, non-gravitating elastic
sphere with a traction-free surface -- TEST INFRASTRUCTURE (a physics
known-answer for the assembled operators and the eigensolver).

Displacement u = grad(phi) + curl curl(r chi), phi = A j_l(h r) Y_lm,
chi = B j_l(k r) Y_lm, h = omega/alpha, k = omega/beta (Lamb 1882; Aki &
Richards, Quantitative Seismology, ch. 8).  Radial and tangential scalars:

    U = A h j_l'(h r) + B l(l+1) j_l(k r)/r
    V = A j_l(h r)/r + B (r j_l(k r))'/r

Spheroidal modes: sigma_rr = lambda div u + 2 mu U' = 0 and
V' - V/r + U/r = 0 at r = a (a 2x2 determinant in A, B; l = 0 is the radial
case with A only).  Toroidal modes: (l - 1) j_l(k a) - k a j_{l+1}(k a) = 0.
Frequencies are returned in mHz for radius in km and velocities in km/s.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.optimize import brentq
from scipy.special import spherical_jn


def _j(l, x, d=0):
    if d == 0:
        return spherical_jn(l, x)
    if d == 1:
        return spherical_jn(l, x, derivative=True)
    j, jp = spherical_jn(l, x), spherical_jn(l, x, derivative=True)
    return -(2.0 / x) * jp - (1.0 - l * (l + 1) / x ** 2) * j


def _spheroidal_det(omega, l, a, alpha, beta, rho):
    h, k = omega / alpha, omega / beta
    lam, mu = rho * (alpha ** 2 - 2 * beta ** 2), rho * beta ** 2
    r = a
    jh, jhp, jhpp = _j(l, h * r), _j(l, h * r, 1), _j(l, h * r, 2)
    jk, jkp, jkpp = _j(l, k * r), _j(l, k * r, 1), _j(l, k * r, 2)
    L = l * (l + 1)
    # column A
    U_A = h * jhp
    Up_A = h * h * jhpp
    V_A = jh / r
    Vp_A = h * jhp / r - jh / r ** 2
    div_A = -h * h * jh
    # column B
    U_B = L * jk / r
    Up_B = L * (k * jkp / r - jk / r ** 2)
    g1 = jk + k * r * jkp           # (r j)'
    g2 = 2 * k * jkp + k * k * r * jkpp  # (r j)''
    V_B = g1 / r
    Vp_B = g2 / r - g1 / r ** 2
    if l == 0:
        return lam * div_A + 2 * mu * Up_A
    m11 = lam * div_A + 2 * mu * Up_A
    m12 = 2 * mu * Up_B
    m21 = Vp_A - V_A / r + U_A / r
    m22 = Vp_B - V_B / r + U_B / r
    return m11 * m22 - m12 * m21


def _toroidal_f(omega, l, a, beta):
    x = omega * a / beta
    return (l - 1) * _j(l, x) - x * _j(l + 1, x)


def _roots(f, wmax, wmin, n=4000):
    """Sign changes of f on (wmin, wmax], refined by Brent's method.  f takes
    arrays.  Below wmin (k a < 1e-2) the determinants vanish like a power of
    omega and their sign is rounding noise, so no root is sought there."""
    w = np.linspace(wmin, wmax, n)
    with np.errstate(all="ignore"):
        v = f(w)
    out = []
    for i in np.flatnonzero(np.isfinite(v[:-1]) & np.isfinite(v[1:]) & (v[:-1] * v[1:] < 0)):
        out.append(brentq(lambda x: float(f(np.array([x]))[0]), w[i], w[i + 1], xtol=1e-14, rtol=1e-14))
    return out


def mode_table(fmax_mhz: float, a=6371.0, alpha=10.0, beta=5.7735, rho=5.51, lmax=30):
    """List of (freq_mHz, kind 'S'|'T', n, l, multiplicity 2l+1) below fmax."""
    wmax = 2 * math.pi * fmax_mhz * 1e-3
    wmin = 1e-2 * beta / a
    modes = []
    for l in range(0, lmax + 1):
        ws = _roots(lambda w: _spheroidal_det(w, l, a, alpha, beta, rho), wmax, wmin)
        for n_, w in enumerate(ws):
            modes.append((w / (2 * math.pi) * 1e3, "S", n_, l, 2 * l + 1))
        if l >= 1:
            wt = _roots(lambda w: _toroidal_f(w, l, a, beta), wmax, wmin)
            for n_, w in enumerate(wt):
                modes.append((w / (2 * math.pi) * 1e3, "T", n_, l, 2 * l + 1))
    modes.sort()
    return modes


def singlet_frequencies(fmax_mhz: float, **kw) -> np.ndarray:
    """Sorted singlet frequencies (each multiplet repeated 2l+1 times)."""
    out = []
    for f, _, _, _, mult in mode_table(fmax_mhz, **kw):
        out += [f] * mult
    return np.array(sorted(out))
