"""The refinement recurrences of the mixed path (refine64, nm_blocksolve.cu)
restated in numpy on a diagonal pencil (B = I, A = diag(lambda), so
A B~^-1 = M = diag(lambda)), against the polynomials they stand for:

* damping:  D_0 = 0, D_1 = alpha R,
            D_{j+1} = 2 l(M) D_j - D_{j-1} + 2 alpha s_j R,  u' = u + D_d / s_d
  gives u' = T_d(l(M)) u / T_d(l(theta));
* with the null-space factor:  E_0 = R, E_1 = alpha M R + (alpha theta - beta) R,
            E_{j+1} = 2 l(M) E_j - E_{j-1} + 2 alpha theta s_j R,
            u' = u + E_d / (theta s_d)
  gives u' = (M / theta) T_d(l(M)) u / T_d(l(theta)), exactly zero on the
  null space;
with R = (M - theta) u, l(x) = alpha x - beta mapping [c, lmax] to [-1, 1]
and s_j = T_j(l(theta))."""
import numpy as np
import pytest


def _cheb(d, t):
    tm1, tj = np.ones_like(t), t.copy()
    if d == 0:
        return tm1
    for _ in range(1, d):
        tm1, tj = tj, 2 * t * tj - tm1
    return tj


@pytest.mark.parametrize("purge", [False, True])
def test_recurrences_apply_the_refinement_polynomial(purge):
    rng = np.random.default_rng(1)
    lam = np.concatenate([np.zeros(20), np.sort(rng.uniform(1e-4, 1e-2, 80)), rng.uniform(0.05, 1.0, 300)])
    u = rng.standard_normal(lam.size)
    theta, lmax, d = 3e-3, 1.0, 40
    c = 8 * theta
    alpha, beta = 2.0 / (lmax - c), (lmax + c) / (lmax - c)
    l = lambda x: alpha * x - beta
    R = (lam - theta) * u
    s = [1.0, l(theta)]
    for _ in range(d):
        s.append(2 * l(theta) * s[-1] - s[-2])
    if purge:
        em1, e = R.copy(), alpha * lam * R + (alpha * theta - beta) * R
        w = theta
    else:
        em1, e = np.zeros_like(R), alpha * R
        w = 1.0
    for j in range(1, d):
        em1, e = e, 2 * l(lam) * e - em1 + 2 * alpha * w * s[j] * R
    got = u + e / (w * s[d])
    h = _cheb(d, l(lam)) / s[d]
    want = (lam / theta if purge else 1.0) * h * u
    assert np.allclose(got, want, rtol=1e-10, atol=1e-12 * np.abs(u).max())
    if purge:
        assert np.max(np.abs(got[:20])) <= 1e-12 * np.abs(u).max()  # null space removed
    # the band [c, lmax] is damped by 1 / T_d(l(theta)) (times lmax / theta with the factor)
    band = lam >= c
    bound = (lmax / theta if purge else 1.0) / abs(s[d])
    assert np.all(np.abs(want[band]) <= bound * np.abs(u[band]) * (1 + 1e-12))
