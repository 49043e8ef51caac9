"""The two recurrences of the mixed path, checked in FP64 numpy on a small
dense SPD pencil (A, B) against direct evaluation:

* range form of the filter: with p(x) = sum_k mu_k T_k((x - cc)/dd),
  p(A B^-1) Z = p(0) Z + A B^-1 Y, where Y = sum_k mu_k E_k,
  E_1 = Z / dd, E_{k+1} = 2 L E_k - E_{k-1} + 2 tau_k Z / dd,
  L = (A B^-1 - cc) / dd, tau_k = T_k(-cc / dd);
* refinement: D_k = T_k(L) B u - T_k(l(theta)) B u obeys
  D_1 = alpha r, D_{k+1} = 2 L D_k - D_{k-1} + 2 alpha tau_k(theta) r with
  r = A u - theta B u, L = alpha A B^-1 - beta, l(x) = alpha x - beta.
"""
import numpy as np


def _pencil(n=40, seed=3):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A = Q @ np.diag(np.concatenate([np.zeros(5), np.linspace(0.01, 2.0, n - 5)])) @ Q.T  # null space of dim 5
    C = rng.standard_normal((n, n))
    B = C @ C.T / n + np.eye(n)
    return A, B


def _cheb_matrix_poly(M, coefs):
    """sum_k coefs[k] T_k(M) by the three-term recurrence."""
    n = M.shape[0]
    Tkm1, Tk = np.eye(n), M.copy()
    out = coefs[0] * Tkm1 + (coefs[1] * Tk if len(coefs) > 1 else 0)
    for k in range(2, len(coefs)):
        Tkm1, Tk = Tk, 2 * M @ Tk - Tkm1
        out = out + coefs[k] * Tk
    return out


def _cheb_scalar(x, k):
    t0, t1 = 1.0, x
    if k == 0:
        return t0
    for _ in range(k - 1):
        t0, t1 = t1, 2 * x * t1 - t0
    return t1


def test_range_form_of_the_filter():
    A, B = _pencil()
    n = A.shape[0]
    Binv = np.linalg.inv(B)
    AB = A @ Binv
    cc, dd, deg = 0.3, 0.9, 12
    mu = np.random.default_rng(1).standard_normal(deg + 1)
    Z = np.random.default_rng(2).standard_normal((n, 4))
    L = (AB - cc * np.eye(n)) / dd
    W_direct = _cheb_matrix_poly(L, mu) @ Z
    l0 = -cc / dd
    tau = [_cheb_scalar(l0, k) for k in range(deg + 1)]
    p0 = sum(mu[k] * tau[k] for k in range(deg + 1))
    Ekm1, Ek = np.zeros_like(Z), Z / dd
    Y = mu[1] * Ek
    for k in range(1, deg):
        Ekp1 = 2 * L @ Ek - Ekm1 + 2 * tau[k] * Z / dd
        Y += mu[k + 1] * Ekp1
        Ekm1, Ek = Ek, Ekp1
    W = p0 * Z + AB @ Y
    assert np.allclose(W, W_direct, rtol=1e-10, atol=1e-10 * np.abs(W_direct).max())
    # the null-space content of W is exactly p(0) times that of Z
    w, V = np.linalg.eigh(A)
    N = V[:, :5]
    assert np.allclose(N.T @ W, p0 * (N.T @ Z), atol=1e-10 * np.abs(W).max())


def test_refinement_recurrence():
    A, B = _pencil()
    n = A.shape[0]
    Binv = np.linalg.inv(B)
    lam_max = np.linalg.eigvalsh(np.linalg.cholesky(Binv).T @ A @ np.linalg.cholesky(Binv)).max()
    c0 = lam_max / 16
    alpha, beta = 2 / (lam_max - c0), (lam_max + c0) / (lam_max - c0)
    u = np.random.default_rng(4).standard_normal(n)
    theta = 0.05
    r = A @ u - theta * B @ u
    L = alpha * A @ Binv - beta * np.eye(n)
    deg = 9
    lt = alpha * theta - beta
    Dkm1, Dk = np.zeros(n), alpha * r
    tkm1, tk = 1.0, lt
    for k in range(1, deg):
        Dkp1 = 2 * L @ Dk - Dkm1 + 2 * alpha * tk * r
        Dkm1, Dk = Dk, Dkp1
        tkm1, tk = tk, 2 * lt * tk - tkm1
    Bu = B @ u
    coefs = np.zeros(deg + 1)
    coefs[deg] = 1.0
    direct = _cheb_matrix_poly(L, coefs) @ Bu - _cheb_scalar(lt, deg) * Bu
    assert np.allclose(Dk, direct, rtol=1e-9, atol=1e-9 * np.abs(direct).max())
    assert np.isclose(tk, _cheb_scalar(lt, deg))


def test_range_form_keeps_the_null_space_exact_in_fp32():
    """Why the mixed path filters in range form: with the recurrence run in
    FP32, the plain form leaves FP32 rounding in the null space of A (the
    zero-frequency fluid modes), which the Lanczos then has to carry; the
    range form p(0) Z + A B^-1 Y, with Y in FP32 and only the last product
    by A in FP64, has exactly p(0) times Z's null-space content, to FP64
    rounding."""
    A, B = _pencil(n=60, seed=7)
    n = A.shape[0]
    Binv = np.linalg.inv(B)
    cc, dd, deg = 1.0, 1.05, 30
    mu = np.random.default_rng(3).standard_normal(deg + 1) / (1 + np.arange(deg + 1))
    Z = np.random.default_rng(4).standard_normal((n, 3))
    L = (A @ Binv - cc * np.eye(n)) / dd
    f32 = np.float32
    L32 = L.astype(f32)
    # plain form, FP32 recurrence
    Tkm1, Tk = Z.astype(f32), (L32 @ Z.astype(f32))
    acc = (f32(mu[0]) * Tkm1 + f32(mu[1]) * Tk)
    for k in range(2, deg + 1):
        Tkm1, Tk = Tk, f32(2) * (L32 @ Tk) - Tkm1
        acc = acc + f32(mu[k]) * Tk
    W_plain = acc.astype(np.float64)
    # range form, FP32 recurrence for Y, final A B^-1 in FP64
    l0 = -cc / dd
    tau = [_cheb_scalar(l0, k) for k in range(deg + 1)]
    p0 = sum(mu[k] * tau[k] for k in range(deg + 1))
    Z32 = Z.astype(f32)
    Ekm1, Ek = np.zeros_like(Z32), Z32 / f32(dd)
    Y = f32(mu[1]) * Ek
    for k in range(1, deg):
        Ekp1 = f32(2) * (L32 @ Ek) - Ekm1 + f32(2 * tau[k] / dd) * Z32
        Y = Y + f32(mu[k + 1]) * Ekp1
        Ekm1, Ek = Ek, Ekp1
    W_range = p0 * Z + A @ (Binv @ Y.astype(np.float64))
    w, V = np.linalg.eigh(A)
    N = V[:, :5]
    exact = p0 * (N.T @ Z)
    scale = np.abs(W_range).max()
    err_plain = np.abs(N.T @ W_plain - exact).max() / scale
    err_range = np.abs(N.T @ W_range - exact).max() / scale
    assert err_plain > 1e-9          # FP32 rounding lands in the null space
    assert err_range < 1e-13         # the range form keeps it at FP64 level
    assert err_plain > 1e4 * err_range
