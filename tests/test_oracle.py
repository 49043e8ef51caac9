"""CPU tests that pin the oracle: the golden fixtures against dense LAPACK
solves of the same pencils, the oracle reproducing its fixtures, and the
assembled operators of a homogeneous ball against the analytic spectrum of a
homogeneous elastic sphere (Lamb 1882)."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden(name):
    return np.load(os.path.join(HERE, "golden", f"{name}.npz"))


@pytest.mark.parametrize("name", ["solid_p1", "fs_p1", "solid_p1_grav", "fs_p1_grav", "const3k_p1", "prem3k_p1"])
def test_golden_fixtures_match_dense_solves(name):
    """The oracle's filtered-Lanczos eigenvalues (the fixtures the GPU tests
    compare with) against scipy.linalg.eigh of the same pencil."""
    g = _golden(name)
    assert len(g["lam"]) == len(g["lam_dense"]) > 0
    assert np.max(np.abs(g["lam"] - g["lam_dense"]) / g["lam_dense"]) < 1e-10
    assert np.max(g["err_ref"]) < 1e-10


@pytest.mark.parametrize("name", ["solid_p1", "solid_p1_grav"])
def test_oracle_reproduces_its_fixture(name):
    import ast

    from normalmodes_gb300.model import Model
    from oracle import oracle as O
    g = _golden(name)
    m = Model.ball(**ast.literal_eval(str(g["model_kw"])))
    op = O.setup_operator(m.operators(), int(g["porder"]), bounds={"B": tuple(g["b_bounds"])})
    lo, hi = (float(x) for x in g["interval"])
    r = O.apply_pevsl(op, lo, hi, ab_bounds=(float(g["xintv"][2]), float(g["xintv"][3])))
    assert r.pol.deg == int(g["pol_deg"])
    assert len(r.lam) == len(g["lam"])
    assert np.max(np.abs(r.lam - g["lam"]) / g["lam"]) < 1e-12


def test_homogeneous_ball_matches_the_analytic_sphere():
    """P2 homogeneous solid ball (vp 10, vs 5.7735 km/s, rho 5.51 g/cm^3):
    six rigid modes at zero, then the lowest 34 singlets within 2 % (6 cells
    per axis) and 1 % (8 cells) of the analytic frequencies, the error
    shrinking with the mesh."""
    from scipy.sparse.linalg import eigsh

    from normalmodes_gb300.model import Model
    from oracle import sphere_modes as S
    fa = S.singlet_frequencies(1.0)
    assert fa[0] == pytest.approx(0.3607351, rel=1e-6)  # 0T2
    mean = {}
    for nc, tol in ((6, 0.02), (8, 0.01)):
        m = Model.ball(n_cells=nc, porder=2, fluid_core=0, homogeneous=1, jitter=0.0)
        A, B = m.csr("A").to_scipy().tocsc(), m.csr("B").to_scipy().tocsc()
        w = np.sort(eigsh(A, k=40, M=B, sigma=2e-6, which="LM", return_eigenvectors=False))
        f = np.sqrt(np.maximum(w, 0.0)) / (2 * np.pi) * 1e3
        assert f[:6].max() < 1e-6
        rel = np.abs(f[6:40] - fa[:34]) / fa[:34]
        assert rel.max() < tol, (nc, rel.max())
        mean[nc] = rel.mean()
    assert mean[8] < 0.6 * mean[6]


@pytest.mark.parametrize("name", ["solid_p1", "fs_p1", "fs_p2"])
def test_oracle_operators_match_sparse_algebra(small_models, name):
    """The C oracle's operators against scipy: D = diag(B)^-1/2 and
    D_p = diag(-Ap)^-1/2 (src/mod_matvec.f90:252-441), B_s x, the solid
    A_s x, and for fluid-solid models D (Ad - E Ap^-1 ET) D x with the exact
    Ap^-1, within the Golub-Varga bound 2 sigma^d of the Chebyshev Ap solve;
    the Chebyshev B solve recovers x from B_s x within 2 sigma^d sqrt(kappa)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla

    from oracle import oracle as O
    d = small_models[name]
    mats = d["mats"]
    op = O.setup_operator(mats, d["porder"])
    B = mats["B"].to_scipy()
    D = 1.0 / np.sqrt(B.diagonal())
    assert np.max(np.abs(op.D - D)) <= 1e-15 * np.max(D)
    Bs = sp.diags(D) @ B @ sp.diags(D)
    x = np.random.default_rng(0).standard_normal(op.n)
    bx = Bs @ x
    assert np.max(np.abs(op.bmv(x) - bx)) <= 1e-14 * np.max(np.abs(bx))

    def bound(cheb):
        lo, hi, deg = cheb
        k = hi / lo
        return 2.0 * ((np.sqrt(k) - 1) / (np.sqrt(k) + 1)) ** deg, k

    eb, kb = bound(op.b_cheb)
    assert np.linalg.norm(op.bsolve(bx) - x) <= eb * np.sqrt(kb) * np.linalg.norm(x)
    if "Ad" in mats:
        Ap = mats["Ap"].to_scipy()
        assert np.max(np.abs(op.Dp - 1.0 / np.sqrt(-Ap.diagonal()))) <= 1e-15 * np.max(op.Dp)
        Ad, E, ET = (mats[k].to_scipy() for k in ("Ad", "E", "ET"))
        exact = D * (Ad @ (D * x) - E @ sla.spsolve(Ap.tocsc(), ET @ (D * x)))
        ea, _ = bound(op.ap_cheb)
        assert np.max(np.abs(op.amv(x) - exact)) <= (ea + 1e-13) * np.max(np.abs(exact))
    else:
        ax = D * (mats["A"].to_scipy() @ (D * x))
        assert np.max(np.abs(op.amv(x) - ax)) <= 1e-14 * np.max(np.abs(ax))


@pytest.mark.parametrize("xintv", [
    [0.2, 0.3, 0.0, 1.0], [3.9e-7, 1.58e-4, -1e-9, 0.6], [1.579e-6, 3.9478e-5, -5e-9, 1.475e-3],
    [0.5, 0.9, 0.0, 1.0], [0.0, 0.05, 0.0, 1.0], [0.9, 1.0, 0.0, 1.0],
])
def test_filter_design_rule(xintv):
    """The filter of pEVSL_FINDPOL_F90 (src/mod_pevsl.f90:108-115) as the
    oracle designs it: p(gamma) = 1; an interior filter is balanced,
    p(a) = p(b); the bar is at or below the threshold (0.8 interior, 0.7 for
    an end interval) and the degree is the smallest that reaches it; on a
    fine grid p stays at or above the bar inside [a, b] and below it
    outside, which is what keeping Ritz values with p(theta) > bar relies on."""
    from oracle import oracle as O
    p = O.find_pol(xintv)
    a, b, lmin, lmax = xintv

    def ev(x):
        return O._cheb_eval(p.mu, (x - p.cc) / p.dd)

    assert abs(O._cheb_eval(p.mu, p.gam) - 1.0) < 1e-12
    thresh = 0.8 if p.kind == "interior" else 0.7
    assert p.bar <= thresh
    if p.kind == "interior":
        assert abs(ev(a) - ev(b)) < 1e-10
    if p.deg > 2:
        q = O.find_pol(xintv, min_deg=p.deg - 1, max_deg=p.deg - 1)
        assert q.bar > thresh
    xs = np.linspace(lmin, lmax, 20001)
    inside = np.array([ev(x) for x in xs if a <= x <= b])
    outside = np.array([ev(x) for x in xs if x < a or x > b])
    assert inside.min() >= p.bar - 1e-12
    assert outside.max() < p.bar


@pytest.mark.parametrize("name", ["solid_p1", "fs_p1"])
def test_lanczos_bounds_bracket_the_spectra(small_models, name):
    """pEVSL_LANBOUNDS_F90 (src/mod_pevsl.f90:84) as the oracle restates it:
    the bounds of B^-1 A, B_s and Ap_s against dense spectra, to 1e-8 of the
    spectral width (the filter and the Chebyshev set-ups only need that)."""
    from scipy.linalg import eigh, eigvalsh

    from oracle import oracle as O
    d = small_models[name]
    op = O.setup_operator(d["mats"], d["porder"])
    A, Bm = O.dense_operator(op)
    w = eigh(A, Bm, eigvals_only=True)
    lo, hi, _ = O.lan_bounds(op.amv, op.n, 3000, 1e-5, solve=op.bsolve)
    width = w[-1] - w[0]
    assert lo <= w[0] + 1e-8 * width and abs(hi - w[-1]) <= 1e-8 * width
    wb = eigvalsh(Bm)
    blo, bhi = op.bounds["B"]
    assert abs(blo - wb[0]) <= 1e-8 * wb[-1] and abs(bhi - wb[-1]) <= 1e-8 * wb[-1]
    if "Ap" in op.bounds:
        Ap = d["mats"]["Ap"].to_scipy().toarray()
        wa = eigvalsh(op.Dp[:, None] * (-Ap) * op.Dp[None, :])
        alo, ahi = op.bounds["Ap"]
        assert abs(alo - wa[0]) <= 1e-8 * wa[-1] and abs(ahi - wa[-1]) <= 1e-8 * wa[-1]
