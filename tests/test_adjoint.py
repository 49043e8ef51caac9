"""CPU checks of the adjoint reference (oracle/adjoint_ref.py): the
per-element eigenvalue sensitivities to density, bulk and shear modulus
against central finite differences of dense generalized eigenvalues of the
re-assembled operators (scipy eigh of A, or of the exact Schur complement
Ad - E Ap^-1 ET, against B).

Degenerate multiplets are compared as sums over clusters of eigenvalues
closer than 1e-3 relative (the per-pair derivative of a degenerate
eigenvalue depends on the basis); steps are 1e-4 of the
element's mean parameter; tolerance 1e-3 relative to the largest group sum.
"""
import numpy as np
import pytest
import scipy.linalg as sl


def _dense_eigs(m):
    ops = m.operators()
    B = ops["B"].to_scipy().toarray()
    if "A" in ops:
        A = ops["A"].to_scipy().toarray()
    else:
        Ap = ops["Ap"].to_scipy().toarray()
        A = ops["Ad"].to_scipy().toarray() - ops["E"].to_scipy().toarray() @ np.linalg.solve(
            Ap, ops["ET"].to_scipy().toarray())
        A = (A + A.T) / 2
    w, V = sl.eigh(A, B)
    return w, V, ops


def _groups(w, tol=1e-6):
    g = [0]
    for i in range(1, len(w)):
        g.append(g[-1] + int(abs(w[i] - w[i - 1]) > tol * abs(w[i - 1])))
    return np.array(g)


@pytest.mark.parametrize("kw", [dict(n_cells=6, porder=1, fluid_core=0), dict(n_cells=8, porder=1)],
                         ids=["solid_p1", "fs_p1"])
def test_reference_gradient_matches_finite_differences(kw):
    from normalmodes_gb300.model import Model
    from oracle import adjoint_ref as AR
    from oracle import fem_ref
    m = Model.ball(**kw)
    mesh = m.mesh()
    R = fem_ref.reference_element(kw["porder"])
    w, V, ops = _dense_eigs(m)
    gr = _groups(w, tol=1e-3)
    i0 = int(np.argmax(w > 1e-7))  # skip rigid-body / zero-frequency fluid modes
    sel = np.where((gr >= gr[i0] + 1) & (gr <= gr[i0] + 4))[0]
    lam, X = w[sel], V[:, sel]
    gsel = gr[sel]
    P = AR.pressure(ops, X) if "Ap" in ops else None
    rng = np.random.default_rng(11)
    els = list(rng.choice(np.where(~mesh["fluid"])[0], 2, replace=False))
    if mesh["fluid"].any():
        els.append(int(rng.choice(np.where(mesh["fluid"])[0])))
    G = AR.gradient(R, mesh, lam, X, P, elements=els)
    for ie, k in enumerate(els):
        for which in (0, 1) if mesh["fluid"][k] else (0, 1, 2):
            h = 1e-4 * AR.element_parameter(mesh, k, which)
            res = []
            for sgn in (1.0, -1.0):
                m.set_material(*AR.perturbed_material(mesh, k, which, sgn * h))
                res.append(_dense_eigs(m)[0][sel])
            m.set_material(mesh["vp"], mesh["vs"], mesh["rho"])
            fd = (res[0] - res[1]) / (2 * h)
            fdg = np.array([fd[gsel == u].sum() for u in np.unique(gsel)])
            gg = np.array([G[gsel == u, ie, which].sum() for u in np.unique(gsel)])
            assert np.max(np.abs(fdg - gg)) <= 1e-3 * np.max(np.abs(gg)), (k, which, fdg, gg)


def test_set_material_rejects_a_phase_change():
    from normalmodes_gb300.model import Model
    m = Model.ball(n_cells=8, porder=1)
    mesh = m.mesh()
    vs = mesh["vs"].copy()
    k = int(np.where(mesh["fluid"])[0][0])
    vs[k] = 1.0
    with pytest.raises(RuntimeError):
        m.set_material(mesh["vp"], vs, mesh["rho"])
