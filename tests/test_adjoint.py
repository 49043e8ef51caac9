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


def _fluid_planet(tmp_path):
    """Homogeneous fluid ball (vs = 0 everywhere) with the reference gravity
    of its density, loaded from the reference's file format."""
    from normalmodes_gb300.model import G_DEMO, Model
    from oracle import gravity_ref
    from tests.test_gravity import _write_reference_files
    src = Model.ball(n_cells=6, porder=1, fluid_core=0, homogeneous=1, assemble=False)
    base = _write_reference_files(src, str(tmp_path), "fluidball", 1, vs_scale=0.0)
    m = Model.load(base, 1, assemble=False)
    m.set_gravity(gravity_ref.ball_gravity(m.mesh(), G_DEMO, 5.51, 0.0, 6371.0))
    return m


def _pick_elements(mesh, R, rng):
    """Two solid elements, a fluid element with a fluid-solid face, an inner
    fluid element and a fluid element on the outer boundary (those present)."""
    from oracle import gravity_ref
    fl = mesh["fluid"]
    els = [int(k) for k in rng.choice(np.where(~fl)[0], 2, replace=False)] if (~fl).any() else []
    if fl.any():
        vt = mesh["tets"][:, R["vord"]]
        six = (mesh["rnum"][vt] == 6).sum(axis=1)
        outer = gravity_ref.boundary_faces(vt).any(axis=1)
        for cand in (fl & (six == 3), fl & (six == 0) & ~outer, fl & outer):
            if cand.any():
                els.append(int(rng.choice(np.where(cand)[0])))
    return els


@pytest.mark.parametrize("case", ["solid_p1", "fs_p1", "fluid_planet"])
def test_reference_gradient_with_gravity(case, tmp_path):
    """JOB = 2: the reference gradient with the gravity terms against
    central finite differences of dense eigenvalues (the gravity field held
    fixed, as the reference takes it as an input).  Steps: 1e-2 of the
    element's parameter in solid elements, where the operators are linear in
    it and only the eigensolver's rounding limits the difference quotient;
    1e-3 in fluid elements, whose free-surface term goes as 1 / rho."""
    from normalmodes_gb300.model import Model
    from oracle import adjoint_ref as AR
    from oracle import fem_ref
    if case == "fluid_planet":
        m = _fluid_planet(tmp_path)
    else:
        kw = dict(n_cells=6, porder=1, fluid_core=0) if case == "solid_p1" else dict(n_cells=8, porder=1)
        m = Model.ball(gravity=True, **kw)
    m.assemble()
    mesh, g0 = m.mesh(), m.gravity()
    R = fem_ref.reference_element(1)
    w, V, ops = _dense_eigs(m)
    gr = _groups(w, tol=1e-3)
    i0 = int(np.argmax(w > 1e-7))
    sel = np.where((gr >= gr[i0] + 1) & (gr <= gr[i0] + 4))[0]
    lam, X = w[sel], V[:, sel]
    gsel = gr[sel]
    P = AR.pressure(ops, X) if "Ap" in ops else None
    els = _pick_elements(mesh, R, np.random.default_rng(7))
    G = AR.gradient(R, mesh, lam, X, P, elements=els, g0=g0)
    for ie, k in enumerate(els):
        for which in (0, 1) if mesh["fluid"][k] else (0, 1, 2):
            h = (1e-3 if mesh["fluid"][k] else 1e-2) * AR.element_parameter(mesh, k, which)
            res = []
            for sgn in (1.0, -1.0):
                m.set_material(*AR.perturbed_material(mesh, k, which, sgn * h))
                res.append(_dense_eigs(m)[0][sel])
            m.set_material(mesh["vp"], mesh["vs"], mesh["rho"])
            fd = (res[0] - res[1]) / (2 * h)
            fdg = np.array([fd[gsel == u].sum() for u in np.unique(gsel)])
            gg = np.array([G[gsel == u, ie, which].sum() for u in np.unique(gsel)])
            assert np.max(np.abs(fdg - gg)) <= 1e-3 * np.max(np.abs(gg)), (case, k, which, fdg, gg)


@pytest.mark.parametrize("case", ["solid_p1", "fs_p1", "fs_p2", "fluid_planet"])
def test_host_gravity_terms_match_the_reference(case, tmp_path):
    """nm_adjoint_gravity (the host code nm_adjoint adds for JOB = 2) against
    the gravity part of the CPU reference gradient, on elements of every kind
    (solid, fluid at the fluid-solid interface, inner fluid, free surface)."""
    from normalmodes_gb300 import nmgpu
    from normalmodes_gb300.model import Model
    from oracle import adjoint_ref as AR
    from oracle import fem_ref
    if case == "fluid_planet":
        m = _fluid_planet(tmp_path)
    else:
        kw = {"solid_p1": dict(n_cells=6, porder=1, fluid_core=0), "fs_p1": dict(n_cells=8, porder=1),
              "fs_p2": dict(n_cells=8, porder=2)}[case]
        m = Model.ball(gravity=True, **kw)
    m.assemble()
    mesh, g0, ref = m.mesh(), m.gravity(), m.reference()
    porder = 2 if case == "fs_p2" else 1
    R = fem_ref.reference_element(porder)
    ops = m.operators()
    rng = np.random.default_rng(3)
    X = rng.standard_normal((ops["B"].shape[0], 3))
    P = AR.pressure(ops, X) if "Ap" in ops else None
    got = nmgpu.adjoint_gravity(mesh, ref, g0, X, P, fluid_solid="Ap" in ops)
    els = sorted(set(_pick_elements(mesh, R, rng)) | set(int(e) for e in rng.choice(len(mesh["fluid"]), 20)))
    want = AR.gradient(R, mesh, np.zeros(3), X, P, elements=els, g0=g0) - \
        AR.gradient(R, mesh, np.zeros(3), X, P, elements=els)
    scale = np.max(np.abs(want))
    assert scale > 0
    assert np.max(np.abs(got[:, els, :] - want)) <= 1e-11 * scale
