"""CPU tests of the reference-gravity (JOB = 2) assembly
(src/mod_cg_create_matrix.f90:192-265, 329-377, 492-705, 866-920,
1057-1160): the C++ operators against the numpy restatement in
oracle/gravity_ref.py, physics known answers of the discrete operators, the
reference's gravity file layout and argument checks."""
import os

import numpy as np
import pytest

from normalmodes_gb300.model import G_DEMO, Model


def _compare(model, porder, g0, floor=0.0):
    """floor: lower limit of the scale the difference is measured against
    (for operators that are sums of cancelling terms)."""
    from oracle import fem_ref, gravity_ref
    ref = gravity_ref.assemble(fem_ref.reference_element(porder), model.mesh(), g0)
    for name, S in ref.items():
        C = model.csr(name).to_scipy()
        assert abs(C - S).max() <= 1e-13 * max(abs(S).max(), floor), name
    return ref


@pytest.mark.parametrize("kw", [
    dict(n_cells=6, porder=1, fluid_core=0),
    dict(n_cells=8, porder=1),
    dict(n_cells=8, porder=2),
    dict(n_cells=8, porder=1, lateral_pert=0.02),
])
def test_assembly_matches_numpy(kw):
    """Global operators with and without the reference gravity."""
    m = Model.ball(gravity=True, **kw)
    g0 = m.gravity()
    assert g0 is not None and g0.shape == (m.info().ntet, m.info().pnp, 3)
    ref = _compare(m, kw["porder"], g0)
    for name in ("A", "Ad", "B", "Ap"):
        if name in ref:
            S = m.csr(name).to_scipy()
            assert abs(S - S.T).max() <= 1e-14 * abs(S).max(), name
    if "E" in ref:
        assert abs(m.csr("E").to_scipy() - m.csr("ET").to_scipy().T).max() == 0.0
    m.set_gravity(None)
    assert m.gravity() is None
    _compare(m, kw["porder"], None)


def test_element_matrices_match_numpy():
    """Element matrices as scattered, solid and fluid (with face terms)."""
    from oracle import fem_ref, gravity_ref
    m = Model.ball(n_cells=8, porder=2, gravity=True)
    me, g0 = m.mesh(), m.gravity()
    R = fem_ref.reference_element(2)
    bface = gravity_ref.boundary_faces(me["tets"][:, R["vord"]])
    fl = np.flatnonzero(me["fluid"])
    for k in [0, 17, int(fl[0]), int(fl[len(fl) // 2]), int(fl[-1]), len(me["fluid"]) - 1]:
        T, M = m.element_matrices(k)
        Tr, Mr = gravity_ref.element_matrices(R, me, k, True, g0, bface)
        assert T.shape == Tr.shape
        assert np.max(np.abs(T - Tr)) <= 1e-12 * np.max(np.abs(Tr))
        assert np.max(np.abs(M - Mr)) <= 1e-12 * np.max(np.abs(Mr))


def test_ball_gravity_field():
    """g = -G M(r) x / r^3 of the radial profile; |g| = 4/3 pi G rho r for a
    homogeneous ball."""
    from oracle import gravity_ref
    m = Model.ball(n_cells=8, porder=2, gravity=True, assemble=False)
    g = m.gravity()
    ga = gravity_ref.ball_gravity(m.mesh(), G_DEMO, 13.0, 3.3 - 13.0, 6371.0)
    assert np.abs(g - ga).max() <= 1e-13 * np.abs(ga).max()
    h = Model.ball(n_cells=6, porder=1, fluid_core=0, homogeneous=1, gravity=True, assemble=False)
    me = h.mesh()
    x = me["xyz"][me["tets"]]
    r = np.linalg.norm(x, axis=2)
    gn = np.linalg.norm(h.gravity(), axis=2)
    assert np.allclose(gn, 4.0 / 3.0 * np.pi * G_DEMO * 5510.0 * r * 1e3, rtol=1e-12, atol=1e-12)
    # pointing inwards
    assert np.all((h.gravity() * x).sum(axis=2) <= 1e-12)


@pytest.mark.parametrize("porder", [1, 2])
def test_rigid_motions_under_gravity(porder):
    """Homogeneous solid ball with the reference gravity of its own density:
    every rigid translation has the Rayleigh quotient 4/3 pi G rho (the
    oscillation frequency of a body in the field of a uniform sphere) and
    every rigid rotation the Rayleigh quotient 0, exactly, on any mesh
    (neither is an exact eigenvector of the polyhedral ball)."""
    m = Model.ball(n_cells=8, porder=porder, fluid_core=0, homogeneous=1, gravity=True)
    A, B = m.csr("A").to_scipy(), m.csr("B").to_scipy()
    xyz = m.mesh()["xyz"]
    n = A.shape[0]
    lam = 4.0 / 3.0 * np.pi * G_DEMO * 5510.0
    for d in range(3):
        u = np.zeros(n)
        u[d::3] = 1.0
        assert abs((u @ (A @ u)) / (u @ (B @ u)) / lam - 1.0) < 1e-12
    for (a, b) in ((0, 1), (1, 2), (0, 2)):
        u = np.zeros(n)
        u[a::3] = -xyz[:, b]
        u[b::3] = xyz[:, a]
        assert abs((u @ (A @ u)) / (u @ (B @ u))) < 1e-12 * lam


def _write_reference_files(model, directory, base, porder, vs_scale=1.0):
    """The model's mesh and material in the reference's input format."""
    me = model.mesh()
    vord = [0, 1, 2, 3] if porder == 1 else [0, 2, 5, 9]
    vt = me["tets"][:, vord]
    verts = np.unique(vt)
    idx = np.full(me["xyz"].shape[0], -1, np.int64)
    idx[verts] = np.arange(len(verts))
    path = os.path.join(directory, base)
    with open(path + "_mesh.header", "w") as f:
        f.write(f"{vt.shape[0]} {len(verts)}\n")
    (idx[vt] + 1).astype(np.int32).tofile(path + "_ele.dat")
    me["xyz"][verts].astype(np.float64).tofile(path + "_node.dat")
    for name, arr in (("vp", me["vp"]), ("vs", me["vs"] * vs_scale), ("rho", me["rho"])):
        np.ascontiguousarray(arr, dtype=np.float64).tofile(path + f"_{name}_pod_{porder}_true.dat")
    return path


@pytest.mark.parametrize("porder", [1, 2])
def test_fluid_planet_free_surface(tmp_path, porder):
    """A fluid planet touches the outer boundary: without gravity the face
    term is undefined (division by the normal gravity) and the assembly
    refuses; with it the free-surface term enters Ap (src/mod_cg_create_matrix.f90:645-666)
    and -Ap stays symmetric positive definite.  N^2 is zero in a fluid planet
    and the inner-face terms of neighbouring elements cancel, so Ad is
    rounding residue: it is compared on the scale of one face term,
    rho |g| h^2 with h the cell size."""
    from oracle import gravity_ref
    src = Model.ball(n_cells=6, porder=porder, fluid_core=0, homogeneous=1, assemble=False)
    base = _write_reference_files(src, str(tmp_path), "fluidball", porder, vs_scale=0.0)
    m = Model.load(base, porder, assemble=False)
    assert m.info().purefluid == 1
    with pytest.raises(RuntimeError, match="without gravity"):
        m.assemble()
    g0 = gravity_ref.ball_gravity(m.mesh(), G_DEMO, 5.51, 0.0, 6371.0)
    m.set_gravity(g0)
    face = 5.51 * 9.8e-3 * (2 * 6371.0 / 6) ** 2
    _compare(m, porder, g0, floor=face)
    assert abs(m.csr("Ad").to_scipy()).max() <= 1e-12 * face
    Ap = m.csr("Ap").to_scipy().toarray()
    assert np.abs(Ap - Ap.T).max() <= 1e-14 * np.abs(Ap).max()
    assert np.linalg.eigvalsh(-Ap).min() > 0


def test_gravity_file_round_trip(tmp_path):
    """<base>_pod_<p>_potential_acceleration_true.dat is float64 Ntet x pNp x 3."""
    src = Model.ball(n_cells=8, porder=2, gravity=True, assemble=False)
    base = _write_reference_files(src, str(tmp_path), "ball", 2)
    g = src.gravity()
    g.astype(np.float64).tofile(base + "_pod_2_potential_acceleration_true.dat")
    m = Model.load(base, 2, gravity=True)
    assert np.array_equal(m.gravity(), g)
    _compare(m, 2, g)


def test_bad_gravity_rejected(tmp_path):
    m = Model.ball(n_cells=6, porder=1, fluid_core=0, assemble=False)
    i = m.info()
    with pytest.raises(ValueError):
        m.set_gravity(np.zeros(5))
    bad = np.zeros((i.ntet, i.pnp, 3))
    bad[3, 1, 2] = np.nan
    with pytest.raises(RuntimeError, match="non-finite"):
        m.set_gravity(bad)
    base = _write_reference_files(m, str(tmp_path), "ball", 1)
    loaded = Model.load(base, 1, assemble=False)
    with pytest.raises(RuntimeError, match="radial density profile"):
        loaded.ball_gravity()
    with pytest.raises(RuntimeError, match="cannot open"):
        Model.load(base, 1, gravity=True)


# The reference's P1 inputs of CONST3k and PREM3k are committed under
# tests/golden/ref_inputs (tests/golden/make_ref_inputs.py); the P2 and
# RTMDWAK8k cases run where NM_REFERENCE_DEMOS names a full demos/models/input.
REF_DEMOS = os.environ.get("NM_REFERENCE_DEMOS",
                           os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_inputs"))


@pytest.mark.parametrize("model,porder", [("PREM3k/prem_3L_3k.1", 1), ("CONST3k/CONST_1L_3k.1", 2),
                                          ("RTMDWAK8k/RTMDWAK_3L_8k.1", 1)])
def test_reference_demo_models(model, porder):
    """The reference's demo models with their own gravity files: the C++
    assembly against the numpy restatement; the CONST3k field is
    4/3 pi G rho r with G = 6.6723e-11."""
    base = os.path.join(REF_DEMOS, model)
    if not os.path.exists(base + f"_vp_pod_{porder}_true.dat"):
        pytest.skip("reference demo model files not present")
    m = Model.load(base, porder, gravity=True)
    g0 = m.gravity()
    _compare(m, porder, g0)
    if "CONST" in model:
        me = m.mesh()
        r = np.linalg.norm(me["xyz"][me["tets"]], axis=2)
        gn = np.linalg.norm(g0, axis=2)
        sel = r > 100.0
        assert np.allclose(gn[sel], 4.0 / 3.0 * np.pi * G_DEMO * 5510.0 * r[sel] * 1e3, rtol=1e-8)


def test_filtered_lanczos_on_gravity_pencil():
    """The pEVSL restatement (the algorithm the GPU path runs) on a JOB = 2
    operator set finds every eigenvalue of the interval that a dense LAPACK
    solve of the same pencil finds, including the near-translation triplet
    that the fixed reference gravity gives a solid ball."""
    from scipy.linalg import eigh

    from oracle import oracle as O
    m = Model.ball(n_cells=6, porder=1, fluid_core=0, gravity=True)
    op = O.setup_operator(m.operators(), 1)
    A, Bm = O.dense_operator(op)
    w = eigh(A, Bm, eigvals_only=True)
    lo, hi = O.interval(0.1, 1.0, w[0], w[-1])[:2]
    ref = w[(w >= lo) & (w <= hi)]
    r = O.apply_pevsl(op, 0.1, 1.0)
    assert len(r.lam) == len(ref) > 3
    assert np.max(np.abs(r.lam - ref) / ref) < 1e-10
    f = O.freq_mhz(ref[:3])[0]
    assert np.ptp(f) < 1e-6 * f[0]  # three-fold degenerate


@pytest.mark.parametrize("model", ["PREM3k/prem_3L_3k.1", "CONST3k/CONST_1L_3k.1", "RTMDWAK8k/RTMDWAK_3L_8k.1"])
def test_boundary_faces_match_the_reference_neighbour_files(model):
    """The outer-boundary faces the gravity face terms use, derived from the
    tetrahedra, are those <base>_neigh.dat marks with -1 (ClNeigh, the
    neighbour opposite vertex i; src/mod_cg_create_matrix.f90:645)."""
    from oracle import gravity_ref
    base = os.path.join(REF_DEMOS, model)
    if not os.path.exists(base + "_neigh.dat"):
        pytest.skip("reference demo models not present")
    nt = int(open(base + "_mesh.header").read().split()[0])
    ele = np.fromfile(base + "_ele.dat", dtype=np.int32).reshape(nt, 4) - 1
    neigh = np.fromfile(base + "_neigh.dat", dtype=np.int32).reshape(nt, 4)
    assert np.array_equal(gravity_ref.boundary_faces(ele), neigh == -1)



@pytest.mark.parametrize("model,porder", [("CONST3k/CONST_1L_3k.1", 1), ("CONST3k/CONST_1L_3k.1", 2),
                                          ("PREM3k/prem_3L_3k.1", 1), ("RTMDWAK8k/RTMDWAK_3L_8k.1", 2)])
def test_model_files_round_trip_byte_for_byte(tmp_path, model, porder):
    """A reference demo model loaded and written back with
    nmm_write_model_files gives the reference's own files, byte for byte:
    header, elements, nodes, neighbours, material and gravity."""
    base = os.path.join(REF_DEMOS, model)
    if not os.path.exists(base + f"_vp_pod_{porder}_true.dat"):
        pytest.skip("reference demo model files not present")
    m = Model.load(base, porder, gravity=True, assemble=False)
    out = str(tmp_path / "copy")
    m.write_model_files(out)
    sfx = ["_mesh.header", "_ele.dat", "_node.dat", "_neigh.dat"] + \
        [f"_{q}_pod_{porder}_true.dat" for q in ("vp", "vs", "rho")] + [f"_pod_{porder}_potential_acceleration_true.dat"]
    for s_ in sfx:
        assert open(base + s_, "rb").read() == open(out + s_, "rb").read(), s_


@pytest.mark.parametrize("porder", [1, 2])
def test_generated_model_through_the_reference_files(tmp_path, porder):
    """A generated fluid-solid ball with gravity, written in the reference's
    files and loaded back, gives the same operators: identical for P1 (same
    node numbering), the same values up to the node numbering for P2."""
    src = Model.ball(n_cells=8, porder=porder, gravity=True)
    base = str(tmp_path / "ball.1")
    src.write_model_files(base)
    back = Model.load(base, porder, gravity=True)
    for name in ("Ad", "B", "Ap", "E", "ET"):
        a, b = src.csr(name), back.csr(name)
        if porder == 1:
            assert np.array_equal(a.rowptr, b.rowptr) and np.array_equal(a.col, b.col)
            assert np.array_equal(a.val, b.val), name
        else:
            assert len(a.val) == len(b.val)
            assert np.allclose(np.sort(a.val), np.sort(b.val), rtol=1e-13, atol=1e-13 * np.abs(a.val).max()), name
    nt = src.info().ntet
    neigh = np.fromfile(base + "_neigh.dat", dtype=np.int32).reshape(nt, 4)
    for k in range(0, nt, 97):
        for f in range(4):
            j = neigh[k, f]
            if j > 0:
                assert k + 1 in neigh[j - 1]
