"""CPU tests of the input side: the layered-ball generator, the reference
element and the CG mixed-FEM assembly (src/mod_cg_create_matrix.f90)."""
import numpy as np
import pytest

from normalmodes_gb300.model import Model


@pytest.fixture(scope="module")
def solid():
    return Model.ball(n_cells=6, porder=1, fluid_core=0, homogeneous=1)


@pytest.fixture(scope="module")
def fs2():
    return Model.ball(n_cells=8, porder=2)


def test_reference_element_p2():
    m = Model.ball(n_cells=6, porder=2, fluid_core=0, assemble=False)
    R = m.reference()
    M = R["M"]
    # mass of the reference tet (volume 4/3) and exact partition of unity
    assert abs(M.sum() - 4.0 / 3.0) < 1e-14
    assert np.allclose(M, M.T, atol=0)
    # derivative of constants vanishes, derivative of r is 1
    r = R["rst"][:, 0]
    for d in range(3):
        assert np.max(np.abs(R["Drst"][d] @ np.ones(10))) < 1e-13
    assert np.max(np.abs(R["Drst"][0] @ r - 1.0)) < 1e-13
    assert np.max(np.abs(R["Drst"][1] @ r)) < 1e-13
    # P2 local order of src/mod_geometry.f90:1707: vertices at 1,3,6,10
    assert np.allclose(R["rst"][[0, 2, 5, 9]], [[-1, -1, -1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]])
    # face masses: each face has area 2 in its projected coordinates
    for f in range(4):
        assert abs(R["MassF"][f].sum() - 2.0) < 1e-14
    # Fmask of face 1 is the slanted face r+s+t=-1 (src/mod_geometry.f90:2402-2404)
    fm = R["Fmask"][0]
    assert np.allclose(R["rst"][fm].sum(axis=1), -1.0)


def test_operators_symmetric(fs2):
    ops = fs2.operators()
    for name in ("Ad", "B", "Ap"):
        S = ops[name].to_scipy()
        assert abs(S - S.T).max() <= 1e-14 * abs(S).max()
    E, ET = ops["E"].to_scipy(), ops["ET"].to_scipy()
    assert abs(E - ET.T).max() == 0.0


def test_rigid_body_null_space(solid):
    A = solid.csr("A").to_scipy()
    xyz = solid.mesh()["xyz"]
    n = A.shape[0]
    scale = abs(A).max()
    for d in range(3):
        u = np.zeros(n)
        u[d::3] = 1.0
        assert np.abs(A @ u).max() < 1e-13 * scale
    for (a, b) in ((0, 1), (1, 2), (0, 2)):
        u = np.zeros(n)
        u[a::3] = -xyz[:, b]
        u[b::3] = xyz[:, a]
        assert np.abs(A @ u).max() < 1e-13 * scale * 6371.0


def test_total_mass(solid):
    # homogeneous ball: sum of B over one component = rho * volume of the polyhedral ball
    B = solid.csr("B").to_scipy()
    mass = B.sum() / 3.0
    vol_ball = 4.0 / 3.0 * np.pi * 6371.0 ** 3
    assert 0.9 * 5.51 * vol_ball < mass < 5.51 * vol_ball


def test_mass_is_scalar_times_identity3(fs2):
    """B(3a+p, 3b+q) = delta_pq M(a, b): the property the GPU mass kernels rely on."""
    B = fs2.csr("B").to_scipy().tocoo()
    assert np.all(B.row % 3 == B.col % 3)
    Bc = B.tocsr()
    M0 = Bc[0::3, 0::3]
    assert abs(Bc[1::3, 1::3] - M0).max() == 0.0
    assert abs(Bc[2::3, 2::3] - M0).max() == 0.0


def test_dof_counts_follow_node_status(fs2):
    me = fs2.mesh()
    i = fs2.info()
    vstat = me["vstat"]
    assert i.n == 3 * len(vstat) + 3 * int(np.sum((vstat == 2) | (vstat == 5)))
    assert i.np == int(np.sum((vstat != 0) & (vstat != 3)))
    # every 6-DOF node touches both solid and fluid tetrahedra
    tets, fluid = me["tets"], me["fluid"]
    has_s = np.zeros(len(vstat), bool)
    has_f = np.zeros(len(vstat), bool)
    has_s[np.unique(tets[~fluid])] = True
    has_f[np.unique(tets[fluid])] = True
    six = (vstat == 2) | (vstat == 5)
    assert np.all(has_s[six] & has_f[six])


def test_positive_orientation(fs2):
    me = fs2.mesh()
    x = me["xyz"]
    t = me["tets"][:, [0, 2, 5, 9]]
    B = np.stack([x[t[:, 1]] - x[t[:, 0]], x[t[:, 2]] - x[t[:, 0]], x[t[:, 3]] - x[t[:, 0]]], axis=1)
    assert np.all(np.linalg.det(B) > 0)


def test_element_matrices_match_numpy_restatement(fs2):
    """Element matrices against an independent numpy restatement of the
    Fortran formulas (oracle/fem_ref.py)."""
    from oracle import fem_ref
    me = fs2.mesh()
    R = fem_ref.reference_element(2)
    for k in [0, 17, int(np.argmax(me["fluid"])), len(me["fluid"]) - 1]:
        T, M = fs2.element_matrices(k)
        Tr, Mr = fem_ref.element_matrices(R, me, k, fluid_solid=True)
        assert T.shape == Tr.shape
        assert np.max(np.abs(T - Tr)) <= 1e-12 * np.max(np.abs(Tr))
        assert np.max(np.abs(M - Mr)) <= 1e-12 * np.max(np.abs(Mr))


def test_global_assembly_matches_numpy(solid):
    """Global A and B of the solid-only path against a dense numpy assembly."""
    from oracle import fem_ref
    me = solid.mesh()
    R = fem_ref.reference_element(1)
    A, B = fem_ref.assemble_solid_dense(R, me)
    Ag = solid.csr("A").to_scipy().toarray()
    Bg = solid.csr("B").to_scipy().toarray()
    assert np.max(np.abs(Ag - A)) <= 1e-12 * np.max(np.abs(A))
    assert np.max(np.abs(Bg - B)) <= 1e-12 * np.max(np.abs(B))


def test_lateral_perturbation_bounded():
    m0 = Model.ball(n_cells=8, porder=1, assemble=False)
    m1 = Model.ball(n_cells=8, porder=1, assemble=False, lateral_pert=0.02)
    a, b = m0.mesh(), m1.mesh()
    for f in ("vp", "rho"):
        r = b[f] / a[f]
        assert np.max(np.abs(r - 1)) <= 0.02 + 1e-12 and np.max(np.abs(r - 1)) > 0.015


def test_thin_fluid_layer_rejected():
    with pytest.raises(RuntimeError):
        Model.ball(n_cells=6, porder=2)


def test_reference_format_roundtrip(tmp_path):
    """Write a model in the reference's binary input format and load it back."""
    m = Model.ball(n_cells=8, porder=1, assemble=True)
    me = m.mesh()
    base = str(tmp_path / "ball")
    ntet, nv = me["tets"].shape[0], me["xyz"].shape[0]
    with open(base + "_mesh.header", "w") as f:
        f.write(f"{ntet} {nv}\n")
    (me["tets"].astype(np.int32) + 1).tofile(base + "_ele.dat")
    me["xyz"].astype(np.float64).tofile(base + "_node.dat")
    for fld in ("vp", "vs", "rho"):
        me[fld].astype(np.float64).tofile(base + f"_{fld}_pod_1_true.dat")
    m2 = Model.load(base, porder=1)
    for name in ("Ad", "B", "Ap", "E", "ET"):
        a, b = m.csr(name), m2.csr(name)
        assert np.array_equal(a.col, b.col) and np.array_equal(a.rowptr, b.rowptr)
        assert np.max(np.abs(a.val - b.val)) <= 1e-14 * np.max(np.abs(a.val))


def test_write_results_reference_layout(tmp_path):
    """Eigenvector files, vlist and vstat in the reference's names and
    formats (src/mod_pevsl.f90:188-247, src/mod_para.f90:269-288)."""
    from normalmodes_gb300.model import Model
    m = Model.ball(n_cells=8, porder=2)
    info = m.info()
    X = np.random.default_rng(2).standard_normal((info.n, 3))
    prefix = m.write_results(str(tmp_path), "ball", 0.1, 2.0, X, job=1, nproc=1)
    assert prefix.endswith("ball_JOB1_pod2_np1_0.100000001_2.00000000")
    for i in range(3):
        y = np.fromfile(f"{prefix}_{i + 1}.dat", dtype=np.float64)
        assert np.array_equal(y, X[:, i])
    vlist = np.fromfile(tmp_path / "ball_pod2_np1_vlist.dat", dtype=np.int32)
    assert np.array_equal(np.sort(vlist), np.arange(1, info.nnode + 1))
    # the input numbering puts the vertices first: their ids are 1..nvert
    mesh = m.mesh()
    vert_nodes = np.unique(mesh["tets"][:, [0, 2, 5, 9]])
    assert vlist[vert_nodes].max() == info.nvert
    vstat = np.fromfile(tmp_path / "ball_pod2_np1_vstat.dat", dtype=np.int32)
    assert vstat.size == info.nnode and vstat.min() >= 0 and vstat.max() <= 5


def test_assembly_does_not_depend_on_the_thread_count():
    """Bitwise-identical operators with 1 and 4 OpenMP threads (elements in
    parallel, scatter in element order), with and without gravity."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = (
        "import sys, hashlib; sys.path.insert(0, %r)\n"
        "from normalmodes_gb300.model import Model\n"
        "h = hashlib.sha256()\n"
        "for g in (False, True):\n"
        "    m = Model.ball(n_cells=8, porder=2, gravity=g)\n"
        "    for k, c in sorted(m.operators().items()):\n"
        "        h.update(c.rowptr.tobytes()); h.update(c.col.tobytes()); h.update(c.val.tobytes())\n"
        "sys.stdout.write(h.hexdigest())\n" % root)
    outs = [subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, check=True, timeout=300,
                           env=dict(os.environ, OMP_NUM_THREADS=nt)).stdout for nt in ("1", "4")]
    assert outs[0] == outs[1] and len(outs[0]) == 64
