"""GPU parity of the C-ABI callbacks and the whole solve against the CPU
FP64 oracle (oracle/) on the same synthetic models.

Tolerances (FP64 path): operators 1e-12 relative in the max norm (the GPU
sums each row in CSR order with FMA; the oracle without), eigenvalues 1e-10
relative, identical eigenvalue counts, and the reference's RMS residual
(src/mod_pevsl.f90:158) below 1e-10.
"""
import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]


@pytest.fixture(scope="module")
def setups(small_models):
    from normalmodes_gb300.nmgpu import Solver
    from oracle import oracle as O
    out = {}
    for name, d in small_models.items():
        op = O.setup_operator(d["mats"], d["porder"])
        sv = Solver(d["mats"], d["porder"], b_bounds=op.bounds["B"], ap_bounds=op.bounds.get("Ap"))
        out[name] = (d, op, sv)
    yield out
    for _, (_, op, sv) in out.items():
        sv.close()
        op.close()


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("name", ["solid_p1", "fs_p1", "fs_p2"])
def test_callbacks_match_oracle(setups, name):
    d, op, sv = setups[name]
    rng = np.random.default_rng(7)
    for _ in range(3):
        x = rng.standard_normal(op.n)
        assert _rel(sv.bmv(x), op.bmv(x)) < 1e-13
        assert _rel(sv.bsolve(x), op.bsolve(x)) < 1e-12
        assert _rel(sv.amv(x), op.amv(x)) < 1e-12


@pytest.mark.parametrize("name", ["solid_p1", "fs_p2"])
def test_block_callbacks(setups, name):
    d, op, sv = setups[name]
    X = np.random.default_rng(3).standard_normal((op.n, 4))
    Y = sv.block("amv", X)
    for j in range(4):
        assert _rel(Y[:, j], op.amv(X[:, j])) < 1e-12
    Yb = sv.block("bsolve", X)
    assert _rel(Yb[:, 2], op.bsolve(X[:, 2])) < 1e-12


def test_device_pointer_callbacks(setups):
    import torch
    from normalmodes_gb300 import nmgpu
    d, op, sv = setups["fs_p1"]
    x = np.random.default_rng(5).standard_normal(op.n)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    torch.cuda.synchronize()
    L = nmgpu.lib()
    assert L.nm_amv_dev(sv._h, xd.data_ptr(), yd.data_ptr()) == 0
    assert L.nm_sync(sv._h) == 0
    assert _rel(yd.cpu().numpy(), op.amv(x)) < 1e-12


def test_bounds_match_oracle(small_models):
    """Lanczos bounds of B_s and Ap_s computed on the GPU agree with the oracle's."""
    from normalmodes_gb300.nmgpu import Solver
    from oracle import oracle as O
    d = small_models["fs_p2"]
    op = O.setup_operator(d["mats"], d["porder"])
    with Solver(d["mats"], d["porder"]) as sv:
        i = sv.info()
        assert abs(i.b_bounds[0] - op.bounds["B"][0]) < 1e-9 * op.bounds["B"][1]
        assert abs(i.b_bounds[1] - op.bounds["B"][1]) < 1e-9 * op.bounds["B"][1]
        assert abs(i.ap_bounds[1] - op.bounds["Ap"][1]) < 1e-9 * op.bounds["Ap"][1]
        assert i.ap_cheb_deg == op.ap_cheb[2]
        assert i.b_cheb_deg == op.b_cheb[2]


def _golden(name):
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", f"{name}.npz")
    if not os.path.exists(path):
        pytest.skip(f"golden fixture {name}.npz missing")
    return np.load(path)


def test_solve_matches_golden_p2(setups):
    """P2 fluid-solid model: the oracle solve takes minutes on a CPU, so the
    GPU is compared with the committed oracle fixture (same seeded model)."""
    d, op, sv = setups["fs_p2"]
    g = _golden("fs_p2")
    lo, hi = g["interval"]
    res = sv.solve(lo, hi, ab_bounds=(float(g["xintv"][2]), float(g["xintv"][3])))
    assert res.pol_deg == int(g["pol_deg"])
    assert len(res.lam) == len(g["lam"]) > 0
    assert np.max(np.abs(res.lam - g["lam"]) / g["lam"]) < 1e-10
    assert np.max(res.err_ref) < 1e-10


@pytest.mark.parametrize("name", ["solid_p1", "fs_p1"])
def test_solve_matches_oracle(setups, name):
    from oracle import oracle as O
    d, op, sv = setups[name]
    lo, hi = d["interval"]
    ref = O.apply_pevsl(op, lo, hi)
    res = sv.solve(lo, hi, ab_bounds=(ref.xintv[2], ref.xintv[3]))
    assert res.pol_deg == ref.pol.deg
    assert len(res.lam) == len(ref.lam) > 0
    assert np.max(np.abs(res.lam - ref.lam) / np.abs(ref.lam)) < 1e-10
    assert np.max(res.err_ref) < 1e-10
    # eigenvectors: B-orthonormal and A-residuals small
    Y = res.vec
    G = np.column_stack([op.bmv(Y[:, j]) for j in range(Y.shape[1])])
    assert np.max(np.abs(Y.T @ G - np.eye(Y.shape[1]))) < 1e-8


def test_solve_matches_dense(setups):
    """Independent pin: dense generalized eigensolve of the same operators."""
    from oracle import oracle as O
    d, op, sv = setups["fs_p1"]
    lo, hi = d["interval"]
    res = sv.solve(lo, hi)
    w, _ = O.dense_reference(op, res.xintv[0], res.xintv[1])
    assert len(w) == len(res.lam)
    assert np.max(np.abs(res.lam - w) / w) < 1e-10


def test_solve_without_graph_identical(setups):
    d, op, sv = setups["solid_p1"]
    lo, hi = d["interval"]
    a = sv.solve(lo, hi, use_graph=True)
    b = sv.solve(lo, hi, use_graph=False)
    assert np.array_equal(a.lam, b.lam)
