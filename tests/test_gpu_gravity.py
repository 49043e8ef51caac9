"""GPU tests of operators assembled with the reference gravity (JOB = 2) and
of the KPM slicer on a context, against the oracle's golden fixtures
(tests/golden/*_grav.npz, made by tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]

SPECS = {
    "solid_p1_grav": dict(n_cells=6, porder=1, fluid_core=0, gravity=True),
    "fs_p1_grav": dict(n_cells=8, porder=1, gravity=True),
}


def _golden(name):
    return np.load(os.path.join(os.path.dirname(__file__), "golden", f"{name}.npz"))


def _lam(f):
    pi = float(np.float32(3.14159265359))
    return (2 * pi * float(np.float32(f))) ** 2 * 1e-6


@pytest.fixture(scope="module")
def grav_models():
    from normalmodes_gb300.model import Model
    return {name: Model.ball(**kw).operators() for name, kw in SPECS.items()}


@pytest.mark.parametrize("name", list(SPECS))
@pytest.mark.parametrize("prec,block", [(0, 0), (0, 32), (1, 32)])
def test_gravity_solve_matches_oracle(grav_models, name, prec, block):
    """FP64 single-vector, FP64 block and mixed block solves of a JOB = 2
    pencil: same count as the oracle, eigenvalues within 1e-10; the
    single-vector path (the reference's algorithm) also at the reference's
    residual level."""
    from normalmodes_gb300.nmgpu import Solver
    g = _golden(name)
    apb = tuple(g["ap_bounds"]) if g["ap_bounds"][1] > 0 else None
    lo, hi = (float(x) for x in g["interval"])
    with Solver(grav_models[name], 1, precision=prec, b_bounds=tuple(g["b_bounds"]), ap_bounds=apb) as sv:
        r = sv.solve(lo, hi, ab_bounds=(float(g["xintv"][2]), float(g["xintv"][3])), block=block)
    assert len(r.lam) == len(g["lam"])
    assert np.max(np.abs(r.lam - g["lam"]) / g["lam"]) < 1e-10
    if block == 0:
        assert r.pol_deg == int(g["pol_deg"])
        assert np.max(r.err_ref) < 1e-10


def test_slice_spectrum_on_a_context(grav_models):
    """nm_slice_spectrum (moments through the context's A-operator and
    B-solve): four slices of 0.1-1.0 mHz whose exact counts (dense solve of
    the oracle's pencil) stay within 40 % of their mean."""
    from normalmodes_gb300.nmgpu import Solver
    g = _golden("solid_p1_grav")
    ab = (float(g["xintv"][2]), float(g["xintv"][3]))
    with Solver(grav_models["solid_p1_grav"], 1, b_bounds=tuple(g["b_bounds"])) as sv:
        sl, counts = sv.slice_spectrum(0.1, 1.0, 4, ab_bounds=ab)
    assert sl[0][0] == pytest.approx(0.1) and sl[-1][1] == pytest.approx(1.0)
    assert all(sl[i][1] == sl[i + 1][0] for i in range(3))
    w = g["lam_dense"]
    per = [int(np.sum((w > _lam(a)) & (w <= _lam(b)))) for a, b in sl]
    assert sum(per) == len(w)
    assert max(abs(c - np.mean(per)) for c in per) <= 0.4 * np.mean(per), per
    assert abs(counts.sum() - len(w)) <= 0.1 * len(w)


@pytest.mark.parametrize("name", list(SPECS))
def test_gravity_adjoint_matches_cpu_reference(name):
    """nm_adjoint with the gravity field (JOB = 2 terms added by
    nm_adjoint_gravity) against the CPU reference gradient on the same
    eigenvectors: within 1e-8 of the largest |gradient| per pair and
    parameter; the gravity terms change the gradient visibly."""
    from normalmodes_gb300.model import Model
    from normalmodes_gb300.nmgpu import Solver
    from oracle import adjoint_ref as AR
    from oracle import fem_ref
    g = _golden(name)
    m = Model.ball(**SPECS[name])
    mats, mesh, ref, g0 = m.operators(), m.mesh(), m.reference(), m.gravity()
    apb = tuple(g["ap_bounds"]) if g["ap_bounds"][1] > 0 else None
    with Solver(mats, 1, b_bounds=tuple(g["b_bounds"]), ap_bounds=apb) as sv:
        r = sv.solve(*(float(x) for x in g["interval"]), ab_bounds=(float(g["xintv"][2]), float(g["xintv"][3])),
                     want_vectors=True, unscale=True)
        k = min(8, len(r.lam))
        lam, X = r.lam[:k], r.vec[:, :k]
        grad, _ = sv.adjoint(mesh, ref, lam, X, g0=g0)
        grad1, _ = sv.adjoint(mesh, ref, lam, X)
    rng = np.random.default_rng(5)
    els = rng.choice(mesh["tets"].shape[0], 40, replace=False)
    if mesh["fluid"].any():
        els = np.concatenate([els, rng.choice(np.where(mesh["fluid"])[0], 10, replace=False)])
    P = AR.pressure(mats, X) if "Ap" in mats else None
    G = AR.gradient(fem_ref.reference_element(1), mesh, lam, X, P, elements=els, g0=g0)
    for j in range(k):
        for c in range(3):
            scale = np.max(np.abs(grad[j, :, c]))
            if scale > 0:
                assert np.max(np.abs(grad[j, els, c] - G[j, :, c])) <= 1e-8 * scale, (j, c)
    assert np.max(np.abs(grad - grad1)) > 1e-3 * np.max(np.abs(grad))
