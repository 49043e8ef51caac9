"""GPU adjoint (nm_adjoint, through the C-ABI) against the FP64 CPU
reference gradient (oracle/adjoint_ref.py) on the same eigenvectors, against
central finite differences of eigenvalues re-solved on the GPU, and through a
torch.autograd.Function wrapper (test harness only).

Tolerances: 1e-8 relative to the largest |gradient| of each eigenpair and
parameter for GPU vs CPU on identical eigenvectors (the GPU pressure uses the
Chebyshev approximation of Ap^-1 that its A-operator applies, the CPU an
exact sparse solve); finite differences with 1e-4 relative steps, compared as
sums over clusters of eigenvalues closer than 1e-3 (relative), 1e-3
relative.
"""
import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]


def _solve(mats, porder, interval, **kw):
    from normalmodes_gb300.nmgpu import Solver
    sv = Solver(mats, porder)
    r = sv.solve(*interval, want_vectors=True, unscale=True, **kw)
    return sv, r


def _groups(w, tol=1e-6):
    g = [0]
    for i in range(1, len(w)):
        g.append(g[-1] + int(abs(w[i] - w[i - 1]) > tol * abs(w[i - 1])))
    return np.array(g)


@pytest.mark.parametrize("name", ["solid_p1", "fs_p1", "fs_p2"])
def test_adjoint_matches_cpu_reference(small_models, name):
    from oracle import adjoint_ref as AR
    from oracle import fem_ref
    d = small_models[name]
    m = d["model"]
    mesh, ref = m.mesh(), m.reference()
    sv, r = _solve(d["mats"], d["porder"], d["interval"])
    try:
        k = min(8, len(r.lam))
        lam, X = r.lam[:k], r.vec[:, :k]
        grad, group = sv.adjoint(mesh, ref, lam, X)
        assert grad.shape == (k, mesh["tets"].shape[0], 3)
        rng = np.random.default_rng(5)
        els = rng.choice(mesh["tets"].shape[0], 40, replace=False)
        if mesh["fluid"].any():
            els = np.concatenate([els, rng.choice(np.where(mesh["fluid"])[0], 10, replace=False)])
        P = AR.pressure(d["mats"], X) if "Ap" in d["mats"] else None
        G = AR.gradient(fem_ref.reference_element(d["porder"]), mesh, lam, X, P, elements=els)
        for j in range(k):
            for c in range(3):
                scale = np.max(np.abs(grad[j, :, c]))
                if scale == 0.0:
                    continue
                err = np.max(np.abs(grad[j, els, c] - G[j, :, c]))
                assert err <= 1e-8 * scale, (j, c, err, scale)
        # fluid elements have no shear sensitivity
        assert np.all(grad[:, mesh["fluid"], 2] == 0.0)
        # multiplet mode sums the pairs of each group
        gm, gr = sv.adjoint(mesh, ref, lam, X, mode=1, tol=1e-6)
        for g in range(gm.shape[0]):
            assert np.allclose(gm[g], grad[gr == g].sum(axis=0), rtol=1e-12, atol=0.0)
    finally:
        sv.close()


def test_adjoint_matches_finite_differences():
    """20 seeded elements of the fluid-solid P1 ball, one parameter each
    (density, bulk, shear in turn; fluid elements density / bulk)."""
    from normalmodes_gb300.model import Model
    from oracle import adjoint_ref as AR
    m = Model.ball(n_cells=8, porder=1)
    mesh, ref = m.mesh(), m.reference()
    interval = (0.2, 1.0)
    sv, r = _solve(m.operators(), 1, interval)
    lam0, X = r.lam, r.vec
    ab = (r.xintv[2], r.xintv[3])
    # clusters closer than 1e-3 (relative) are summed: a perturbation of
    # this size moves eigenvalues by ~1e-6 relative and can mix pairs whose
    # gap is of that order, while a cluster sum stays smooth
    gr = _groups(lam0, tol=1e-3)
    full = [g for g in np.unique(gr)]
    grad, _ = sv.adjoint(mesh, ref, lam0, X)
    sv.close()
    rng = np.random.default_rng(20)
    els = rng.choice(mesh["tets"].shape[0], 20, replace=False)
    for i, k in enumerate(els):
        which = i % (2 if mesh["fluid"][k] else 3)
        h = 1e-4 * AR.element_parameter(mesh, k, which)
        lam_pm = []
        for sgn in (1.0, -1.0):
            m.set_material(*AR.perturbed_material(mesh, k, which, sgn * h))
            s2, r2 = _solve(m.operators(), 1, interval, ab_bounds=ab)
            s2.close()
            assert len(r2.lam) == len(lam0)
            lam_pm.append(r2.lam)
        m.set_material(mesh["vp"], mesh["vs"], mesh["rho"])
        fd = (lam_pm[0] - lam_pm[1]) / (2 * h)
        fdg = np.array([fd[gr == g].sum() for g in full])
        gg = np.array([grad[gr == g, k, which].sum() for g in full])
        assert np.max(np.abs(fdg - gg)) <= 1e-3 * np.max(np.abs(gg)), (k, which, fdg, gg)


def test_autograd_function_wrapper(small_models):
    """d(sum of one multiplet)/d(per-element parameter shifts) through a
    torch.autograd.Function whose backward calls nm_adjoint."""
    import torch
    from normalmodes_gb300.model import Model
    from oracle import adjoint_ref as AR
    from oracle import fem_ref

    m = Model.ball(n_cells=6, porder=1, fluid_core=0)
    mesh, ref = m.mesh(), m.reference()
    interval = (0.2, 1.0)

    class Eigenvalues(torch.autograd.Function):
        @staticmethod
        def forward(ctx, shifts):
            assert float(shifts.abs().max()) == 0.0  # evaluated at the assembled material
            sv, r = _solve(m.operators(), 1, interval)
            ctx.sv, ctx.lam, ctx.X = sv, r.lam, r.vec
            return torch.from_numpy(r.lam.copy())

        @staticmethod
        def backward(ctx, g):
            grad, _ = ctx.sv.adjoint(mesh, ref, ctx.lam, ctx.X)
            ctx.sv.close()
            return torch.einsum("j,jec->ec", g.double(), torch.from_numpy(grad))

    shifts = torch.zeros(mesh["tets"].shape[0], 3, dtype=torch.float64, requires_grad=True)
    lam = Eigenvalues.apply(shifts)
    gr = _groups(lam.detach().numpy())
    sel = torch.from_numpy(gr == gr[len(gr) // 2])
    lam[sel].sum().backward()
    # the multiplet sum is basis independent: compare with the CPU reference
    sv, r = _solve(m.operators(), 1, interval)
    sv.close()
    idx = np.where(sel.numpy())[0]
    els = np.arange(0, mesh["tets"].shape[0], 37)
    G = AR.gradient(fem_ref.reference_element(1), mesh, r.lam[idx], r.vec[:, idx], None, elements=els).sum(axis=0)
    got = shifts.grad.numpy()[els]
    assert np.max(np.abs(got - G)) <= 1e-8 * np.max(np.abs(G))
