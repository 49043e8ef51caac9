"""nm_solve_batched: adjacent spectrum slices give together the eigenpairs
of the whole interval (count equal, eigenvalues within 1e-10 relative), for
the single-vector FP64 path and the block mixed path."""
import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]


@pytest.mark.parametrize("block,prec,tol", [(0, 0, 1e-10), (32, 1, 1e-9)], ids=["fp64", "mixed-block"])
def test_slices_cover_the_interval(small_models, block, prec, tol):
    from normalmodes_gb300.nmgpu import Solver
    d = small_models["fs_p1"]
    lo, hi = d["interval"]
    mid = 0.5 * (lo + hi)
    with Solver(d["mats"], d["porder"], precision=prec) as sv:
        whole = sv.solve(lo, hi, block=block, want_vectors=False)
        parts = sv.solve_batched([(lo, mid), (mid, hi)], block=block, want_vectors=False)
    lam = np.concatenate([p.lam for p in parts])
    assert len(lam) == len(whole.lam)
    assert np.max(np.abs(np.sort(lam) - whole.lam) / np.abs(whole.lam)) < tol
    assert all(p.pol_deg > 0 for p in parts)


def test_bad_slice_is_rejected(small_models):
    from normalmodes_gb300.nmgpu import NmError, Solver
    d = small_models["solid_p1"]
    with Solver(d["mats"], d["porder"]) as sv:
        with pytest.raises(NmError):
            sv.solve_batched([(0.5, 0.4)])
