"""nm_bsolve_dev_noalloc (scratch array compiled into the library, no device
allocation) against nm_bsolve_dev on the same context, through the C-ABI.

The two entry points run the same Chebyshev semi-iteration in the same
summation order, so the results are expected to agree to the last bit; the
test allows a relative max-norm difference of 1e-13.  Each model makes two
calls in a row with different right-hand sides, so the second call must not
depend on what the first left in the shared scratch.
"""
import numpy as np
import pytest

TOL = 1e-13


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["solid_p1", "fs_p1"])
def test_noalloc_bsolve_matches_bsolve_dev(small_models, name):
    import torch
    from normalmodes_gb300 import nmgpu

    d = small_models[name]
    L = nmgpu.lib()
    with nmgpu.Solver(d["mats"], d["porder"]) as sv:
        n = sv.info().n
        assert n <= 1310720
        rng = np.random.default_rng(11)
        for call in range(2):
            x = torch.from_numpy(rng.standard_normal(n)).cuda()
            y_ref = torch.empty_like(x)
            y_new = torch.full_like(x, float("nan"))
            torch.cuda.synchronize()
            assert L.nm_bsolve_dev(sv._h, x.data_ptr(), y_ref.data_ptr()) == 0
            rc = L.nm_bsolve_dev_noalloc(sv._h, x.data_ptr(), y_new.data_ptr())
            assert rc == 0, L.nm_last_error(sv._h)
            assert L.nm_sync(sv._h) == 0
            a, b = y_new.cpu().numpy(), y_ref.cpu().numpy()
            assert np.all(np.isfinite(a)), f"call {call}"
            assert _rel(a, b) <= TOL, f"call {call}: {_rel(a, b)}"
