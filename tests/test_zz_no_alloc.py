"""nm_bsolve_dev_noalloc (scratch array compiled into the library, no device
allocation) against nm_bsolve_dev on the same context, through the C-ABI.

The two entry points run the same Chebyshev semi-iteration in the same
summation order, so the results are expected to agree to the last bit; the
test allows a relative max-norm difference of 1e-13.  Each model makes two
calls in a row with different right-hand sides, so the second call must not
depend on what the first left in the shared scratch; around the second call
the device's free memory (cudaMemGetInfo) must not move.  A context with
more rows than the scratch holds is refused with NM_ERR_ARG.
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
            assert L.nm_sync(sv._h) == 0
            free0 = torch.cuda.mem_get_info()[0]
            rc = L.nm_bsolve_dev_noalloc(sv._h, x.data_ptr(), y_new.data_ptr())
            assert rc == 0, L.nm_last_error(sv._h)
            assert L.nm_sync(sv._h) == 0
            if call == 1:  # the first call may load the library's module on this device
                assert torch.cuda.mem_get_info()[0] == free0, "the no-allocation call changed free device memory"
            a, b = y_new.cpu().numpy(), y_ref.cpu().numpy()
            assert np.all(np.isfinite(a)), f"call {call}"
            assert _rel(a, b) <= TOL, f"call {call}: {_rel(a, b)}"


@pytest.mark.gpu
def test_noalloc_refuses_more_rows_than_the_scratch():
    """n = NM_NOALLOC_MAX_ROWS + 32 rows (a diagonal pencil, cheap to build):
    the call is refused with NM_ERR_ARG and a message naming the limit, and
    nothing is launched."""
    import scipy.sparse as sp
    from normalmodes_gb300 import nmgpu
    from normalmodes_gb300.model import Csr

    import torch

    n = 1310720 + 32
    eye = sp.identity(n, format="csr", dtype=np.float64)
    mk = lambda m: Csr(m.indptr.astype(np.int32), m.indices.astype(np.int32), m.data.copy(), m.shape)
    L = nmgpu.lib()
    with nmgpu.Solver({"A": mk(2.0 * eye), "B": mk(eye)}, 1, b_bounds=(0.5, 2.0)) as sv:
        x = torch.ones(n, dtype=torch.float64, device="cuda")
        y = torch.zeros_like(x)
        torch.cuda.synchronize()
        rc = L.nm_bsolve_dev_noalloc(sv._h, x.data_ptr(), y.data_ptr())
        assert rc == -1
        msg = L.nm_last_error(sv._h).decode()
        assert "1310720" in msg and "exceeds" in msg, msg
        assert L.nm_sync(sv._h) == 0
        assert float(y.abs().max()) == 0.0  # nothing was written
