"""Failure detection of the bounded device-side waits, without a GPU fault:
a one-block kernel waits at the grid barrier for a block that is never
launched (a flag nothing sets), gives up after a short spin limit and sets
the status word; the host turns it into NM_ERR_TIMEOUT.  The GPU stays
usable: a new context computes a correct B-product afterwards."""
import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]


def test_barrier_wait_times_out_and_reports(small_models):
    from normalmodes_gb300 import nmgpu
    from oracle import oracle as O
    d = small_models["solid_p1"]
    L = nmgpu.lib()
    with nmgpu.Solver(d["mats"], d["porder"]) as sv:
        assert L.nm_test_barrier_timeout(sv._h, 1 << 16) == -5  # NM_ERR_TIMEOUT
        assert b"timed out" in L.nm_last_error(sv._h)
    op = O.setup_operator(d["mats"], d["porder"])
    try:
        x = np.random.default_rng(1).standard_normal(op.n)
        with nmgpu.Solver(d["mats"], d["porder"]) as sv2:
            y = sv2.bmv(x)
        ref = op.bmv(x)
        assert np.max(np.abs(y - ref)) <= 1e-12 * np.max(np.abs(ref))
    finally:
        op.close()
