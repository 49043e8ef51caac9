"""Element-level assembly on the GPU (nm_assemble, JOB = 1) against the
host assembly (nmm_assemble) of the same model into the same CSR
structures: solid and fluid-solid layered balls (P1 and P2) and the
reference's CONST3k / PREM3k inputs.  The element formulas are the same, so
the values agree up to the order of the floating-point additions: 1e-13 of
the largest entry of each operator."""
import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]


@pytest.mark.parametrize("name", ["solid_p1", "fs_p1", "fs_p2", "const3k_p1", "prem3k_p1"])
def test_device_assembly_matches_host(small_models, name):
    from normalmodes_gb300 import nmgpu
    if name in small_models:
        m = small_models[name]["model"]
    else:
        from tests.golden.make_golden import load_model
        m = load_model(name)
    vals, sec = nmgpu.assemble(m)
    mats = m.operators()
    worst = 0.0
    for nm, v in vals.items():
        ref = mats[nm].val
        err = np.max(np.abs(v - ref)) / max(np.max(np.abs(ref)), 1e-300)
        worst = max(worst, err)
        assert err <= 1e-13, (nm, err)
    print(f"{name}: {m.info().ntet} elements assembled on the GPU in {sec * 1e3:.2f} ms, max rel diff {worst:.1e}")
