"""GPU tests of the batched (block) filtered Lanczos: FP64 block filter and
FP32 (mixed precision) block filter against the oracle's golden eigenvalues."""
import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]


def _golden(name):
    import os
    return np.load(os.path.join(os.path.dirname(__file__), "golden", f"{name}.npz"))


@pytest.mark.parametrize("name", ["solid_p1", "fs_p1", "fs_p2"])
def test_block_fp64_matches_oracle(small_models, name):
    from normalmodes_gb300.nmgpu import Solver
    d = small_models[name]
    g = _golden(name)
    with Solver(d["mats"], d["porder"], b_bounds=tuple(g["b_bounds"]),
                ap_bounds=tuple(g["ap_bounds"]) if name != "solid_p1" else None) as sv:
        lo, hi = g["interval"]
        res = sv.solve(lo, hi, ab_bounds=(float(g["xintv"][2]), float(g["xintv"][3])), block=32)
    assert res.pol_deg == int(g["pol_deg"])
    assert len(res.lam) == len(g["lam"])
    assert np.max(np.abs(res.lam - g["lam"]) / g["lam"]) < 1e-10
    assert np.max(res.err_ref) < 1e-10


@pytest.mark.parametrize("name", ["fs_p1", "fs_p2"])
def test_block_mixed_precision(small_models, name):
    """FP32 filter, FP64 Lanczos/Rayleigh-Ritz and the adaptive refinement:
    same eigenpairs, eigenvalues within 1e-10 and the reference's RMS
    residual (src/mod_pevsl.f90:158) within 1e-10."""
    from normalmodes_gb300.nmgpu import Solver, NM_PREC_MIXED
    d = small_models[name]
    g = _golden(name)
    with Solver(d["mats"], d["porder"], precision=NM_PREC_MIXED, b_bounds=tuple(g["b_bounds"]),
                ap_bounds=tuple(g["ap_bounds"])) as sv:
        lo, hi = g["interval"]
        res = sv.solve(lo, hi, ab_bounds=(float(g["xintv"][2]), float(g["xintv"][3])), block=32)
    assert len(res.lam) == len(g["lam"])
    rel = np.abs(res.lam - g["lam"]) / g["lam"]
    print(f"{name}: mixed eigenvalue rel err max {rel.max():.2e}, err_ref max {res.err_ref.max():.2e}, "
          f"{res.counts['refine_passes']} refinement passes, {res.counts['refine_guards']} guards")
    assert rel.max() < 1e-10
    assert res.err_ref.max() <= 1e-10
    assert res.counts["refine_guards"] > 0


@pytest.mark.parametrize("name", ["fs_p1", "fs_p2"])
def test_mixed_polish_reaches_fp64_eigenvalues(small_models, name):
    """Mixed path with the range-form filter (no FP32 rounding in the
    zero-frequency fluid modes), with the adaptive refinement (polish 0)
    against without it (polish -1): every refined eigenvalue within 1e-10 of
    the FP64 golden values, and the largest residual brought from FP32 level
    to the 1e-10 gate."""
    from normalmodes_gb300.nmgpu import Solver, NM_PREC_MIXED
    d = small_models[name]
    g = _golden(name)
    lo, hi = g["interval"]
    out = {}
    for pol in (-1, 0):
        with Solver(d["mats"], d["porder"], precision=NM_PREC_MIXED, b_bounds=tuple(g["b_bounds"]),
                    ap_bounds=tuple(g["ap_bounds"])) as sv:
            out[pol] = sv.solve(lo, hi, ab_bounds=(float(g["xintv"][2]), float(g["xintv"][3])), block=32,
                                polish=pol)
    for pol, res in out.items():
        assert len(res.lam) == len(g["lam"])
    rel = np.abs(out[0].lam - g["lam"]) / g["lam"]
    print(f"{name}: polished eigenvalue rel err max {rel.max():.2e}, err_ref max {out[0].err_ref.max():.2e} "
          f"(unpolished {out[-1].err_ref.max():.2e})")
    assert rel.max() <= 1e-10
    assert out[0].err_ref.max() <= 1e-10 < out[-1].err_ref.max()
