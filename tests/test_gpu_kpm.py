"""GPU tests of the device KPM moments (nm_kpm_moments_ctx): the same
Rademacher vectors and estimator as the host routine nm_kpm_moments, with
B^-1 A applied to 32-column blocks on the device.

* FP64 context: the device moments equal the host moments taken through the
  same context's block callbacks (nm_amv_block + nm_bsolve_block) within
  1e-10 of the largest moment (different kernels, same arithmetic);
* mixed-precision context (FP32 block operators): within 1e-4, far below
  the estimator's own sampling error (~1 / sqrt(n nvec));
* the slices nm_slice_spectrum cuts from them on a fluid-solid ball hold the
  oracle's eigenvalue count.
"""
import os

import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden(name):
    return np.load(os.path.join(HERE, "golden", f"{name}.npz"))


def _lam(f):
    pi = float(np.float32(3.14159265359))
    f = float(np.float32(f))
    return (2 * pi * f) ** 2 * 1e-6


@pytest.mark.parametrize("name", ["fs_p1", "fs_p2"])
def test_device_moments_match_host_moments(small_models, name):
    from normalmodes_gb300 import nmgpu
    from normalmodes_gb300.nmgpu import NM_PREC_MIXED, Solver
    d = small_models[name]
    g = _golden(name)
    lmin, lmax = float(g["xintv"][2]), float(g["xintv"][3]) * 1.005
    deg, nvec = 300, 16
    with Solver(d["mats"], d["porder"], b_bounds=tuple(g["b_bounds"]), ap_bounds=tuple(g["ap_bounds"])) as sv:
        mu_dev = sv.kpm_moments(lmin, lmax, deg, nvec)
        n = sv.n
        mu_host = nmgpu.kpm_moments(lambda X: sv.block("bsolve", sv.block("amv", X)), n, lmin, lmax, deg, nvec)
    scale = np.max(np.abs(mu_host))
    err64 = np.max(np.abs(mu_dev - mu_host)) / scale
    with Solver(d["mats"], d["porder"], precision=NM_PREC_MIXED, b_bounds=tuple(g["b_bounds"]),
                ap_bounds=tuple(g["ap_bounds"])) as sm:
        mu32 = sm.kpm_moments(lmin, lmax, deg, nvec)
    err32 = np.max(np.abs(mu32 - mu_host)) / scale
    print(f"{name}: device vs host moments, FP64 {err64:.2e}, FP32 {err32:.2e}")
    assert err64 <= 1e-10
    assert err32 <= 1e-4


def test_device_slices_hold_the_oracle_count(small_models):
    from normalmodes_gb300.nmgpu import Solver
    d = small_models["fs_p1"]
    g = _golden("fs_p1")
    ab = (float(g["xintv"][2]), float(g["xintv"][3]))
    with Solver(d["mats"], 1, b_bounds=tuple(g["b_bounds"]), ap_bounds=tuple(g["ap_bounds"])) as sv:
        sl, counts = sv.slice_spectrum(0.2, 1.0, 3, ab_bounds=ab)
    w = g["lam"]
    per = [int(np.sum((w > _lam(a)) & (w <= _lam(b)))) for a, b in sl]
    assert sum(per) == len(w)
    assert abs(counts.sum() - len(w)) <= 0.15 * len(w), (counts, len(w))
