"""CPU tests of bench.py's host logic: the clock-sample summary that decides
whether a run is kept, the Gershgorin intervals of the CPU sample, and the
roofline inputs (measured peak, ncu traffic per launch)."""
import importlib.util
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    argv, sys.argv = sys.argv, ["bench.py"]
    try:
        spec.loader.exec_module(mod)
    finally:
        sys.argv = argv
    return mod


def test_clock_summary(bench):
    c = bench.Clocks(0)
    rows = [
        "0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 1200.5, 0x4, Not Active, Not Active, Not Active, Active",
        "0, [N/A], 2070, 10.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
        "0, 2040, 2070, 1390.0, 0x8, Active, Not Active, Not Active, Not Active",
    ]
    c.f.write(("\n".join(rows) + "\n").encode())
    c.f.close()
    s = c.summary()
    assert s["samples"] == 3 and s["sm_mhz"] == 2055.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"]
    assert not os.path.exists(c.f.name)


def test_gershgorin_intervals_contain_the_spectra(bench, small_models):
    mats = small_models["fs_p1"]["mats"]
    b = bench.gershgorin_bounds(mats)
    for name, sign in (("B", 1.0), ("Ap", -1.0)):
        A = mats[name].to_scipy().toarray() * sign
        d = 1.0 / np.sqrt(np.diag(A))
        w = np.linalg.eigvalsh(d[:, None] * A * d[None, :])
        lo, hi = b[name]
        assert hi >= w.max() * (1 - 1e-12)
        assert 0 < lo <= w.min() * (1 + 1e-12) or lo == pytest.approx(1e-3 * hi)


def test_roofline_inputs(bench):
    peak, kind = bench.peaks()
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        assert kind == "measured" and peak == float(json.load(open(path))["hbm_gbs"])
    else:
        assert (peak, kind) == (6800.0, "fallback")
    tr = bench.traffic_per_launch("k_mass_cheb_block32_fp32")
    d = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
    assert tr == float(d["k_mass_cheb_block32_fp32"]["bytes_per_launch"]) > 0
    assert bench.traffic_per_launch("no_such_kernel") is None


def test_step_cuts(bench):
    """The K steps of the timed solve: equal shares of the block-Lanczos
    steps, the set-up in the first step and the closing phases in the last,
    covering [t0, t_end] exactly."""
    blocks = [1.0 + 0.5 * i for i in range(1, 41)]  # 40 block steps ending at 1.5 .. 21.0
    cuts = bench.step_cuts(0.0, 30.0, blocks, 4)
    assert cuts == [0.0, blocks[9], blocks[19], blocks[29], 30.0]
    assert len(bench.step_cuts(0.0, 30.0, blocks, 20)) == 21
    assert bench.step_cuts(0.0, 8.0, blocks[:2], 4) == [0.0, 2.0, 4.0, 6.0, 8.0]
    c = bench.step_cuts(0.0, 30.0, blocks, 1)
    assert c == [0.0, 30.0]
