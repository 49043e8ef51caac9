"""CPU tests of the KPM spectrum slicer (nm_kpm_* in libnmgpu): the moment
recurrence, the weighted count and the slices, driven through the block
operator callback by exact diagonal operators and by the oracle's B^-1 A."""
import math
import os
import subprocess
import sys

import numpy as np
import pytest

from normalmodes_gb300 import nmgpu


def _lam(f):
    """Frequency (mHz) to eigenvalue as the reference maps it (src/mod_pevsl.f90:93-99)."""
    pi = float(np.float32(3.14159265359))
    f = float(np.float32(f))
    return (2 * pi * f) ** 2 * 1e-6


def test_moments_of_a_diagonal_operator_are_exact():
    """With Rademacher vectors v' D v = tr(D) for diagonal D, so the
    estimate equals tr(T_k(S) Lambda) / n exactly."""
    rng = np.random.default_rng(3)
    lam = np.sort(rng.uniform(0.0, 2.0, 500))
    lam[:40] = 0.0  # a null space
    lmin, lmax = 0.0, 2.0
    deg = 60
    mu = nmgpu.kpm_moments(lambda X: lam[:, None] * X, len(lam), lmin, lmax, deg, nvec=3)
    t = (lam - 1.0) / 1.0
    ref = np.array([np.mean(np.cos(k * np.arccos(np.clip(t, -1, 1))) * lam) for k in range(deg + 1)])
    assert np.max(np.abs(mu - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_weighted_count_ignores_the_null_space():
    """500 zero eigenvalues next to an interval starting at 4e-7: the count
    of the interval is that of its own eigenvalues."""
    rng = np.random.default_rng(5)
    nz = 500
    inside = np.sort(rng.uniform(_lam(0.1), _lam(2.0), 200))
    bulk = rng.uniform(_lam(2.0) * 1.2, 0.6, 3000)
    lam = np.concatenate([np.zeros(nz), inside, bulk])
    n, lmin, lmax = len(lam), 0.0, 0.6 * 1.005
    deg = nmgpu.kpm_degree(lmin, lmax, _lam(0.1), _lam(2.0), 4)
    assert 50 <= deg <= 2000
    mu = nmgpu.kpm_moments(lambda X: lam[:, None] * X, n, lmin, lmax, deg, nvec=2)
    est = nmgpu.kpm_count(mu, n, lmin, lmax, _lam(0.1), _lam(2.0))
    assert abs(est - 200) < 0.1 * 200
    sl, counts = nmgpu.kpm_slices(mu, n, lmin, lmax, 0.1, 2.0, 4)
    assert sl[0][0] == 0.1 and sl[-1][1] == 2.0
    assert all(sl[i][1] == sl[i + 1][0] for i in range(3))
    exact = [np.sum((lam > _lam(a)) & (lam <= _lam(b))) for a, b in sl]
    # exact moments here: what is left is the resolution of the degree rule
    assert max(abs(c - 50) for c in exact) <= 0.35 * 50, exact


def test_degree_rule():
    # Jackson width pi / d = a quarter of the mean slice width in theta = acos(t)
    for lmax, ns in ((0.0044, 6), (0.05, 4), (0.6, 8)):
        a, b = _lam(0.1), _lam(2.0)
        d = nmgpu.kpm_degree(0.0, lmax, a, b, ns)
        c = e = lmax / 2
        dth = math.acos((a - c) / e) - math.acos((b - c) / e)
        assert d == max(50, min(4000, math.ceil(4 * math.pi * ns / dth)))
    assert nmgpu.kpm_degree(0.0, 0.6, _lam(2.0), _lam(0.1), 8) == 0


@pytest.mark.parametrize("name,slices", [("solid_p1", 5), ("fs_p1", 6)])
def test_slices_of_small_models(small_models, name, slices):
    """Against a dense solve of the oracle's pencil: the estimated count of
    [0.1, 2.0] mHz within 10 %, and every slice within 35 % of the mean."""
    from scipy.linalg import eigh

    from oracle import oracle as O
    d = small_models[name]
    op = O.setup_operator(d["mats"], d["porder"])
    A, Bm = O.dense_operator(op)
    w = eigh(A, Bm, eigvals_only=True)
    lmin, lmax = w[0], w[-1] * 1.005

    def apply(X):
        return np.stack([op.bsolve(op.amv(X[:, j])) for j in range(X.shape[1])], axis=1)

    lo, hi = _lam(0.1), _lam(2.0)
    deg = nmgpu.kpm_degree(lmin, lmax, lo, hi, slices)
    mu = nmgpu.kpm_moments(apply, op.n, lmin, lmax, deg, nvec=16)
    exact = int(np.sum((w > lo) & (w <= hi)))
    assert abs(nmgpu.kpm_count(mu, op.n, lmin, lmax, lo, hi) - exact) <= 0.1 * exact
    sl, counts = nmgpu.kpm_slices(mu, op.n, lmin, lmax, 0.1, 2.0, slices)
    per = [int(np.sum((w > _lam(a)) & (w <= _lam(b)))) for a, b in sl]
    assert sum(per) == exact
    assert max(abs(c - exact / slices) for c in per) <= 0.35 * exact / slices, per
    assert abs(counts.sum() - exact) <= 0.1 * exact


def test_bad_arguments():
    mu = np.ones(10)
    with pytest.raises(nmgpu.NmError):
        nmgpu.kpm_slices(mu, 100, 0.0, 1.0, 0.0, 1.0, 3)  # lower frequency 0
    with pytest.raises(nmgpu.NmError):
        nmgpu.kpm_count(mu, 100, 1.0, 1.0, 0.1, 0.2)  # empty bounds
    with pytest.raises(nmgpu.NmError):
        nmgpu.kpm_moments(lambda X: X, 10, 0.0, 1.0, 0, 2)  # degree 0
    def broken(X):
        raise ValueError("operator failed")

    with pytest.raises(ValueError, match="operator failed"):
        nmgpu.kpm_moments(broken, 10, 0.0, 1.0, 3, 2)  # operator errors surface


def test_moments_do_not_depend_on_the_thread_count():
    """Bitwise-identical moments with 1 and 4 OpenMP threads (fixed-chunk
    partial sums), so the slices are the same on any host."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = (
        "import sys, numpy as np; sys.path.insert(0, %r)\n"
        "from normalmodes_gb300 import nmgpu\n"
        "rng = np.random.default_rng(1); lam = rng.uniform(0, 1, 300000)\n"
        "mu = nmgpu.kpm_moments(lambda X: lam[:, None] * X, len(lam), 0.0, 1.0, 30, nvec=2)\n"
        "sys.stdout.write(mu.tobytes().hex())\n" % root)
    outs = []
    for nt in ("1", "4"):
        env = dict(os.environ, OMP_NUM_THREADS=nt)
        outs.append(subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                                   check=True, timeout=300).stdout)
    assert outs[0] == outs[1] and len(outs[0]) > 0
