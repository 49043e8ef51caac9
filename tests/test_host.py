"""CPU tests of libnmgpu's host side: the C-ABI loads and exports every
symbol of include/nmgpu.h, the filter design and the tridiagonal solver
agree with the oracle and with LAPACK, and the library fails loudly
without a GPU (there is no CPU fallback)."""
import os
import re

import numpy as np
import pytest

from normalmodes_gb300 import nmgpu
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_exports_every_declared_symbol():
    hdr = open(os.path.join(ROOT, "include", "nmgpu.h")).read()
    declared = set(re.findall(r"\b(nm_[a-z_0-9]+)\s*\(", hdr))
    L = nmgpu.lib()
    missing = [s for s in sorted(declared) if not hasattr(L, s)]
    assert not missing, missing
    assert set(nmgpu.EXPORTS) <= declared
    # and the model library exports what include/nmmodel.h declares
    from normalmodes_gb300 import model
    mh = open(os.path.join(ROOT, "include", "nmmodel.h")).read()
    mdecl = set(re.findall(r"\b(nmm_[a-z_0-9]+)\s*\(", mh))
    assert {"nmm_set_gravity", "nmm_load_gravity", "nmm_ball_gravity", "nmm_get_gravity"} <= mdecl
    ML = model.lib()
    assert not [f for f in sorted(mdecl) if not hasattr(ML, f)]


def test_start_vector_matches_oracle():
    assert np.array_equal(nmgpu.start_vector(4097), O.start_vector(4097))


@pytest.mark.parametrize("xintv", [
    [1.579e-6, 3.9478e-5, -5e-9, 1.475e-3],      # interior, P1-like
    [3.9e-7, 1.58e-4, -1e-8, 0.6],               # interior, P2-like (high degree)
    [-1e-9, 1e-5, 0.0, 0.01],                    # left end interval
    [0.5e-2, 0.02, 0.0, 0.01],                   # right end interval
])
def test_find_pol_matches_oracle(xintv):
    deg, mu, (cc, dd, gam, bar) = nmgpu.find_pol(xintv)
    p = O.find_pol(xintv)
    assert deg == p.deg
    assert abs(bar - p.bar) < 1e-12 and abs(gam - p.gam) < 1e-12
    assert np.max(np.abs(mu - p.mu)) < 1e-12
    # the degree is the smallest one whose filter drops to the threshold
    thr = 0.8 if p.kind == "interior" else 0.7
    assert bar <= thr


def test_tridiagonal_matches_lapack():
    from scipy.linalg import eigh_tridiagonal
    rng = np.random.default_rng(1)
    for k in (3, 64, 500):
        d = rng.standard_normal(k)
        e = rng.standard_normal(k - 1)
        d[:6] = 0.9
        e[:5] = 1e-11  # a near-degenerate cluster
        w, V = nmgpu.tridiag_eig(d, e, 0.1, 1e9)
        ws = eigh_tridiagonal(d, e, eigvals_only=True)
        ws = ws[ws >= 0.1]
        assert len(w) == len(ws)
        assert np.max(np.abs(w - ws)) < 1e-12 * max(1, np.max(np.abs(ws)))
        T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
        assert np.max(np.abs(T @ V - V * w)) < 1e-12
        assert np.max(np.abs(V.T @ V - np.eye(len(w)))) < 1e-10


def test_sell_packing():
    import ctypes as C
    rng = np.random.default_rng(2)
    nr = 77
    lens = rng.integers(0, 9, size=nr)
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    col = rng.integers(0, 50, size=rp[-1]).astype(np.int32)
    val = rng.standard_normal(rp[-1])
    rl = np.zeros(nr, np.int32)
    sp = np.zeros((nr + 31) // 32 + 1, np.int64)
    L = nmgpu.lib()
    stored = L.nm_test_sell(nr, 50, rp.ctypes.data_as(C.POINTER(C.c_int)), col.ctypes.data_as(C.POINTER(C.c_int)),
                            val.ctypes.data_as(C.POINTER(C.c_double)), rl.ctypes.data_as(C.POINTER(C.c_int)),
                            sp.ctypes.data_as(C.POINTER(C.c_longlong)))
    assert np.array_equal(rl, lens)
    widths = [lens[s * 32:(s + 1) * 32].max() for s in range(len(sp) - 1)]
    assert stored == 32 * sum(widths) == sp[-1]


def _sell_reference(rp, col, val, dl, dr, sign, S=32):
    """SELL-S layout: slices of S rows padded to their longest row, stored
    column-major within a slice; padding repeats the row's last column with
    value 0; values scaled as sign * dl[r] * a_rc * dr[c]."""
    nr = len(rp) - 1
    lens = np.diff(rp)
    ns = (nr + S - 1) // S
    width = [int(lens[s * S:(s + 1) * S].max()) for s in range(ns)]
    ptr = np.concatenate([[0], np.cumsum(np.array(width) * S)])
    C_ = np.zeros(ptr[-1], np.int32)
    V = np.zeros(ptr[-1])
    for r in range(nr):
        base = ptr[r // S] + r % S
        cols = col[rp[r]:rp[r + 1]]
        vals = sign * val[rp[r]:rp[r + 1]] * dr[cols] * dl[r]
        for k in range(width[r // S]):
            C_[base + k * S] = cols[k] if k < len(cols) else (cols[-1] if len(cols) else 0)
            V[base + k * S] = vals[k] if k < len(cols) else 0.0
    return C_, V


@pytest.mark.parametrize("seed", [0, 1])
def test_sell_arrays_match_the_layout(seed):
    """The packed indices and scaled values (what nm_create uploads) against a
    direct restatement of the layout, element for element; empty rows and a
    ragged last slice included."""
    import ctypes as C
    rng = np.random.default_rng(seed)
    nr, nc = 1000 + 37 * seed, 300
    lens = rng.integers(0, 12, size=nr)
    lens[rng.integers(0, nr, 20)] = 0
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    col = rng.integers(0, nc, size=rp[-1]).astype(np.int32)
    val = rng.standard_normal(rp[-1])
    dl, dr = rng.uniform(0.5, 2.0, nr), rng.uniform(0.5, 2.0, nc)
    L = nmgpu.lib()
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    rl = np.zeros(nr, np.int32)
    sp = np.zeros((nr + 31) // 32 + 1, np.int64)
    stored = L.nm_test_sell(nr, nc, ip(rp), ip(col), fp(val), ip(rl), sp.ctypes.data_as(C.POINTER(C.c_longlong)))
    Cg, Vg = np.zeros(stored, np.int32), np.zeros(stored)
    L.nm_test_sell_arrays(nr, nc, ip(rp), ip(col), fp(val), fp(dl), fp(dr), -1.0, ip(Cg), fp(Vg))
    Cr, Vr = _sell_reference(rp, col, val, dl, dr, -1.0)
    assert np.array_equal(Cg, Cr)
    assert np.array_equal(Vg, Vr)


def test_no_gpu_fails_loudly(small_models):
    from tests.conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    d = small_models["solid_p1"]
    with pytest.raises(nmgpu.NmError) as ei:
        nmgpu.Solver(d["mats"], d["porder"])
    assert ei.value.code == -2  # NM_ERR_CUDA


def test_bad_arguments_rejected(small_models):
    """Shape errors are caught on the host before any device work."""
    import copy
    d = small_models["fs_p1"]
    mats = dict(d["mats"])
    bad = copy.copy(mats["E"])
    bad.shape = (bad.shape[0], bad.shape[1] + 1)
    mats["E"] = bad
    with pytest.raises(nmgpu.NmError) as ei:
        nmgpu.Solver(mats, d["porder"])
    assert ei.value.code == -1  # NM_ERR_ARG


@pytest.mark.parametrize("which,fault,code", [
    ("B", "rowptr0", -1), ("Ad", "rowptr_order", -1), ("E", "col_range", -1),
    ("Ad", "nan", -6), ("ET", "inf", -6), ("Ap", "nan", -6),
])
def test_corrupted_inputs_rejected_on_the_host(small_models, which, fault, code):
    """Host-side fault injection: corrupted CSR (NM_ERR_ARG) and NaN / Inf
    values (NM_ERR_NUMERIC) planted in host copies of the operators are
    rejected by nm_create's validator before any device work, so the codes
    are the same with or without a GPU."""
    import copy
    d = small_models["fs_p1"]
    mats = dict(d["mats"])
    m = copy.deepcopy(mats[which])
    if fault == "rowptr0":
        m.rowptr = m.rowptr.copy()
        m.rowptr[0] = 1
    elif fault == "rowptr_order":
        m.rowptr = m.rowptr.copy()
        m.rowptr[5], m.rowptr[6] = m.rowptr[6], m.rowptr[5] - 1
    elif fault == "col_range":
        m.col = m.col.copy()
        m.col[7] = m.shape[1]
    else:
        m.val = m.val.copy()
        m.val[len(m.val) // 2] = np.nan if fault == "nan" else np.inf
    mats[which] = m
    with pytest.raises(nmgpu.NmError) as ei:
        nmgpu.Solver(mats, d["porder"])
    assert ei.value.code == code
