"""CPU check of the mixed path's refinement design, in FP32 emulation on a
small pencil with its dense eigendecomposition.

The GPU refinement (`refine64`) is restated here in numpy: the three-term
recurrence in correction form, E_0 = R, E_1 = alpha A B~^-1 R + (alpha theta
- beta) R, E_{j+1} = 2 l(A B~^-1) E_j - E_{j-1} + 2 alpha theta s_j R, with
A, B and the Chebyshev B~^-1 in float32 and the residual R, the update and
the Rayleigh-Ritz in float64.  The band start and the degree of every block
come from the library itself (nm_test_refine_band), so the test exercises
its host decisions.  The start vectors are the exact eigenvectors plus white
noise of 1e-6 relative, the character of the FP32 filter's Ritz vectors.

It shows the two facts the design rests on:

* a refinement that damps [8 theta, lmax] only leaves the noise in the modes
  just above b, and the reference's RMS residual stalls far above 1e-10;
* with guard vectors for the modes in (b, 1.5 b] and passes whose band starts
  at 1.05 x the top guarded value, every pair meets err_ref <= 1e-10, and
  the eigenvalues stay within 1e-10 of the dense ones.
"""
import ctypes as C
import math
import os

import numpy as np
import pytest
from scipy.linalg import eigh

from normalmodes_gb300 import nmgpu
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
F32 = np.float32


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@pytest.fixture(scope="module")
def pencil():
    from normalmodes_gb300.model import Model
    g = np.load(os.path.join(HERE, "golden", "solid_p1.npz"))
    mats = Model.ball(n_cells=6, porder=1, fluid_core=0).operators()
    op = O.setup_operator(mats, 1, bounds={"B": tuple(g["b_bounds"])})
    A, B = O.dense_operator(op)
    w, X = eigh(A, B)
    return dict(A=A, B=B, w=w, X=X, g=g)


class _Emu:
    def __init__(self, p):
        self.A, self.B, g = p["A"], p["B"], p["g"]
        self.A32, self.B32 = self.A.astype(F32), self.B.astype(F32)
        self.lmax = float(g["xintv"][3])
        self.bl, self.bh = (float(x) for x in g["b_bounds"])
        k = self.bh / self.bl
        s = (math.sqrt(k) - 1) / (math.sqrt(k) + 1)
        self.dB = max(1, min(25, math.ceil(math.log(2.0 ** -24 / 2) / math.log(s))))
        self.n = self.A.shape[0]
        self.tol = 0.5e-10 * math.sqrt(self.n)

    def bsolve(self, v):
        """FP32 Chebyshev semi-iteration for B x = v (the B~^-1 of the filter)."""
        th, de = 0.5 * (self.bh + self.bl), 0.5 * (self.bh - self.bl)
        sig = th / de
        rho = 1 / sig
        v = v.astype(F32)
        x, r, d = np.zeros_like(v), v.copy(), v / F32(th)
        for _ in range(self.dB):
            x = x + d
            r = r - self.B32 @ d
            rn = 1 / (2 * sig - rho)
            d = F32(rn * rho) * d + F32(2 * rn / de) * r
            rho = rn
        return x + d

    def resid(self, U, th):
        R = self.A @ U - (self.B @ U) * th
        return R, np.linalg.norm(R, axis=0) / np.abs(th)

    def rr(self, U):
        GA, GB = U.T @ (self.A @ U), U.T @ (self.B @ U)
        th, Q = eigh(0.5 * (GA + GA.T), 0.5 * (GB + GB.T))
        return U @ Q, th

    def refine(self, U, th, want, near_c=0.0, low_x=0.0):
        U = U.copy()
        for j0 in range(0, U.shape[1], 32):
            cols = slice(j0, min(U.shape[1], j0 + 32))
            t = np.ascontiguousarray(th[cols])
            R, rb = self.resid(U[:, cols], t)
            # guards aim at 100x the target: scale their residuals to match
            rs = np.ascontiguousarray(np.where(want[cols], rb, rb / 100.0))
            if not np.any(rs > self.tol):
                continue
            out = np.zeros(4)
            nmgpu.lib().nm_test_refine_band(_dp(t), _dp(rs), len(t), self.lmax, self.tol, near_c, low_x, _dp(out))
            c0, deg = out[0], int(out[1])
            if deg <= 0:
                continue
            al, be = 2 / (self.lmax - c0), (self.lmax + c0) / (self.lmax - c0)
            lt = al * t - be

            def aop(v):
                return self.A32 @ self.bsolve(v)

            Rf = R.astype(F32)
            Em1 = Rf.copy()
            E = (F32(al) * aop(Rf) - F32(be) * Rf + (al * t).astype(F32) * Rf).astype(F32)
            tm1, tj = np.ones_like(t), lt.copy()
            for _ in range(1, deg):
                En = (F32(2 * al) * aop(E) - F32(2 * be) * E - Em1 + (2 * al * t * tj).astype(F32) * Rf).astype(F32)
                tm1, tj = tj, 2 * lt * tj - tm1
                Em1, E = E, En
            U[:, cols] += self.bsolve(E).astype(np.float64) / (t * tj)
        return U


def _start(p, idx, eps, rng):
    X = p["X"][:, idx]
    return X + eps * rng.standard_normal(X.shape) * np.linalg.norm(X, axis=0) / math.sqrt(X.shape[0])


def _report(emu, p, U, th, a, b):
    inn = (th >= a * (1 - 1e-9)) & (th <= b * (1 + 1e-9))
    _, r2 = emu.resid(U[:, inn], th[inn])
    w = p["w"]
    k = np.array([np.argmin(np.abs(w - t)) for t in th[inn]])
    return int(inn.sum()), float(r2.max() / math.sqrt(emu.n)), float(np.max(np.abs(th[inn] - w[k]) / w[k]))


def test_band_only_refinement_stalls_above_the_gate(pencil):
    p = pencil
    emu = _Emu(p)
    lam = p["g"]["lam"]
    a, b, w = lam.min(), lam.max(), p["w"]
    sel = np.where((w >= a * (1 - 1e-9)) & (w <= b * (1 + 1e-9)))[0]
    U, th = emu.rr(_start(p, sel, 1e-6, np.random.default_rng(7)))
    errs = []
    for _ in range(3):
        want = np.ones(len(th), bool)
        U, th = emu.rr(emu.refine(U, th, want))
        nin, err, _ = _report(emu, p, U, th, a, b)
        errs.append(err)
    assert nin == len(lam)
    assert min(errs) > 1e-9, errs  # stuck at the noise of the modes above b


def test_guards_and_near_passes_reach_the_gate(pencil):
    p = pencil
    emu = _Emu(p)
    lam = p["g"]["lam"]
    a, b, w = lam.min(), lam.max(), p["w"]
    rng = np.random.default_rng(7)
    sel = np.where((w >= a * (1 - 1e-9)) & (w <= b * (1 + 1e-9)))[0]
    gi = np.where(((w > b * (1 + 1e-9)) & (w <= 1.5 * b)) | ((w < a * (1 - 1e-9)) & (w >= a / 1.5) & (w > 0)))[0]
    assert len(gi) > 0
    U, th = emu.rr(np.concatenate([_start(p, sel, 1e-6, rng), _start(p, gi, 1e-6, rng)], axis=1))
    for sw in range(4):
        want = (th >= a * (1 - 1e-9)) & (th <= b * (1 + 1e-9))
        near = 1.05 * th.max() if sw > 0 else 0.0
        U, th = emu.rr(emu.refine(U, th, want, near, th.min() if sw > 0 else 0.0))
        keep = (th >= a / 1.5) & (th <= 1.5 * b)
        U, th = U[:, keep], th[keep]
    nin, err, eig = _report(emu, p, U, th, a, b)
    print(f"guards + near passes: {nin} pairs, err_ref max {err:.2e}, eigenvalue error max {eig:.2e}")
    assert nin == len(lam)
    assert err <= 1e-10
    assert eig <= 1e-10
