"""CPU FP64 oracle for the NormalModes eigensolve path -- TEST INFRASTRUCTURE.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use this module, and only as the checker / timed CPU baseline.  The
product (``normalmodes_gb300`` + ``libnmgpu.so``) never imports it.

What is restated, and from where (paths within js1019/NormalModes):

* operators and diagonal scaling -- ``nm_oracle.c`` (src/mod_matvec.f90:252-520)
* the solve driver ``pnm_apply_pevsl`` -- :func:`apply_pevsl`
  (src/mod_pevsl.f90:43-186): bounds of B^-1 A, the mHz -> lambda interval
  (:93-103, with the single-precision PI literal of :43 and the default-real
  frequencies of src/mod_para.f90:51-52), filter thresholds 0.8 / 0.7
  (:108-109), NEV = 802, MLAN = max(4 NEV, 2000), MAXIT = 3 MLAN, TOL = 1e-5
  (:113-119), the per-pair RMS residual (:144-162) and the ascending sort
  (:164-186).
* operator set-up ``setupmatvec`` -- :func:`setup_operator`
  (src/mod_matvec.f90:75-95,152-174): Lanczos bounds of B_s (1000 steps,
  tol 1e-12) and Ap_s (2000 steps, tol 1e-12), Chebyshev degrees 45/25 for B
  and max(min(int(cond),15)*3,100)/25 for Ap.
* pEVSL internals (not vendored in the reference; restated from the
  published methods): Lanczos bounds (:func:`lan_bounds`), the
  Chebyshev-Jackson delta filter with balanced centre and degree selection
  (:func:`find_pol`, Li, Xi, Vecharynski, Yang, Saad, SISC 38 (2016)), and
  polynomial-filtered non-restarted Lanczos with full reorthogonalisation in
  the B^-1 inner product (:func:`cheb_lan_nr`, EVSL, Li, Xi, Erlandson, Saad,
  SISC 41 (2019)).  The choices the reference does not pin (start vector,
  convergence-check cadence, two Gram-Schmidt passes, Jackson damping) are
  stated where they are made and are shared with the CUDA library.

Parity status: the reference ships no eigenvalues or eigenvectors for any
model and cannot be built here (Fortran + MPI + un-vendored pEVSL), so the
pEVSL-level parity is unpinned.  The oracle is pinned instead against an
independent dense generalized eigensolve of the same operators
(:func:`dense_reference`), against rigid-body null modes, and against the
analytic spectrum of a homogeneous sphere.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
import time
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "nm_oracle.c")

# Parameters of src/mod_pevsl.f90:43-52,108-119 and src/mod_matvec.f90:83-92,160-171
PI_REF = float(np.float32(3.14159265359))  # default-real literal assigned to real*8
TOL_SOLVE = 1.0e-5
MLAN_AB, LANSTEP_AB = 3000, 5000
THRE_INT, THRE_EXT = 0.8, 0.7
EVINT = 800
NEV = EVINT + 2
MLAN = max(4 * NEV, 2000)
MAXIT = 3 * MLAN
B_MLAN, B_LANSTEP, B_TOL = 1000, 2000, 1.0e-12
AP_MLAN, AP_LANSTEP, AP_TOL = 2000, 3000, 1.0e-12
# Build decisions for the unpinned pEVSL internals (shared with libnmgpu)
BOUNDS_CHECK_EVERY = 10
LAN_NTEST, LAN_CYCLE = 50, 50
GS_PASSES = 2
START_SEED = 0x5EED5EED


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.run(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", LIB, SRC, "-lm"], check=True)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        ip, dp, vp = C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_void_p
        L.or_create.restype = vp
        L.or_create.argtypes = [C.c_int, C.c_int, C.c_int] + [ip, ip, dp] * 5
        L.or_destroy.argtypes = [vp]
        for f in ("or_bmv", "or_apmv", "or_bsolve", "or_apsolve", "or_amv"):
            getattr(L, f).argtypes = [vp, dp, dp]
        L.or_set_cheb.argtypes = [vp, C.c_int, C.c_double, C.c_double, C.c_int]
        L.or_chebav.argtypes = [vp, C.c_int, dp, C.c_double, C.c_double, dp, dp]
        L.or_get_scaling.argtypes = [vp, dp, dp]
        L.or_get_scaled_values.argtypes = [vp, dp, dp]
        L.or_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _p(a, ct=C.c_double):
    return a.ctypes.data_as(C.POINTER(ct))


def start_vector(n: int, seed: int = START_SEED) -> np.ndarray:
    """Deterministic start vector in [-1, 1): splitmix64 of (seed, i).
    The CUDA library generates the same vector."""
    i = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = (np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15)) + i + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        x = x ^ (x >> np.uint64(31))
    u = (x >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return 2.0 * u - 1.0


# --------------------------------------------------------------------------- operator
class Operator:
    """Scaled operators of one model (what ``setupmatvec`` builds)."""

    def __init__(self, mats: dict):
        self.fs = "Ad" in mats
        A = mats["Ad"] if self.fs else mats["A"]
        B = mats["B"]
        self.n = B.shape[0]
        self.np = mats["Ap"].shape[0] if self.fs else 0
        self._keep = []

        def csr(c):
            rp = np.ascontiguousarray(c.rowptr, dtype=np.int32)
            ci = np.ascontiguousarray(c.col, dtype=np.int32)
            v = np.ascontiguousarray(c.val, dtype=np.float64)
            self._keep += [rp, ci, v]
            return [_p(rp, C.c_int), _p(ci, C.c_int), _p(v)]

        dummy = [C.POINTER(C.c_int)(), C.POINTER(C.c_int)(), C.POINTER(C.c_double)()]
        args = csr(A) + csr(B)
        if self.fs:
            args += csr(mats["Ap"]) + csr(mats["E"]) + csr(mats["ET"])
        else:
            args += dummy * 3
        self._h = lib().or_create(int(self.fs), self.n, self.np, *args)
        if not self._h:
            raise ValueError("non-positive diagonal in B or -Ap")
        self.D = np.empty(self.n)
        self.Dp = np.empty(max(self.np, 1))
        lib().or_get_scaling(self._h, _p(self.D), _p(self.Dp))
        self.Dp = self.Dp[: self.np]
        self.b_cheb = None
        self.ap_cheb = None
        self.nmatvec = {"A": 0, "B": 0, "Bsolve": 0}

    def set_cheb(self, which: str, lmin: float, lmax: float, deg: int) -> None:
        lib().or_set_cheb(self._h, 0 if which == "B" else 1, lmin, lmax, int(deg))
        if which == "B":
            self.b_cheb = (lmin, lmax, int(deg))
        else:
            self.ap_cheb = (lmin, lmax, int(deg))

    def _call(self, fn, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.np if fn in ("or_apmv", "or_apsolve") else self.n)
        getattr(lib(), fn)(self._h, _p(x), _p(y))
        return y

    def amv(self, x):
        self.nmatvec["A"] += 1
        return self._call("or_amv", x)

    def bmv(self, x):
        self.nmatvec["B"] += 1
        return self._call("or_bmv", x)

    def bsolve(self, x):
        self.nmatvec["Bsolve"] += 1
        return self._call("or_bsolve", x)

    def apmv(self, x):
        return self._call("or_apmv", x)

    def apsolve(self, x):
        return self._call("or_apsolve", x)

    def chebav(self, pol: "Pol", v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        y = np.empty(self.n)
        mu = np.ascontiguousarray(pol.mu, dtype=np.float64)
        lib().or_chebav(self._h, pol.deg, _p(mu), pol.cc, pol.dd, _p(v), _p(y))
        self.nmatvec["A"] += pol.deg
        self.nmatvec["Bsolve"] += pol.deg
        return y

    def close(self):
        if self._h:
            lib().or_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --------------------------------------------------------------------------- Lanczos bounds
def _tri_eig(alpha, beta, vectors=False):
    from scipy.linalg import eigh_tridiagonal
    if len(alpha) == 1:
        return (np.array(alpha), np.ones((1, 1))) if vectors else np.array(alpha)
    if vectors:
        return eigh_tridiagonal(alpha, beta[: len(alpha) - 1])
    return eigh_tridiagonal(alpha, beta[: len(alpha) - 1], eigvals_only=True)


def lan_bounds(matvec, n, msteps, tol, solve=None, v0=None):
    """Extreme eigenvalue bounds by Lanczos with full reorthogonalisation.

    Standard form (``solve is None``): Lanczos on ``matvec``.  Generalized
    form: Lanczos on solve(matvec(.)) = B~^-1 A in the B~^-1 inner product,
    carrying z = B~ v as ChebLanNr does.  Every BOUNDS_CHECK_EVERY steps the
    extreme Ritz values theta and their residual estimates |beta s_k| are
    checked against tol * max|theta|; the bounds are theta_min - |beta s| and
    theta_max + |beta s|.  Returns (lmin, lmax, steps)."""
    msteps = min(msteps, n)
    v = start_vector(n) if v0 is None else v0.copy()
    gen = solve is not None
    if gen:
        z = v
        v = solve(z)
        t = math.sqrt(float(v @ z))
        z = z / t
        v = v / t
    else:
        v = v / np.linalg.norm(v)
        z = v
    V = np.zeros((n, msteps + 1))
    Z = np.zeros((n, msteps + 1)) if gen else V
    V[:, 0] = v
    if gen:
        Z[:, 0] = z
    alpha = np.zeros(msteps)
    beta = np.zeros(msteps)
    lmin = lmax = None
    k = 0
    for k in range(msteps):
        znew = matvec(V[:, k])
        if k > 0:
            znew -= beta[k - 1] * Z[:, k - 1]
        a = float(V[:, k] @ znew)
        alpha[k] = a
        znew -= a * Z[:, k]
        for _ in range(GS_PASSES):
            znew -= Z[:, : k + 1] @ (V[:, : k + 1].T @ znew)
        if gen:
            vnew = solve(znew)
            b = math.sqrt(max(float(vnew @ znew), 0.0))
        else:
            b = float(np.linalg.norm(znew))
            vnew = znew
        beta[k] = b
        last = k == msteps - 1 or b == 0.0
        if (k + 1) % BOUNDS_CHECK_EVERY == 0 or last:
            th, S = _tri_eig(alpha[: k + 1], beta[: k + 1], vectors=True)
            rmin = abs(b * S[-1, 0])
            rmax = abs(b * S[-1, -1])
            scale = max(abs(th[0]), abs(th[-1]))
            lmin, lmax = th[0] - rmin, th[-1] + rmax
            if (rmin <= tol * scale and rmax <= tol * scale) or last:
                break
        V[:, k + 1] = vnew / b
        if gen:
            Z[:, k + 1] = znew / b
    return lmin, lmax, k + 1


# --------------------------------------------------------------------------- filter
@dataclass
class Pol:
    deg: int
    mu: np.ndarray
    cc: float
    dd: float
    gam: float
    bar: float
    kind: str  # "interior" | "left" | "right"


def damping_coefs(m: int, kind: int = 1) -> np.ndarray:
    """Damping factors g_k (k = 0..m) times the 1/2 of the zeroth Chebyshev
    term.  kind 0 or 1: Jackson (KPM form, Weisse et al. RMP 78 (2006));
    kind 2: Lanczos sigma factors; kind 3: none."""
    k = np.arange(m + 1, dtype=np.float64)
    if kind in (0, 1):
        th = math.pi / (m + 2)
        g = ((m + 2 - k) * np.cos(k * th) + np.sin(k * th) / math.tan(th)) / (m + 2)
    elif kind == 2:
        th = math.pi / (m + 1)
        g = np.ones(m + 1)
        g[1:] = np.sin(k[1:] * th) / (k[1:] * th)
    else:
        g = np.ones(m + 1)
    g[0] *= 0.5
    return g


def _cheb_eval(mu: np.ndarray, t: float) -> float:
    th = math.acos(max(-1.0, min(1.0, t)))
    return float(np.sum(mu * np.cos(np.arange(len(mu)) * th)))


def _balance(g: np.ndarray, tha: float, thb: float) -> float:
    """theta_c in [thb, tha] with p(a) = p(b) for p = sum g_k cos(k thc) T_k."""
    k = np.arange(len(g), dtype=np.float64)
    w = g * (np.cos(k * tha) - np.cos(k * thb))

    def f(th):
        return float(np.sum(w * np.cos(k * th)))

    def fp(th):
        return float(-np.sum(w * k * np.sin(k * th)))

    lo, hi = thb, tha
    flo, fhi = f(lo), f(hi)
    if flo * fhi > 0:
        return 0.5 * (lo + hi)
    th = 0.5 * (lo + hi)
    for _ in range(200):
        ft = f(th)
        if ft == 0.0:
            break
        if (ft < 0) == (flo < 0):
            lo, flo = th, ft
        else:
            hi, fhi = th, ft
        d = fp(th)
        nt = th - ft / d if d != 0.0 else 0.5 * (lo + hi)
        if not (lo < nt < hi):
            nt = 0.5 * (lo + hi)
        if abs(nt - th) <= 1e-15 * max(1.0, abs(th)) or hi - lo <= 1e-15:
            th = nt
            break
        th = nt
    return th


def find_pol(xintv, thresh_int=THRE_INT, thresh_ext=THRE_EXT, min_deg=2, max_deg=10000, damping=1) -> Pol:
    """Chebyshev delta-function filter for [a, b] inside [lmin, lmax]
    (pEVSL_FINDPOL_F90 at src/mod_pevsl.f90:115).  The degree is the smallest
    m >= min_deg for which the filter, normalised to p(gamma) = 1, drops to the
    threshold at the interval ends; bar = min(p(a), p(b))."""
    a, b, lmin, lmax = map(float, xintv)
    cc = 0.5 * (lmax + lmin)
    dd = 0.5 * (lmax - lmin)
    aa = max((a - cc) / dd, -1.0)
    bb = min((b - cc) / dd, 1.0)
    tha, thb = math.acos(aa), math.acos(bb)
    if aa <= -1.0:
        kind, thresh = "left", thresh_ext
    elif bb >= 1.0:
        kind, thresh = "right", thresh_ext
    else:
        kind, thresh = "interior", thresh_int
    mu = None
    gam = -1.0 if kind == "left" else 1.0
    vals = (1.0, 1.0)
    m = min_deg
    for m in range(min_deg, max_deg + 1):
        g = damping_coefs(m, damping)
        if kind == "interior":
            gam = math.cos(_balance(g, tha, thb))
        thc = math.acos(gam)
        mu = g * np.cos(np.arange(m + 1) * thc)
        mu = mu / _cheb_eval(mu, gam)
        vals = (_cheb_eval(mu, aa), _cheb_eval(mu, bb))
        if kind == "interior" and max(vals) <= thresh:
            break
        if kind == "left" and vals[1] <= thresh:
            break
        if kind == "right" and vals[0] <= thresh:
            break
    bar = min(vals) if kind == "interior" else (vals[1] if kind == "left" else vals[0])
    return Pol(m, mu, cc, dd, gam, bar, kind)


# --------------------------------------------------------------------------- ChebLanNr
@dataclass
class LanResult:
    lam: np.ndarray
    Y: np.ndarray
    res: np.ndarray
    steps: int
    nritz_above_bar: int
    stats: dict = field(default_factory=dict)


def cheb_lan_nr(op: Operator, xintv, maxit: int, tol: float, pol: Pol, v0=None) -> LanResult:
    """Polynomial-filtered non-restart Lanczos with full reorthogonalisation
    (pEVSL_CHEBLANNR_F90 at src/mod_pevsl.f90:122), generalized form."""
    n = op.n
    maxit = min(maxit, n)
    aa, bb = float(xintv[0]), float(xintv[1])
    bar = pol.bar
    V = np.zeros((n, maxit + 1))
    Z = np.zeros((n, maxit + 1))
    z = start_vector(n) if v0 is None else v0.copy()
    v = op.bsolve(z)
    t = 1.0 / math.sqrt(float(v @ z))
    Z[:, 0] = z * t
    V[:, 0] = v * t
    dT = np.zeros(maxit)
    eT = np.zeros(maxit)
    beta = 0.0
    tr0 = 0.0
    k = 0
    kdim = 0
    t_filter = 0.0
    for k in range(maxit):
        t0 = time.perf_counter()
        znew = op.chebav(pol, Z[:, k])
        t_filter += time.perf_counter() - t0
        if k > 0:
            znew -= beta * Z[:, k - 1]
        alpha = float(V[:, k] @ znew)
        dT[k] = alpha
        znew -= alpha * Z[:, k]
        for _ in range(GS_PASSES):
            znew -= Z[:, : k + 1] @ (V[:, : k + 1].T @ znew)
        vnew = op.bsolve(znew)
        beta = math.sqrt(max(float(vnew @ znew), 0.0))
        if beta == 0.0:
            kdim = k + 1
            break
        V[:, k + 1] = vnew / beta
        Z[:, k + 1] = znew / beta
        eT[k] = beta
        kdim = k + 1
        if (k < LAN_NTEST or (k - LAN_NTEST) % LAN_CYCLE != 0) and k != maxit - 1:
            continue
        ev = _tri_eig(dT[:kdim], eT[:kdim])
        sel = ev[ev + np.finfo(float).eps >= bar]
        tr1 = float(sel.sum())
        if abs(tr1 - tr0) < 2e-12 or abs(tr1) + abs(tr0) < 1e-10:
            break
        tr0 = tr1
    ev, S = _tri_eig(dT[:kdim], eT[:kdim], vectors=True)
    keep = np.where(ev >= bar)[0]
    lam, Ys, res = [], [], []
    for i in keep:
        u = V[:, :kdim] @ S[:, i]
        w2 = op.bmv(u)
        tn = math.sqrt(float(u @ w2))
        if tn == 0.0:
            continue
        u = u / tn
        w2 = w2 / tn
        w = op.amv(u)
        th = float(w @ u)
        if th < aa - np.finfo(float).eps or th > bb + np.finfo(float).eps:
            continue
        r = float(np.linalg.norm(w - th * w2))
        if r < tol:
            lam.append(th)
            Ys.append(u)
            res.append(r)
    Y = np.array(Ys).T if Ys else np.zeros((n, 0))
    return LanResult(np.array(lam), Y, np.array(res), kdim, len(keep), {"t_filter": t_filter})


# --------------------------------------------------------------------------- drivers
def interval(lowfreq_mhz: float, upfreq_mhz: float, lmin: float, lmax: float):
    """XINTV of src/mod_pevsl.f90:93-103 (frequencies are default REAL)."""
    lo = float(np.float32(lowfreq_mhz))
    hi = float(np.float32(upfreq_mhz))
    x = [(2.0 * PI_REF * lo) ** 2 * 1.0e-6, (2.0 * PI_REF * hi) ** 2 * 1.0e-6, lmin, lmax]
    if x[0] < 1.0e-10:
        x[0] = lmin
    return x


def cheb_degrees(porder: int, ap_lmin: float | None = None, ap_lmax: float | None = None):
    """CHEBDEG for B and Ap (src/mod_matvec.f90:88-92,167-171)."""
    dB = 45 if porder == 2 else 25
    if ap_lmin is None:
        return dB, None
    dAp = max(min(int(ap_lmax / ap_lmin), 15) * 3, 100) if porder == 2 else 25
    return dB, dAp


def setup_operator(mats: dict, porder: int, bounds: dict | None = None) -> Operator:
    """setupmatvec: scaling, bounds of B_s (and Ap_s) and Chebyshev set-ups.
    ``bounds`` may give {'B': (lmin, lmax), 'Ap': (lmin, lmax)} to skip the
    Lanczos bound estimation."""
    op = Operator(mats)
    bounds = dict(bounds or {})
    if "B" not in bounds:
        lo, hi, _ = lan_bounds(op.bmv, op.n, B_MLAN, B_TOL)
        bounds["B"] = (lo, hi)
    dB, _ = cheb_degrees(porder)
    op.set_cheb("B", bounds["B"][0], bounds["B"][1], dB)
    if op.fs:
        if "Ap" not in bounds:
            lo, hi, _ = lan_bounds(op.apmv, op.np, AP_MLAN, AP_TOL)
            bounds["Ap"] = (lo, hi)
        _, dAp = cheb_degrees(porder, *bounds["Ap"])
        op.set_cheb("Ap", bounds["Ap"][0], bounds["Ap"][1], dAp)
    op.bounds = bounds
    return op


@dataclass
class SolveResult:
    lam: np.ndarray          # ascending
    Y: np.ndarray            # scaled eigenvectors (columns), B_s-normalised
    err_ref: np.ndarray      # sqrt(sum r^2 / N) / |lam|  (src/mod_pevsl.f90:158)
    res2: np.ndarray         # ||A y - lam B y||_2 / |lam|
    xintv: list
    pol: Pol
    steps: int
    times: dict


def apply_pevsl(op: Operator, lowfreq: float, upfreq: float, ab_bounds=None, maxit: int = MAXIT,
                damping: int = 1) -> SolveResult:
    """pnm_apply_pevsl (src/mod_pevsl.f90:16-186) on a prepared operator."""
    t0 = time.perf_counter()
    if ab_bounds is None:
        lmin, lmax, _ = lan_bounds(op.amv, op.n, MLAN_AB, TOL_SOLVE, solve=op.bsolve)
    else:
        lmin, lmax = ab_bounds
    t1 = time.perf_counter()
    xintv = interval(lowfreq, upfreq, lmin, lmax)
    pol = find_pol(xintv, THRE_INT, THRE_EXT, damping=damping)
    r = cheb_lan_nr(op, xintv, maxit, TOL_SOLVE, pol)
    t2 = time.perf_counter()
    lam, Y = r.lam, r.Y
    err = np.zeros(len(lam))
    res2 = np.zeros(len(lam))
    for j in range(len(lam)):
        ay = op.amv(Y[:, j])
        by = op.bmv(Y[:, j])
        rr = ay - lam[j] * by
        err[j] = math.sqrt(float(rr @ rr) / op.n) / abs(lam[j])
        res2[j] = float(np.linalg.norm(rr)) / abs(lam[j])
    order = np.argsort(lam, kind="stable")
    t3 = time.perf_counter()
    return SolveResult(lam[order], Y[:, order], err[order], res2[order], xintv, pol, r.steps,
                       {"bounds": t1 - t0, "lanczos": t2 - t1, "residual": t3 - t2,
                        "filter": r.stats["t_filter"]})


def freq_mhz(lam):
    """Eigenvalue -> frequency in mHz and period in s (src/mod_pevsl.f90:177-183)."""
    lam = np.asarray(lam, dtype=np.float64)
    return np.sqrt(lam) / PI_REF / 2.0 * 1.0e3, 2.0 * PI_REF / np.sqrt(lam)


def dense_operator(op: Operator) -> tuple[np.ndarray, np.ndarray]:
    """Dense A_op (the reference's operator, Chebyshev Ap^-1 included) and B_s."""
    n = op.n
    A = np.empty((n, n))
    Bm = np.empty((n, n))
    e = np.zeros(n)
    for j in range(n):
        e[j] = 1.0
        A[:, j] = op.amv(e)
        Bm[:, j] = op.bmv(e)
        e[j] = 0.0
    return 0.5 * (A + A.T), 0.5 * (Bm + Bm.T)


def dense_reference(op: Operator, lo: float, hi: float):
    """All eigenvalues of (A_op, B_s) in [lo, hi] by a dense FP64 solve
    (scipy/LAPACK), independent of the filter and the Lanczos."""
    from scipy.linalg import eigh
    A, Bm = dense_operator(op)
    w, X = eigh(A, Bm)
    sel = (w >= lo) & (w <= hi)
    return w[sel], X[:, sel]
