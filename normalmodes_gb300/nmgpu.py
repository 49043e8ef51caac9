"""Python host binding of ``libnmgpu.so`` (ctypes over the C-ABI of
``include/nmgpu.h``).

:class:`Solver` mirrors the reference's solve driver: construction is
``setupmatvec`` (src/mod_matvec.f90:24-250), :meth:`Solver.amv`,
:meth:`Solver.bmv`, :meth:`Solver.bsolve` are the callbacks
``sparseAV``/``sparsefsAV``, ``sparseBV``, ``solveBV`` (src/mod_matvec.f90:445-520)
and :meth:`Solver.solve` is ``pnm_apply_pevsl`` (src/mod_pevsl.f90:16-222).

There is no CPU fallback: if the CUDA library cannot be loaded or no GPU is
usable, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

NM_PREC_FP64 = 0
NM_PREC_MIXED = 1

ERRORS = {0: "NM_OK", -1: "NM_ERR_ARG", -2: "NM_ERR_CUDA", -3: "NM_ERR_OOM", -4: "NM_ERR_NOCONV",
          -5: "NM_ERR_TIMEOUT", -6: "NM_ERR_NUMERIC"}

EXPORTS = [
    "nm_create", "nm_destroy", "nm_default_opts", "nm_default_solve_opts", "nm_amv", "nm_bmv", "nm_bsolve",
    "nm_amv_dev", "nm_bmv_dev", "nm_bsolve_dev", "nm_amv_block", "nm_bmv_block", "nm_bsolve_block", "nm_solve",
    "nm_result_free", "nm_get_info", "nm_get_stream", "nm_last_error", "nm_sync", "nm_time_op",
    "nm_bsolve_dev_noalloc", "nm_adjoint", "nm_solve_batched",
]


class NmCsr(C.Structure):
    _fields_ = [("nrows", C.c_int), ("ncols", C.c_int), ("rowptr", C.POINTER(C.c_int)),
                ("col", C.POINTER(C.c_int)), ("val", C.POINTER(C.c_double))]


class NmOpts(C.Structure):
    _fields_ = [("porder", C.c_int), ("device", C.c_int), ("b_cheb_deg", C.c_int), ("ap_cheb_deg", C.c_int),
                ("b_bounds", C.c_double * 2), ("ap_bounds", C.c_double * 2), ("precision", C.c_int),
                ("verbose", C.c_int), ("filter_form", C.c_int), ("orth", C.c_int), ("inner_tol", C.c_double),
                ("autotune", C.c_int)]


class NmSolveOpts(C.Structure):
    _fields_ = [("maxit", C.c_int), ("tol", C.c_double), ("thresh_int", C.c_double), ("thresh_ext", C.c_double),
                ("mlan_bounds", C.c_int), ("ab_bounds", C.c_double * 2), ("damping", C.c_int),
                ("want_vectors", C.c_int), ("unscale", C.c_int), ("use_graph", C.c_int), ("block", C.c_int),
                ("polish", C.c_int), ("resid_tol", C.c_double), ("refine_sweeps", C.c_int),
                ("refine_maxdeg", C.c_int), ("refine_band", C.c_double), ("refine_purge", C.c_int),
                ("progress", C.c_void_p), ("progress_data", C.c_void_p), ("refine_guard", C.c_double),
                ("refine_near", C.c_double), ("refine_growth", C.c_double)]


# void (*)(void* data, int phase, int done, int total)
NM_PROGRESS_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_int, C.c_int)
NM_PHASE_BOUNDS, NM_PHASE_LANCZOS, NM_PHASE_RITZ, NM_PHASE_REFINE, NM_PHASE_DONE = range(5)


class NmResult(C.Structure):
    _fields_ = [("nev", C.c_int), ("n", C.c_int), ("lam", C.POINTER(C.c_double)), ("vec", C.POINTER(C.c_double)),
                ("err_ref", C.POINTER(C.c_double)), ("res2", C.POINTER(C.c_double)), ("xintv", C.c_double * 4),
                ("pol_deg", C.c_int), ("pol_gam", C.c_double), ("pol_bar", C.c_double),
                ("lanczos_steps", C.c_int), ("nritz_above_bar", C.c_int),
                ("t_bounds", C.c_double), ("t_filter_design", C.c_double), ("t_lanczos", C.c_double),
                ("t_ritz", C.c_double), ("t_total", C.c_double),
                ("n_amv", C.c_longlong), ("n_bsolve", C.c_longlong), ("n_spmv", C.c_longlong),
                ("n_kernels", C.c_longlong), ("t_filter", C.c_double), ("t_orth", C.c_double),
                ("t_eig", C.c_double), ("refine_passes", C.c_int), ("refine_blocks", C.c_int),
                ("refine_maxdeg", C.c_int), ("refine_steps", C.c_longlong), ("res2_before_refine", C.c_double),
                ("refine_guards", C.c_int)]


class NmElemModel(C.Structure):
    _fields_ = [("ntet", C.c_int), ("pnp", C.c_int), ("nnode", C.c_int), ("fluid_solid", C.c_int),
                ("tets", C.c_void_p), ("xyz", C.c_void_p), ("fluid", C.c_void_p), ("vstt", C.c_void_p),
                ("rnum", C.c_void_p), ("pstt", C.c_void_p), ("vp", C.c_void_p), ("vs", C.c_void_p),
                ("rho", C.c_void_p), ("ref_mass", C.c_void_p), ("ref_drst", C.c_void_p), ("g0", C.c_void_p),
                ("ref_massf", C.c_void_p), ("ref_fmask", C.c_void_p)]


def _elem_model(mesh: dict, ref: dict, fluid_solid: bool, g0=None):
    """nm_elem_model over contiguous copies of the arrays; returns the struct
    and the copies (keep them alive for the call)."""
    nt, pnp = mesh["tets"].shape
    keep = {
        "tets": np.ascontiguousarray(mesh["tets"], dtype=np.int32),
        "xyz": np.ascontiguousarray(mesh["xyz"], dtype=np.float64),
        "fluid": np.ascontiguousarray(mesh["fluid"], dtype=np.uint8),
        "vstt": np.ascontiguousarray(mesh["vstt"], dtype=np.int32),
        "rnum": np.ascontiguousarray(mesh["rnum"], dtype=np.int32),
        "pstt": np.ascontiguousarray(mesh["pstt"], dtype=np.int32),
        "vp": np.ascontiguousarray(mesh["vp"], dtype=np.float64),
        "vs": np.ascontiguousarray(mesh["vs"], dtype=np.float64),
        "rho": np.ascontiguousarray(mesh["rho"], dtype=np.float64),
        "M": np.ascontiguousarray(ref["M"], dtype=np.float64),
        "D": np.ascontiguousarray(ref["Drst"], dtype=np.float64),
        "MF": np.ascontiguousarray(ref["MassF"], dtype=np.float64),
        "FM": np.ascontiguousarray(ref["Fmask"], dtype=np.int32),
    }
    gp = None
    if g0 is not None:
        keep["g0"] = np.ascontiguousarray(g0, dtype=np.float64)
        gp = keep["g0"].ctypes.data
    em = NmElemModel(nt, pnp, mesh["xyz"].shape[0], int(fluid_solid),
                     *[keep[q].ctypes.data for q in ("tets", "xyz", "fluid", "vstt", "rnum", "pstt", "vp", "vs",
                                                     "rho", "M", "D")],
                     gp, keep["MF"].ctypes.data, keep["FM"].ctypes.data)
    return em, keep


def assemble(model) -> tuple:
    """nm_assemble: the JOB = 1 operators of `model` (normalmodes_gb300.model.Model)
    assembled element by element on the GPU into the model's own CSR
    structures.  Returns ({name: values}, kernel seconds)."""
    mats = model.operators()
    fs = "Ad" in mats
    em, keep = _elem_model(model.mesh(), model.reference(), fs)
    names = ["Ad", "B", "Ap", "E", "ET"] if fs else ["A", "B"]
    vals, fills = {}, {}
    for nm in names:
        m = mats[nm]
        rp = np.ascontiguousarray(m.rowptr, dtype=np.int32)
        ci = np.ascontiguousarray(m.col, dtype=np.int32)
        vals[nm] = np.zeros(len(ci))
        keep[nm + "_rp"], keep[nm + "_ci"] = rp, ci
        fills[nm] = NmCsrFill(m.shape[0], rp.ctypes.data_as(C.POINTER(C.c_int)), ci.ctypes.data_as(C.POINTER(C.c_int)),
                              _dp(vals[nm]))
    ref = lambda k: C.byref(fills[k]) if k in fills else None
    sec = C.c_double()
    rc = lib().nm_assemble(C.byref(em), ref("Ad" if fs else "A"), ref("B"), ref("Ap"), ref("E"), ref("ET"),
                           C.byref(sec))
    if rc != 0:
        raise NmError(rc, "nm_assemble failed")
    return vals, sec.value


def adjoint_gravity(mesh: dict, ref: dict, g0, X, P=None, fluid_solid: bool = False) -> np.ndarray:
    """nm_adjoint_gravity (host code, no GPU): the reference-gravity terms of
    the per-pair sensitivities, (k, ntet, 3)."""
    X = np.asfortranarray(X, dtype=np.float64)
    if X.ndim == 1:
        X = X[:, None]
    k = X.shape[1]
    em, keep = _elem_model(mesh, ref, fluid_solid, g0)
    grad = np.zeros((k, mesh["tets"].shape[0], 3))
    Pp, ldp = None, 0
    if P is not None:
        P = np.asfortranarray(P, dtype=np.float64).reshape(-1, k)
        Pp, ldp = _dp(P), P.shape[0]
    rc = lib().nm_adjoint_gravity(C.byref(em), k, _dp(X), X.shape[0], Pp, ldp, _dp(grad))
    if rc != 0:
        raise NmError(rc, "nm_adjoint_gravity failed")
    return grad


class NmCsrFill(C.Structure):
    _fields_ = [("nrows", C.c_int), ("rowptr", C.POINTER(C.c_int)), ("col", C.POINTER(C.c_int)),
                ("val", C.POINTER(C.c_double))]


class NmSlice(C.Structure):
    _fields_ = [("f_lo_mhz", C.c_double), ("f_hi_mhz", C.c_double)]


class NmKpmOpts(C.Structure):
    _fields_ = [("degree", C.c_int), ("nvec", C.c_int), ("seed", C.c_ulonglong), ("ab_bounds", C.c_double * 2)]


# int (*)(void* data, const double* X, double* Y, int ncols, int ld)
NM_BLOCK_OP = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int, C.c_int)

NM_ADJ_PAIR = 0
NM_ADJ_MULTIPLET = 1


class NmInfo(C.Structure):
    _fields_ = [("n", C.c_int), ("np", C.c_int), ("fs", C.c_int), ("porder", C.c_int), ("precision", C.c_int),
                ("nnz_a", C.c_longlong), ("nnz_b", C.c_longlong), ("nnz_ap", C.c_longlong),
                ("nnz_e", C.c_longlong), ("nnz_et", C.c_longlong), ("b_bounds", C.c_double * 2),
                ("ap_bounds", C.c_double * 2), ("b_cheb_deg", C.c_int), ("ap_cheb_deg", C.c_int),
                ("t_setup", C.c_double), ("h2d_bytes", C.c_longlong), ("device_bytes", C.c_size_t),
                ("mass_vec", C.c_int), ("mass_threads", C.c_int), ("ap_vec", C.c_int), ("ap_threads", C.c_int),
                ("mass_sweep", C.c_int), ("ap_sweep", C.c_int), ("aop_threads", C.c_int), ("aop_sweep", C.c_int)]


_lib = None


def lib_path() -> str:
    return os.path.join(_build.LIBDIR, "libnmgpu.so")


def lib() -> C.CDLL:
    """Load libnmgpu.so (building it if this is a fresh tree)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            path = _build.build_gpu()
        L = C.CDLL(path)
        vp, dp = C.c_void_p, C.POINTER(C.c_double)
        L.nm_create.argtypes = [C.POINTER(vp)] + [C.POINTER(NmCsr)] * 5 + [C.POINTER(NmOpts)]
        L.nm_destroy.argtypes = [vp]
        L.nm_default_opts.argtypes = [C.POINTER(NmOpts)]
        L.nm_default_solve_opts.argtypes = [C.POINTER(NmSolveOpts)]
        for f in ("nm_amv", "nm_bmv", "nm_bsolve", "nm_amv_dev", "nm_bmv_dev", "nm_bsolve_dev",
                  "nm_bsolve_dev_noalloc"):
            getattr(L, f).argtypes = [vp, C.c_void_p, C.c_void_p]
        for f in ("nm_amv_block", "nm_bmv_block", "nm_bsolve_block"):
            getattr(L, f).argtypes = [vp, dp, dp, C.c_int, C.c_int]
        L.nm_solve.argtypes = [vp, C.c_double, C.c_double, C.POINTER(NmSolveOpts), C.POINTER(NmResult)]
        L.nm_result_free.argtypes = [C.POINTER(NmResult)]
        L.nm_get_info.argtypes = [vp, C.POINTER(NmInfo)]
        L.nm_get_stream.argtypes = [vp]
        L.nm_get_stream.restype = C.c_void_p
        L.nm_last_error.argtypes = [vp]
        L.nm_last_error.restype = C.c_char_p
        L.nm_sync.argtypes = [vp]
        L.nm_time_op.argtypes = [vp, C.c_int, C.c_int, dp, dp, C.POINTER(C.c_int)]
        L.nm_test_barrier_timeout.argtypes = [vp, C.c_longlong]
        L.nm_test_cheb_degree.argtypes = [C.c_double, C.c_double, C.c_int, C.c_double]
        L.nm_test_cheb_degree.restype = C.c_int
        L.nm_test_filter_at_zero.argtypes = [dp, C.c_double, C.c_double, C.c_int]
        L.nm_test_filter_at_zero.restype = C.c_double
        L.nm_test_polish_plan.argtypes = [dp, C.c_int, C.POINTER(C.c_int), dp]
        L.nm_test_refine_band.argtypes = [dp, dp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, dp]
        L.nm_test_ritz_first.argtypes = [dp, C.c_int, C.c_double, C.c_double, C.c_int]
        L.nm_test_ritz_first.restype = C.c_int
        L.nm_test_window_range.argtypes = [dp, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_int)]
        L.nm_test_filter_value.argtypes = [dp, C.c_double, C.c_double, C.c_int, C.c_double]
        L.nm_test_filter_value.restype = C.c_double
        L.nm_test_polish_block.argtypes = [dp, C.c_int, C.c_double, C.c_double, dp]
        L.nm_test_polish_block.restype = C.c_int
        L.nm_solve_batched.argtypes = [vp, C.POINTER(NmSlice), C.c_int, C.POINTER(NmSolveOpts), C.POINTER(NmResult)]
        L.nm_adjoint.argtypes = [vp, C.POINTER(NmElemModel), C.c_int, dp, dp, C.c_int, C.c_int, C.c_double, dp,
                                 C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.nm_adjoint_gravity.argtypes = [C.POINTER(NmElemModel), C.c_int, dp, C.c_int, dp, C.c_int, dp]
        L.nm_test_find_pol.argtypes = [dp, C.c_double, C.c_double, C.c_int, dp, C.c_int, dp]
        L.nm_test_tridiag.argtypes = [dp, dp, C.c_int, C.c_double, C.c_double, dp, dp, C.c_int]
        L.nm_test_sell.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), dp,
                                   C.POINTER(C.c_int), C.POINTER(C.c_longlong)]
        L.nm_test_sell.restype = C.c_longlong
        L.nm_test_start_vector.argtypes = [C.c_int, dp]
        L.nm_test_sell_arrays.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), dp, dp, dp,
                                          C.c_double, C.POINTER(C.c_int), dp]
        L.nm_default_kpm_opts.argtypes = [C.POINTER(NmKpmOpts)]
        L.nm_kpm_degree.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
        L.nm_kpm_moments.argtypes = [NM_BLOCK_OP, C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int,
                                     C.c_ulonglong, dp]
        L.nm_kpm_moments_ctx.argtypes = [vp, C.c_double, C.c_double, C.c_int, C.c_int, C.c_ulonglong, dp]
        L.nm_test_gather_shape.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int]
        L.nm_assemble.argtypes = [C.POINTER(NmElemModel)] + [C.POINTER(NmCsrFill)] * 5 + [dp]
        L.nm_test_gs_tc.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        L.nm_kpm_count.argtypes = [dp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, dp]
        L.nm_kpm_slices.argtypes = [dp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                    C.POINTER(NmSlice), dp]
        L.nm_slice_spectrum.argtypes = [vp, C.c_double, C.c_double, C.c_int, C.POINTER(NmKpmOpts),
                                        C.POINTER(NmSlice), dp]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class NmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


@dataclass
class SolveResult:
    lam: np.ndarray
    vec: np.ndarray | None
    err_ref: np.ndarray
    res2: np.ndarray
    xintv: tuple
    pol_deg: int
    pol_gam: float
    pol_bar: float
    lanczos_steps: int
    nritz_above_bar: int
    times: dict
    counts: dict


class Solver:
    """Operators of one model on one GPU and the filtered-Lanczos solve."""

    def __init__(self, mats: dict, porder: int, device: int = 0, precision: int = NM_PREC_FP64,
                 b_bounds=None, ap_bounds=None, b_cheb_deg: int = 0, ap_cheb_deg: int = 0, verbose: bool = False,
                 filter_form: int = 0, orth: int = 0, inner_tol: float = 0.0, autotune: int = 0):
        L = lib()
        self.fs = "Ad" in mats
        self._keep = []

        def csr(m):
            rp = np.ascontiguousarray(m.rowptr, dtype=np.int32)
            ci = np.ascontiguousarray(m.col, dtype=np.int32)
            v = np.ascontiguousarray(m.val, dtype=np.float64)
            self._keep += [rp, ci, v]
            return NmCsr(m.shape[0], m.shape[1], rp.ctypes.data_as(C.POINTER(C.c_int)),
                         ci.ctypes.data_as(C.POINTER(C.c_int)), _dp(v))

        A = csr(mats["Ad"] if self.fs else mats["A"])
        B = csr(mats["B"])
        Ap = csr(mats["Ap"]) if self.fs else None
        E = csr(mats["E"]) if self.fs else None
        ET = csr(mats["ET"]) if self.fs else None
        o = NmOpts()
        L.nm_default_opts(C.byref(o))
        o.porder = porder
        o.device = device
        o.precision = precision
        o.verbose = int(verbose)
        o.b_cheb_deg = b_cheb_deg
        o.ap_cheb_deg = ap_cheb_deg
        o.filter_form = filter_form
        o.orth = orth
        o.inner_tol = inner_tol
        o.autotune = autotune
        if b_bounds is not None:
            o.b_bounds[0], o.b_bounds[1] = b_bounds
        if ap_bounds is not None:
            o.ap_bounds[0], o.ap_bounds[1] = ap_bounds
        h = C.c_void_p()
        ref = lambda x: C.byref(x) if x is not None else None
        rc = L.nm_create(C.byref(h), ref(A), ref(B), ref(Ap), ref(E), ref(ET), C.byref(o))
        self._h = h
        if rc != 0:
            msg = L.nm_last_error(h).decode() if h else "nm_create failed"
            L.nm_destroy(h)
            self._h = C.c_void_p()
            raise NmError(rc, msg)
        self._keep = []  # the library copied the arrays
        self.n = mats["B"].shape[0]

    # -- callbacks (host vectors)
    def _call(self, fn, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        rc = getattr(lib(), fn)(self._h, x.ctypes.data, y.ctypes.data)
        self._check(rc)
        return y

    def _check(self, rc):
        if rc != 0:
            raise NmError(rc, lib().nm_last_error(self._h).decode())

    def amv(self, x):
        return self._call("nm_amv", x)

    def bmv(self, x):
        return self._call("nm_bmv", x)

    def bsolve(self, x):
        return self._call("nm_bsolve", x)

    def block(self, which: str, X: np.ndarray) -> np.ndarray:
        X = np.asfortranarray(X, dtype=np.float64)
        Y = np.empty_like(X)
        fn = {"amv": "nm_amv_block", "bmv": "nm_bmv_block", "bsolve": "nm_bsolve_block"}[which]
        self._check(getattr(lib(), fn)(self._h, _dp(X), _dp(Y), X.shape[1], X.shape[0]))
        return Y

    def info(self) -> NmInfo:
        i = NmInfo()
        self._check(lib().nm_get_info(self._h, C.byref(i)))
        return i

    @property
    def stream(self) -> int:
        return lib().nm_get_stream(self._h)

    def time_op(self, which: int, reps: int = 20):
        ms, by, la = C.c_double(), C.c_double(), C.c_int()
        self._check(lib().nm_time_op(self._h, which, reps, C.byref(ms), C.byref(by), C.byref(la)))
        return ms.value, by.value, la.value

    @staticmethod
    def _solve_opts(maxit=0, tol=0.0, ab_bounds=None, want_vectors=True, unscale=False, use_graph=True, damping=1,
                    mlan_bounds=0, block=0, polish=0, resid_tol=0.0, refine_sweeps=0, refine_maxdeg=0,
                    progress=None, refine_band=0.0, refine_purge=0, refine_guard=0.0,
                    refine_near=0.0, refine_growth=0.0) -> "NmSolveOpts":
        o = NmSolveOpts()
        lib().nm_default_solve_opts(C.byref(o))
        o.resid_tol = resid_tol
        o.refine_sweeps = refine_sweeps
        o.refine_maxdeg = refine_maxdeg
        o.refine_band = refine_band
        o.refine_purge = refine_purge
        o.refine_guard = refine_guard
        o.refine_near = refine_near
        o.refine_growth = refine_growth
        if progress is not None:  # an NM_PROGRESS_FN the caller keeps alive for the call
            o.progress = C.cast(progress, C.c_void_p)
        o.maxit = maxit
        o.tol = tol
        o.want_vectors = int(want_vectors)
        o.unscale = int(unscale)
        o.use_graph = int(use_graph)
        o.damping = damping
        o.mlan_bounds = mlan_bounds
        o.block = block
        o.polish = polish
        if ab_bounds is not None:
            o.ab_bounds[0], o.ab_bounds[1] = ab_bounds
        return o

    @staticmethod
    def _result(r: "NmResult", want_vectors: bool) -> SolveResult:
        nev, n = r.nev, r.n
        arr = lambda p: np.ctypeslib.as_array(p, shape=(max(nev, 1),))[:nev].copy() if nev else np.zeros(0)
        vec = None
        if want_vectors and nev:
            vec = np.ctypeslib.as_array(r.vec, shape=(nev * n,)).reshape(nev, n).T.copy()
        return SolveResult(arr(r.lam), vec, arr(r.err_ref), arr(r.res2), tuple(r.xintv), r.pol_deg, r.pol_gam,
                           r.pol_bar, r.lanczos_steps, r.nritz_above_bar,
                           {"bounds": r.t_bounds, "filter_design": r.t_filter_design, "lanczos": r.t_lanczos,
                            "ritz": r.t_ritz, "total": r.t_total, "filter": r.t_filter, "orth": r.t_orth,
                            "eig": r.t_eig},
                           {"amv": r.n_amv, "bsolve": r.n_bsolve, "spmv": r.n_spmv, "kernels": r.n_kernels,
                            "refine_passes": r.refine_passes, "refine_blocks": r.refine_blocks,
                            "refine_maxdeg": r.refine_maxdeg, "refine_steps": r.refine_steps,
                            "res2_before_refine": r.res2_before_refine, "refine_guards": r.refine_guards})

    def solve(self, lowfreq: float, upfreq: float, maxit: int = 0, tol: float = 0.0, ab_bounds=None,
              want_vectors: bool = True, unscale: bool = False, use_graph: bool = True, damping: int = 1,
              mlan_bounds: int = 0, allow_noconv: bool = False, block: int = 0, polish: int = 0,
              resid_tol: float = 0.0, refine_sweeps: int = 0, refine_maxdeg: int = 0,
              progress=None, refine_band: float = 0.0, refine_purge: int = 0, refine_guard: float = 0.0,
              refine_near: float = 0.0, refine_growth: float = 0.0) -> SolveResult:
        """nm_solve on [lowfreq, upfreq] mHz.  `progress`, if given, is a
        Python callable progress(phase, done, total) called at the solve's
        phase and block boundaries (NM_PHASE_*), stream drained."""
        L = lib()
        cb = None
        if progress is not None:
            cb = NM_PROGRESS_FN(lambda _d, ph, done, tot: progress(ph, done, tot))
        o = self._solve_opts(maxit, tol, ab_bounds, want_vectors, unscale, use_graph, damping, mlan_bounds, block,
                             polish, resid_tol, refine_sweeps, refine_maxdeg, cb, refine_band, refine_purge,
                             refine_guard, refine_near, refine_growth)
        r = NmResult()
        rc = L.nm_solve(self._h, lowfreq, upfreq, C.byref(o), C.byref(r))
        try:
            if rc != 0 and not (allow_noconv and rc == -4):
                self._check(rc)
            return self._result(r, want_vectors)
        finally:
            L.nm_result_free(C.byref(r))

    def solve_batched(self, slices, allow_noconv: bool = False, **kw) -> list:
        """nm_solve_batched over [(f_lo, f_hi), ...] mHz; one SolveResult per
        slice.  Keyword options as for solve()."""
        L = lib()
        want = kw.get("want_vectors", True)
        o = self._solve_opts(**kw)
        arr = (NmSlice * len(slices))(*[NmSlice(lo, hi) for lo, hi in slices])
        res = (NmResult * len(slices))()
        rc = L.nm_solve_batched(self._h, arr, len(slices), C.byref(o), res)
        try:
            if rc != 0 and not (allow_noconv and rc == -4):
                self._check(rc)
            return [self._result(res[i], want) for i in range(len(slices))]
        finally:
            for i in range(len(slices)):
                L.nm_result_free(C.byref(res[i]))

    def kpm_moments(self, lmin: float, lmax: float, degree: int, nvec: int = 16, seed: int = 0x4B504D):
        """nm_kpm_moments_ctx: the KPM moments mu[0..degree] of the
        lambda-weighted density of B^-1 A on the device block operators."""
        mu = np.zeros(degree + 1)
        self._check(lib().nm_kpm_moments_ctx(self._h, lmin, lmax, degree, nvec, seed, _dp(mu)))
        return mu

    def slice_spectrum(self, lowfreq: float, upfreq: float, nslices: int, degree: int = 0, nvec: int = 16,
                       seed: int = 0x4B504D, ab_bounds=None):
        """nm_slice_spectrum: nslices [(f_lo, f_hi), ...] mHz slices of the
        interval with equal estimated eigenvalue counts, and the estimates."""
        o = NmKpmOpts()
        lib().nm_default_kpm_opts(C.byref(o))
        o.degree, o.nvec, o.seed = degree, nvec, seed
        if ab_bounds is not None:
            o.ab_bounds[0], o.ab_bounds[1] = ab_bounds
        out = (NmSlice * nslices)()
        counts = np.zeros(nslices)
        self._check(lib().nm_slice_spectrum(self._h, lowfreq, upfreq, nslices, C.byref(o), out, _dp(counts)))
        return [(out[i].f_lo_mhz, out[i].f_hi_mhz) for i in range(nslices)], counts

    def adjoint(self, mesh: dict, ref: dict, lam, X, mode: int = NM_ADJ_PAIR, tol: float = 1e-6, g0=None):
        """Per-element sensitivities (rho, kappa, mu) of the eigenvalues `lam`
        with unscaled, B-normalised eigenvectors X (n x k), through
        nm_adjoint.  `mesh` is Model.mesh(), `ref` Model.reference(), `g0`
        Model.gravity() for operators assembled with the reference gravity.
        Returns (grad[k or ngroups, ntet, 3], group[k])."""
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        X = np.asfortranarray(X, dtype=np.float64)
        k = lam.size
        nt = mesh["tets"].shape[0]
        em, keep = _elem_model(mesh, ref, bool(self.info().fs), g0)
        grad = np.zeros((k, nt, 3))
        group = np.zeros(k, dtype=np.int32)
        ng = C.c_int()
        self._check(lib().nm_adjoint(self._h, C.byref(em), k, _dp(lam), _dp(X), X.shape[0], mode, tol, _dp(grad),
                                     group.ctypes.data_as(C.POINTER(C.c_int)), C.byref(ng)))
        return grad[: ng.value], group

    def close(self):
        if self._h:
            lib().nm_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# -- host-only helpers (no GPU needed)
def find_pol(xintv, thresh_int=0.8, thresh_ext=0.7, damping=1, max_deg=10000):
    mu = np.zeros(max_deg + 1)
    out = np.zeros(4)
    x = np.ascontiguousarray(xintv, dtype=np.float64)
    deg = lib().nm_test_find_pol(_dp(x), thresh_int, thresh_ext, damping, _dp(mu), max_deg, _dp(out))
    return deg, mu[: deg + 1].copy(), tuple(out)


def tridiag_eig(d, e, lo, hi, cap=None):
    d = np.ascontiguousarray(d, dtype=np.float64)
    e = np.ascontiguousarray(e, dtype=np.float64)
    k = len(d)
    cap = cap or k
    lam = np.zeros(cap)
    vec = np.zeros(cap * k)
    m = lib().nm_test_tridiag(_dp(d), _dp(e if len(e) else np.zeros(1)), k, lo, hi, _dp(lam), _dp(vec), cap)
    return lam[:m].copy(), vec[: m * k].reshape(m, k).T.copy()


def start_vector(n: int) -> np.ndarray:
    out = np.zeros(n)
    lib().nm_test_start_vector(n, _dp(out))
    return out


# ---------------------------------------------------------------- KPM slicing
def kpm_degree(lmin: float, lmax: float, lam_lo: float, lam_hi: float, nslices: int) -> int:
    return lib().nm_kpm_degree(lmin, lmax, lam_lo, lam_hi, nslices)


def kpm_moments(apply, n: int, lmin: float, lmax: float, degree: int, nvec: int = 16,
                seed: int = 0x4B504D) -> np.ndarray:
    """nm_kpm_moments through a Python block operator: apply(X) returns
    B^-1 A X for an n x ncols array."""
    err = []

    def cb(data, X, Y, ncols, ld):
        try:
            x = np.ctypeslib.as_array(X, shape=(ncols * ld,)).reshape(ncols, ld).T[:n]
            y = np.ctypeslib.as_array(Y, shape=(ncols * ld,)).reshape(ncols, ld).T
            y[:n] = apply(np.array(x))
            return 0
        except Exception as e:  # reported after the call
            err.append(e)
            return -1

    f = NM_BLOCK_OP(cb)
    mu = np.zeros(degree + 1)
    rc = lib().nm_kpm_moments(f, None, n, lmin, lmax, degree, nvec, seed, _dp(mu))
    if err:
        raise err[0]
    if rc != 0:
        raise NmError(rc, "nm_kpm_moments failed")
    return mu


def kpm_count(mu, n: int, lmin: float, lmax: float, lam_lo: float, lam_hi: float) -> float:
    mu = np.ascontiguousarray(mu, dtype=np.float64)
    out = np.zeros(1)
    rc = lib().nm_kpm_count(_dp(mu), len(mu) - 1, n, lmin, lmax, lam_lo, lam_hi, _dp(out))
    if rc != 0:
        raise NmError(rc, "nm_kpm_count: bad arguments")
    return float(out[0])


def kpm_slices(mu, n: int, lmin: float, lmax: float, lowfreq: float, upfreq: float, nslices: int):
    mu = np.ascontiguousarray(mu, dtype=np.float64)
    out = (NmSlice * nslices)()
    counts = np.zeros(nslices)
    rc = lib().nm_kpm_slices(_dp(mu), len(mu) - 1, n, lmin, lmax, lowfreq, upfreq, nslices, out, _dp(counts))
    if rc != 0:
        raise NmError(rc, "nm_kpm_slices: bad arguments")
    return [(out[i].f_lo_mhz, out[i].f_hi_mhz) for i in range(nslices)], counts

