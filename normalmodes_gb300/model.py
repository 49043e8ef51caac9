"""Python bindings (ctypes) for ``libnmmodel.so``: synthetic planet models,
the reference's binary input format and the CG mixed-FEM assembly.

A :class:`Model` owns the native model; :meth:`Model.csr` returns numpy views
or copies of the assembled operators with the names the reference uses
(``A``, ``B``, ``Ad``, ``Ap``, ``E``, ``ET`` -- src/mod_cg_datatype.f90:61-66).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

_MATS = {"A": 0, "B": 1, "Ad": 2, "Ap": 3, "E": 4, "ET": 5}

# Gravitational constant (m^3 kg^-1 s^-2) with which the reference's demo
# gravity files are computed: |g| = 4/3 pi G rho r on the homogeneous CONST3k
# model holds with this value to 1e-9.
G_DEMO = 6.6723e-11


class BallOpts(C.Structure):
    _fields_ = [
        ("n_cells", C.c_int),
        ("porder", C.c_int),
        ("radius", C.c_double),
        ("r_icb", C.c_double),
        ("r_cmb", C.c_double),
        ("jitter", C.c_double),
        ("seed", C.c_ulonglong),
        ("fluid_core", C.c_int),
        ("homogeneous", C.c_int),
        ("vp0", C.c_double),
        ("vs0", C.c_double),
        ("rho0", C.c_double),
        ("lateral_pert", C.c_double),
        ("lateral_lmax", C.c_int),
    ]


class Info(C.Structure):
    _fields_ = [
        ("porder", C.c_int), ("pnp", C.c_int), ("nfp", C.c_int),
        ("nvert", C.c_int), ("ntet", C.c_int), ("nnode", C.c_int),
        ("n_fluid_tets", C.c_int), ("fsexist", C.c_int), ("purefluid", C.c_int),
        ("n", C.c_int), ("np", C.c_int), ("nnz", C.c_longlong * 6), ("assembled", C.c_int),
    ]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = os.path.join(_build.LIBDIR, "libnmmodel.so")
        if not os.path.exists(path):
            path = _build.build_model()
        L = C.CDLL(path)
        vp = C.c_void_p
        L.nmm_ball_default_opts.argtypes = [C.POINTER(BallOpts)]
        L.nmm_ball_create.argtypes = [C.POINTER(BallOpts), C.POINTER(vp)]
        L.nmm_load_files.argtypes = [C.c_char_p, C.c_int, C.POINTER(vp)]
        L.nmm_assemble.argtypes = [vp]
        L.nmm_info.argtypes = [vp, C.POINTER(Info)]
        L.nmm_get_csr.argtypes = [vp, C.c_int, C.POINTER(C.POINTER(C.c_int)), C.POINTER(C.POINTER(C.c_int)),
                                  C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(C.c_longlong)]
        L.nmm_mesh_arrays.argtypes = [vp] + [C.c_void_p] * 10
        L.nmm_element_matrices.argtypes = [vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                           C.POINTER(C.c_int)]
        L.nmm_reference.argtypes = [vp] + [C.c_void_p] * 5
        L.nmm_write_results.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_double, C.c_double,
                                        C.c_int, C.POINTER(C.c_double), C.c_longlong, C.c_char_p, C.c_int]
        L.nmm_set_material.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.nmm_set_gravity.argtypes = [vp, C.POINTER(C.c_double)]
        L.nmm_load_gravity.argtypes = [vp, C.c_char_p]
        L.nmm_ball_gravity.argtypes = [vp, C.c_double]
        L.nmm_get_gravity.argtypes = [vp, C.POINTER(C.POINTER(C.c_double))]
        L.nmm_write_model_files.argtypes = [vp, C.c_char_p]
        L.nmm_write_vector.argtypes = [C.c_char_p, C.POINTER(C.c_double), C.c_longlong]
        L.nmm_last_error.restype = C.c_char_p
        L.nmm_destroy.argtypes = [vp]
        _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != 0:
        raise RuntimeError(f"nmmodel error {rc}: {lib().nmm_last_error().decode()}")


@dataclass
class Csr:
    rowptr: np.ndarray
    col: np.ndarray
    val: np.ndarray
    shape: tuple

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.val, self.col, self.rowptr), shape=self.shape)


def write_vector(path: str, x) -> None:
    """One raw float64 vector file, as the reference writes eigenvectors."""
    a = np.ascontiguousarray(x, dtype=np.float64)
    _check(lib().nmm_write_vector(path.encode(), a.ctypes.data_as(C.POINTER(C.c_double)), a.size))


def default_opts(**kw) -> BallOpts:
    o = BallOpts()
    lib().nmm_ball_default_opts(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class Model:
    """A synthetic (or loaded) planet model with its assembled operators."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)

    @classmethod
    def ball(cls, n_cells: int = 12, porder: int = 1, assemble: bool = True, gravity: bool = False,
             **kw) -> "Model":
        """Layered ball; ``gravity=True`` adds the reference gravity of its
        radial density profile (JOB = 2)."""
        o = default_opts(n_cells=n_cells, porder=porder, **kw)
        h = C.c_void_p()
        _check(lib().nmm_ball_create(C.byref(o), C.byref(h)))
        m = cls(h.value)
        if gravity:
            m.ball_gravity(assemble=False)
        if assemble:
            m.assemble()
        return m

    @classmethod
    def load(cls, base_path: str, porder: int = 1, assemble: bool = True, gravity: bool = False) -> "Model":
        """Model in the reference's input files; ``gravity=True`` also reads
        ``<base>_pod_<p>_potential_acceleration_true.dat`` (JOB = 2)."""
        h = C.c_void_p()
        _check(lib().nmm_load_files(base_path.encode(), porder, C.byref(h)))
        m = cls(h.value)
        if gravity:
            _check(lib().nmm_load_gravity(m._h, base_path.encode()))
        if assemble:
            m.assemble()
        return m

    def set_gravity(self, g0, assemble: bool = True) -> None:
        """Reference gravity (ntet x pnp x 3, m/s^2) or None for JOB = 1."""
        if g0 is None:
            _check(lib().nmm_set_gravity(self._h, None))
        else:
            i = self.info()
            a = np.ascontiguousarray(g0, dtype=np.float64).ravel()
            if a.size != 3 * i.pnp * i.ntet:
                raise ValueError(f"gravity needs {3 * i.pnp * i.ntet} values, got {a.size}")
            _check(lib().nmm_set_gravity(self._h, a.ctypes.data_as(C.POINTER(C.c_double))))
        if assemble:
            self.assemble()

    def ball_gravity(self, G: float = G_DEMO, assemble: bool = True) -> None:
        _check(lib().nmm_ball_gravity(self._h, G))
        if assemble:
            self.assemble()

    def write_model_files(self, base_path: str) -> None:
        """The model in the reference's input files (nmm_write_model_files):
        Model.load(base_path, p, gravity=...) reads it back."""
        _check(lib().nmm_write_model_files(self._h, base_path.encode()))

    def gravity(self):
        """The reference gravity (ntet x pnp x 3, m/s^2), or None (JOB = 1)."""
        ptr = C.POINTER(C.c_double)()
        _check(lib().nmm_get_gravity(self._h, C.byref(ptr)))
        if not ptr:
            return None
        i = self.info()
        return np.ctypeslib.as_array(ptr, shape=(3 * i.pnp * i.ntet,)).copy().reshape(i.ntet, i.pnp, 3)

    def assemble(self) -> None:
        _check(lib().nmm_assemble(self._h))

    def info(self) -> Info:
        i = Info()
        _check(lib().nmm_info(self._h, C.byref(i)))
        return i

    @property
    def fluid_solid(self) -> bool:
        i = self.info()
        return bool(i.fsexist or i.purefluid)

    def csr(self, name: str, copy: bool = True) -> Csr:
        rp = C.POINTER(C.c_int)()
        cl = C.POINTER(C.c_int)()
        vl = C.POINTER(C.c_double)()
        nr, nc, nnz = C.c_int(), C.c_int(), C.c_longlong()
        _check(lib().nmm_get_csr(self._h, _MATS[name], C.byref(rp), C.byref(cl), C.byref(vl),
                                 C.byref(nr), C.byref(nc), C.byref(nnz)))
        r = np.ctypeslib.as_array(rp, shape=(nr.value + 1,))
        c = np.ctypeslib.as_array(cl, shape=(max(nnz.value, 1),))[: nnz.value]
        v = np.ctypeslib.as_array(vl, shape=(max(nnz.value, 1),))[: nnz.value]
        if copy:
            r, c, v = r.copy(), c.copy(), v.copy()
        return Csr(r, c, v, (nr.value, nc.value))

    def operators(self) -> dict:
        names = ["Ad", "B", "Ap", "E", "ET"] if self.fluid_solid else ["A", "B"]
        return {n: self.csr(n) for n in names}

    def mesh(self) -> dict:
        i = self.info()
        ptrs = [C.c_void_p() for _ in range(10)]
        _check(lib().nmm_mesh_arrays(self._h, *[C.byref(p) for p in ptrs]))

        def arr(p, ctype, n):
            return np.ctypeslib.as_array(C.cast(p, C.POINTER(ctype)), shape=(n,)).copy()

        nn, nt, pnp = i.nnode, i.ntet, i.pnp
        return {
            "xyz": arr(ptrs[0], C.c_double, 3 * nn).reshape(nn, 3),
            "tets": arr(ptrs[1], C.c_int, pnp * nt).reshape(nt, pnp),
            "fluid": arr(ptrs[2], C.c_ubyte, nt).astype(bool),
            "vstat": arr(ptrs[3], C.c_int, nn),
            "vstt": arr(ptrs[4], C.c_int, nn),
            "rnum": arr(ptrs[5], C.c_int, nn),
            "pstt": arr(ptrs[6], C.c_int, nn),
            "vp": arr(ptrs[7], C.c_double, pnp * nt).reshape(nt, pnp),
            "vs": arr(ptrs[8], C.c_double, pnp * nt).reshape(nt, pnp),
            "rho": arr(ptrs[9], C.c_double, pnp * nt).reshape(nt, pnp),
        }

    def set_material(self, vp, vs, rho, assemble: bool = True) -> None:
        """Replace the per-element nodal material (ntet x pnp arrays) and
        re-assemble; the solid / fluid split must not change."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (vp, vs, rho)]
        _check(lib().nmm_set_material(self._h, *[a.ctypes.data_as(C.POINTER(C.c_double)) for a in arrs]))
        if assemble:
            self.assemble()

    def write_results(self, outputdir: str, basename: str, lowfreq: float, upfreq: float, X,
                      job: int = 1, nproc: int = 1) -> str:
        """Write eigenvectors (n x k, unscaled) and the node lists in the
        reference's file layout; returns the eigenvector file prefix."""
        X = np.asfortranarray(X, dtype=np.float64)
        if X.ndim == 1:
            X = X[:, None]
        buf = C.create_string_buffer(4096)
        d = outputdir if outputdir.endswith("/") or not outputdir else outputdir + "/"
        _check(lib().nmm_write_results(self._h, d.encode(), basename.encode(), job, nproc, lowfreq, upfreq,
                                       X.shape[1], X.ctypes.data_as(C.POINTER(C.c_double)), X.shape[0], buf,
                                       len(buf)))
        return buf.value.decode()

    def element_matrices(self, k: int):
        i = self.info()
        d = 4 * i.pnp
        T = np.zeros(d * d)
        M = np.zeros(d * d)
        dim = C.c_int()
        _check(lib().nmm_element_matrices(self._h, k, T.ctypes.data_as(C.POINTER(C.c_double)),
                                          M.ctypes.data_as(C.POINTER(C.c_double)), C.byref(dim)))
        n = dim.value
        return T[: n * n].reshape(n, n), M[: n * n].reshape(n, n)

    def reference(self) -> dict:
        i = self.info()
        p, f = i.pnp, i.nfp
        ptrs = [C.c_void_p() for _ in range(5)]
        _check(lib().nmm_reference(self._h, *[C.byref(x) for x in ptrs]))

        def arr(ptr, ctype, n):
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(n,)).copy()

        return {
            "rst": arr(ptrs[0], C.c_double, 3 * p).reshape(p, 3),
            "M": arr(ptrs[1], C.c_double, p * p).reshape(p, p),
            "Drst": arr(ptrs[2], C.c_double, 3 * p * p).reshape(3, p, p),
            "MassF": arr(ptrs[3], C.c_double, 4 * f * f).reshape(4, f, f),
            "Fmask": arr(ptrs[4], C.c_int, 4 * f).reshape(4, f),
        }

    def close(self) -> None:
        if self._h:
            lib().nmm_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
