"""Numpy restatement of the reference-gravity (JOB = 2) terms of the CG
mixed FEM and a sparse assembly of the fluid-solid operators -- TEST
INFRASTRUCTURE (checks the C++ assembly of normalmodes_gb300/csrc/model).

Follows the Fortran statements, with the products written as the matrices
they are (the reference symmetrises several of them, A + A^T over 2 where A
is already symmetric; those steps change only rounding):

* per-element gravity quantities (gk1 = g0 / 1e3, least-squares gradients of
  g and rho over the element's nodes, N^2, unit g):
  src/mod_cg_create_matrix.f90:192-265 (CGFSE3D_ISO), :1057-1083 (CGE3D_ISO)
* solid gravity block OPrho: :329-377, :1118-1160
* fluid N^2 block and the rho g / kappa part of the coupling: :492-608
* fluid face terms (free surface, inner faces): :643-705
* fluid-solid interface gravity term (SCM): :866-920, with the JOB = 1
  interface coupling of E / ET (:922-952)
* face normals and sJac: face_normal, src/mod_geometry.f90:2265-2304 and
  :1418-1428
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from . import fem_ref

EPS0 = 1.0e-15  # src/mod_cg_create_matrix.f90:30


def face_normals(x4):
    """Outward unit normals and sJac (area / 2, i.e. |cross| / 4) of the four
    faces of a tet; face i is opposite vertex i."""
    n = np.zeros((4, 3))
    sj = np.zeros(4)
    for i in range(4):
        v = [x4[j] for j in range(4) if j != i]
        c = np.cross(v[1] - v[0], v[2] - v[0])
        a = np.linalg.norm(c)
        c = c / a
        if np.dot(x4[i] - v[0], c) > 0:
            c = -c
        n[i] = c
        sj[i] = a / 4.0
    return n, sj


def boundary_faces(tets_vertices):
    """bface[k, f]: face f (opposite vertex f) of tet k has no neighbour."""
    nt = tets_vertices.shape[0]
    count = {}
    for k in range(nt):
        for f in range(4):
            key = tuple(sorted(int(tets_vertices[k, v]) for v in range(4) if v != f))
            count[key] = count.get(key, 0) + 1
    out = np.zeros((nt, 4), bool)
    for k in range(nt):
        for f in range(4):
            key = tuple(sorted(int(tets_vertices[k, v]) for v in range(4) if v != f))
            out[k, f] = count[key] == 1
    return out


def _lsq_gradient(X, f):
    """(dism' dism)^-1 dism' (f - mean f), dism = X - mean X: rows are d/dx_a."""
    d = X - X.mean(axis=0)
    return np.linalg.solve(d.T @ d, d.T @ (f - f.mean(axis=0)))


def element_gravity(X, g0, rho, lam=None, purefluid=False):
    """gk1 (pnp x 3, km/s^2), dg (3 x 3, dg[a, c] = d g_c / d x_a) and, given
    lam (kappa), N^2 and the unit vector along g at the nodes."""
    gk = g0 / 1.0e3
    out = {"g": gk, "dg": _lsq_gradient(X, gk)}
    if lam is not None:
        drho = _lsq_gradient(X, rho[:, None])[:, 0]
        ng = np.linalg.norm(gk, axis=1)
        n2 = (gk @ drho) / rho - ng ** 2 / lam * rho
        n2[ng < EPS0] = 0.0
        if purefluid:
            n2[:] = 0.0
        out["n2"] = n2
        out["unit"] = gk / np.maximum(ng, EPS0)[:, None]
    return out


def solid_gravity(M, D, ge, rho):
    """3 x 3 blocks of OPrho (before detJ)."""
    R = np.diag(rho)
    G = [np.diag(ge["g"][:, c]) for c in range(3)]
    out = [[None] * 3 for _ in range(3)]
    for i in range(3):
        for j in range(3):
            X = (D[i].T @ M @ G[j] + G[i] @ M @ D[j]) / 2 \
                - M * (ge["dg"][i, j] + ge["dg"][j, i]) / 2 \
                - (D[j].T @ G[i] @ M + M @ G[j] @ D[i]) / 2
            out[i][j] = (X @ R + R @ X) / 2
    return out


def _mesh_geometry(R, mesh, k):
    invJ, detJ = fem_ref.geometry(R, mesh, k)
    D = [sum(invJ[i, j] * R["D"][j] for j in range(3)) for i in range(3)]
    x4 = mesh["xyz"][mesh["tets"][k, R["vord"]]]
    n, sj = face_normals(x4)
    return D, detJ, n, sj


def element_matrices(R, mesh, k, fluid_solid, g0, bface, purefluid=False):
    """Element matrices with the reference gravity, as the assembly scatters
    them (JOB = 1 part from fem_ref plus the gravity terms; for a fluid
    element the face terms of :643-705 are included)."""
    T, Mm = fem_ref.element_matrices(R, mesh, k, fluid_solid)
    p = R["pnp"]
    M = R["M"]
    rho = mesh["rho"][k]
    vp, vs = mesh["vp"][k], mesh["vs"][k]
    mu = rho * vs ** 2
    lam = rho * vp ** 2 - 2 * mu
    X = mesh["xyz"][mesh["tets"][k]]
    D, detJ, n, sj = _mesh_geometry(R, mesh, k)
    if T.shape[0] == 3 * p:
        ge = element_gravity(X, g0[k], rho)
        blocks = solid_gravity(M, D, ge, rho)
        for i in range(3):
            for j in range(3):
                T[i * p:(i + 1) * p, j * p:(j + 1) * p] += detJ * blocks[i][j]
        return T, Mm
    ge = element_gravity(X, g0[k], rho, lam, purefluid)
    U = ge["unit"]
    W = U * (ge["n2"] * rho)[:, None]
    for i in range(3):
        for j in range(3):
            blk = (np.diag(U[:, i]) @ M @ np.diag(W[:, j]) + np.diag(W[:, i]) @ M @ np.diag(U[:, j])) / 2
            T[i * p:(i + 1) * p, j * p:(j + 1) * p] = detJ * blk
        cpl = detJ * (M @ np.diag(rho / lam * ge["g"][:, i]))
        T[i * p:(i + 1) * p, 3 * p:] -= cpl
        T[3 * p:, i * p:(i + 1) * p] -= cpl.T
    rnum = mesh["rnum"]
    tets = mesh["tets"]
    for f in range(4):
        Fm = np.asarray(R["Fmask"][f])
        MF = R["MF"][f]
        gn = ge["g"][Fm] @ n[f]
        srho = rho[Fm].mean()
        if bface[k, f]:
            sgn = np.abs(gn).mean()
            T[np.ix_(3 * p + Fm, 3 * p + Fm)] -= MF / sgn / srho * sj[f]
        else:
            cout = sum(1 for v in range(4) if v != f and rnum[tets[k, R["vord"][v]]] == 6)
            if cout < 3:
                for j in range(3):
                    T[np.ix_(j * p + Fm, j * p + Fm)] += MF * gn.mean() * srho * sj[f] * n[f][j] ** 2
    return T, Mm


def assemble(R, mesh, g0=None):
    """Sparse operators of a model: {"A", "B"} for a solid-only model,
    {"Ad", "B", "Ap", "E", "ET"} for a fluid(-solid) model, with the
    reference gravity when g0 (ntet x pnp x 3, m/s^2) is given.  The DOF
    numbering (vstt, rnum, pstt) is taken from the mesh dict."""
    tets, fluid = mesh["tets"], mesh["fluid"]
    vstt, rnum, pstt = mesh["vstt"], mesh["rnum"], mesh["pstt"]
    nt, p = tets.shape
    n = int(np.max(vstt + rnum))
    general = bool(np.any(fluid))
    purefluid = bool(np.all(fluid))
    vt = tets[:, R["vord"]]
    bface = boundary_faces(vt)
    trip = {k: ([], [], []) for k in ("A", "B", "Ap", "E", "ET")}

    def add(name, rows, cols, vals):
        t = trip[name]
        t[0].append(np.asarray(rows).ravel())
        t[1].append(np.asarray(cols).ravel())
        t[2].append(np.asarray(vals).ravel())

    for k in range(nt):
        nodes = tets[k]
        if g0 is None:
            T, Mm = fem_ref.element_matrices(R, mesh, k, general)
        else:
            T, Mm = element_matrices(R, mesh, k, general, g0, bface, purefluid)
        if T.shape[0] == 3 * p:
            dof = np.concatenate([vstt[nodes] + c for c in range(3)])  # solid copy
            add("A", dof[:, None].repeat(3 * p, 1), dof[None, :].repeat(3 * p, 0), T)
            add("B", dof[:, None].repeat(3 * p, 1), dof[None, :].repeat(3 * p, 0), Mm)
            continue
        udof = np.concatenate([vstt[nodes] + rnum[nodes] - 3 + c for c in range(3)])  # fluid copy
        pdof = pstt[nodes]
        Tuu, Tup, Tpu, Tpp = T[:3 * p, :3 * p], T[:3 * p, 3 * p:], T[3 * p:, :3 * p], T[3 * p:, 3 * p:]
        add("A", udof[:, None].repeat(3 * p, 1), udof[None, :].repeat(3 * p, 0), Tuu)
        add("B", udof[:, None].repeat(3 * p, 1), udof[None, :].repeat(3 * p, 0), Mm[:3 * p, :3 * p])
        add("E", udof[:, None].repeat(p, 1), pdof[None, :].repeat(3 * p, 0), Tup)
        add("ET", pdof[:, None].repeat(3 * p, 1), udof[None, :].repeat(p, 0), Tpu)
        add("Ap", pdof[:, None].repeat(p, 1), pdof[None, :].repeat(p, 0), Tpp)
        six = [v for v in range(4) if rnum[vt[k, v]] == 6]
        if len(six) != 3:
            continue
        fc = [v for v in range(4) if rnum[vt[k, v]] != 6][0]
        _, _, nrm, sj = _mesh_geometry(R, mesh, k)
        Fm = np.asarray(R["Fmask"][fc])
        MF = R["MF"][fc]
        fn = nodes[Fm]
        for c in range(3):
            # E(solid dof c of node a, pressure of node b) -= n_c sJac MF(a, b); ET is its transpose
            add("E", (vstt[fn] + c)[:, None].repeat(len(Fm), 1), pstt[fn][None, :].repeat(len(Fm), 0),
                -nrm[fc][c] * sj[fc] * MF)
            add("ET", pstt[fn][:, None].repeat(len(Fm), 1), (vstt[fn] + c)[None, :].repeat(len(Fm), 0),
                -nrm[fc][c] * sj[fc] * MF.T)
        if g0 is not None:
            gk = g0[k][Fm] / 1.0e3
            rhof = mesh["rho"][k][Fm].mean()
            for a_ in range(3):
                for b_ in range(3):
                    scm = rhof * sj[fc] * (nrm[fc][a_] * MF * gk[None, :, b_] + nrm[fc][b_] * gk[:, None, a_] * MF) / 2
                    add("A", (vstt[fn] + a_)[:, None].repeat(len(Fm), 1),
                        (vstt[fn] + b_)[None, :].repeat(len(Fm), 0), -scm)

    def build(name, shape):
        r, c, v = (np.concatenate(x) if x else np.zeros(0) for x in trip[name])
        return sp.csr_matrix((v, (r.astype(np.int64), c.astype(np.int64))), shape=shape)

    if not general:
        return {"A": build("A", (n, n)), "B": build("B", (n, n))}
    npr = int(np.max(pstt)) + 1
    return {"Ad": build("A", (n, n)), "B": build("B", (n, n)), "Ap": build("Ap", (npr, npr)),
            "E": build("E", (n, npr)), "ET": build("ET", (npr, n))}


def ball_gravity(mesh, G, a, b, R):
    """-G M(r) x / r^3 at every element node for rho = a + b r / R (r in km,
    rho in g/cm^3, g in m/s^2)."""
    X = mesh["xyz"][mesh["tets"]]
    r = np.linalg.norm(X, axis=2)
    gr = G * 4 * np.pi * 1e6 * (a * r / 3 + b * r ** 2 / (4 * R))
    with np.errstate(invalid="ignore", divide="ignore"):
        g = -gr[..., None] * X / r[..., None]
    g[r == 0] = 0.0
    return g
