"""Numpy restatement of the reference element and the element matrices of
the CG mixed FEM -- TEST INFRASTRUCTURE (checks the C++ assembly of
normalmodes_gb300/csrc/model).

It is written independently of the C++ code: the nodal basis comes from a
monomial Vandermonde inverse (as Build_reference does with its orthonormal
basis, src/mod_geometry.f90:2461-2487) and the integrals from collapsed
Gauss-Legendre quadrature, while the C++ side integrates barycentric
monomials exactly.  The element formulas follow the Fortran statements:

* solid:  src/mod_cg_create_matrix.f90:1043-1219 (CGE3D_ISO) and :279-409
  (solid branch of CGFSE3D_ISO, mean-density mass of :293)
* fluid:  src/mod_cg_create_matrix.f90:456-639 (JOB = 1)
* geometry: transfMat src/mod_geometry.f90:2216-2240, Jacobians :1401-1407
"""
from __future__ import annotations

import itertools

import numpy as np


def _nodes(p):
    out = []
    for i in range(1, p + 2):
        for j in range(1, p + 3 - i):
            for k in range(1, p + 4 - i - j):
                out.append((-1 + (k - 1) * 2.0 / p, -1 + (j - 1) * 2.0 / p, -1 + (i - 1) * 2.0 / p))
    return np.array(out)


def _monos(p, dim):
    return [e for e in itertools.product(range(p + 1), repeat=dim) if sum(e) <= p]


def _quad_tet(order=8):
    g, w = np.polynomial.legendre.leggauss(order)
    g = 0.5 * (g + 1)
    w = 0.5 * w
    pts, wts = [], []
    for a, wa in zip(g, w):
        for b, wb in zip(g, w):
            for c, wc in zip(g, w):
                x = a
                y = b * (1 - a)
                z = c * (1 - a) * (1 - b)
                pts.append((-1 + 2 * x, -1 + 2 * y, -1 + 2 * z))
                wts.append(wa * wb * wc * (1 - a) ** 2 * (1 - b) * 8.0)
    return np.array(pts), np.array(wts)


def _quad_tri(order=8):
    g, w = np.polynomial.legendre.leggauss(order)
    g = 0.5 * (g + 1)
    w = 0.5 * w
    pts, wts = [], []
    for a, wa in zip(g, w):
        for b, wb in zip(g, w):
            pts.append((-1 + 2 * a, -1 + 2 * b * (1 - a)))
            wts.append(wa * wb * (1 - a) * 4.0)
    return np.array(pts), np.array(wts)


def reference_element(p: int) -> dict:
    X = _nodes(p)
    mon = _monos(p, 3)
    V = np.array([[np.prod(np.power(x, e)) for e in mon] for x in X])
    Vinv = np.linalg.inv(V)
    qp, qw = _quad_tet()
    Pq = np.array([[np.prod(np.power(x, e)) for e in mon] for x in qp]) @ Vinv  # basis at quad points
    M = (Pq * qw[:, None]).T @ Pq

    def dmono(x, e, d):
        if e[d] == 0:
            return 0.0
        ee = list(e)
        ee[d] -= 1
        return e[d] * np.prod(np.power(x, ee))

    D = np.array([np.array([[dmono(x, e, d) for e in mon] for x in X]) @ Vinv for d in range(3)])
    tol = 1e-8
    fm = [[], [], [], []]
    for n, (r, s, t) in enumerate(X):
        if abs(1 + r + s + t) <= tol:
            fm[0].append(n)
        if abs(1 + r) <= tol:
            fm[1].append(n)
        if abs(1 + s) <= tol:
            fm[2].append(n)
        if abs(1 + t) <= tol:
            fm[3].append(n)
    coords = [(1, 2), (1, 2), (0, 2), (0, 1)]
    mon2 = _monos(p, 2)
    tp, tw = _quad_tri()
    MF = []
    for f in range(4):
        c = X[fm[f]][:, list(coords[f])]
        V2 = np.array([[np.prod(np.power(x, e)) for e in mon2] for x in c])
        B2 = np.array([[np.prod(np.power(x, e)) for e in mon2] for x in tp]) @ np.linalg.inv(V2)
        MF.append((B2 * tw[:, None]).T @ B2)
    vord = [0, 1, 2, 3] if p == 1 else [0, 2, 5, 9]
    return {"p": p, "pnp": len(X), "nodes": X, "M": M, "D": D, "Fmask": [np.array(x) for x in fm],
            "MF": MF, "vord": vord}


def geometry(R, mesh, k):
    x = mesh["xyz"][mesh["tets"][k, R["vord"]]]
    B = np.array([x[1] - x[0], x[2] - x[0], x[3] - x[0]])
    invJ = 2.0 * np.linalg.inv(B)
    detJ = np.linalg.det(B) / 8.0
    return invJ, detJ


def solid_stiffness(R, D, detJ, lam, mu):
    """Solid element stiffness for nodal Lame lambda / mu (the TM of
    CGE3D_ISO, src/mod_cg_create_matrix.f90:1043-1219)."""
    p = R["pnp"]
    M = R["M"]
    Ml = M @ np.diag(lam)
    Ml = (Ml + Ml.T) / 2
    Mm = M @ np.diag(mu)
    Mm = (Mm + Mm.T) / 2
    OP1 = [Ml @ D[i] for i in range(3)]
    OP2 = [Mm @ D[i] for i in range(3)]
    OPt = [D[i].T @ OP2[i] for i in range(3)]
    OPs = OPt[0] + OPt[1] + OPt[2]
    TM = np.zeros((3 * p, 3 * p))
    for i in range(3):
        for j in range(3):
            if i == j:
                O = OPs + OPt[i] + D[i].T @ OP1[i]
                O = (O + O.T) / 2
            else:
                tmp = D[i].T @ OP1[j] + D[j].T @ OP2[i]
                trs = D[j].T @ OP1[i] + D[i].T @ OP2[j]
                O = (trs.T + tmp) / 2
            TM[i * p:(i + 1) * p, j * p:(j + 1) * p] = O * detJ
    return TM


def element_matrices(R, mesh, k, fluid_solid: bool):
    p = R["pnp"]
    M = R["M"]
    rho = mesh["rho"][k]
    vp, vs = mesh["vp"][k], mesh["vs"][k]
    mu = rho * vs ** 2
    lam = rho * vp ** 2 - 2 * mu
    invJ, detJ = geometry(R, mesh, k)
    D = [sum(invJ[i, j] * R["D"][j] for j in range(3)) for i in range(3)]
    if (not fluid_solid) or mu.max() >= 1e-8:
        Ml = M @ np.diag(lam)
        Ml = (Ml + Ml.T) / 2
        Mm = M @ np.diag(mu)
        Mm = (Mm + Mm.T) / 2
        OP1 = [Ml @ D[i] for i in range(3)]
        OP2 = [Mm @ D[i] for i in range(3)]
        OPt = [D[i].T @ OP2[i] for i in range(3)]
        OPs = OPt[0] + OPt[1] + OPt[2]
        if fluid_solid:
            Mrho = M * rho.sum() / p
        else:
            Mrho = (np.diag(rho) @ M + M @ np.diag(rho)) / 2
        TM = np.zeros((3 * p, 3 * p))
        MM = np.zeros((3 * p, 3 * p))
        for i in range(3):
            for j in range(3):
                if i == j:
                    O = OPs + OPt[i] + D[i].T @ OP1[i]
                    O = (O + O.T) / 2
                    MM[i * p:(i + 1) * p, j * p:(j + 1) * p] = Mrho * detJ
                else:
                    tmp = D[i].T @ OP1[j] + D[j].T @ OP2[i]
                    trs = D[j].T @ OP1[i] + D[i].T @ OP2[j]
                    O = (trs.T + tmp) / 2
                TM[i * p:(i + 1) * p, j * p:(j + 1) * p] = O * detJ
        return TM, MM
    lamiv = 1.0 / np.sqrt(lam)
    flam = np.diag(lamiv) @ M @ np.diag(lamiv)
    Mrho = M * rho.sum() / p
    FT = np.zeros((4 * p, 4 * p))
    FM = np.zeros((4 * p, 4 * p))
    for i in range(3):
        FM[i * p:(i + 1) * p, i * p:(i + 1) * p] = Mrho * detJ
        Oij = (M @ D[i] + (D[i].T @ M).T) / 2
        FT[i * p:(i + 1) * p, 3 * p:] = Oij * detJ
        FT[3 * p:, i * p:(i + 1) * p] = Oij.T * detJ
    FT[3 * p:, 3 * p:] = -detJ * flam
    return FT, FM


def assemble_solid_dense(R, mesh):
    """Dense A, B of the solid-only path (3 DOFs per node, node-major)."""
    nn = mesh["xyz"].shape[0]
    p = R["pnp"]
    A = np.zeros((3 * nn, 3 * nn))
    B = np.zeros((3 * nn, 3 * nn))
    for k in range(mesh["tets"].shape[0]):
        TM, MM = element_matrices(R, mesh, k, fluid_solid=False)
        nodes = mesh["tets"][k]
        idx = np.concatenate([3 * nodes + c for c in range(3)])
        A[np.ix_(idx, idx)] += TM
        B[np.ix_(idx, idx)] += MM
    return A, B
