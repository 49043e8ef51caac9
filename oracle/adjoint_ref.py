"""FP64 CPU reference for the adjoint eigenvalue sensitivities --
TEST INFRASTRUCTURE (the checker of nm_adjoint).

For an eigenpair (lam, x) of the reference's pencil, x^T B x = 1, and its
pressure p = -Ap^-1 ET x (fluid-solid models), the sensitivity to a uniform
shift of the nodal values of m in element e is

    dlam/dm_e = z_e^T dT_e/dm z_e - lam x_e^T dM_e/dm x_e,   z_e = [x_e; p_e],

with the element matrices of src/mod_cg_create_matrix.f90 (CGE3D_ISO
:1043-1219, CGFSE3D_ISO :279-409 solid branch, :453-640 fluid, JOB = 1)
differentiated here independently of the CUDA code: the solid stiffness is
rebuilt by :func:`fem_ref.solid_stiffness` with unit coefficients (it is
linear in the nodal Lame lambda and mu; bulk / shear at fixed other modulus
via lambda = kappa - 2 mu / 3), the fluid pressure block
-detJ diag(l^-1/2) M diag(l^-1/2) is differentiated entrywise in l = kappa,
and the mass with unit density is M detJ per component.
"""
from __future__ import annotations

import numpy as np

from oracle import fem_ref


def element_dofs(mesh, k, fluid: bool, p: int):
    nodes = mesh["tets"][k]
    off = (mesh["rnum"][nodes] - 3) if fluid else np.zeros(len(nodes), dtype=int)
    u = np.concatenate([mesh["vstt"][nodes] + off + c for c in range(3)])
    pr = mesh["pstt"][nodes] if fluid else None
    return u, pr


def element_derivatives(R, mesh, k, fluid: bool):
    """(dT_rho, dT_kappa, dT_mu, dM_rho) for element k; stiffness matrices of
    size 3p (solid) or 4p (fluid, pressure last)."""
    p = R["pnp"]
    M = R["M"]
    invJ, detJ = fem_ref.geometry(R, mesh, k)
    D = [sum(invJ[i, j] * R["D"][j] for j in range(3)) for i in range(3)]
    one, zero = np.ones(p), np.zeros(p)
    if not fluid:
        dT_kappa = fem_ref.solid_stiffness(R, D, detJ, one, zero)
        dT_mu = fem_ref.solid_stiffness(R, D, detJ, -2.0 / 3.0 * one, one)
        dM = np.kron(np.eye(3), M) * detJ
        return np.zeros_like(dT_kappa), dT_kappa, dT_mu, dM
    rho, vp, vs = mesh["rho"][k], mesh["vp"][k], mesh["vs"][k]
    lam = rho * vp ** 2 - 2 * rho * vs ** 2
    a, b = lam ** -1.5, lam ** -0.5
    dflam = -0.5 * (np.outer(a, b) + np.outer(b, a)) * M
    dT_kappa = np.zeros((4 * p, 4 * p))
    dT_kappa[3 * p:, 3 * p:] = -detJ * dflam
    dM = np.zeros((4 * p, 4 * p))
    dM[:3 * p, :3 * p] = np.kron(np.eye(3), M) * detJ
    return np.zeros_like(dT_kappa), dT_kappa, np.zeros_like(dT_kappa), dM


def pressure(mats, X):
    """p = -Ap^-1 ET x for every column of X (dense solve; small models)."""
    import scipy.sparse.linalg as sla
    Ap = mats["Ap"].to_scipy().tocsc()
    ET = mats["ET"].to_scipy()
    lu = sla.splu(Ap)
    return -lu.solve(np.asarray(ET @ X))


def gradient(R, mesh, lam, X, P=None, elements=None):
    """grad[j, e, :] = (d/drho, d/dkappa, d/dmu) of eigenvalue j for the
    listed elements (all if None)."""
    lam = np.atleast_1d(lam)
    X = X.reshape(X.shape[0], -1)
    els = range(mesh["tets"].shape[0]) if elements is None else elements
    out = np.zeros((X.shape[1], len(els), 3))
    for ie, k in enumerate(els):
        fl = bool(mesh["fluid"][k])
        u, pr = element_dofs(mesh, k, fl, R["pnp"])
        dTr, dTk, dTm, dM = element_derivatives(R, mesh, k, fl)
        for j in range(X.shape[1]):
            xe = X[u, j]
            z = np.concatenate([xe, P[pr, j]]) if fl else xe
            mass = xe @ (dM[:len(xe), :len(xe)] @ xe)
            out[j, ie, 0] = -lam[j] * mass
            out[j, ie, 1] = z @ dTk @ z
            out[j, ie, 2] = z @ dTm @ z
    return out


def perturbed_material(mesh, k, which: int, h: float):
    """Nodal (vp, vs, rho) with parameter `which` (0 rho, 1 kappa, 2 mu) of
    element k shifted by h at every node, the other two held fixed."""
    vp, vs, rho = mesh["vp"].copy(), mesh["vs"].copy(), mesh["rho"].copy()
    r, a, b = rho[k], vp[k], vs[k]
    mu = r * b ** 2
    kap = r * a ** 2 - 4.0 / 3.0 * mu
    if which == 0:
        r = r + h
    elif which == 1:
        kap = kap + h
    else:
        mu = mu + h
    rho[k] = r
    vs[k] = np.sqrt(mu / r)
    vp[k] = np.sqrt((kap + 4.0 / 3.0 * mu) / r)
    return vp, vs, rho


def element_parameter(mesh, k, which: int) -> float:
    """Mean nodal value of rho / kappa / mu in element k."""
    r, a, b = mesh["rho"][k], mesh["vp"][k], mesh["vs"][k]
    mu = r * b ** 2
    return float(np.mean([r, r * a ** 2 - 4.0 / 3.0 * mu, mu][which]))
