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


def gravity_derivatives(R, mesh, k, g0, bface, purefluid=False):
    """(dT_rho, dT_kappa) of the reference-gravity terms (JOB = 2) of element
    k, in its element layout (3p solid, 4p fluid with the pressure last),
    differentiated by hand from oracle/gravity_ref.py (the gravity field is
    an input, held fixed; a uniform shift leaves the least-squares density
    gradient unchanged):
      solid: OPrho = (X R + R X)/2 -> dT_rho = detJ X (blocks of X with R = I);
      fluid: W_j = g^_j N^2 rho with N^2 rho = grad rho . g - |g|^2 rho^2 / kappa
             -> d(N^2 rho) = -2 |g|^2 rho / kappa (rho), |g|^2 rho^2 / kappa^2 (kappa);
             coupling -M diag(rho g_i / kappa) -> -M diag(g_i / kappa) (rho),
             M diag(rho g_i / kappa^2) (kappa);
             free surface -MF sJac / (|g.n| rho_f) -> MF sJac / (|g.n| rho_f^2) (rho);
             inner faces MF sJac (g.n) rho_f n_j^2 -> MF sJac (g.n) n_j^2 (rho).
    The fluid-solid interface term is added in `gradient` (it sits on the
    solid copies of the face nodes)."""
    from oracle import gravity_ref as GR
    p = R["pnp"]
    M = R["M"]
    rho, vp, vs = mesh["rho"][k], mesh["vp"][k], mesh["vs"][k]
    lam = rho * vp ** 2 - 2 * rho * vs ** 2
    X = mesh["xyz"][mesh["tets"][k]]
    invJ, detJ = fem_ref.geometry(R, mesh, k)
    D = [sum(invJ[i, j] * R["D"][j] for j in range(3)) for i in range(3)]
    if not mesh["fluid"][k]:
        ge = GR.element_gravity(X, g0[k], rho)
        blocks = GR.solid_gravity(M, D, ge, np.ones(p))
        dTr = np.zeros((3 * p, 3 * p))
        for i in range(3):
            for j in range(3):
                dTr[i * p:(i + 1) * p, j * p:(j + 1) * p] = detJ * blocks[i][j]
        return dTr, np.zeros_like(dTr)
    ge = GR.element_gravity(X, g0[k], rho, lam, purefluid)
    g, U = ge["g"], ge["unit"]
    g2 = np.sum(g ** 2, axis=1)
    live = (np.sqrt(g2) >= GR.EPS0) & (not purefluid)  # where N^2 is not forced to 0
    d_rho = np.where(live, -2.0 * g2 * rho / lam, 0.0)
    d_kap = np.where(live, g2 * rho ** 2 / lam ** 2, 0.0)
    out = []
    for d, cpl in ((d_rho, -g / lam[:, None]), (d_kap, rho[:, None] * g / lam[:, None] ** 2)):
        T = np.zeros((4 * p, 4 * p))
        W = U * d[:, None]
        for i in range(3):
            for j in range(3):
                T[i * p:(i + 1) * p, j * p:(j + 1) * p] = detJ * (
                    np.diag(U[:, i]) @ M @ np.diag(W[:, j]) + np.diag(W[:, i]) @ M @ np.diag(U[:, j])) / 2
            c = detJ * (M @ np.diag(cpl[:, i]))
            T[i * p:(i + 1) * p, 3 * p:] += c
            T[3 * p:, i * p:(i + 1) * p] += c.T
        out.append(T)
    dTr, dTk = out
    x4 = mesh["xyz"][mesh["tets"][k, R["vord"]]]
    nrm, sj = GR.face_normals(x4)
    rnum, tets = mesh["rnum"], mesh["tets"]
    for f in range(4):
        Fm = np.asarray(R["Fmask"][f])
        MF = R["MF"][f]
        gn = g[Fm] @ nrm[f]
        srho = rho[Fm].mean()
        if bface[k, f]:
            dTr[np.ix_(3 * p + Fm, 3 * p + Fm)] += MF * sj[f] / (np.abs(gn).mean() * srho ** 2)
        elif sum(1 for v in range(4) if v != f and rnum[tets[k, R["vord"][v]]] == 6) < 3:
            for j in range(3):
                dTr[np.ix_(j * p + Fm, j * p + Fm)] += MF * sj[f] * gn.mean() * nrm[f][j] ** 2
    return dTr, dTk


def _interface_gravity_rho(R, mesh, k, g0, X):
    """d/drho of the fluid-solid interface gravity term of fluid element k,
    -sJac (u.n)' MF (g.u) on the solid copies of the face nodes, per column
    of X (0 if element k has no interface face)."""
    from oracle import gravity_ref as GR
    tets, rnum, vstt = mesh["tets"], mesh["rnum"], mesh["vstt"]
    six = [v for v in range(4) if rnum[tets[k, R["vord"][v]]] == 6]
    if len(six) != 3:
        return np.zeros(X.shape[1])
    fc = [v for v in range(4) if v not in six][0]
    nrm, sj = GR.face_normals(mesh["xyz"][tets[k, R["vord"]]])
    Fm = np.asarray(R["Fmask"][fc])
    fn = tets[k][Fm]
    gk = g0[k][Fm] / 1.0e3
    U = np.stack([X[vstt[fn] + c] for c in range(3)], axis=0)  # 3 x nfp x ncols
    un = np.einsum("c,cfj->fj", nrm[fc], U)
    gu = np.einsum("fc,cfj->fj", gk, U)
    return -sj[fc] * np.einsum("fj,fg,gj->j", un, R["MF"][fc], gu)


def pressure(mats, X):
    """p = -Ap^-1 ET x for every column of X (dense solve; small models)."""
    import scipy.sparse.linalg as sla
    Ap = mats["Ap"].to_scipy().tocsc()
    ET = mats["ET"].to_scipy()
    lu = sla.splu(Ap)
    return -lu.solve(np.asarray(ET @ X))


def gradient(R, mesh, lam, X, P=None, elements=None, g0=None):
    """grad[j, e, :] = (d/drho, d/dkappa, d/dmu) of eigenvalue j for the
    listed elements (all if None); with g0 (ntet x pnp x 3, m/s^2) the
    operators are those of the reference gravity (JOB = 2)."""
    lam = np.atleast_1d(lam)
    X = X.reshape(X.shape[0], -1)
    els = range(mesh["tets"].shape[0]) if elements is None else elements
    out = np.zeros((X.shape[1], len(els), 3))
    bface = None
    if g0 is not None:
        from oracle import gravity_ref as GR
        bface = GR.boundary_faces(mesh["tets"][:, R["vord"]])
        purefluid = bool(np.all(mesh["fluid"]))
    for ie, k in enumerate(els):
        fl = bool(mesh["fluid"][k])
        u, pr = element_dofs(mesh, k, fl, R["pnp"])
        dTr, dTk, dTm, dM = element_derivatives(R, mesh, k, fl)
        if g0 is not None:
            gr, gk = gravity_derivatives(R, mesh, k, g0, bface, purefluid)
            dTr, dTk = dTr + gr, dTk + gk
            if fl:
                out[:, ie, 0] += _interface_gravity_rho(R, mesh, k, g0, X)
        for j in range(X.shape[1]):
            xe = X[u, j]
            z = np.concatenate([xe, P[pr, j]]) if fl else xe
            mass = xe @ (dM[:len(xe), :len(xe)] @ xe)
            out[j, ie, 0] += -lam[j] * mass + z @ dTr @ z
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
