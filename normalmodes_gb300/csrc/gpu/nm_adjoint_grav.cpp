// Reference-gravity (JOB = 2) terms of the eigenvalue sensitivities: added
// to what k_adjoint computes for the JOB = 1 element matrices when the
// element model carries the gravity field.  The gravity field is an input of
// the reference (src/mod_cg_models.f90:366-429) and is held fixed; a uniform
// shift of rho in an element leaves its least-squares density gradient
// unchanged.  Per element e and eigenvector (x, p), with g in km/s^2, M the
// reference mass, D_k the nodal derivative matrices, G_j = diag(g_j):
//
//  solid (OPrho = (X R + R X)/2, src/mod_cg_create_matrix.f90:329-377,
//  :1118-1160, so dT/drho = detJ X):
//    dlam/drho += detJ [ div' M gu - sum_ij s_ij u_i' M u_j - sum_k u_k' M w_k ]
//    div = sum_i D_i u_i, gu = sum_j g_j u_j, w_k = sum_m g_m (D_k u_m),
//    s_ij = (dg_ij + dg_ji) / 2 the symmetric least-squares gradient of g;
//  fluid (:492-608), s = sum_i (g_i / |g|) u_i, N^2 rho = grad rho . g - |g|^2 rho^2 / kappa:
//    N^2 block:  detJ s' M (d(N^2 rho) s),  d/drho = -2 |g|^2 rho / kappa,
//                d/dkappa = |g|^2 rho^2 / kappa^2 (0 where N^2 is forced to 0);
//    coupling:   2 detJ sum_i u_i' M (c_i p),  c_i = -g_i / kappa (rho),
//                rho g_i / kappa^2 (kappa);
//    faces (:643-705): outer  + sJac p_F' MF p_F / (mean|g.n| rho_F^2)   (rho)
//                      inner  + sJac mean(g.n) sum_j n_j^2 u_jF' MF u_jF (rho);
//  fluid-solid face of a fluid element (:866-920):
//    dlam/drho -= sJac (u.n)_F' MF (g.u)_F on the solid copies of the nodes.
// Host code (OpenMP over elements): the arrays are host arrays of the call.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <vector>

#include "nm_internal.h"

namespace {

constexpr double kEps0 = 1.0e-15;  // eps0, src/mod_cg_create_matrix.f90:30

bool inv3(const double A[3][3], double X[3][3]) {
  const double det = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) -
                     A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
                     A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
  if (!(det != 0.0) || !std::isfinite(det)) return false;
  X[0][0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]) / det;
  X[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) / det;
  X[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) / det;
  X[1][0] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) / det;
  X[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) / det;
  X[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) / det;
  X[2][0] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]) / det;
  X[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) / det;
  X[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) / det;
  return true;
}

// x' M y for a p x p row-major M
inline double qf(const double* M, const double* x, const double* y, int p) {
  double s = 0.0;
  for (int a = 0; a < p; ++a) {
    double t = 0.0;
    for (int b = 0; b < p; ++b) t += M[a * p + b] * y[b];
    s += x[a] * t;
  }
  return s;
}

// Outer-boundary faces (face f of tet e opposite local vertex f).
std::vector<unsigned char> boundary_faces(const nm_elem_model* em, const int vord[4]) {
  const int P = em->pnp, nt = em->ntet;
  std::vector<std::pair<std::array<int, 3>, int>> faces((size_t)nt * 4);
  for (int e = 0; e < nt; ++e)
    for (int f = 0; f < 4; ++f) {
      std::array<int, 3> a;
      int q = 0;
      for (int v = 0; v < 4; ++v)
        if (v != f) a[q++] = em->tets[(size_t)e * P + vord[v]];
      std::sort(a.begin(), a.end());
      faces[(size_t)e * 4 + f] = {a, e * 4 + f};
    }
  std::sort(faces.begin(), faces.end());
  std::vector<unsigned char> b((size_t)nt * 4, 0);
  for (size_t i = 0; i < faces.size();) {
    size_t j = i + 1;
    while (j < faces.size() && faces[j].first == faces[i].first) ++j;
    if (j - i == 1) b[faces[i].second] = 1;
    i = j;
  }
  return b;
}

}  // namespace

extern "C" int nm_adjoint_gravity(const nm_elem_model* em, int k, const double* X, int ldx, const double* P,
                                  int ldp, double* grad) {
  if (!em || !X || !grad || k < 0 || !em->g0 || !em->ref_massf || !em->ref_fmask || !em->tets || !em->xyz ||
      !em->fluid || !em->vstt || !em->rnum || !em->vp || !em->vs || !em->rho || !em->ref_mass || !em->ref_drst)
    return NM_ERR_ARG;
  const int p = em->pnp, nt = em->ntet;
  if (p != 4 && p != 10) return NM_ERR_ARG;
  const int nfp = p == 4 ? 3 : 6;
  const int vord[4] = {0, p == 4 ? 1 : 2, p == 4 ? 2 : 5, p == 4 ? 3 : 9};
  bool anyfluid = false, allfluid = nt > 0;
  for (int e = 0; e < nt; ++e) {
    anyfluid = anyfluid || em->fluid[e];
    allfluid = allfluid && em->fluid[e];
  }
  if (anyfluid && (!P || !em->pstt)) return NM_ERR_ARG;
  if (k == 0 || nt == 0) return NM_OK;
  const std::vector<unsigned char> bface = boundary_faces(em, vord);
  const double* M = em->ref_mass;
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : bad)
  for (int e = 0; e < nt; ++e) {
    const int* nodes = em->tets + (size_t)e * p;
    double xe[10][3], g[10][3], rho[10], kap[10];
    for (int a = 0; a < p; ++a) {
      for (int c = 0; c < 3; ++c) {
        xe[a][c] = em->xyz[3 * (size_t)nodes[a] + c];
        g[a][c] = em->g0[3 * ((size_t)e * p + a) + c] / 1.0e3;
      }
      const size_t q = (size_t)e * p + a;
      rho[a] = em->rho[q];
      kap[a] = em->rho[q] * em->vp[q] * em->vp[q] - 2.0 * em->rho[q] * em->vs[q] * em->vs[q];
    }
    // geometry (invJ = 2 B^-1, detJ = det B / 8) and face normals / sJac
    double Bm[3][3], invB[3][3];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) Bm[r][c] = xe[vord[r + 1]][c] - xe[vord[0]][c];
    if (!inv3(Bm, invB)) {
      ++bad;
      continue;
    }
    const double detJ = (Bm[0][0] * (Bm[1][1] * Bm[2][2] - Bm[1][2] * Bm[2][1]) -
                         Bm[0][1] * (Bm[1][0] * Bm[2][2] - Bm[1][2] * Bm[2][0]) +
                         Bm[0][2] * (Bm[1][0] * Bm[2][1] - Bm[1][1] * Bm[2][0])) / 8.0;
    double invJ[3][3];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) invJ[r][c] = 2.0 * invB[r][c];
    double fn[4][3], sJac[4];
    for (int f = 0; f < 4; ++f) {
      const double* w[3];
      int q = 0;
      for (int v = 0; v < 4; ++v)
        if (v != f) w[q++] = xe[vord[v]];
      double a1[3], a2[3], nn[3];
      for (int c = 0; c < 3; ++c) {
        a1[c] = w[1][c] - w[0][c];
        a2[c] = w[2][c] - w[0][c];
      }
      nn[0] = a1[1] * a2[2] - a1[2] * a2[1];
      nn[1] = a1[2] * a2[0] - a1[0] * a2[2];
      nn[2] = a1[0] * a2[1] - a1[1] * a2[0];
      const double len = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
      double dot = 0.0;
      for (int c = 0; c < 3; ++c) {
        nn[c] /= len;
        dot += (xe[vord[f]][c] - w[0][c]) * nn[c];
      }
      for (int c = 0; c < 3; ++c) fn[f][c] = dot > 0 ? -nn[c] : nn[c];
      sJac[f] = len / 4.0;
    }
    const bool fl = em->fluid[e] != 0;
    // least-squares gradient of g over the element's nodes (solid term)
    double sym[3][3] = {};
    if (!fl) {
      double xm[3] = {0, 0, 0}, gm[3] = {0, 0, 0};
      for (int a = 0; a < p; ++a)
        for (int c = 0; c < 3; ++c) {
          xm[c] += xe[a][c] / p;
          gm[c] += g[a][c] / p;
        }
      double N[3][3] = {}, Ni[3][3], Rg[3][3] = {}, dg[3][3];
      for (int a = 0; a < p; ++a)
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) {
            N[r][c] += (xe[a][r] - xm[r]) * (xe[a][c] - xm[c]);
            Rg[r][c] += (xe[a][r] - xm[r]) * (g[a][c] - gm[c]);
          }
      if (!inv3(N, Ni)) {
        ++bad;
        continue;
      }
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          dg[r][c] = 0.0;
          for (int t = 0; t < 3; ++t) dg[r][c] += Ni[r][t] * Rg[t][c];
        }
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) sym[r][c] = (dg[r][c] + dg[c][r]) / 2.0;
    }
    // nodal derivative matrices D_k = sum_j invJ[k][j] Dr_j
    std::vector<double> Dk(3 * (size_t)p * p);
    for (int kk = 0; kk < 3; ++kk)
      for (int q = 0; q < p * p; ++q)
        Dk[(size_t)kk * p * p + q] = invJ[kk][0] * em->ref_drst[q] + invJ[kk][1] * em->ref_drst[p * p + q] +
                                     invJ[kk][2] * em->ref_drst[2 * p * p + q];
    // fluid-solid interface face of a fluid element
    int fcid = -1;
    if (fl) {
      int six = 0;
      for (int v = 0; v < 4; ++v) {
        if (em->rnum[nodes[vord[v]]] == 6) ++six;
        else fcid = v;
      }
      if (six != 3) fcid = -1;
    }
    for (int j = 0; j < k; ++j) {
      const double* x = X + (size_t)j * ldx;
      double u[3][10];
      for (int a = 0; a < p; ++a) {
        const int base = em->vstt[nodes[a]] + (fl ? em->rnum[nodes[a]] - 3 : 0);
        for (int i = 0; i < 3; ++i) u[i][a] = x[base + i];
      }
      double* o = grad + ((size_t)j * nt + e) * 3;
      if (!fl) {
        double du[3][3][10];  // du[kk][i] = D_kk u_i
        for (int kk = 0; kk < 3; ++kk)
          for (int i = 0; i < 3; ++i)
            for (int a = 0; a < p; ++a) {
              double s = 0.0;
              for (int b = 0; b < p; ++b) s += Dk[(size_t)kk * p * p + a * p + b] * u[i][b];
              du[kk][i][a] = s;
            }
        double div[10], gu[10];
        for (int a = 0; a < p; ++a) {
          div[a] = du[0][0][a] + du[1][1][a] + du[2][2][a];
          gu[a] = g[a][0] * u[0][a] + g[a][1] * u[1][a] + g[a][2] * u[2][a];
        }
        double q = qf(M, div, gu, p);
        for (int i = 0; i < 3; ++i)
          for (int jj = 0; jj < 3; ++jj) q -= sym[i][jj] * qf(M, u[i], u[jj], p);
        for (int kk = 0; kk < 3; ++kk) {
          double w[10];
          for (int a = 0; a < p; ++a) w[a] = g[a][0] * du[kk][0][a] + g[a][1] * du[kk][1][a] + g[a][2] * du[kk][2][a];
          q -= qf(M, u[kk], w, p);
        }
        o[0] += detJ * q;
        continue;
      }
      const double* pj = P + (size_t)j * ldp;
      double pv[10], s[10], sdr[10], sdk[10];
      for (int a = 0; a < p; ++a) {
        pv[a] = pj[em->pstt[nodes[a]]];
        const double g2 = g[a][0] * g[a][0] + g[a][1] * g[a][1] + g[a][2] * g[a][2], ng = std::sqrt(g2);
        const double inv = 1.0 / std::max(ng, kEps0);
        s[a] = (g[a][0] * u[0][a] + g[a][1] * u[1][a] + g[a][2] * u[2][a]) * inv;
        const bool live = ng >= kEps0 && !allfluid;
        sdr[a] = live ? s[a] * (-2.0 * g2 * rho[a] / kap[a]) : 0.0;
        sdk[a] = live ? s[a] * (g2 * rho[a] * rho[a] / (kap[a] * kap[a])) : 0.0;
      }
      double dr = qf(M, s, sdr, p), dk = qf(M, s, sdk, p);
      for (int i = 0; i < 3; ++i) {
        double cr[10], ck[10];
        for (int a = 0; a < p; ++a) {
          cr[a] = -g[a][i] / kap[a] * pv[a];
          ck[a] = rho[a] * g[a][i] / (kap[a] * kap[a]) * pv[a];
        }
        dr += 2.0 * qf(M, u[i], cr, p);
        dk += 2.0 * qf(M, u[i], ck, p);
      }
      dr *= detJ;
      dk *= detJ;
      for (int f = 0; f < 4; ++f) {
        const int* Fm = em->ref_fmask + f * nfp;
        const double* MF = em->ref_massf + (size_t)f * nfp * nfp;
        double srho = 0.0, sgn = 0.0, sabs = 0.0;
        for (int a = 0; a < nfp; ++a) {
          const double gn = g[Fm[a]][0] * fn[f][0] + g[Fm[a]][1] * fn[f][1] + g[Fm[a]][2] * fn[f][2];
          srho += rho[Fm[a]] / nfp;
          sgn += gn / nfp;
          sabs += std::fabs(gn) / nfp;
        }
        double pf[6], uf[3][6];
        for (int a = 0; a < nfp; ++a) {
          pf[a] = pv[Fm[a]];
          for (int i = 0; i < 3; ++i) uf[i][a] = u[i][Fm[a]];
        }
        if (bface[(size_t)e * 4 + f]) {
          dr += sJac[f] * qf(MF, pf, pf, nfp) / (sabs * srho * srho);
        } else {
          int cout = 0;
          for (int v = 0; v < 4; ++v)
            if (v != f && em->rnum[nodes[vord[v]]] == 6) ++cout;
          if (cout < 3)
            for (int i = 0; i < 3; ++i) dr += sJac[f] * sgn * fn[f][i] * fn[f][i] * qf(MF, uf[i], uf[i], nfp);
        }
      }
      if (fcid >= 0) {
        const int* Fm = em->ref_fmask + fcid * nfp;
        const double* MF = em->ref_massf + (size_t)fcid * nfp * nfp;
        double un[6], gu[6];
        for (int a = 0; a < nfp; ++a) {
          const int nd = nodes[Fm[a]];
          double us[3];
          for (int c = 0; c < 3; ++c) us[c] = x[em->vstt[nd] + c];  // solid copy
          un[a] = us[0] * fn[fcid][0] + us[1] * fn[fcid][1] + us[2] * fn[fcid][2];
          gu[a] = us[0] * g[Fm[a]][0] + us[1] * g[Fm[a]][1] + us[2] * g[Fm[a]][2];
        }
        dr -= sJac[fcid] * qf(MF, un, gu, nfp);
      }
      o[0] += dr;
      o[1] += dk;
    }
  }
  return bad ? NM_ERR_NUMERIC : NM_OK;
}
