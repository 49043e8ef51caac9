// Synthetic layered-ball models, the reference element and the CG mixed-FEM
// assembly (JOB = 1, and JOB = 2 with the reference gravity) that produce the
// CSR operators of the eigensolve path.
//
// The formulas follow the reference's assembly statement by statement:
//   reference element   src/mod_geometry.f90:2307-2523 (nodes, MassM, Drst,
//                       Fmask, MassF, vord); src/mod_utility.f90:494-539
//                       (equispaced node order for pOrder <= 2)
//   element geometry    src/mod_geometry.f90:2216-2240 (transfMat),
//                       :1401-1407 (invJ = 2 B^-1, detJ = det B / 8),
//                       :2265-2304 + :1418-1428 (face normals, sJac / 4)
//   solid elements      src/mod_cg_create_matrix.f90:980-1266 (CGE3D_ISO) and
//                       :279-452 (solid branch of CGFSE3D_ISO)
//   fluid elements      src/mod_cg_create_matrix.f90:453-801
//   f-s interface faces src/mod_cg_create_matrix.f90:803-953
//   reference gravity   src/mod_cg_create_matrix.f90:192-265, 329-377,
//                       492-608, 643-705, 866-920, 1057-1160 (JOB = 2)
//   CSR structure       src/mod_cg_create_matrix.f90:1269-1455, 1458-2033
//   node status         src/mod_geometry.f90:284-312, 672-680
// The reference element is built from the exact Lagrange basis on the
// equispaced nodes instead of an orthonormal Vandermonde inverse; for
// pOrder <= 2 both give the same matrices up to rounding.
#include "../../../include/nmmodel.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_err;
int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

// ---------------------------------------------------------------- reference
// Polynomial in the four barycentric coordinates L1..L4 of the reference tet.
struct BaryTerm {
  double c;
  int e[4];
};
using BaryPoly = std::vector<BaryTerm>;

double fact(int k) {
  double f = 1.0;
  for (int i = 2; i <= k; ++i) f *= i;
  return f;
}

BaryPoly poly_mul(const BaryPoly& a, const BaryPoly& b) {
  BaryPoly r;
  for (const auto& x : a)
    for (const auto& y : b) {
      BaryTerm t;
      t.c = x.c * y.c;
      for (int i = 0; i < 4; ++i) t.e[i] = x.e[i] + y.e[i];
      r.push_back(t);
    }
  return r;
}

// Integral over the reference tet (volume 4/3) of prod L_i^e_i.
double integrate_tet(const BaryPoly& p) {
  const double vol = 4.0 / 3.0;
  double s = 0.0;
  for (const auto& t : p) {
    int tot = t.e[0] + t.e[1] + t.e[2] + t.e[3];
    s += t.c * 6.0 * vol * fact(t.e[0]) * fact(t.e[1]) * fact(t.e[2]) * fact(t.e[3]) /
         fact(tot + 3);
  }
  return s;
}

// Integral over face f (L_f = 0), measured on the projected reference
// triangle of area 2 (the measure MassF is built on).
double integrate_face(const BaryPoly& p, int f) {
  const double area = 2.0;
  double s = 0.0;
  for (const auto& t : p) {
    if (t.e[f] != 0) continue;
    int tot = 0;
    double num = 1.0;
    for (int i = 0; i < 4; ++i)
      if (i != f) {
        tot += t.e[i];
        num *= fact(t.e[i]);
      }
    s += t.c * 2.0 * area * num / fact(tot + 2);
  }
  return s;
}

// d/dL_k of a barycentric polynomial evaluated at barycentric point b.
double eval_poly(const BaryPoly& p, const double* b) {
  double s = 0.0;
  for (const auto& t : p) {
    double v = t.c;
    for (int i = 0; i < 4; ++i)
      for (int q = 0; q < t.e[i]; ++q) v *= b[i];
    s += v;
  }
  return s;
}
double eval_dpoly(const BaryPoly& p, int k, const double* b) {
  double s = 0.0;
  for (const auto& t : p) {
    if (t.e[k] == 0) continue;
    double v = t.c * t.e[k];
    for (int i = 0; i < 4; ++i) {
      int ex = t.e[i] - (i == k ? 1 : 0);
      for (int q = 0; q < ex; ++q) v *= b[i];
    }
    s += v;
  }
  return s;
}

struct RefElem {
  int p = 1, pnp = 4, nfp = 3;
  std::vector<double> rst;      // 3*pnp, node (r,s,t)
  std::vector<double> M;        // pnp*pnp row-major: MassM
  std::vector<double> D[3];     // Drst(:,:,d): D[d][i*pnp+j] = dphi_j/dr_d (node i)
  std::vector<int> fmask[4];    // nfp each, 0-based, increasing node index
  std::vector<double> MF[4];    // nfp*nfp face mass matrices
  int vord[4];                  // local positions of the 4 vertices
};

// dL_i/d(r,s,t) for L1 = -(1+r+s+t)/2, L2 = (1+r)/2, L3 = (1+s)/2, L4 = (1+t)/2.
const double kDL[4][3] = {{-0.5, -0.5, -0.5}, {0.5, 0.0, 0.0}, {0.0, 0.5, 0.0}, {0.0, 0.0, 0.5}};

RefElem build_reference(int porder) {
  RefElem R;
  R.p = porder;
  R.pnp = (porder + 1) * (porder + 2) * (porder + 3) / 6;
  R.nfp = (porder + 1) * (porder + 2) / 2;
  const int pnp = R.pnp;
  // Equispaced node order of src/mod_utility.f90:529-539: t outer, s, r inner.
  for (int i = 1; i <= porder + 1; ++i)
    for (int j = 1; j <= porder + 2 - i; ++j)
      for (int k = 1; k <= porder + 3 - i - j; ++k) {
        R.rst.push_back(-1.0 + (k - 1) * 2.0 / porder);
        R.rst.push_back(-1.0 + (j - 1) * 2.0 / porder);
        R.rst.push_back(-1.0 + (i - 1) * 2.0 / porder);
      }
  // Lagrange basis in barycentric form.
  std::vector<BaryPoly> phi(pnp);
  std::vector<std::array<double, 4>> bary(pnp);
  for (int n = 0; n < pnp; ++n) {
    double r = R.rst[3 * n], s = R.rst[3 * n + 1], t = R.rst[3 * n + 2];
    double b[4] = {-(1 + r + s + t) / 2, (1 + r) / 2, (1 + s) / 2, (1 + t) / 2};
    for (int i = 0; i < 4; ++i) bary[n][i] = b[i];
    if (porder == 1) {
      int v = -1;
      for (int i = 0; i < 4; ++i)
        if (std::fabs(b[i] - 1.0) < 1e-12) v = i;
      BaryTerm t1{1.0, {0, 0, 0, 0}};
      t1.e[v] = 1;
      phi[n] = {t1};
    } else {
      int ones = -1, h0 = -1, h1 = -1;
      for (int i = 0; i < 4; ++i) {
        if (std::fabs(b[i] - 1.0) < 1e-12) ones = i;
        if (std::fabs(b[i] - 0.5) < 1e-12) {
          if (h0 < 0) h0 = i; else h1 = i;
        }
      }
      if (ones >= 0) {  // vertex: L(2L-1)
        BaryTerm a{2.0, {0, 0, 0, 0}}, c{-1.0, {0, 0, 0, 0}};
        a.e[ones] = 2;
        c.e[ones] = 1;
        phi[n] = {a, c};
      } else {  // edge: 4 La Lb
        BaryTerm a{4.0, {0, 0, 0, 0}};
        a.e[h0] = 1;
        a.e[h1] = 1;
        phi[n] = {a};
      }
    }
  }
  R.M.assign(pnp * pnp, 0.0);
  for (int i = 0; i < pnp; ++i)
    for (int j = 0; j < pnp; ++j) R.M[i * pnp + j] = integrate_tet(poly_mul(phi[i], phi[j]));
  for (int d = 0; d < 3; ++d) {
    R.D[d].assign(pnp * pnp, 0.0);
    for (int i = 0; i < pnp; ++i)
      for (int j = 0; j < pnp; ++j) {
        double v = 0.0;
        for (int k = 0; k < 4; ++k) v += eval_dpoly(phi[j], k, bary[i].data()) * kDL[k][d];
        R.D[d][i * pnp + j] = v;
      }
  }
  // Fmask: face f holds the nodes with L_f = 0 (face f lacks vertex f),
  // src/mod_geometry.f90:2391-2405.
  for (int f = 0; f < 4; ++f) {
    for (int n = 0; n < pnp; ++n)
      if (std::fabs(bary[n][f]) < 1e-12) R.fmask[f].push_back(n);
    R.MF[f].assign(R.nfp * R.nfp, 0.0);
    for (int a = 0; a < R.nfp; ++a)
      for (int b = 0; b < R.nfp; ++b)
        R.MF[f][a * R.nfp + b] =
            integrate_face(poly_mul(phi[R.fmask[f][a]], phi[R.fmask[f][b]]), f);
  }
  if (porder == 1) {
    R.vord[0] = 0; R.vord[1] = 1; R.vord[2] = 2; R.vord[3] = 3;
  } else {
    R.vord[0] = 0; R.vord[1] = 2; R.vord[2] = 5; R.vord[3] = 9;
  }
  (void)eval_poly;
  return R;
}

// ---------------------------------------------------------------- small dense
using Mat = std::vector<double>;  // row-major n x n

inline Mat mm(const Mat& A, const Mat& B, int n) {
  Mat C(n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s += A[i * n + k] * B[k * n + j];
      C[i * n + j] = s;
    }
  return C;
}
inline Mat tr(const Mat& A, int n) {
  Mat C(n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) C[i * n + j] = A[j * n + i];
  return C;
}

// ---------------------------------------------------------------- geometry
struct ElemGeom {
  double invJ[3][3];
  double detJ;
  double n[4][3];
  double sJac[4];
};

bool elem_geometry(const double v[4][3], ElemGeom& g) {
  double B[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) B[r][c] = v[r + 1][c] - v[0][c];
  double det = B[0][0] * (B[1][1] * B[2][2] - B[1][2] * B[2][1]) -
               B[0][1] * (B[1][0] * B[2][2] - B[1][2] * B[2][0]) +
               B[0][2] * (B[1][0] * B[2][1] - B[1][1] * B[2][0]);
  if (det == 0.0) return false;
  double inv[3][3];
  inv[0][0] = (B[1][1] * B[2][2] - B[1][2] * B[2][1]) / det;
  inv[0][1] = (B[0][2] * B[2][1] - B[0][1] * B[2][2]) / det;
  inv[0][2] = (B[0][1] * B[1][2] - B[0][2] * B[1][1]) / det;
  inv[1][0] = (B[1][2] * B[2][0] - B[1][0] * B[2][2]) / det;
  inv[1][1] = (B[0][0] * B[2][2] - B[0][2] * B[2][0]) / det;
  inv[1][2] = (B[0][2] * B[1][0] - B[0][0] * B[1][2]) / det;
  inv[2][0] = (B[1][0] * B[2][1] - B[1][1] * B[2][0]) / det;
  inv[2][1] = (B[0][1] * B[2][0] - B[0][0] * B[2][1]) / det;
  inv[2][2] = (B[0][0] * B[1][1] - B[0][1] * B[1][0]) / det;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) g.invJ[r][c] = inv[r][c] * 2.0;
  g.detJ = det / 8.0;
  // face_normal: face i is spanned by the other three vertices in order.
  for (int i = 0; i < 4; ++i) {
    const double* vr = v[i];
    const double* w[3];
    int k = 0;
    for (int j = 0; j < 4; ++j)
      if (j != i) w[k++] = v[j];
    double a[3], b[3], nn[3];
    for (int c = 0; c < 3; ++c) {
      a[c] = w[1][c] - w[0][c];
      b[c] = w[2][c] - w[0][c];
    }
    nn[0] = a[1] * b[2] - a[2] * b[1];
    nn[1] = a[2] * b[0] - a[0] * b[2];
    nn[2] = a[0] * b[1] - a[1] * b[0];
    double sj = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
    for (int c = 0; c < 3; ++c) nn[c] /= sj;
    double dot = 0.0;
    for (int c = 0; c < 3; ++c) dot += (vr[c] - w[0][c]) * nn[c];
    if (dot > 0) for (int c = 0; c < 3; ++c) nn[c] = -nn[c];
    for (int c = 0; c < 3; ++c) g.n[i][c] = nn[c];
    g.sJac[i] = sj / 4.0;
  }
  return true;
}

// ---------------------------------------------------------------- RNG
inline uint64_t splitmix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
inline double u01(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed) {}
  double uniform() {
    s = splitmix(s);
    return u01(s);
  }
  double normal() {
    double a = uniform(), b = uniform();
    if (a < 1e-300) a = 1e-300;
    return std::sqrt(-2.0 * std::log(a)) * std::cos(2.0 * M_PI * b);
  }
};

// Real spherical-harmonic field of degrees 1..L with Gaussian coefficients.
struct ShField {
  int L = 0;
  std::vector<double> c;  // (l, m) with m in -l..l
  double scale = 1.0;
  void init(int lmax, uint64_t seed) {
    L = lmax;
    Rng rng(seed);
    for (int l = 1; l <= L; ++l)
      for (int m = -l; m <= l; ++m) c.push_back(rng.normal());
  }
  double eval(double x, double y, double z) const {
    double r = std::sqrt(x * x + y * y + z * z);
    if (r == 0.0) return 0.0;
    double ct = z / r, st = std::sqrt(std::max(0.0, 1.0 - ct * ct));
    double ph = std::atan2(y, x);
    // Schmidt-like normalised associated Legendre P_l^m(ct) by recurrence.
    std::vector<double> P((L + 1) * (L + 1), 0.0);
    auto idx = [&](int l, int m) { return l * (L + 1) + m; };
    P[idx(0, 0)] = 1.0;
    for (int m = 1; m <= L; ++m)
      P[idx(m, m)] = P[idx(m - 1, m - 1)] * st * std::sqrt((2.0 * m - 1.0) / (2.0 * m));
    for (int m = 0; m < L; ++m) P[idx(m + 1, m)] = ct * std::sqrt(2.0 * m + 1.0) * P[idx(m, m)];
    for (int m = 0; m <= L; ++m)
      for (int l = m + 2; l <= L; ++l) {
        double a = std::sqrt((double)(l * l - m * m));
        double b = std::sqrt((double)((l - 1) * (l - 1) - m * m));
        P[idx(l, m)] = ((2.0 * l - 1.0) * ct * P[idx(l - 1, m)] - b * P[idx(l - 2, m)]) / a;
      }
    double s = 0.0;
    int k = 0;
    for (int l = 1; l <= L; ++l)
      for (int m = -l; m <= l; ++m, ++k) {
        int am = std::abs(m);
        double ang = m >= 0 ? std::cos(am * ph) : std::sin(am * ph);
        s += c[k] * P[idx(l, am)] * ang;
      }
    return s * scale;
  }
};

}  // namespace

// ---------------------------------------------------------------- model
struct Csr {
  int nrows = 0, ncols = 0;
  std::vector<int> rowptr, col;
  std::vector<double> val;
  long long nnz() const { return (long long)col.size(); }
};

struct nmm_model {
  RefElem ref;
  int porder = 1, pnp = 4, nfp = 3;
  int nvert = 0, ntet = 0, nnode = 0;
  std::vector<double> xyz;           // 3*nnode
  std::vector<int> tet;              // pnp*ntet
  std::vector<double> vp, vs, rho;   // pnp*ntet
  std::vector<unsigned char> fluid;  // ntet
  std::vector<unsigned char> bface;  // 4*ntet: face on the outer boundary
  std::vector<int> vstat, rnum, pnum, vstt, pstt;
  std::vector<int> orig;  // per node: its id in the input numbering (vertices, then edge nodes)
  // Reference gravity (JOB = 2): acceleration at every element node,
  // 3*pnp*ntet in m/s^2 ([tet][node][xyz]); empty for JOB = 1.
  std::vector<double> g0;
  // Radial density profile of a generated ball, rho = rho_a + rho_b r / R.
  bool has_profile = false;
  double prof_a = 0.0, prof_b = 0.0, prof_R = 1.0;
  int n = 0, np = 0;
  bool fsexist = false, purefluid = false, assembled = false;
  int n_cout4 = 0;
  Csr A, B, Ad, Ap, E, ET;
};

namespace {

// P2: add edge nodes (sorted by endpoint pair), fill the reference local
// order 1=v1 2=e12 3=v2 4=e13 5=e23 6=v3 7=e14 8=e24 9=e34 10=v4.
void add_p2_nodes(nmm_model* m, const std::vector<int>& tv) {
  std::vector<std::pair<long long, int>> keys;
  keys.reserve((size_t)m->ntet * 6);
  static const int ep[6][2] = {{0, 1}, {0, 2}, {1, 2}, {0, 3}, {1, 3}, {2, 3}};
  for (int k = 0; k < m->ntet; ++k)
    for (int e = 0; e < 6; ++e) {
      int a = tv[4 * k + ep[e][0]], b = tv[4 * k + ep[e][1]];
      if (a > b) std::swap(a, b);
      keys.push_back({(long long)a * m->nvert + b, 0});
    }
  std::vector<long long> uk(keys.size());
  for (size_t i = 0; i < keys.size(); ++i) uk[i] = keys[i].first;
  std::sort(uk.begin(), uk.end());
  uk.erase(std::unique(uk.begin(), uk.end()), uk.end());
  int nedge = (int)uk.size();
  m->nnode = m->nvert + nedge;
  m->xyz.resize(3 * (size_t)m->nnode);
  for (int e = 0; e < nedge; ++e) {
    int a = (int)(uk[e] / m->nvert), b = (int)(uk[e] % m->nvert);
    for (int c = 0; c < 3; ++c)
      m->xyz[3 * (size_t)(m->nvert + e) + c] = 0.5 * (m->xyz[3 * (size_t)a + c] + m->xyz[3 * (size_t)b + c]);
  }
  m->tet.assign((size_t)m->ntet * 10, 0);
  static const int pos_v[4] = {0, 2, 5, 9};
  static const int pos_e[6] = {1, 3, 4, 6, 7, 8};
  for (int k = 0; k < m->ntet; ++k) {
    for (int v = 0; v < 4; ++v) m->tet[10 * (size_t)k + pos_v[v]] = tv[4 * k + v];
    for (int e = 0; e < 6; ++e) {
      int a = tv[4 * k + ep[e][0]], b = tv[4 * k + ep[e][1]];
      if (a > b) std::swap(a, b);
      long long key = (long long)a * m->nvert + b;
      int id = (int)(std::lower_bound(uk.begin(), uk.end(), key) - uk.begin());
      m->tet[10 * (size_t)k + pos_e[e]] = m->nvert + id;
    }
  }
}

void mark_boundary_faces(nmm_model* m, const std::vector<int>& tv) {
  // face f of tet k is opposite local vertex f
  std::vector<std::pair<std::array<int, 3>, int>> faces;
  faces.reserve((size_t)m->ntet * 4);
  for (int k = 0; k < m->ntet; ++k)
    for (int f = 0; f < 4; ++f) {
      std::array<int, 3> a;
      int q = 0;
      for (int v = 0; v < 4; ++v)
        if (v != f) a[q++] = tv[4 * k + v];
      std::sort(a.begin(), a.end());
      faces.push_back({a, 4 * k + f});
    }
  std::sort(faces.begin(), faces.end());
  m->bface.assign((size_t)m->ntet * 4, 0);
  for (size_t i = 0; i < faces.size();) {
    size_t j = i + 1;
    while (j < faces.size() && faces[j].first == faces[i].first) ++j;
    if (j - i == 1) m->bface[faces[i].second] = 1;
    i = j;
  }
}

// Node status, DOF counts and offsets (src/mod_geometry.f90:284-312,672-680;
// src/mod_cg_create_matrix.f90:1467-1499,1581-1613).
void classify_nodes(nmm_model* m, const std::vector<int>& tv) {
  std::vector<int> has_s(m->nvert, 0), has_f(m->nvert, 0);
  for (int k = 0; k < m->ntet; ++k)
    for (int v = 0; v < 4; ++v) (m->fluid[k] ? has_f : has_s)[tv[4 * k + v]] = 1;
  m->vstat.assign(m->nnode, 0);
  int maxstat = 0;
  for (int i = 0; i < m->nvert; ++i) {
    m->vstat[i] = (has_f[i] && !has_s[i]) ? 1 : (has_f[i] && has_s[i]) ? 2 : 0;
    maxstat = std::max(maxstat, m->vstat[i]);
  }
  if (m->porder == 2) {
    static const int ep[6][2] = {{0, 1}, {0, 2}, {1, 2}, {0, 3}, {1, 3}, {2, 3}};
    static const int pos_e[6] = {1, 3, 4, 6, 7, 8};
    for (int k = 0; k < m->ntet; ++k)
      for (int e = 0; e < 6; ++e) {
        int a = tv[4 * k + ep[e][0]], b = tv[4 * k + ep[e][1]];
        int mn = std::min(m->vstat[a], m->vstat[b]);
        m->vstat[m->tet[10 * (size_t)k + pos_e[e]]] = mn == 0 ? 3 : mn == 1 ? 4 : 5;
      }
  }
  m->fsexist = maxstat == 2;
  m->purefluid = maxstat == 1;
  m->rnum.assign(m->nnode, 3);
  m->pnum.assign(m->nnode, 0);
  const bool general = m->fsexist || m->purefluid;
  for (int i = 0; i < m->nnode; ++i) {
    if (general && (m->vstat[i] == 2 || m->vstat[i] == 5)) m->rnum[i] = 6;
    if (general && m->vstat[i] != 0 && m->vstat[i] != 3) m->pnum[i] = 1;
  }
  m->vstt.assign(m->nnode, 0);
  m->pstt.assign(m->nnode, -1);
  int acc = 0, pacc = 0;
  for (int i = 0; i < m->nnode; ++i) {
    m->vstt[i] = acc;
    acc += m->rnum[i];
    if (m->pnum[i]) m->pstt[i] = pacc++;
  }
  m->n = acc;
  m->np = pacc;
}

// Node status from the tetrahedra alone (works for any node numbering):
// vertices by their incident elements, P2 edge nodes by the statuses of the
// edge's two vertices (src/mod_geometry.f90:284-312, 672-680).
void classify_from_tets(nmm_model* m) {
  const int p = m->pnp;
  std::vector<char> has_s(m->nnode, 0), has_f(m->nnode, 0), isv(m->nnode, 0);
  for (int k = 0; k < m->ntet; ++k)
    for (int v = 0; v < 4; ++v) {
      const int node = m->tet[(size_t)p * k + m->ref.vord[v]];
      isv[node] = 1;
      (m->fluid[k] ? has_f : has_s)[node] = 1;
    }
  m->vstat.assign(m->nnode, 0);
  int maxstat = 0;
  for (int i = 0; i < m->nnode; ++i)
    if (isv[i]) {
      m->vstat[i] = (has_f[i] && !has_s[i]) ? 1 : (has_f[i] && has_s[i]) ? 2 : 0;
      maxstat = std::max(maxstat, m->vstat[i]);
    }
  if (m->porder == 2) {
    static const int ep[6][2] = {{0, 1}, {0, 2}, {1, 2}, {0, 3}, {1, 3}, {2, 3}};
    static const int pos_e[6] = {1, 3, 4, 6, 7, 8};
    for (int k = 0; k < m->ntet; ++k)
      for (int e = 0; e < 6; ++e) {
        const int a = m->tet[(size_t)p * k + m->ref.vord[ep[e][0]]];
        const int b = m->tet[(size_t)p * k + m->ref.vord[ep[e][1]]];
        const int mn = std::min(m->vstat[a], m->vstat[b]);
        m->vstat[m->tet[(size_t)p * k + pos_e[e]]] = mn == 0 ? 3 : mn == 1 ? 4 : 5;
      }
  }
  m->fsexist = maxstat == 2;
  m->purefluid = maxstat == 1;
  m->rnum.assign(m->nnode, 3);
  m->pnum.assign(m->nnode, 0);
  const bool general = m->fsexist || m->purefluid;
  for (int i = 0; i < m->nnode; ++i) {
    if (general && (m->vstat[i] == 2 || m->vstat[i] == 5)) m->rnum[i] = 6;
    if (general && m->vstat[i] != 0 && m->vstat[i] != 3) m->pnum[i] = 1;
  }
  m->vstt.assign(m->nnode, 0);
  m->pstt.assign(m->nnode, -1);
  int acc = 0, pacc = 0;
  for (int i = 0; i < m->nnode; ++i) {
    m->vstt[i] = acc;
    acc += m->rnum[i];
    if (m->pnum[i]) m->pstt[i] = pacc++;
  }
  m->n = acc;
  m->np = pacc;
}

// Renumber nodes along a Morton (Z-order) curve of their doubled grid
// coordinates, so that consecutive rows of the operators are close in space
// (the GPU kernels then find a row's neighbours in cache).
void renumber_morton(nmm_model* m, const std::vector<std::array<int, 3>>& gv) {
  const int p = m->pnp;
  std::vector<std::array<int, 3>> g2(m->nnode, {-1, -1, -1});
  for (int k = 0; k < m->ntet; ++k)
    for (int v = 0; v < 4; ++v) {
      const int node = m->tet[(size_t)p * k + m->ref.vord[v]];
      g2[node] = {2 * gv[node][0], 2 * gv[node][1], 2 * gv[node][2]};
    }
  if (m->porder == 2) {
    static const int ep[6][2] = {{0, 1}, {0, 2}, {1, 2}, {0, 3}, {1, 3}, {2, 3}};
    static const int pos_e[6] = {1, 3, 4, 6, 7, 8};
    for (int k = 0; k < m->ntet; ++k)
      for (int e = 0; e < 6; ++e) {
        const int a = m->tet[(size_t)p * k + m->ref.vord[ep[e][0]]];
        const int b = m->tet[(size_t)p * k + m->ref.vord[ep[e][1]]];
        const int node = m->tet[(size_t)p * k + pos_e[e]];
        for (int c = 0; c < 3; ++c) g2[node][c] = gv[a][c] + gv[b][c];
      }
  }
  auto spread = [](uint64_t x) {
    uint64_t r = 0;
    for (int b = 0; b < 21; ++b) r |= ((x >> b) & 1ull) << (3 * b);
    return r;
  };
  std::vector<std::pair<uint64_t, int>> key(m->nnode);
  for (int i = 0; i < m->nnode; ++i)
    key[i] = {spread((uint64_t)g2[i][0]) | (spread((uint64_t)g2[i][1]) << 1) | (spread((uint64_t)g2[i][2]) << 2), i};
  std::sort(key.begin(), key.end());
  std::vector<int> newid(m->nnode);
  for (int r = 0; r < m->nnode; ++r) newid[key[r].second] = r;
  std::vector<int> orig(m->nnode);
  for (int i = 0; i < m->nnode; ++i) orig[newid[i]] = m->orig[i];
  m->orig.swap(orig);
  std::vector<double> xyz(m->xyz.size());
  for (int i = 0; i < m->nnode; ++i)
    for (int c = 0; c < 3; ++c) xyz[3 * (size_t)newid[i] + c] = m->xyz[3 * (size_t)i + c];
  m->xyz.swap(xyz);
  for (auto& t : m->tet) t = newid[t];
}

void finish_mesh(nmm_model* m, const std::vector<int>& tv, const std::vector<std::array<int, 3>>* grid = nullptr) {
  if (m->porder == 2) {
    add_p2_nodes(m, tv);
  } else {
    m->nnode = m->nvert;
    m->tet = tv;
  }
  mark_boundary_faces(m, tv);
  m->orig.resize(m->nnode);
  for (int i = 0; i < m->nnode; ++i) m->orig[i] = i;
  if (grid) {
    std::vector<std::array<int, 3>> gv(m->nnode, {0, 0, 0});
    for (int i = 0; i < m->nvert; ++i) gv[i] = (*grid)[i];
    renumber_morton(m, gv);
  }
  classify_from_tets(m);
}

}  // namespace

extern "C" {

const char* nmm_last_error(void) { return g_err.c_str(); }

void nmm_ball_default_opts(nmm_ball_opts* o) {
  std::memset(o, 0, sizeof(*o));
  o->n_cells = 12;
  o->porder = 1;
  o->radius = 6371.0;
  o->r_icb = 1221.0;
  o->r_cmb = 3480.0;
  o->jitter = 0.1;
  o->seed = 20240501ull;
  o->fluid_core = 1;
  o->homogeneous = 0;
  o->vp0 = 10.0;
  o->vs0 = 5.7735;
  o->rho0 = 5.51;
  o->lateral_pert = 0.0;
  o->lateral_lmax = 8;
}

// Layered ball: the cube [-m, m]^3 (m = n/2) is cut into unit cells, each
// cell into 6 tetrahedra along the diagonal pointing away from the centre
// (mirrored Freudenthal/Kuhn subdivision, conforming across octants), and
// the cube shell |p|_inf = s is mapped to the sphere of radius R(s) with the
// equiangular cubed-sphere projection.  R is piecewise linear with the inner
// core boundary and the core-mantle boundary on whole shells, so both
// interfaces are conforming triangulated shells and every tetrahedron lies in
// one layer.  Each tetrahedron meets a shell in at most one of its faces, so
// the vertex-status rules of the reference classify fluid-solid faces and P2
// edge nodes exactly.
int nmm_ball_create(const nmm_ball_opts* o, nmm_model** out) {
  if (!o || !out) return fail(NMM_ERR_ARG, "null argument");
  if (o->n_cells < 2 || (o->n_cells % 2)) return fail(NMM_ERR_ARG, "n_cells must be even and >= 2");
  if (o->porder != 1 && o->porder != 2) return fail(NMM_ERR_ARG, "porder must be 1 or 2");
  if (!(o->radius > o->r_cmb && o->r_cmb > o->r_icb && o->r_icb > 0))
    return fail(NMM_ERR_ARG, "need 0 < r_icb < r_cmb < radius");
  const int mh = o->n_cells / 2;
  int s1 = (int)std::lround(mh * o->r_icb / o->radius);
  int s2 = (int)std::lround(mh * o->r_cmb / o->radius);
  s1 = std::max(1, s1);
  // A fluid layer one cell thick would give P2 edge nodes joining the two
  // interfaces the fluid-solid status 5 of src/mod_geometry.f90:677-678
  // although they belong to no solid element; keep it at least two cells.
  s2 = std::max(s1 + (o->fluid_core ? 2 : 1), s2);
  if (s2 >= mh) return fail(NMM_ERR_ARG, "n_cells too small to resolve three layers");
  auto Rmap = [&](int s) -> double {
    if (s <= s1) return o->r_icb * s / s1;
    if (s <= s2) return o->r_icb + (o->r_cmb - o->r_icb) * (s - s1) / (double)(s2 - s1);
    return o->r_cmb + (o->radius - o->r_cmb) * (s - s2) / (double)(mh - s2);
  };
  auto* m = new nmm_model();
  m->porder = o->porder;
  m->ref = build_reference(o->porder);
  m->pnp = m->ref.pnp;
  m->nfp = m->ref.nfp;
  const int g = o->n_cells + 1;
  m->nvert = g * g * g;
  auto vid = [&](int i, int j, int k) { return ((i + mh) * g + (j + mh)) * g + (k + mh); };
  std::vector<double> X(3 * (size_t)m->nvert);
  std::vector<int> shell(m->nvert);
  for (int i = -mh; i <= mh; ++i)
    for (int j = -mh; j <= mh; ++j)
      for (int k = -mh; k <= mh; ++k) {
        int id = vid(i, j, k);
        int s = std::max(std::abs(i), std::max(std::abs(j), std::abs(k)));
        shell[id] = s;
        double* x = &X[3 * (size_t)id];
        if (s == 0) {
          x[0] = x[1] = x[2] = 0.0;
          continue;
        }
        int p[3] = {i, j, k};
        int ax = std::abs(i) == s ? 0 : std::abs(j) == s ? 1 : 2;
        double d[3];
        for (int c = 0; c < 3; ++c) {
          if (c == ax) {
            d[c] = p[c] > 0 ? 1.0 : -1.0;
          } else {
            double u = (double)p[c] / s;
            d[c] = std::abs(p[c]) == s ? (p[c] > 0 ? 1.0 : -1.0) : std::tan(0.25 * M_PI * u);
          }
        }
        double nr = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        double R = Rmap(s);
        for (int c = 0; c < 3; ++c) x[c] = d[c] / nr * R;
      }
  // Tetrahedra.
  std::vector<int> tv;
  std::vector<int> layer;
  tv.reserve((size_t)o->n_cells * o->n_cells * o->n_cells * 24);
  static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  for (int a = -mh; a < mh; ++a)
    for (int b = -mh; b < mh; ++b)
      for (int c = -mh; c < mh; ++c) {
        int lo[3] = {a, b, c}, inner[3], step[3];
        int sout = 0;
        for (int d = 0; d < 3; ++d) {
          if (lo[d] >= 0) { inner[d] = lo[d]; step[d] = 1; }
          else { inner[d] = lo[d] + 1; step[d] = -1; }
          sout = std::max(sout, std::max(std::abs(lo[d]), std::abs(lo[d] + 1)));
        }
        int lay = sout <= s1 ? 0 : sout <= s2 ? 1 : 2;
        for (int pi = 0; pi < 6; ++pi) {
          int cur[3] = {inner[0], inner[1], inner[2]};
          int v[4];
          v[0] = vid(cur[0], cur[1], cur[2]);
          for (int q = 0; q < 3; ++q) {
            cur[perms[pi][q]] += step[perms[pi][q]];
            v[q + 1] = vid(cur[0], cur[1], cur[2]);
          }
          tv.insert(tv.end(), v, v + 4);
          layer.push_back(lay);
        }
      }
  m->ntet = (int)(tv.size() / 4);
  auto tetdet = [&](const std::vector<double>& P, int k) {
    const double* v0 = &P[3 * (size_t)tv[4 * k]];
    double B[3][3];
    for (int r = 0; r < 3; ++r)
      for (int cc = 0; cc < 3; ++cc) B[r][cc] = P[3 * (size_t)tv[4 * k + r + 1] + cc] - v0[cc];
    return B[0][0] * (B[1][1] * B[2][2] - B[1][2] * B[2][1]) -
           B[0][1] * (B[1][0] * B[2][2] - B[1][2] * B[2][0]) +
           B[0][2] * (B[1][0] * B[2][1] - B[1][1] * B[2][0]);
  };
  // Positive orientation (detJ > 0) as the reference's meshes have.
  for (int k = 0; k < m->ntet; ++k)
    if (tetdet(X, k) < 0) std::swap(tv[4 * k + 2], tv[4 * k + 3]);
  // Jitter interior vertices (not on the interfaces, the surface or the centre).
  std::vector<double> hmin(m->nvert, 1e300);
  static const int te[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
  for (int k = 0; k < m->ntet; ++k)
    for (int e = 0; e < 6; ++e) {
      int a = tv[4 * k + te[e][0]], b = tv[4 * k + te[e][1]];
      double d2 = 0;
      for (int cc = 0; cc < 3; ++cc) {
        double t = X[3 * (size_t)a + cc] - X[3 * (size_t)b + cc];
        d2 += t * t;
      }
      double d = std::sqrt(d2);
      hmin[a] = std::min(hmin[a], d);
      hmin[b] = std::min(hmin[b], d);
    }
  std::vector<double> X0 = X;
  if (o->jitter > 0) {
    for (int id = 0; id < m->nvert; ++id) {
      int s = shell[id];
      if (s == 0 || s == s1 || s == s2 || s == mh) continue;
      for (int cc = 0; cc < 3; ++cc) {
        double u = u01(splitmix(o->seed * 0x9E3779B97F4A7C15ull + 3ull * id + cc));
        X[3 * (size_t)id + cc] += (2.0 * u - 1.0) * o->jitter * hmin[id];
      }
    }
    // Undo the jitter around any tetrahedron that lost more than 90 % of its volume.
    for (int pass = 0; pass < 8; ++pass) {
      int bad = 0;
      for (int k = 0; k < m->ntet; ++k)
        if (tetdet(X, k) < 0.1 * tetdet(X0, k)) {
          ++bad;
          for (int v = 0; v < 4; ++v) {
            int id = tv[4 * k + v];
            for (int cc = 0; cc < 3; ++cc) X[3 * (size_t)id + cc] = X0[3 * (size_t)id + cc];
          }
        }
      if (!bad) break;
    }
  }
  for (int k = 0; k < m->ntet; ++k)
    if (!(tetdet(X, k) > 0)) {
      delete m;
      return fail(NMM_ERR_MESH, "inverted tetrahedron after mapping");
    }
  m->xyz = X;
  m->fluid.assign(m->ntet, 0);
  for (int k = 0; k < m->ntet; ++k) m->fluid[k] = (o->fluid_core && layer[k] == 1) ? 1 : 0;
  std::vector<std::array<int, 3>> grid(m->nvert);
  for (int i = -mh; i <= mh; ++i)
    for (int j = -mh; j <= mh; ++j)
      for (int k = -mh; k <= mh; ++k) grid[vid(i, j, k)] = {i + mh, j + mh, k + mh};
  finish_mesh(m, tv, &grid);
  // Per-element nodal material.
  ShField fvp, fvs, frho;
  const bool pert = o->lateral_pert != 0.0;
  if (pert) {
    fvp.init(o->lateral_lmax, o->seed ^ 0x1111ull);
    fvs.init(o->lateral_lmax, o->seed ^ 0x2222ull);
    frho.init(o->lateral_lmax, o->seed ^ 0x3333ull);
    for (ShField* f : {&fvp, &fvs, &frho}) {
      double mx = 0.0;
      for (int id = 0; id < m->nnode; ++id) {
        const double* x = &m->xyz[3 * (size_t)id];
        mx = std::max(mx, std::fabs(f->eval(x[0], x[1], x[2])));
      }
      f->scale = mx > 0 ? 1.0 / mx : 1.0;
    }
  }
  const int pnp = m->pnp;
  m->has_profile = true;
  m->prof_R = o->radius;
  m->prof_a = o->homogeneous ? o->rho0 : 13.0;
  m->prof_b = o->homogeneous ? 0.0 : 3.3 - 13.0;
  m->vp.resize((size_t)pnp * m->ntet);
  m->vs.resize((size_t)pnp * m->ntet);
  m->rho.resize((size_t)pnp * m->ntet);
  for (int k = 0; k < m->ntet; ++k)
    for (int l = 0; l < pnp; ++l) {
      const double* x = &m->xyz[3 * (size_t)m->tet[(size_t)pnp * k + l]];
      double r = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]) / o->radius;
      double vp, vs, rho;
      if (o->homogeneous) {
        vp = o->vp0; vs = o->vs0; rho = o->rho0;
      } else {
        rho = 13.0 + (3.3 - 13.0) * r;
        vp = 11.0 + (8.0 - 11.0) * r;
        vs = 3.5 + (4.5 - 3.5) * r;
      }
      if (m->fluid[k]) vs = 0.0;
      if (pert) {
        vp *= 1.0 + o->lateral_pert * fvp.eval(x[0], x[1], x[2]);
        if (vs != 0.0) vs *= 1.0 + o->lateral_pert * fvs.eval(x[0], x[1], x[2]);
        rho *= 1.0 + o->lateral_pert * frho.eval(x[0], x[1], x[2]);
      }
      size_t q = (size_t)pnp * k + l;
      m->vp[q] = vp;
      m->vs[q] = vs;
      m->rho[q] = rho;
    }
  *out = m;
  return NMM_OK;
}

int nmm_load_files(const char* base, int porder, nmm_model** out) {
  if (!base || !out) return fail(NMM_ERR_ARG, "null argument");
  if (porder != 1 && porder != 2) return fail(NMM_ERR_ARG, "porder must be 1 or 2");
  std::string b(base);
  int ntet = 0, nvert = 0;
  {
    FILE* f = std::fopen((b + "_mesh.header").c_str(), "r");
    if (!f) return fail(NMM_ERR_IO, "cannot open " + b + "_mesh.header");
    int ok = std::fscanf(f, "%d %d", &ntet, &nvert);
    std::fclose(f);
    if (ok != 2 || ntet <= 0 || nvert <= 0) return fail(NMM_ERR_IO, "bad mesh header");
  }
  auto readall = [&](const std::string& path, void* dst, size_t bytes) -> bool {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    size_t got = std::fread(dst, 1, bytes, f);
    std::fclose(f);
    return got == bytes;
  };
  auto* m = new nmm_model();
  m->porder = porder;
  m->ref = build_reference(porder);
  m->pnp = m->ref.pnp;
  m->nfp = m->ref.nfp;
  m->nvert = nvert;
  m->ntet = ntet;
  std::vector<int> tv(4 * (size_t)ntet);
  m->xyz.resize(3 * (size_t)nvert);
  if (!readall(b + "_ele.dat", tv.data(), tv.size() * 4) ||
      !readall(b + "_node.dat", m->xyz.data(), m->xyz.size() * 8)) {
    delete m;
    return fail(NMM_ERR_IO, "cannot read ele/node files for " + b);
  }
  for (auto& v : tv) {
    v -= 1;
    if (v < 0 || v >= nvert) {
      delete m;
      return fail(NMM_ERR_IO, "vertex index out of range in ele file");
    }
  }
  const int pnp = m->pnp;
  m->vp.resize((size_t)pnp * ntet);
  m->vs.resize((size_t)pnp * ntet);
  m->rho.resize((size_t)pnp * ntet);
  std::string ps = std::to_string(porder);
  if (!readall(b + "_vp_pod_" + ps + "_true.dat", m->vp.data(), m->vp.size() * 8) ||
      !readall(b + "_vs_pod_" + ps + "_true.dat", m->vs.data(), m->vs.size() * 8) ||
      !readall(b + "_rho_pod_" + ps + "_true.dat", m->rho.data(), m->rho.size() * 8)) {
    delete m;
    return fail(NMM_ERR_IO, "cannot read material files for " + b);
  }
  m->fluid.assign(ntet, 0);
  for (int k = 0; k < ntet; ++k) {
    double mx = 0.0;
    for (int l = 0; l < pnp; ++l) mx = std::max(mx, m->vs[(size_t)pnp * k + l]);
    m->fluid[k] = mx < 1e-6 ? 1 : 0;  // src/mod_geometry.f90:286
  }
  finish_mesh(m, tv);
  *out = m;
  return NMM_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- assembly
namespace {

void elem_vertices(const nmm_model* m, int k, double v[4][3]) {
  for (int j = 0; j < 4; ++j) {
    int node = m->tet[(size_t)m->pnp * k + m->ref.vord[j]];
    for (int c = 0; c < 3; ++c) v[j][c] = m->xyz[3 * (size_t)node + c];
  }
}

// ---------------------------------------------------------------- gravity
// Reference gravity (JOB = 2) quantities of one element
// (src/mod_cg_create_matrix.f90:192-265 in CGFSE3D_ISO, :1057-1083 in
// CGE3D_ISO): the nodal acceleration gk1 = g0 / 1e3 (km/s^2), its
// least-squares gradient dgk1 over the element's nodes and, for the fluid
// terms, the least-squares density gradient, N^2 and the unit vector along g.
constexpr double kEps0 = 1.0e-15;  // eps0, src/mod_cg_create_matrix.f90:30

struct GravElem {
  std::vector<double> g;     // pnp x 3, km/s^2
  double dg[3][3] = {};      // dg[a][c] = d g_c / d x_a
  double drho[3] = {};       // d rho / d x_a
  std::vector<double> n2;    // pnp: buoyancy frequency squared (fluid)
  std::vector<double> unit;  // pnp x 3: g / max(|g|, eps0)
};

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

// lam: nodal lambda (kappa in a fluid); the N^2 fields are filled for fluid
// elements only.  N^2 = (grad rho . g) / rho - |g|^2 rho / lambda, zero where
// |g| < eps0 and everywhere in a pure-fluid planet (:233-255).
bool grav_elem(const nmm_model* m, int k, const std::vector<double>& lam, bool fluid, GravElem& ge) {
  const int p = m->pnp;
  ge.g.assign(3 * (size_t)p, 0.0);
  double xm[3] = {0, 0, 0}, gm[3] = {0, 0, 0}, rm = 0.0;
  std::vector<double> X(3 * (size_t)p);
  for (int l = 0; l < p; ++l) {
    const double* x = &m->xyz[3 * (size_t)m->tet[(size_t)p * k + l]];
    const double* g = &m->g0[3 * ((size_t)p * k + l)];
    for (int c = 0; c < 3; ++c) {
      X[3 * l + c] = x[c];
      ge.g[3 * l + c] = g[c] / 1.0e3;
      xm[c] += x[c];
      gm[c] += ge.g[3 * l + c];
    }
    rm += m->rho[(size_t)p * k + l];
  }
  for (int c = 0; c < 3; ++c) {
    xm[c] /= p;
    gm[c] /= p;
  }
  rm /= p;
  // dism = X - mean(X); dgk1 = (dism' dism)^-1 dism' (g - mean g)
  double N[3][3] = {}, Ni[3][3], Rg[3][3] = {}, Rr[3] = {};
  for (int l = 0; l < p; ++l) {
    double d[3];
    for (int c = 0; c < 3; ++c) d[c] = X[3 * l + c] - xm[c];
    const double rd = m->rho[(size_t)p * k + l] - rm;
    for (int a = 0; a < 3; ++a) {
      for (int b = 0; b < 3; ++b) {
        N[a][b] += d[a] * d[b];
        Rg[a][b] += d[a] * (ge.g[3 * l + b] - gm[b]);
      }
      Rr[a] += d[a] * rd;
    }
  }
  if (!inv3(N, Ni)) return false;
  for (int a = 0; a < 3; ++a) {
    ge.drho[a] = 0.0;
    for (int c = 0; c < 3; ++c) {
      ge.dg[a][c] = 0.0;
      for (int b = 0; b < 3; ++b) ge.dg[a][c] += Ni[a][b] * Rg[b][c];
    }
    for (int b = 0; b < 3; ++b) ge.drho[a] += Ni[a][b] * Rr[b];
  }
  if (fluid) {
    ge.n2.assign(p, 0.0);
    ge.unit.assign(3 * (size_t)p, 0.0);
    for (int l = 0; l < p; ++l) {
      const double* g = &ge.g[3 * l];
      const double rho = m->rho[(size_t)p * k + l];
      const double ng = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
      double n2 = (ge.drho[0] * g[0] + ge.drho[1] * g[1] + ge.drho[2] * g[2]) / rho - ng * ng / lam[l] * rho;
      if (ng < kEps0 || m->purefluid) n2 = 0.0;
      ge.n2[l] = n2;
      for (int c = 0; c < 3; ++c) ge.unit[3 * l + c] = g[c] / std::max(ng, kEps0);
    }
  }
  return true;
}

// Gravity block (i, j) of a solid element, before the detJ factor
// (src/mod_cg_create_matrix.f90:329-377, :1118-1160), G_j = diag(g_j):
//   X = (D_i' M G_j + G_i M D_j) / 2 - M (dg_ij + dg_ji) / 2
//       - (D_j' G_i M + M G_j D_i) / 2,   OPrho = (X R + R X) / 2, R = diag(rho).
Mat solid_gravity_block(const RefElem& R, const Mat* D, const GravElem& ge, const std::vector<double>& rhot, int i,
                        int j) {
  const int p = R.pnp;
  const Mat& M = R.M;
  const double s = (ge.dg[i][j] + ge.dg[j][i]) / 2.0;
  Mat X(p * p);
  for (int a = 0; a < p; ++a)
    for (int b = 0; b < p; ++b) {
      double t1 = 0.0, t2 = 0.0, t3 = 0.0, t4 = 0.0;
      for (int c = 0; c < p; ++c) {
        t1 += D[i][c * p + a] * M[c * p + b];                      // (D_i' M)(a, b)
        t2 += M[a * p + c] * D[j][c * p + b];                      // (M D_j)(a, b)
        t3 += D[j][c * p + a] * ge.g[3 * c + i] * M[c * p + b];    // (D_j' G_i M)(a, b)
        t4 += M[a * p + c] * ge.g[3 * c + j] * D[i][c * p + b];    // (M G_j D_i)(a, b)
      }
      t1 *= ge.g[3 * b + j];
      t2 *= ge.g[3 * a + i];
      X[a * p + b] = (t1 + t2) / 2.0 - M[a * p + b] * s - (t3 + t4) / 2.0;
    }
  Mat O(p * p);
  for (int a = 0; a < p; ++a)
    for (int b = 0; b < p; ++b) O[a * p + b] = (X[a * p + b] * rhot[b] + rhot[a] * X[a * p + b]) / 2.0;
  return O;
}

// Solid element: TM (3pnp)^2 and MM (3pnp)^2.  `sym_mass` selects the
// diag(rho)-symmetrised mass of CGE3D_ISO (src/mod_cg_create_matrix.f90:1089-1091)
// instead of the mean-density mass of CGFSE3D_ISO (:293).
bool solid_element(const nmm_model* m, int k, const ElemGeom& g, bool sym_mass, double* TM, double* MM) {
  const int p = m->pnp, les = 3 * p;
  const RefElem& R = m->ref;
  std::vector<double> lam(p), mu(p), rhot(p);
  for (int l = 0; l < p; ++l) {
    size_t q = (size_t)p * k + l;
    double c44 = m->rho[q] * m->vs[q] * m->vs[q];
    double c33 = m->rho[q] * m->vp[q] * m->vp[q] - 2 * c44;
    lam[l] = c33;
    mu[l] = c44;
    rhot[l] = m->rho[q];
  }
  Mat D[3], TD[3], OP1[3], OP2[3], OPt[3];
  for (int i = 0; i < 3; ++i) {
    D[i].assign(p * p, 0.0);
    for (int a = 0; a < p * p; ++a)
      D[i][a] = g.invJ[i][0] * R.D[0][a] + g.invJ[i][1] * R.D[1][a] + g.invJ[i][2] * R.D[2][a];
  }
  Mat Ml(p * p), Mm(p * p);
  for (int a = 0; a < p; ++a)
    for (int b = 0; b < p; ++b) {
      Ml[a * p + b] = R.M[a * p + b] * lam[b];
      Mm[a * p + b] = R.M[a * p + b] * mu[b];
    }
  {
    Mat t1 = tr(Ml, p), t2 = tr(Mm, p);
    for (int a = 0; a < p * p; ++a) {
      Ml[a] = (Ml[a] + t1[a]) / 2.0;
      Mm[a] = (Mm[a] + t2[a]) / 2.0;
    }
  }
  Mat OPs(p * p, 0.0);
  for (int i = 0; i < 3; ++i) {
    OP1[i] = mm(Ml, D[i], p);
    OP2[i] = mm(Mm, D[i], p);
    TD[i] = tr(D[i], p);
    OPt[i] = mm(TD[i], OP2[i], p);
    for (int a = 0; a < p * p; ++a) OPs[a] += OPt[i][a];
  }
  Mat Mrho(p * p);
  if (sym_mass) {
    for (int a = 0; a < p; ++a)
      for (int b = 0; b < p; ++b)
        Mrho[a * p + b] = (rhot[a] * R.M[a * p + b] + R.M[a * p + b] * rhot[b]) / 2.0;
  } else {
    double srho = 0.0;
    for (int l = 0; l < p; ++l) srho += rhot[l];
    for (int a = 0; a < p * p; ++a) Mrho[a] = R.M[a] * srho / (double)p;
  }
  GravElem ge;
  const bool grav = !m->g0.empty();
  if (grav && !grav_elem(m, k, lam, false, ge)) return false;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      Mat OPij(p * p);
      if (i == j) {
        Mat OPtmp = mm(TD[i], OP1[i], p);
        for (int a = 0; a < p * p; ++a) OPij[a] = OPs[a] + OPt[i][a] + OPtmp[a];
        Mat t = tr(OPij, p);
        for (int a = 0; a < p * p; ++a) OPij[a] = (OPij[a] + t[a]) / 2.0;
      } else {
        Mat a1 = mm(TD[i], OP1[j], p), a2 = mm(TD[j], OP2[i], p);
        Mat b1 = mm(TD[j], OP1[i], p), b2 = mm(TD[i], OP2[j], p);
        Mat OPtrsT(p * p);
        for (int a = 0; a < p; ++a)
          for (int b = 0; b < p; ++b)
            OPtrsT[a * p + b] = b1[b * p + a] + b2[b * p + a];
        for (int a = 0; a < p * p; ++a) OPij[a] = (OPtrsT[a] + (a1[a] + a2[a])) / 2.0;
      }
      if (grav) {
        const Mat Og = solid_gravity_block(R, D, ge, rhot, i, j);
        for (int a = 0; a < p * p; ++a) OPij[a] += Og[a];
      }
      for (int a = 0; a < p; ++a)
        for (int b = 0; b < p; ++b) {
          TM[(size_t)(i * p + a) * les + (j * p + b)] = OPij[a * p + b] * g.detJ;
          MM[(size_t)(i * p + a) * les + (j * p + b)] = (i == j) ? Mrho[a * p + b] * g.detJ : 0.0;
        }
    }
  return true;
}

// Fluid element: FT and FM of dimension 3 pnp + pnp
// (src/mod_cg_create_matrix.f90:453-640).  With the reference gravity
// (JOB = 2) FT also carries
//   * the N^2 displacement block (:492-608): (U_i M W_j + W_i M U_j) / 2 with
//     U_i = diag(g_i / |g|), W_j = diag(g_j / |g| N^2 rho);
//   * the density-gradient part of the coupling (:541-570): M D_i becomes
//     M D_i - M diag(rho g_i / kappa);
//   * the face terms of :643-705: on the outer boundary the pressure block
//     gets -MassF sJac / (mean|g.n| mean rho) (free surface of a fluid); on an
//     inner face that is not a fluid-solid face the displacement blocks get
//     MassF sJac mean(g.n) mean(rho) n_j^2.
// Without gravity the face terms vanish: they are built from the gravity
// (zero in JOB = 1).  Returns NMM_OK or an error code.
int fluid_element(const nmm_model* m, int k, const ElemGeom& g, double* FT, double* FM) {
  const int p = m->pnp, lef = 4 * p;
  const RefElem& R = m->ref;
  std::vector<double> lamiv(p), lam(p), rhot(p);
  double srho = 0.0;
  for (int l = 0; l < p; ++l) {
    size_t q = (size_t)p * k + l;
    double c44 = m->rho[q] * m->vs[q] * m->vs[q];
    double c33 = m->rho[q] * m->vp[q] * m->vp[q] - 2 * c44;
    lam[l] = c33;
    lamiv[l] = 1.0 / std::sqrt(c33);
    rhot[l] = m->rho[q];
    srho += rhot[l];
  }
  GravElem ge;
  const bool grav = !m->g0.empty();
  if (grav && !grav_elem(m, k, lam, true, ge)) return fail(NMM_ERR_MESH, "degenerate element in the gravity gradient");
  std::fill(FT, FT + (size_t)lef * lef, 0.0);
  std::fill(FM, FM + (size_t)lef * lef, 0.0);
  Mat flam(p * p), Mrho(p * p);
  for (int a = 0; a < p; ++a)
    for (int b = 0; b < p; ++b) flam[a * p + b] = (lamiv[a] * R.M[a * p + b]) * lamiv[b];
  for (int a = 0; a < p * p; ++a) Mrho[a] = R.M[a] * srho / (double)p;
  for (int i = 0; i < 3; ++i) {
    Mat D(p * p);
    for (int a = 0; a < p * p; ++a)
      D[a] = g.invJ[i][0] * R.D[0][a] + g.invJ[i][1] * R.D[1][a] + g.invJ[i][2] * R.D[2][a];
    Mat G = mm(R.M, D, p);
    Mat Ot = mm(tr(D, p), R.M, p);
    Mat Oij(p * p);
    for (int a = 0; a < p; ++a)
      for (int b = 0; b < p; ++b) Oij[a * p + b] = (G[a * p + b] + Ot[b * p + a]) / 2.0;
    if (grav)
      for (int a = 0; a < p; ++a)
        for (int b = 0; b < p; ++b) Oij[a * p + b] -= R.M[a * p + b] * (rhot[b] / lam[b] * ge.g[3 * b + i]);
    for (int a = 0; a < p; ++a)
      for (int b = 0; b < p; ++b) {
        FM[(size_t)(i * p + a) * lef + (i * p + b)] = Mrho[a * p + b] * g.detJ;
        FT[(size_t)(i * p + a) * lef + (3 * p + b)] = Oij[a * p + b] * g.detJ;
        FT[(size_t)(3 * p + a) * lef + (i * p + b)] = Oij[b * p + a] * g.detJ;
      }
  }
  for (int a = 0; a < p; ++a)
    for (int b = 0; b < p; ++b) FT[(size_t)(3 * p + a) * lef + (3 * p + b)] = -(g.detJ * flam[a * p + b]);
  if (!grav) return NMM_OK;
  // N^2 block
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int a = 0; a < p; ++a)
        for (int b = 0; b < p; ++b) {
          const double wj = ge.unit[3 * b + j] * ge.n2[b] * rhot[b];
          const double wi = ge.unit[3 * a + i] * ge.n2[a] * rhot[a];
          const double v = (ge.unit[3 * a + i] * R.M[a * p + b] * wj + wi * R.M[a * p + b] * ge.unit[3 * b + j]) / 2.0;
          FT[(size_t)(i * p + a) * lef + (j * p + b)] = v * g.detJ;
        }
  // face terms
  const int nfp = m->nfp;
  for (int f = 0; f < 4; ++f) {
    const std::vector<int>& Fm = R.fmask[f];
    const std::vector<double>& MF = R.MF[f];
    const double* nf = g.n[f];
    double surfrho = 0.0, sgn = 0.0;
    const bool outer = m->bface[4 * (size_t)k + f] != 0;
    for (int a = 0; a < nfp; ++a) {
      const double* gk = &ge.g[3 * Fm[a]];
      const double gn = gk[0] * nf[0] + gk[1] * nf[1] + gk[2] * nf[2];
      surfrho += rhot[Fm[a]];
      sgn += outer ? std::sqrt(gn * gn) : gn;
    }
    surfrho /= nfp;
    sgn /= nfp;
    if (outer) {
      if (!(sgn > 0.0)) return fail(NMM_ERR_MESH, "fluid boundary face without normal gravity");
      for (int a = 0; a < nfp; ++a)
        for (int b = 0; b < nfp; ++b)
          FT[(size_t)(3 * p + Fm[a]) * lef + (3 * p + Fm[b])] -= MF[a * nfp + b] / sgn / surfrho * g.sJac[f];
    } else {
      int cout = 0;
      for (int v = 0; v < 4; ++v)
        if (v != f && m->rnum[m->tet[(size_t)p * k + R.vord[v]]] == 6) ++cout;
      if (cout >= 3) continue;
      for (int j = 0; j < 3; ++j)
        for (int a = 0; a < nfp; ++a)
          for (int b = 0; b < nfp; ++b)
            FT[(size_t)(j * p + Fm[a]) * lef + (j * p + Fm[b])] +=
                MF[a * nfp + b] * sgn * surfrho * g.sJac[f] * (nf[j] * nf[j]);
    }
  }
  return NMM_OK;
}

// Sorted-neighbour lists (v2v, including the node itself).
std::vector<std::vector<int>> node_adjacency(const nmm_model* m) {
  const int p = m->pnp;
  std::vector<int> cnt(m->nnode + 1, 0);
  for (int k = 0; k < m->ntet; ++k)
    for (int l = 0; l < p; ++l) cnt[m->tet[(size_t)p * k + l] + 1]++;
  for (int i = 0; i < m->nnode; ++i) cnt[i + 1] += cnt[i];
  std::vector<int> n2e(cnt[m->nnode]);
  std::vector<int> fill(cnt.begin(), cnt.end() - 1);
  for (int k = 0; k < m->ntet; ++k)
    for (int l = 0; l < p; ++l) n2e[fill[m->tet[(size_t)p * k + l]]++] = k;
  std::vector<std::vector<int>> adj(m->nnode);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < m->nnode; ++i) {
    std::vector<int> v;
    for (int q = cnt[i]; q < cnt[i + 1]; ++q) {
      int k = n2e[q];
      for (int l = 0; l < p; ++l) v.push_back(m->tet[(size_t)p * k + l]);
    }
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    adj[i] = std::move(v);
  }
  return adj;
}

void csr_from_rows(Csr& C, int ncols, std::vector<std::vector<int>>& rows) {
  C.nrows = (int)rows.size();
  C.ncols = ncols;
  C.rowptr.assign(C.nrows + 1, 0);
  for (int r = 0; r < C.nrows; ++r) C.rowptr[r + 1] = C.rowptr[r] + (int)rows[r].size();
  C.col.resize(C.rowptr[C.nrows]);
  for (int r = 0; r < C.nrows; ++r) {
    std::sort(rows[r].begin(), rows[r].end());
    std::copy(rows[r].begin(), rows[r].end(), C.col.begin() + C.rowptr[r]);
  }
  C.val.assign(C.col.size(), 0.0);
}

// CSR structure for the solid-only path (src/mod_cg_create_matrix.f90:1269-1455).
void structure_solid(nmm_model* m, const std::vector<std::vector<int>>& adj) {
  std::vector<std::vector<int>> ra(m->n), rb(m->n);
  for (int i = 0; i < m->nnode; ++i)
    for (int j = 0; j < 3; ++j) {
      auto& a = ra[m->vstt[i] + j];
      auto& b = rb[m->vstt[i] + j];
      for (int nb : adj[i]) {
        for (int c = 0; c < 3; ++c) a.push_back(m->vstt[nb] + c);
        b.push_back(m->vstt[nb] + j);
      }
    }
  csr_from_rows(m->A, m->n, ra);
  csr_from_rows(m->B, m->n, rb);
}

// CSR structure for the fluid / fluid-solid path (src/mod_cg_create_matrix.f90:1458-2033).
int structure_general(nmm_model* m, const std::vector<std::vector<int>>& adj) {
  std::vector<std::vector<int>> rad(m->n), rb(m->n), re(m->n), rap(m->np), ret(m->np);
  for (int i = 0; i < m->nnode; ++i) {
    const auto& nb = adj[i];
    const int v0 = m->vstt[i];
    if (m->pnum[i] == 1 && m->rnum[i] == 3) {  // pure fluid
      for (int b : nb)
        if (m->pnum[b] != 1) return fail(NMM_ERR_MESH, "pure fluid node next to a node without pressure");
      auto& ap = rap[m->pstt[i]];
      auto& et = ret[m->pstt[i]];
      for (int b : nb) {
        ap.push_back(m->pstt[b]);
        for (int c = 0; c < 3; ++c) et.push_back(m->vstt[b] + c + m->rnum[b] - 3);
      }
      for (int j = 0; j < 3; ++j) {
        for (int b : nb) {
          for (int c = 0; c < 3; ++c) rad[v0 + j].push_back(m->vstt[b] + c + m->rnum[b] - 3);
          rb[v0 + j].push_back(m->vstt[b] + j + m->rnum[b] - 3);
          re[v0 + j].push_back(m->pstt[b]);
        }
      }
    } else if (m->pnum[i] == 1) {  // fluid-solid node: solid rows then fluid rows
      for (int j = 0; j < 3; ++j)
        for (int b : nb) {
          if (m->pnum[b] == 0 || m->rnum[b] == 6) {
            for (int c = 0; c < 3; ++c) rad[v0 + j].push_back(m->vstt[b] + c);
            rb[v0 + j].push_back(m->vstt[b] + j);
          }
          if (m->rnum[b] == 6) re[v0 + j].push_back(m->pstt[b]);
        }
      auto& ap = rap[m->pstt[i]];
      auto& et = ret[m->pstt[i]];
      for (int b : nb)
        if (m->pnum[b] == 1) {
          ap.push_back(m->pstt[b]);
          for (int c = 0; c < m->rnum[b]; ++c) et.push_back(m->vstt[b] + c);
        }
      for (int j = 0; j < 3; ++j)
        for (int b : nb)
          if (m->pnum[b] == 1) {
            for (int c = 0; c < 3; ++c) rad[v0 + 3 + j].push_back(m->vstt[b] + c + m->rnum[b] - 3);
            rb[v0 + 3 + j].push_back(m->vstt[b] + j + m->rnum[b] - 3);
            re[v0 + 3 + j].push_back(m->pstt[b]);
          }
    } else {  // pure solid
      if (m->rnum[i] != 3) return fail(NMM_ERR_MESH, "solid node with 6 DOFs");
      for (int j = 0; j < 3; ++j)
        for (int b : nb) {
          for (int c = 0; c < 3; ++c) rad[v0 + j].push_back(m->vstt[b] + c);
          rb[v0 + j].push_back(m->vstt[b] + j);
        }
    }
  }
  csr_from_rows(m->Ad, m->n, rad);
  csr_from_rows(m->B, m->n, rb);
  csr_from_rows(m->E, m->np, re);
  csr_from_rows(m->Ap, m->np, rap);
  csr_from_rows(m->ET, m->n, ret);
  return NMM_OK;
}

inline int find_col(const Csr& C, int row, int col) {
  const int* b = C.col.data() + C.rowptr[row];
  const int* e = C.col.data() + C.rowptr[row + 1];
  const int* it = std::lower_bound(b, e, col);
  if (it == e || *it != col) return -1;
  return (int)(it - C.col.data());
}

}  // namespace

extern "C" int nmm_element_matrices(const nmm_model* m, int k, double* T, double* Mo, int* dim) {
  if (!m || !T || !Mo || !dim || k < 0 || k >= m->ntet) return fail(NMM_ERR_ARG, "bad argument");
  double v[4][3];
  elem_vertices(m, k, v);
  ElemGeom g;
  if (!elem_geometry(v, g)) return fail(NMM_ERR_MESH, "flat tetrahedron");
  const bool general = m->fsexist || m->purefluid;
  double maxmu = 0.0;
  for (int l = 0; l < m->pnp; ++l) {
    size_t q = (size_t)m->pnp * k + l;
    maxmu = std::max(maxmu, m->rho[q] * m->vs[q] * m->vs[q]);
  }
  if (!general || maxmu >= 1e-8) {
    *dim = 3 * m->pnp;
    if (!solid_element(m, k, g, !general, T, Mo)) return fail(NMM_ERR_MESH, "degenerate element in the gravity gradient");
    return NMM_OK;
  }
  *dim = 4 * m->pnp;
  return fluid_element(m, k, g, T, Mo);
}

extern "C" int nmm_assemble(nmm_model* m) {
  if (!m) return fail(NMM_ERR_ARG, "null model");
  if (m->assembled) return NMM_OK;
  const bool general = m->fsexist || m->purefluid;
  const int p = m->pnp;
  // Fluid element on the outer boundary: the face term divides by the normal
  // gravity there (src/mod_cg_create_matrix.f90:645-666), zero in JOB = 1.
  if (m->g0.empty())
    for (int k = 0; k < m->ntet; ++k)
      if (m->fluid[k])
        for (int f = 0; f < 4; ++f)
          if (m->bface[4 * (size_t)k + f])
            return fail(NMM_ERR_MESH, "fluid element on the outer boundary is not supported without gravity");
  auto adj = node_adjacency(m);
  if (general) {
    int rc = structure_general(m, adj);
    if (rc) return rc;
  } else {
    structure_solid(m, adj);
  }
  adj.clear();
  adj.shrink_to_fit();
  Csr& Amat = general ? m->Ad : m->A;
  const int lef = 4 * p, les = 3 * p;
  const int chunk = 8192;
  std::vector<double> T((size_t)chunk * lef * lef), Mm((size_t)chunk * lef * lef);
  std::vector<unsigned char> is_solid(chunk);
  std::vector<ElemGeom> geo(chunk);
  m->n_cout4 = 0;
  for (int k0 = 0; k0 < m->ntet; k0 += chunk) {
    int k1 = std::min(m->ntet, k0 + chunk);
    int bad = 0, badg = 0, badf = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad, badg, badf)
    for (int k = k0; k < k1; ++k) {
      double v[4][3];
      elem_vertices(m, k, v);
      ElemGeom& g = geo[k - k0];
      if (!elem_geometry(v, g)) { ++bad; continue; }
      double maxmu = 0.0;
      for (int l = 0; l < p; ++l) {
        size_t q = (size_t)p * k + l;
        maxmu = std::max(maxmu, m->rho[q] * m->vs[q] * m->vs[q]);
      }
      bool solid = !general || maxmu >= 1e-8;  // src/mod_cg_create_matrix.f90:279
      is_solid[k - k0] = solid;
      double* Tk = &T[(size_t)(k - k0) * lef * lef];
      double* Mk = &Mm[(size_t)(k - k0) * lef * lef];
      if (solid) {
        if (!solid_element(m, k, g, !general, Tk, Mk)) ++badg;
      } else if (fluid_element(m, k, g, Tk, Mk) != NMM_OK) {
        ++badf;
      }
    }
    if (bad) return fail(NMM_ERR_MESH, "flat tetrahedron");
    if (badg) return fail(NMM_ERR_MESH, "degenerate element in the gravity gradient");
    if (badf) return fail(NMM_ERR_MESH, "fluid element: degenerate gravity gradient or boundary face without normal gravity");
    for (int k = k0; k < k1; ++k) {
      const int* nodes = &m->tet[(size_t)p * k];
      const double* Tk = &T[(size_t)(k - k0) * lef * lef];
      const double* Mk = &Mm[(size_t)(k - k0) * lef * lef];
      if (is_solid[k - k0]) {
        for (int mm_ = 0; mm_ < p; ++mm_) {
          int a = nodes[mm_];
          for (int pp = 0; pp < 3; ++pp) {
            int row = m->vstt[a] + pp;
            for (int nn = 0; nn < p; ++nn) {
              int b = nodes[nn];
              int pos = find_col(Amat, row, m->vstt[b]);
              if (pos < 0) return fail(NMM_ERR_STATE, "A/Ad structure miss");
              for (int q = 0; q < 3; ++q)
                Amat.val[pos + q] += Tk[(size_t)(pp * p + mm_) * les + (q * p + nn)];
            }
            for (int nn = 0; nn < p; ++nn) {
              int b = nodes[nn];
              int pos = find_col(m->B, row, m->vstt[b] + pp);
              if (pos < 0) return fail(NMM_ERR_STATE, "B structure miss");
              m->B.val[pos] += Mk[(size_t)(pp * p + mm_) * les + (pp * p + nn)];
            }
          }
        }
      } else {
        for (int mm_ = 0; mm_ < p; ++mm_) {
          int a = nodes[mm_];
          int prow = m->pstt[a];
          for (int nn = 0; nn < p; ++nn) {
            int pos = find_col(m->Ap, prow, m->pstt[nodes[nn]]);
            if (pos < 0) return fail(NMM_ERR_STATE, "Ap structure miss");
            m->Ap.val[pos] += Tk[(size_t)(3 * p + mm_) * lef + (3 * p + nn)];
          }
          for (int nn = 0; nn < p; ++nn) {
            int b = nodes[nn];
            int pos = find_col(m->ET, prow, m->vstt[b] + m->rnum[b] - 3);
            if (pos < 0) return fail(NMM_ERR_STATE, "ET structure miss");
            for (int q = 0; q < 3; ++q) m->ET.val[pos + q] += Tk[(size_t)(3 * p + mm_) * lef + (q * p + nn)];
          }
          for (int pp = 0; pp < 3; ++pp) {
            int row = m->vstt[a] + m->rnum[a] - 3 + pp;
            for (int nn = 0; nn < p; ++nn) {
              int b = nodes[nn];
              int pos = find_col(m->Ad, row, m->vstt[b] + m->rnum[b] - 3);
              if (pos < 0) return fail(NMM_ERR_STATE, "Ad structure miss (fluid)");
              for (int q = 0; q < 3; ++q) m->Ad.val[pos + q] += Tk[(size_t)(pp * p + mm_) * lef + (q * p + nn)];
            }
            for (int nn = 0; nn < p; ++nn) {
              int b = nodes[nn];
              int pos = find_col(m->B, row, m->vstt[b] + pp + m->rnum[b] - 3);
              if (pos < 0) return fail(NMM_ERR_STATE, "B structure miss (fluid)");
              m->B.val[pos] += Mk[(size_t)(pp * p + mm_) * lef + (pp * p + nn)];
            }
            for (int nn = 0; nn < p; ++nn) {
              int pos = find_col(m->E, row, m->pstt[nodes[nn]]);
              if (pos < 0) return fail(NMM_ERR_STATE, "E structure miss");
              m->E.val[pos] += Tk[(size_t)(pp * p + mm_) * lef + (3 * p + nn)];
            }
          }
        }
        // Fluid-solid interface face: three of the four vertices carry 6 DOFs
        // (src/mod_cg_create_matrix.f90:804-952).
        int cout = 0, fcid = -1;
        for (int v = 0; v < 4; ++v) {
          if (m->rnum[nodes[m->ref.vord[v]]] == 6) ++cout;
          else fcid = v;
        }
        if (cout == 4) ++m->n_cout4;
        if (cout == 3) {
          const ElemGeom& g = geo[k - k0];
          const int nfp = m->nfp;
          const std::vector<int>& Fm = m->ref.fmask[fcid];
          const std::vector<double>& MF = m->ref.MF[fcid];
          for (int a = 0; a < nfp; ++a) {
            int na = nodes[Fm[a]];
            int prow = m->pstt[na];
            for (int b = 0; b < nfp; ++b) {
              int nb = nodes[Fm[b]];
              int pos = find_col(m->ET, prow, m->vstt[nb]);
              if (pos < 0) return fail(NMM_ERR_STATE, "ET interface structure miss");
              for (int q = 0; q < 3; ++q)
                m->ET.val[pos + q] -= g.n[fcid][q] * g.sJac[fcid] * MF[b * nfp + a];
            }
            for (int pp = 0; pp < 3; ++pp) {
              int row = m->vstt[na] + pp;
              for (int b = 0; b < nfp; ++b) {
                int pos = find_col(m->E, row, m->pstt[nodes[Fm[b]]]);
                if (pos < 0) return fail(NMM_ERR_STATE, "E interface structure miss");
                m->E.val[pos] -= g.n[fcid][pp] * g.sJac[fcid] * MF[a * nfp + b];
              }
            }
          }
          // Reference gravity on the interface (src/mod_cg_create_matrix.f90:866-920):
          // the solid rows and columns of the face nodes lose
          // rho_f sJac (n_p MF(a,b) g_q(b) + n_q g_p(a) MF(a,b)) / 2.
          if (!m->g0.empty()) {
            const double* nf = g.n[fcid];
            double rhof = 0.0;
            for (int a = 0; a < nfp; ++a) rhof += m->rho[(size_t)p * k + Fm[a]];
            rhof /= nfp;
            const double* gk = &m->g0[3 * (size_t)p * k];
            for (int a = 0; a < nfp; ++a) {
              const int na = nodes[Fm[a]];
              for (int pp = 0; pp < 3; ++pp) {
                const int row = m->vstt[na] + pp;
                for (int b = 0; b < nfp; ++b) {
                  const int pos = find_col(m->Ad, row, m->vstt[nodes[Fm[b]]]);
                  if (pos < 0) return fail(NMM_ERR_STATE, "Ad interface structure miss");
                  const double mf = MF[a * nfp + b];
                  for (int q = 0; q < 3; ++q) {
                    const double gq = gk[3 * Fm[b] + q] / 1.0e3, gp = gk[3 * Fm[a] + pp] / 1.0e3;
                    m->Ad.val[pos + q] -= rhof * g.sJac[fcid] * (nf[pp] * mf * gq + nf[q] * gp * mf) / 2.0;
                  }
                }
              }
            }
          }
        }
      }
    }
  }
  m->assembled = true;
  return NMM_OK;
}

extern "C" {

int nmm_info(const nmm_model* m, nmm_info_t* info) {
  if (!m || !info) return fail(NMM_ERR_ARG, "null argument");
  std::memset(info, 0, sizeof(*info));
  info->porder = m->porder;
  info->pnp = m->pnp;
  info->nfp = m->nfp;
  info->nvert = m->nvert;
  info->ntet = m->ntet;
  info->nnode = m->nnode;
  for (auto f : m->fluid) info->n_fluid_tets += f;
  info->fsexist = m->fsexist;
  info->purefluid = m->purefluid;
  info->n = m->n;
  info->np = m->np;
  const Csr* mats[6] = {&m->A, &m->B, &m->Ad, &m->Ap, &m->E, &m->ET};
  for (int i = 0; i < 6; ++i) info->nnz[i] = mats[i]->nnz();
  info->assembled = m->assembled;
  return NMM_OK;
}

int nmm_get_csr(const nmm_model* m, int which, const int** rowptr, const int** col, const double** val,
                int* nrows, int* ncols, long long* nnz) {
  if (!m) return fail(NMM_ERR_ARG, "null model");
  if (!m->assembled) return fail(NMM_ERR_STATE, "model not assembled");
  const Csr* mats[6] = {&m->A, &m->B, &m->Ad, &m->Ap, &m->E, &m->ET};
  if (which < 0 || which > 5) return fail(NMM_ERR_ARG, "bad matrix selector");
  const Csr* C = mats[which];
  if (C->nrows == 0) return fail(NMM_ERR_ARG, "matrix not present in this model");
  if (rowptr) *rowptr = C->rowptr.data();
  if (col) *col = C->col.data();
  if (val) *val = C->val.data();
  if (nrows) *nrows = C->nrows;
  if (ncols) *ncols = C->ncols;
  if (nnz) *nnz = C->nnz();
  return NMM_OK;
}

int nmm_mesh_arrays(const nmm_model* m, const double** xyz, const int** tets, const unsigned char** fluid,
                    const int** vstat, const int** vstt, const int** rnum, const int** pstt,
                    const double** vp, const double** vs, const double** rho) {
  if (!m) return fail(NMM_ERR_ARG, "null model");
  if (xyz) *xyz = m->xyz.data();
  if (tets) *tets = m->tet.data();
  if (fluid) *fluid = m->fluid.data();
  if (vstat) *vstat = m->vstat.data();
  if (vstt) *vstt = m->vstt.data();
  if (rnum) *rnum = m->rnum.data();
  if (pstt) *pstt = m->pstt.data();
  if (vp) *vp = m->vp.data();
  if (vs) *vs = m->vs.data();
  if (rho) *rho = m->rho.data();
  return NMM_OK;
}

int nmm_set_material(nmm_model* m, const double* vp, const double* vs, const double* rho) {
  if (!m || !vp || !vs || !rho) return fail(NMM_ERR_ARG, "null argument");
  const size_t len = (size_t)m->pnp * m->ntet;
  // the solid / fluid split (and with it the DOF structure) must not change
  for (int k = 0; k < m->ntet; ++k) {
    double mx = 0.0, mxold = 0.0;
    for (int l = 0; l < m->pnp; ++l) {
      const size_t q = (size_t)m->pnp * k + l;
      if (!(vp[q] > 0.0) || !(rho[q] > 0.0) || vs[q] < 0.0) return fail(NMM_ERR_ARG, "non-physical material");
      mx = std::max(mx, rho[q] * vs[q] * vs[q]);
      mxold = std::max(mxold, m->rho[q] * m->vs[q] * m->vs[q]);
    }
    if ((mx >= 1e-8) != (mxold >= 1e-8)) return fail(NMM_ERR_ARG, "material change would turn a solid element fluid or back");
  }
  m->vp.assign(vp, vp + len);
  m->vs.assign(vs, vs + len);
  m->rho.assign(rho, rho + len);
  m->assembled = false;
  return NMM_OK;
}

int nmm_set_gravity(nmm_model* m, const double* g0) {
  if (!m) return fail(NMM_ERR_ARG, "null model");
  const size_t len = 3 * (size_t)m->pnp * m->ntet;
  if (g0) {
    for (size_t i = 0; i < len; ++i)
      if (!std::isfinite(g0[i])) return fail(NMM_ERR_ARG, "non-finite gravity value");
    m->g0.assign(g0, g0 + len);
  } else {
    m->g0.clear();
  }
  m->assembled = false;
  return NMM_OK;
}

int nmm_load_gravity(nmm_model* m, const char* base) {
  if (!m || !base) return fail(NMM_ERR_ARG, "null argument");
  const std::string path = std::string(base) + "_pod_" + std::to_string(m->porder) + "_potential_acceleration_true.dat";
  std::vector<double> buf(3 * (size_t)m->pnp * m->ntet);
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return fail(NMM_ERR_IO, "cannot open " + path);
  const size_t got = std::fread(buf.data(), sizeof(double), buf.size(), f);
  std::fclose(f);
  if (got != buf.size()) return fail(NMM_ERR_IO, "short gravity file " + path);
  return nmm_set_gravity(m, buf.data());
}

// g(r) = G M(r) / r^2 with M(r) = 4 pi (a r^3 / 3 + b r^4 / (4 R)) for
// rho = a + b r / R; r in km, rho in g/cm^3, so M in 1e12 kg and g in m/s^2
// is G 4 pi 1e6 (a r / 3 + b r^2 / (4 R)).
int nmm_ball_gravity(nmm_model* m, double G) {
  if (!m) return fail(NMM_ERR_ARG, "null model");
  if (!m->has_profile) return fail(NMM_ERR_STATE, "model has no radial density profile (load a gravity file instead)");
  if (!(G > 0.0)) return fail(NMM_ERR_ARG, "G must be positive");
  const int p = m->pnp;
  std::vector<double> g0(3 * (size_t)p * m->ntet);
  for (int k = 0; k < m->ntet; ++k)
    for (int l = 0; l < p; ++l) {
      const double* x = &m->xyz[3 * (size_t)m->tet[(size_t)p * k + l]];
      const double r = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
      const double gr = G * 4.0 * M_PI * 1.0e6 * (m->prof_a * r / 3.0 + m->prof_b * r * r / (4.0 * m->prof_R));
      for (int c = 0; c < 3; ++c) g0[3 * ((size_t)p * k + l) + c] = r > 0.0 ? -gr * x[c] / r : 0.0;
    }
  return nmm_set_gravity(m, g0.data());
}

// The model in the reference's input files (the files nmm_load_files and
// nmm_load_gravity read; src/mod_geometry.f90:83-425, src/mod_cg_models.f90:301-429):
// vertices are numbered by increasing node id among the nodes at vertex
// positions (for P1 models, the model's own numbering), tetrahedra keep
// their order, the neighbour file lists the tetrahedron opposite each
// vertex (1-based, -1 on the outer boundary) and the nodal material and
// gravity keep the reference element's local order.
int nmm_write_model_files(const nmm_model* m, const char* base) {
  if (!m || !base) return fail(NMM_ERR_ARG, "null argument");
  const std::string b(base), ps = std::to_string(m->porder);
  const int p = m->pnp;
  std::vector<int> vid(m->nnode, -1);
  for (int k = 0; k < m->ntet; ++k)
    for (int v = 0; v < 4; ++v) vid[m->tet[(size_t)p * k + m->ref.vord[v]]] = 0;
  int nv = 0;
  for (int i = 0; i < m->nnode; ++i)
    if (vid[i] == 0) vid[i] = nv++;
  std::vector<int> ele(4 * (size_t)m->ntet);
  for (int k = 0; k < m->ntet; ++k)
    for (int v = 0; v < 4; ++v) ele[4 * (size_t)k + v] = vid[m->tet[(size_t)p * k + m->ref.vord[v]]];
  std::vector<double> xyz(3 * (size_t)nv);
  for (int i = 0; i < m->nnode; ++i)
    if (vid[i] >= 0)
      for (int c = 0; c < 3; ++c) xyz[3 * (size_t)vid[i] + c] = m->xyz[3 * (size_t)i + c];
  // neighbours across the face opposite each vertex
  std::vector<std::pair<std::array<int, 3>, int>> faces((size_t)m->ntet * 4);
  for (int k = 0; k < m->ntet; ++k)
    for (int f = 0; f < 4; ++f) {
      std::array<int, 3> a;
      int q = 0;
      for (int v = 0; v < 4; ++v)
        if (v != f) a[q++] = ele[4 * (size_t)k + v];
      std::sort(a.begin(), a.end());
      faces[4 * (size_t)k + f] = {a, 4 * k + f};
    }
  std::sort(faces.begin(), faces.end());
  std::vector<int> neigh(4 * (size_t)m->ntet, -1);
  for (size_t i = 0; i < faces.size();) {
    size_t j = i + 1;
    while (j < faces.size() && faces[j].first == faces[i].first) ++j;
    if (j - i > 2) return fail(NMM_ERR_MESH, "a face shared by more than two tetrahedra");
    if (j - i == 2) {
      neigh[faces[i].second] = faces[i + 1].second / 4 + 1;
      neigh[faces[i + 1].second] = faces[i].second / 4 + 1;
    }
    i = j;
  }
  for (auto& e : ele) ++e;  // 1-based
  auto put = [&](const std::string& path, const void* data, size_t bytes) -> int {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return fail(NMM_ERR_IO, "cannot open " + path);
    const size_t w = bytes ? std::fwrite(data, 1, bytes, f) : 0;
    std::fclose(f);
    return w == bytes ? NMM_OK : fail(NMM_ERR_IO, "short write " + path);
  };
  const std::string hdr = std::to_string(m->ntet) + " " + std::to_string(nv);
  const size_t nm = (size_t)p * m->ntet * sizeof(double);
  int rc;
  if ((rc = put(b + "_mesh.header", hdr.data(), hdr.size())) ||
      (rc = put(b + "_ele.dat", ele.data(), ele.size() * sizeof(int))) ||
      (rc = put(b + "_node.dat", xyz.data(), xyz.size() * sizeof(double))) ||
      (rc = put(b + "_neigh.dat", neigh.data(), neigh.size() * sizeof(int))) ||
      (rc = put(b + "_vp_pod_" + ps + "_true.dat", m->vp.data(), nm)) ||
      (rc = put(b + "_vs_pod_" + ps + "_true.dat", m->vs.data(), nm)) ||
      (rc = put(b + "_rho_pod_" + ps + "_true.dat", m->rho.data(), nm)))
    return rc;
  if (!m->g0.empty() &&
      (rc = put(b + "_pod_" + ps + "_potential_acceleration_true.dat", m->g0.data(), m->g0.size() * sizeof(double))))
    return rc;
  return NMM_OK;
}

int nmm_get_gravity(const nmm_model* m, const double** g0) {
  if (!m || !g0) return fail(NMM_ERR_ARG, "null argument");
  *g0 = m->g0.empty() ? nullptr : m->g0.data();
  return NMM_OK;
}

int nmm_reference(const nmm_model* m, const double** nodes_rst, const double** massm, const double** drst,
                  const double** massf, const int** fmask) {
  if (!m) return fail(NMM_ERR_ARG, "null model");
  static thread_local std::vector<double> dcat, fcat;
  static thread_local std::vector<int> mcat;
  const RefElem& R = m->ref;
  dcat.clear();
  for (int d = 0; d < 3; ++d) dcat.insert(dcat.end(), R.D[d].begin(), R.D[d].end());
  fcat.clear();
  mcat.clear();
  for (int f = 0; f < 4; ++f) {
    fcat.insert(fcat.end(), R.MF[f].begin(), R.MF[f].end());
    mcat.insert(mcat.end(), R.fmask[f].begin(), R.fmask[f].end());
  }
  if (nodes_rst) *nodes_rst = R.rst.data();
  if (massm) *massm = R.M.data();
  if (drst) *drst = dcat.data();
  if (massf) *massf = fcat.data();
  if (fmask) *fmask = mcat.data();
  return NMM_OK;
}

int nmm_write_vector(const char* path, const double* x, long long n) {
  if (!path || (!x && n > 0) || n < 0) return fail(NMM_ERR_ARG, "bad argument");
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(NMM_ERR_IO, std::string("cannot open ") + path);
  size_t w = std::fwrite(x, 8, (size_t)n, f);
  std::fclose(f);
  return w == (size_t)n ? NMM_OK : fail(NMM_ERR_IO, "short write");
}

// Fortran list-directed output of a REAL(4) value as gfortran writes it
// (nine significant digits, F form for 0.1 <= |x| < 1e9, else E form), which
// is how the reference spells the frequencies in its output file names
// (src/mod_para.f90:282-288).
static std::string fortran_real4(double v) {
  const double x = (double)(float)v;
  const double ax = std::fabs(x);
  char buf[64];
  if (ax == 0.0) {
    std::snprintf(buf, sizeof buf, "0.00000000");
  } else if (ax >= 0.1 && ax < 1e9) {
    const int e = (int)std::floor(std::log10(ax));
    std::snprintf(buf, sizeof buf, "%.*f", std::max(0, 8 - e), x);
  } else {
    std::snprintf(buf, sizeof buf, "%.8E", x);
  }
  return buf;
}

int nmm_write_results(const nmm_model* m, const char* outputdir, const char* basename, int job, int nproc,
                      double lowfreq, double upfreq, int nev, const double* X, long long ldx, char* prefix_out,
                      int prefix_len) {
  if (!m || !outputdir || !basename || nev < 0 || (nev > 0 && !X) || ldx < m->n || nproc < 1)
    return fail(NMM_ERR_ARG, "bad argument");
  const std::string p = std::to_string(m->porder), np = std::to_string(nproc);
  const std::string dir = outputdir, base = dir + basename;
  const std::string data = base + "_JOB" + std::to_string(job) + "_pod" + p + "_np" + np + "_" +
                           fortran_real4(lowfreq) + "_" + fortran_real4(upfreq);
  for (int i = 0; i < nev; ++i) {
    const std::string f = data + "_" + std::to_string(i + 1) + ".dat";
    const int rc = nmm_write_vector(f.c_str(), X + (size_t)i * ldx, m->n);
    if (rc) return rc;
  }
  // node lists in DOF order: the input id (1-based) and the status of every
  // node, int32 (src/mod_pevsl.f90:225-247)
  auto write_i32 = [&](const std::string& f, const std::vector<int>& v) -> int {
    FILE* fp = std::fopen(f.c_str(), "wb");
    if (!fp) return fail(NMM_ERR_IO, "cannot open " + f);
    const size_t w = std::fwrite(v.data(), 4, v.size(), fp);
    std::fclose(fp);
    return w == v.size() ? NMM_OK : fail(NMM_ERR_IO, "short write");
  };
  std::vector<int> vlist(m->nnode);
  for (int i = 0; i < m->nnode; ++i) vlist[i] = (m->orig.empty() ? i : m->orig[i]) + 1;
  int rc = write_i32(base + "_pod" + p + "_np" + np + "_vlist.dat", vlist);
  if (rc) return rc;
  if (m->fsexist && (rc = write_i32(base + "_pod" + p + "_np" + np + "_vstat.dat", m->vstat))) return rc;
  if (prefix_out && prefix_len > 0) {
    std::snprintf(prefix_out, (size_t)prefix_len, "%s", data.c_str());
  }
  return NMM_OK;
}

void nmm_destroy(nmm_model* m) { delete m; }

}  // extern "C"
