// Host-side numerics of libnmgpu: SELL-32 packing of the scaled operators,
// Chebyshev semi-iteration coefficients, the polynomial-filter design
// (pEVSL_FINDPOL_F90, src/mod_pevsl.f90:115) and the symmetric tridiagonal
// eigen-solver (Sturm bisection + inverse iteration) used by the Lanczos
// drivers.  None of this touches the GPU, so it is unit-tested on the CPU
// through the nm_test_* entry points at the end of the file.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#include "nm_internal.h"

namespace nmg {

SellHost sell_from_csr(const nm_csr* m, const double* dl, const double* dr, double sign) {
  SellHost h;
  h.nrows = m->nrows;
  h.ncols = m->ncols;
  h.nslices = (m->nrows + kSlice - 1) / kSlice;
  h.nnz = m->rowptr[m->nrows];
  h.slice_ptr.assign(h.nslices + 1, 0);
  h.row_len.resize(m->nrows);
  // Every row fills its own slots, so rows (and slices) are packed in
  // parallel; the result does not depend on the thread count.
#pragma omp parallel for schedule(static)
  for (int r = 0; r < m->nrows; ++r) h.row_len[r] = m->rowptr[r + 1] - m->rowptr[r];
#pragma omp parallel for schedule(static)
  for (int s = 0; s < h.nslices; ++s) {
    int w = 0;
    for (int r = s * kSlice; r < std::min(m->nrows, (s + 1) * kSlice); ++r) w = std::max(w, h.row_len[r]);
    h.slice_ptr[s + 1] = (long long)w * kSlice;
  }
  for (int s = 0; s < h.nslices; ++s) h.slice_ptr[s + 1] += h.slice_ptr[s];
  h.nstored = h.slice_ptr[h.nslices];
  h.col.assign(h.nstored, 0);
  h.val.assign(h.nstored, 0.0);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int r = 0; r < m->nrows; ++r) {
    const long long base = h.slice_ptr[r / kSlice] + (r % kSlice);
    for (int k = 0; k < h.row_len[r]; ++k) {
      const int q = m->rowptr[r] + k;
      const int c = m->col[q];
      double v = sign * m->val[q];
      if (dr) v = v * dr[c];
      if (dl) v = v * dl[r];
      h.col[base + (long long)k * kSlice] = c;
      h.val[base + (long long)k * kSlice] = v;
    }
    // padding columns point at the row's own last column (never read)
    for (long long k = h.row_len[r]; k * kSlice + base < h.slice_ptr[r / kSlice + 1]; ++k)
      h.col[base + k * kSlice] = h.row_len[r] ? h.col[base + (long long)(h.row_len[r] - 1) * kSlice] : 0;
  }
  return h;
}

// Coefficients of the Chebyshev semi-iteration (Saad, Alg. 12.1):
// theta = (lmax+lmin)/2, delta = (lmax-lmin)/2, sigma = theta/delta,
// rho_0 = 1/sigma, rho_{k+1} = 1/(2 sigma - rho_k), a_k = rho_{k+1} rho_k,
// c_k = 2 rho_{k+1} / delta.
void cheb_coefs(ChebSetup& s) {
  const double theta = 0.5 * (s.lmax + s.lmin), delta = 0.5 * (s.lmax - s.lmin);
  const double sigma = theta / delta;
  double rho = 1.0 / sigma;
  s.a.resize(s.deg);
  s.c.resize(s.deg);
  for (int k = 0; k < s.deg; ++k) {
    const double rn = 1.0 / (2.0 * sigma - rho);
    s.a[k] = rn * rho;
    s.c[k] = 2.0 * rn / delta;
    rho = rn;
  }
  s.inv_theta = 1.0 / theta;
}

void start_vector(std::vector<double>& v, int n, uint64_t seed) {
  v.resize(n);
  const uint64_t g = 0x9E3779B97F4A7C15ull;
  for (int i = 0; i < n; ++i) {
    uint64_t x = seed * g + (uint64_t)i + g;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x = x ^ (x >> 31);
    v[i] = 2.0 * ((double)(x >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
  }
}

// ---------------------------------------------------------------- filter design
namespace {

std::vector<double> damping(int m, int kind) {
  std::vector<double> g(m + 1, 1.0);
  if (kind == 2) {
    const double th = M_PI / (m + 1);
    for (int k = 1; k <= m; ++k) g[k] = std::sin(k * th) / (k * th);
  } else if (kind != 3) {  // Jackson (default)
    const double th = M_PI / (m + 2);
    for (int k = 0; k <= m; ++k) g[k] = ((m + 2 - k) * std::cos(k * th) + std::sin(k * th) / std::tan(th)) / (m + 2);
  }
  g[0] *= 0.5;
  return g;
}

double cheb_eval(const std::vector<double>& mu, double t) {
  const double th = std::acos(std::max(-1.0, std::min(1.0, t)));
  double s = 0.0;
  for (size_t k = 0; k < mu.size(); ++k) s += mu[k] * std::cos(k * th);
  return s;
}

double balance(const std::vector<double>& g, double tha, double thb) {
  const int m1 = (int)g.size();
  std::vector<double> w(m1);
  for (int k = 0; k < m1; ++k) w[k] = g[k] * (std::cos(k * tha) - std::cos(k * thb));
  auto f = [&](double th) {
    double s = 0.0;
    for (int k = 0; k < m1; ++k) s += w[k] * std::cos(k * th);
    return s;
  };
  auto fp = [&](double th) {
    double s = 0.0;
    for (int k = 0; k < m1; ++k) s -= w[k] * k * std::sin(k * th);
    return s;
  };
  double lo = thb, hi = tha, flo = f(lo), fhi = f(hi);
  if (flo * fhi > 0) return 0.5 * (lo + hi);
  double th = 0.5 * (lo + hi);
  for (int it = 0; it < 200; ++it) {
    const double ft = f(th);
    if (ft == 0.0) break;
    if ((ft < 0) == (flo < 0)) {
      lo = th;
      flo = ft;
    } else {
      hi = th;
      fhi = ft;
    }
    const double d = fp(th);
    double nt = d != 0.0 ? th - ft / d : 0.5 * (lo + hi);
    if (!(lo < nt && nt < hi)) nt = 0.5 * (lo + hi);
    if (std::fabs(nt - th) <= 1e-15 * std::max(1.0, std::fabs(th)) || hi - lo <= 1e-15) {
      th = nt;
      break;
    }
    th = nt;
  }
  (void)fhi;
  return th;
}

}  // namespace

// Chebyshev delta-function filter for [a, b] inside [lmin, lmax]: smallest
// degree m >= min_deg whose normalised filter (p(gamma) = 1) has dropped to
// the threshold at the interval ends; for an interior interval gamma is the
// balancing centre with p(a) = p(b).  bar = min(p(a), p(b)).
Pol find_pol(const double xintv[4], double thresh_int, double thresh_ext, int min_deg, int max_deg, int damp) {
  Pol P;
  const double a = xintv[0], b = xintv[1], lmin = xintv[2], lmax = xintv[3];
  P.cc = 0.5 * (lmax + lmin);
  P.dd = 0.5 * (lmax - lmin);
  const double aa = std::max((a - P.cc) / P.dd, -1.0);
  const double bb = std::min((b - P.cc) / P.dd, 1.0);
  const double tha = std::acos(aa), thb = std::acos(bb);
  double thresh;
  if (aa <= -1.0) {
    P.kind = 1;
    thresh = thresh_ext;
  } else if (bb >= 1.0) {
    P.kind = 2;
    thresh = thresh_ext;
  } else {
    P.kind = 0;
    thresh = thresh_int;
  }
  double gam = P.kind == 1 ? -1.0 : 1.0;
  double va = 1.0, vb = 1.0;
  int m = min_deg;
  std::vector<double> mu;
  for (m = min_deg; m <= max_deg; ++m) {
    std::vector<double> g = damping(m, damp);
    if (P.kind == 0) gam = std::cos(balance(g, tha, thb));
    const double thc = std::acos(gam);
    mu.assign(m + 1, 0.0);
    for (int k = 0; k <= m; ++k) mu[k] = g[k] * std::cos(k * thc);
    const double t = cheb_eval(mu, gam);
    for (auto& x : mu) x /= t;
    va = cheb_eval(mu, aa);
    vb = cheb_eval(mu, bb);
    if (P.kind == 0 && std::max(va, vb) <= thresh) break;
    if (P.kind == 1 && vb <= thresh) break;
    if (P.kind == 2 && va <= thresh) break;
  }
  if (m > max_deg) m = max_deg;
  P.deg = m;
  P.mu = mu;
  P.gam = gam;
  P.bar = P.kind == 0 ? std::min(va, vb) : (P.kind == 1 ? vb : va);
  return P;
}

// ---------------------------------------------------------------- tridiagonal
namespace {

// number of eigenvalues < x (Sturm sequence)
int sturm_count(const std::vector<double>& d, const std::vector<double>& e, double x, double pivmin) {
  const int k = (int)d.size();
  int cnt = 0;
  double q = d[0] - x;
  if (std::fabs(q) < pivmin) q = -pivmin;
  if (q < 0) ++cnt;
  for (int i = 1; i < k; ++i) {
    q = d[i] - x - e[i - 1] * e[i - 1] / q;
    if (std::fabs(q) < pivmin) q = -pivmin;
    if (q < 0) ++cnt;
  }
  return cnt;
}

void gersh(const std::vector<double>& d, const std::vector<double>& e, double& lo, double& hi, double& pivmin) {
  const int k = (int)d.size();
  lo = 1e300;
  hi = -1e300;
  double emax = 0.0;
  for (int i = 0; i < k; ++i) {
    double r = (i > 0 ? std::fabs(e[i - 1]) : 0.0) + (i < k - 1 ? std::fabs(e[i]) : 0.0);
    lo = std::min(lo, d[i] - r);
    hi = std::max(hi, d[i] + r);
    if (i < k - 1) emax = std::max(emax, e[i] * e[i]);
  }
  const double span = std::max(hi - lo, 1e-300);
  lo -= 2.1 * span * std::numeric_limits<double>::epsilon() * k + 2.1 * std::numeric_limits<double>::min();
  hi += 2.1 * span * std::numeric_limits<double>::epsilon() * k + 2.1 * std::numeric_limits<double>::min();
  pivmin = std::numeric_limits<double>::min() * std::max(1.0, emax);
}

double bisect_index(const std::vector<double>& d, const std::vector<double>& e, int idx, double lo, double hi,
                    double pivmin) {
  // smallest x with count(x) > idx
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (sturm_count(d, e, mid, pivmin) > idx) hi = mid;
    else lo = mid;
  }
  return 0.5 * (lo + hi);
}

struct TriLU {
  std::vector<double> u0, u1, u2, f;
  std::vector<char> piv;
};

void tri_factor(const std::vector<double>& d, const std::vector<double>& e, double sigma, double tiny, TriLU& L) {
  const int k = (int)d.size();
  L.u0.assign(k, 0.0);
  L.u1.assign(k, 0.0);
  L.u2.assign(k, 0.0);
  L.f.assign(k, 0.0);
  L.piv.assign(k, 0);
  double cd = d[0] - sigma, cu = k > 1 ? e[0] : 0.0;
  for (int i = 0; i < k - 1; ++i) {
    const double nd = e[i], nd1 = d[i + 1] - sigma, nd2 = (i + 1 < k - 1) ? e[i + 1] : 0.0;
    if (std::fabs(cd) >= std::fabs(nd)) {
      const double f = cd != 0.0 ? nd / cd : 0.0;
      L.u0[i] = cd == 0.0 ? tiny : cd;
      L.u1[i] = cu;
      L.u2[i] = 0.0;
      L.f[i] = f;
      cd = nd1 - f * cu;
      cu = nd2;
    } else {
      const double f = cd / nd;
      L.piv[i] = 1;
      L.u0[i] = nd;
      L.u1[i] = nd1;
      L.u2[i] = nd2;
      L.f[i] = f;
      const double ndd = cu - f * nd1, nuu = -f * nd2;
      cd = ndd;
      cu = nuu;
    }
  }
  L.u0[k - 1] = cd == 0.0 ? tiny : cd;
}

void tri_solve(const TriLU& L, std::vector<double>& y) {
  const int k = (int)y.size();
  for (int i = 0; i < k - 1; ++i) {
    if (L.piv[i]) std::swap(y[i], y[i + 1]);
    y[i + 1] -= L.f[i] * y[i];
  }
  y[k - 1] /= L.u0[k - 1];
  if (k > 1) y[k - 2] = (y[k - 2] - L.u1[k - 2] * y[k - 1]) / L.u0[k - 2];
  for (int i = k - 3; i >= 0; --i) y[i] = (y[i] - L.u1[i] * y[i + 1] - L.u2[i] * y[i + 2]) / L.u0[i];
}

}  // namespace

std::vector<double> tri_eigs_range(const std::vector<double>& d, const std::vector<double>& e, double lo, double hi) {
  const int k = (int)d.size();
  std::vector<double> out;
  if (k == 0) return out;
  double glo, ghi, pivmin;
  gersh(d, e, glo, ghi, pivmin);
  lo = std::max(lo, glo);
  hi = std::min(hi, ghi);
  if (lo > hi) return out;
  const int c0 = sturm_count(d, e, lo, pivmin), c1 = sturm_count(d, e, hi, pivmin);
  out.resize(std::max(0, c1 - c0));
#pragma omp parallel for schedule(dynamic, 4)
  for (int i = c0; i < c1; ++i) out[i - c0] = bisect_index(d, e, i, glo, ghi, pivmin);
  return out;
}

std::vector<double> tri_eigs_above(const std::vector<double>& d, const std::vector<double>& e, double lo) {
  return tri_eigs_range(d, e, lo, 1e300);
}

double tri_eig_index(const std::vector<double>& d, const std::vector<double>& e, int idx) {
  double glo, ghi, pivmin;
  gersh(d, e, glo, ghi, pivmin);
  return bisect_index(d, e, idx, glo, ghi, pivmin);
}

// Inverse iteration with Gram-Schmidt inside clusters of close eigenvalues
// (the scheme of LAPACK's xSTEIN, written from its published description).
void tri_eigvecs(const std::vector<double>& d, const std::vector<double>& e, const std::vector<double>& lam,
                 std::vector<double>& S) {
  const int k = (int)d.size(), m = (int)lam.size();
  S.assign((size_t)k * m, 0.0);
  if (k == 0 || m == 0) return;
  double tnorm = 0.0;
  for (int i = 0; i < k; ++i)
    tnorm = std::max(tnorm, std::fabs(d[i]) + (i > 0 ? std::fabs(e[i - 1]) : 0) + (i < k - 1 ? std::fabs(e[i]) : 0));
  const double eps = std::numeric_limits<double>::epsilon();
  const double ortol = 1e-3 * tnorm, pertol = 10.0 * eps * tnorm, tiny = eps * tnorm;
  // clusters of consecutive eigenvalues closer than ortol
  std::vector<int> cstart;
  for (int j = 0; j < m; ++j)
    if (j == 0 || lam[j] - lam[j - 1] > ortol) cstart.push_back(j);
  cstart.push_back(m);
  const int ncl = (int)cstart.size() - 1;
#pragma omp parallel for schedule(dynamic, 1)
  for (int cl = 0; cl < ncl; ++cl) {
    TriLU L;
    std::vector<double> x(k);
    double prev = -1e300;
    for (int j = cstart[cl]; j < cstart[cl + 1]; ++j) {
      double sigma = lam[j];
      if (j > cstart[cl] && sigma - prev < pertol) sigma = prev + pertol;
      prev = sigma;
      tri_factor(d, e, sigma, tiny, L);
      std::vector<double> sv;
      start_vector(sv, k, 0xA5A5ull + (uint64_t)j);
      x = sv;
      for (int it = 0; it < 4; ++it) {
        tri_solve(L, x);
        for (int q = cstart[cl]; q < j; ++q) {
          const double* s = &S[(size_t)q * k];
          double dp = 0.0;
          for (int i = 0; i < k; ++i) dp += s[i] * x[i];
          for (int i = 0; i < k; ++i) x[i] -= dp * s[i];
        }
        double nrm = 0.0;
        for (int i = 0; i < k; ++i) nrm += x[i] * x[i];
        nrm = std::sqrt(nrm);
        if (nrm == 0.0) {
          x = sv;
          continue;
        }
        for (int i = 0; i < k; ++i) x[i] /= nrm;
      }
      std::copy(x.begin(), x.end(), S.begin() + (size_t)j * k);
    }
  }
}

}  // namespace nmg

// ---------------------------------------------------------------- CPU test hooks
extern "C" {

// Filter design without a GPU (for the CPU test-suite).  mu_out needs
// max_deg + 1 entries.  Returns the degree.
int nm_test_find_pol(const double* xintv, double thresh_int, double thresh_ext, int damping, double* mu_out,
                     int max_deg, double* cc_dd_gam_bar) {
  nmg::Pol P = nmg::find_pol(xintv, thresh_int, thresh_ext, 2, max_deg, damping);
  for (int k = 0; k <= P.deg && k <= max_deg; ++k) mu_out[k] = P.mu[k];
  cc_dd_gam_bar[0] = P.cc;
  cc_dd_gam_bar[1] = P.dd;
  cc_dd_gam_bar[2] = P.gam;
  cc_dd_gam_bar[3] = P.bar;
  return P.deg;
}

// Eigenvalues of a symmetric tridiagonal in [lo, hi] and their vectors
// (k x m column-major).  Returns m (<= cap).
int nm_test_tridiag(const double* d, const double* e, int k, double lo, double hi, double* lam, double* vec, int cap) {
  std::vector<double> dd(d, d + k), ee(e, e + (k > 0 ? k - 1 : 0));
  std::vector<double> w = nmg::tri_eigs_range(dd, ee, lo, hi);
  int m = std::min((int)w.size(), cap);
  w.resize(m);
  std::vector<double> S;
  nmg::tri_eigvecs(dd, ee, w, S);
  std::copy(w.begin(), w.end(), lam);
  if (vec) std::copy(S.begin(), S.end(), vec);
  return m;
}

// SELL packing check: returns stored element count and fills row lengths.
long long nm_test_sell(int nrows, int ncols, const int* rowptr, const int* col, const double* val, int* row_len,
                       long long* slice_ptr) {
  nm_csr m{nrows, ncols, rowptr, col, val};
  nmg::SellHost h = nmg::sell_from_csr(&m, nullptr, nullptr, 1.0);
  std::copy(h.row_len.begin(), h.row_len.end(), row_len);
  std::copy(h.slice_ptr.begin(), h.slice_ptr.end(), slice_ptr);
  return h.nstored;
}

// SELL packing with scaling: the packed column indices and values
// (nstored each, returned by nm_test_sell for the same matrix).
void nm_test_sell_arrays(int nrows, int ncols, const int* rowptr, const int* col, const double* val,
                         const double* dl, const double* dr, double sign, int* col_out, double* val_out) {
  nm_csr m{nrows, ncols, rowptr, col, val};
  nmg::SellHost h = nmg::sell_from_csr(&m, dl, dr, sign);
  std::copy(h.col.begin(), h.col.end(), col_out);
  std::copy(h.val.begin(), h.val.end(), val_out);
}

void nm_test_start_vector(int n, double* out) {
  std::vector<double> v;
  nmg::start_vector(v, n, nmg::kStartSeed);
  std::copy(v.begin(), v.end(), out);
}

}  // extern "C"
