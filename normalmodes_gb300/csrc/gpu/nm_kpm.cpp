// Spectrum slicing by a kernel-polynomial (KPM) estimate of the eigenvalue
// density of B^-1 A.  The reference solves one interval per job and has no
// slicer; pEVSL's own slicer (kpmdos + spslicer) follows Lin, Saad & Yang,
// "Approximating spectral densities of large matrices", SIAM Review 58 (2016)
// and Li, Xi, Erlandson & Saad, "The eigenvalues slicing library (EVSL)",
// SIAM J. Sci. Comput. 41 (2019).  This is a restatement of that method with
// one change for the normal-mode pencils:
//
// The fluid-solid pencils have a large null space (the zero-frequency fluid
// modes, thousands of eigenvalues at 0 next to an interval that starts at
// 0.1 mHz, i.e. lambda ~ 4e-7).  A degree-d Chebyshev expansion smears the
// cluster over ~ (lmax - lmin) pi^2 / (2 d^2) and the plain count of
// [a, b] is then dominated by it.  So the moments are those of the
// lambda-weighted density psi(l) = sum_i lambda_i delta(l - lambda_i):
//   mu_k = tr(T_k(S) B^-1 A) / n,   S = (B^-1 A - c) / e,
// estimated with Rademacher vectors v as  v' T_k(S) (B^-1 A v)  (Hutchinson;
// unbiased for the trace of any matrix), and the count of (a, b] is
//   n / pi  int_{theta_b}^{theta_a} sum_k h_k g_k mu_k cos(k theta)
//                                   / (c + e cos theta) d theta,
// with t = cos theta, h_0 = 1, h_k = 2 and g_k the Jackson kernel.  Zero
// eigenvalues carry zero weight whatever the polynomial does at 0.  The
// slicer then cuts [a, b] at equal counts.
//
// nm_kpm_moments is host code over a block-operator callback (as pEVSL takes
// its matvecs through registered callbacks), so it runs on the CPU against
// any operator; nm_kpm_moments_ctx (nm_blocksolve.cu) runs the same estimator
// on the device block operators, and nm_slice_spectrum uses it whenever the
// context has them.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "nm_block.h"
#include "nm_internal.h"
#include "nm_ops.h"

namespace {

// Jackson kernel coefficients for degree m (g_0 = 1).
std::vector<double> jackson(int m) {
  std::vector<double> g(m + 1);
  const double th = M_PI / (m + 2);
  for (int k = 0; k <= m; ++k) g[k] = ((m + 2 - k) * std::cos(k * th) + std::sin(k * th) / std::tan(th)) / (m + 2);
  return g;
}

// The single-precision PI literal and REAL(4) frequencies of the reference's
// interval mapping (src/mod_pevsl.f90:93-99), as nm_solve uses them.
const double kPi = (double)3.14159265359f;
inline double lam_of_f(double f) {
  const double ff = (double)(float)f;
  return (2.0 * kPi * ff) * (2.0 * kPi * ff) * 1.0e-6;
}
inline double f_of_lam(double l) { return std::sqrt(l / 1.0e-6) / (2.0 * kPi); }

bool bad_bounds(double lmin, double lmax) { return !(lmax > lmin) || !std::isfinite(lmin) || !std::isfinite(lmax); }

// Cumulative count N(lambda) of (a, lambda] on a grid uniform in theta from
// theta(a) down to theta(b) (lambda increasing); running maximum so that it
// is monotone.
void cumulative(const double* mu, int m, int n, double lmin, double lmax, double a, double b, int npts,
                std::vector<double>& lam, std::vector<double>& N) {
  const double c = 0.5 * (lmax + lmin), e = 0.5 * (lmax - lmin);
  const std::vector<double> g = jackson(m);
  std::vector<double> coef(m + 1);
  for (int k = 0; k <= m; ++k) coef[k] = (k == 0 ? 1.0 : 2.0) * g[k] * mu[k];
  const double ta = std::max(-1.0, std::min(1.0, (a - c) / e)), tb = std::max(-1.0, std::min(1.0, (b - c) / e));
  const double tha = std::acos(ta), thb = std::acos(tb);
  lam.assign(npts, 0.0);
  N.assign(npts, 0.0);
  std::vector<double> f(npts);
  for (int i = 0; i < npts; ++i) {
    const double th = tha + (thb - tha) * i / (npts - 1);
    const double t = std::cos(th);
    // Clenshaw for sum_k coef_k T_k(t)
    double b1 = 0.0, b2 = 0.0;
    for (int k = m; k >= 1; --k) {
      const double b0 = coef[k] + 2.0 * t * b1 - b2;
      b2 = b1;
      b1 = b0;
    }
    const double s = coef[0] + t * b1 - b2;
    lam[i] = c + e * t;
    f[i] = s / lam[i];
  }
  const double dth = (tha - thb) / (npts - 1);
  for (int i = 1; i < npts; ++i) N[i] = N[i - 1] + 0.5 * (f[i] + f[i - 1]) * dth / M_PI * n;
  for (int i = 1; i < npts; ++i) N[i] = std::max(N[i], N[i - 1]);
}

int grid_points(int m) { return std::max(2001, 16 * m + 1); }

struct CtxOp {
  nm_ctx* c;
  std::vector<double> tmp;
};

int ctx_op(void* data, const double* X, double* Y, int ncols, int ld) {
  CtxOp* o = static_cast<CtxOp*>(data);
  int rc = nm_amv_block(o->c, X, o->tmp.data(), ncols, ld);
  if (rc) return rc;
  return nm_bsolve_block(o->c, o->tmp.data(), Y, ncols, ld);
}

}  // namespace

extern "C" {

void nm_default_kpm_opts(nm_kpm_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->nvec = 16;
  o->seed = 0x4B504Dull;
}

int nm_kpm_degree(double lmin, double lmax, double lam_lo, double lam_hi, int nslices) {
  if (bad_bounds(lmin, lmax) || !(lam_hi > lam_lo) || nslices < 1) return 0;
  // The Jackson kernel of degree d is about pi / d wide in theta = acos(t):
  // make that a quarter of the mean slice width in theta.
  const double c = 0.5 * (lmax + lmin), e = 0.5 * (lmax - lmin);
  const double ta = std::max(-1.0, std::min(1.0, (lam_lo - c) / e));
  const double tb = std::max(-1.0, std::min(1.0, (lam_hi - c) / e));
  const double dth = std::acos(ta) - std::acos(tb);
  if (!(dth > 0.0)) return 4000;
  const double d = std::ceil(4.0 * M_PI * nslices / dth);
  return (int)std::max(50.0, std::min(4000.0, d));
}

int nm_kpm_moments(nm_block_op op, void* data, int n, double lmin, double lmax, int degree, int nvec,
                   unsigned long long seed, double* mu) {
  if (!op || n <= 0 || degree < 1 || nvec < 1 || !mu || bad_bounds(lmin, lmax)) return NM_ERR_ARG;
  const double c = 0.5 * (lmax + lmin), e = 0.5 * (lmax - lmin);
  const size_t len = (size_t)n * nvec;
  std::vector<double> V(len), W0(len), W1(len), T(len);
  for (int j = 0; j < nvec; ++j)
    for (int i = 0; i < n; ++i) V[(size_t)j * n + i] = nmg::rademacher(seed, j, n, i);
  // v'w as partial sums over fixed chunks added in order: the moments, and
  // with them the slices, do not depend on the thread count.
  constexpr long long kChunk = 1 << 16;
  const long long nchunk = ((long long)len + kChunk - 1) / kChunk;
  std::vector<double> part(nchunk);
  auto dot = [&](const std::vector<double>& W) {
#pragma omp parallel for schedule(static)
    for (long long b = 0; b < nchunk; ++b) {
      double s = 0.0;
      const long long e = std::min((long long)len, (b + 1) * kChunk);
      for (long long i = b * kChunk; i < e; ++i) s += V[i] * W[i];
      part[b] = s;
    }
    double s = 0.0;
    for (long long b = 0; b < nchunk; ++b) s += part[b];
    return s;
  };
  int rc;
  if ((rc = op(data, V.data(), W0.data(), nvec, n))) return rc;  // B^-1 A V
  mu[0] = dot(W0);
  if ((rc = op(data, W0.data(), T.data(), nvec, n))) return rc;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)len; ++i) W1[i] = (T[i] - c * W0[i]) / e;
  mu[1] = dot(W1);
  for (int k = 2; k <= degree; ++k) {
    if ((rc = op(data, W1.data(), T.data(), nvec, n))) return rc;
    // W0 <- 2 S W1 - W0, then swap so that W1 holds T_k
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)len; ++i) W0[i] = 2.0 * (T[i] - c * W1[i]) / e - W0[i];
    std::swap(W0, W1);
    mu[k] = dot(W1);
  }
  for (int k = 0; k <= degree; ++k) mu[k] /= (double)len;
  return NM_OK;
}

int nm_kpm_count(const double* mu, int degree, int n, double lmin, double lmax, double lam_lo, double lam_hi,
                 double* count) {
  if (!mu || degree < 1 || n <= 0 || !count || bad_bounds(lmin, lmax) || !(lam_lo > 0.0) || !(lam_hi > lam_lo))
    return NM_ERR_ARG;
  std::vector<double> lam, N;
  cumulative(mu, degree, n, lmin, lmax, lam_lo, lam_hi, grid_points(degree), lam, N);
  *count = N.back();
  return NM_OK;
}

int nm_kpm_slices(const double* mu, int degree, int n, double lmin, double lmax, double f_lo_mhz, double f_hi_mhz,
                  int nslices, nm_slice* out, double* counts) {
  if (!mu || degree < 1 || n <= 0 || nslices < 1 || !out || bad_bounds(lmin, lmax) || !(f_lo_mhz < f_hi_mhz))
    return NM_ERR_ARG;
  const double a = lam_of_f(f_lo_mhz), b = lam_of_f(f_hi_mhz);
  if (!(a >= 1.0e-10)) return NM_ERR_ARG;  // the weighted count needs a > 0
  std::vector<double> lam, N;
  cumulative(mu, degree, n, lmin, lmax, a, b, grid_points(degree), lam, N);
  const double tot = N.back();
  std::vector<double> cut(nslices + 1);
  cut[0] = a;
  cut[nslices] = b;
  size_t i = 1;
  for (int s = 1; s < nslices; ++s) {
    const double target = tot * s / nslices;
    while (i + 1 < N.size() && N[i] < target) ++i;
    const double n0 = N[i - 1], n1 = N[i];
    const double w = n1 > n0 ? (target - n0) / (n1 - n0) : 0.5;
    cut[s] = std::max(cut[s - 1], lam[i - 1] + w * (lam[i] - lam[i - 1]));
  }
  for (int s = 0; s < nslices; ++s) {
    out[s].f_lo_mhz = s == 0 ? f_lo_mhz : out[s - 1].f_hi_mhz;
    out[s].f_hi_mhz = s == nslices - 1 ? f_hi_mhz : f_of_lam(cut[s + 1]);
  }
  if (counts)
    for (int s = 0; s < nslices; ++s) {
      const double l0 = s == 0 ? a : lam_of_f(out[s].f_lo_mhz), l1 = s == nslices - 1 ? b : lam_of_f(out[s].f_hi_mhz);
      double cnt = 0.0;
      if (l1 > l0 && nm_kpm_count(mu, degree, n, lmin, lmax, l0, l1, &cnt) != NM_OK) cnt = 0.0;
      counts[s] = cnt;
    }
  return NM_OK;
}

int nm_slice_spectrum(nm_ctx* c, double f_lo_mhz, double f_hi_mhz, int nslices, const nm_kpm_opts* opts,
                      nm_slice* out, double* counts) {
  if (!c) return NM_ERR_ARG;
  if (!out || nslices < 1 || !(f_lo_mhz < f_hi_mhz)) return nmg::set_err(c, NM_ERR_ARG, "bad slicing arguments");
  if (!(lam_of_f(f_lo_mhz) >= 1.0e-10))
    return nmg::set_err(c, NM_ERR_ARG, "slicing counts eigenvalues above 0: the lower frequency must be positive");
  nm_kpm_opts o;
  if (opts) o = *opts;
  else nm_default_kpm_opts(&o);
  double lmin, lmax;
  int rc;
  if (o.ab_bounds[1] > 0) {
    lmin = o.ab_bounds[0];
    lmax = o.ab_bounds[1];
  } else {
    int steps;
    if ((rc = nmg::lan_bounds_gen(c, 3000, 1e-5, &lmin, &lmax, &steps))) return rc;
  }
  if (bad_bounds(lmin, lmax)) return nmg::set_err(c, NM_ERR_ARG, "bad bounds of B^-1 A");
  lmax += 0.005 * (lmax - lmin);  // the polynomial must not see eigenvalues above lmax
  const int deg = o.degree > 0 ? o.degree
                               : nm_kpm_degree(lmin, lmax, lam_of_f(f_lo_mhz), lam_of_f(f_hi_mhz), nslices);
  const int nvec = o.nvec > 0 ? o.nvec : 16;
  std::vector<double> mu(deg + 1);
  // moments on the device block path when the context has it (no host
  // round trip per degree), else through the host block callbacks
  rc = nm_kpm_moments_ctx(c, lmin, lmax, deg, nvec, o.seed, mu.data());
  if (rc == NM_ERR_ARG && nmg::block_path_missing(c)) {
    CtxOp data{c, std::vector<double>((size_t)c->n * nvec)};
    rc = nm_kpm_moments(ctx_op, &data, c->n, lmin, lmax, deg, nvec, o.seed, mu.data());
  }
  if (rc) return rc;
  if ((rc = nm_kpm_slices(mu.data(), deg, c->n, lmin, lmax, f_lo_mhz, f_hi_mhz, nslices, out, counts)))
    return nmg::set_err(c, rc, "slicing failed");
  return NM_OK;
}

}  // extern "C"
