/*
 * nm_oracle.c -- CPU FP64 restatement of the operator layer of the
 * NormalModes eigensolve path.  TEST INFRASTRUCTURE ONLY: it is the parity
 * checker for the CUDA library and the timed CPU baseline; nothing in the
 * product links or calls it.
 *
 * Restated from the reference (file:line within js1019/NormalModes):
 *   Bdiagscaling   src/mod_matvec.f90:252-342   D = diag(B)^-1/2, B_s = D B D
 *   Apdiagscaling  src/mod_matvec.f90:345-441   Ap := -Ap (:137), D_p, Ap_s
 *   sparseAV       src/mod_matvec.f90:445-458   w = D (A (D v))
 *   sparseBV       src/mod_matvec.f90:461-472   w = B_s v
 *   solveBV        src/mod_matvec.f90:475-483   w = Cheb_{B_s}(v)
 *   sparseApV      src/mod_matvec.f90:485-496   w = Ap_s v
 *   sparsefsAV     src/mod_matvec.f90:498-520   w = D(Ad D v + E D_p Cheb_{Ap_s}(D_p ET D v))
 * The Chebyshev semi-iteration (pEVSL chebiter, not vendored in the
 * reference) follows the published method (Golub & Varga 1961; Saad,
 * "Iterative Methods for Sparse Linear Systems", Alg. 12.1) with a zero
 * initial guess and `deg` matrix-vector products; the polynomial filter
 * application (pEVSL ChebAv) is the Chebyshev three-term recurrence of the
 * EVSL papers (Li, Xi, Vecharynski, Yang, Saad, SISC 2016) applied to
 * A B~^-1 as in the generalized-eigenproblem form.
 *
 * Parity is pinned against independent dense eigensolves of the same
 * operators and against analytic spectra; the reference publishes no golden
 * vectors for this path.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  int nrows, ncols;
  int* rp;
  int* ci;
  double* v;
} ocsr;

typedef struct {
  int fs; /* 1: fluid-solid operator (sparsefsAV); 0: sparseAV */
  int n, np;
  ocsr A;  /* A or Ad (unscaled) */
  ocsr Bs; /* scaled B */
  ocsr Aps;
  ocsr E, ET;
  double* D;  /* n */
  double* Dp; /* np */
  /* Chebyshev solve parameters */
  double b_lmin, b_lmax;
  int b_deg;
  double ap_lmin, ap_lmax;
  int ap_deg;
  double* wk; /* workspace */
} octx;

static void csr_copy(ocsr* dst, int nr, int nc, const int* rp, const int* ci, const double* v) {
  long long nnz = rp[nr];
  dst->nrows = nr;
  dst->ncols = nc;
  dst->rp = (int*)malloc(sizeof(int) * (nr + 1));
  dst->ci = (int*)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
  dst->v = (double*)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
  memcpy(dst->rp, rp, sizeof(int) * (nr + 1));
  if (nnz) {
    memcpy(dst->ci, ci, sizeof(int) * nnz);
    memcpy(dst->v, v, sizeof(double) * nnz);
  }
}

static void csr_free(ocsr* c) {
  free(c->rp);
  free(c->ci);
  free(c->v);
  memset(c, 0, sizeof(*c));
}

/* y = C x */
static void spmv(const ocsr* c, const double* x, double* y) {
#pragma omp parallel for schedule(static) if (c->nrows > 20000)
  for (int i = 0; i < c->nrows; ++i) {
    double s = 0.0;
    for (int k = c->rp[i]; k < c->rp[i + 1]; ++k) s += c->v[k] * x[c->ci[k]];
    y[i] = s;
  }
}

/* diag(C)^-1/2 with sign flip option (Bdiagscaling :270-279, Apdiagscaling :356-365) */
static int inv_sqrt_diag(const ocsr* c, double sign, double* d) {
  for (int i = 0; i < c->nrows; ++i) {
    double dv = 0.0;
    int found = 0;
    for (int k = c->rp[i]; k < c->rp[i + 1]; ++k)
      if (c->ci[k] == i) {
        dv = sign * c->v[k];
        found = 1;
      }
    if (!found || !(dv > 0)) return -1;
    d[i] = 1.0 / sqrt(dv);
  }
  return 0;
}

octx* or_create(int fs, int n, int np, const int* a_rp, const int* a_ci, const double* a_v, const int* b_rp,
                const int* b_ci, const double* b_v, const int* ap_rp, const int* ap_ci, const double* ap_v,
                const int* e_rp, const int* e_ci, const double* e_v, const int* et_rp, const int* et_ci,
                const double* et_v) {
  octx* c = (octx*)calloc(1, sizeof(octx));
  c->fs = fs;
  c->n = n;
  c->np = np;
  csr_copy(&c->A, n, n, a_rp, a_ci, a_v);
  csr_copy(&c->Bs, n, n, b_rp, b_ci, b_v);
  c->D = (double*)malloc(sizeof(double) * n);
  if (inv_sqrt_diag(&c->Bs, 1.0, c->D)) {
    free(c);
    return NULL;
  }
  /* B_s(i,j) = B(i,j) D_j D_i  (src/mod_matvec.f90:336) */
  for (int i = 0; i < n; ++i)
    for (int k = c->Bs.rp[i]; k < c->Bs.rp[i + 1]; ++k) c->Bs.v[k] = c->Bs.v[k] * c->D[c->Bs.ci[k]] * c->D[i];
  if (fs) {
    csr_copy(&c->Aps, np, np, ap_rp, ap_ci, ap_v);
    csr_copy(&c->E, n, np, e_rp, e_ci, e_v);
    csr_copy(&c->ET, np, n, et_rp, et_ci, et_v);
    c->Dp = (double*)malloc(sizeof(double) * (np > 0 ? np : 1));
    if (inv_sqrt_diag(&c->Aps, -1.0, c->Dp)) {
      free(c);
      return NULL;
    }
    /* Ap_s(i,j) = -Ap(i,j) Dp_j Dp_i  (src/mod_matvec.f90:422) */
    for (int i = 0; i < np; ++i)
      for (int k = c->Aps.rp[i]; k < c->Aps.rp[i + 1]; ++k)
        c->Aps.v[k] = -c->Aps.v[k] * c->Dp[c->Aps.ci[k]] * c->Dp[i];
  }
  size_t wn = (size_t)(n > np ? n : np);
  c->wk = (double*)malloc(sizeof(double) * wn * 16);
  return c;
}

void or_destroy(octx* c) {
  if (!c) return;
  csr_free(&c->A);
  csr_free(&c->Bs);
  csr_free(&c->Aps);
  csr_free(&c->E);
  csr_free(&c->ET);
  free(c->D);
  free(c->Dp);
  free(c->wk);
  free(c);
}

void or_get_scaling(const octx* c, double* D, double* Dp) {
  if (D) memcpy(D, c->D, sizeof(double) * c->n);
  if (Dp && c->fs) memcpy(Dp, c->Dp, sizeof(double) * c->np);
}

void or_get_scaled_values(const octx* c, double* bs_v, double* aps_v) {
  if (bs_v) memcpy(bs_v, c->Bs.v, sizeof(double) * c->Bs.rp[c->n]);
  if (aps_v && c->fs) memcpy(aps_v, c->Aps.v, sizeof(double) * c->Aps.rp[c->np]);
}

void or_set_cheb(octx* c, int which, double lmin, double lmax, int deg) {
  if (which == 0) {
    c->b_lmin = lmin;
    c->b_lmax = lmax;
    c->b_deg = deg;
  } else {
    c->ap_lmin = lmin;
    c->ap_lmax = lmax;
    c->ap_deg = deg;
  }
}

/* Chebyshev semi-iteration for M z = b, x0 = 0, `deg` products with M.
 * Iterate k = 0..deg-1:  x += d;  r -= M d;  rho' = 1/(2 sigma - rho);
 * d = rho' rho d + (2 rho'/delta) r.  Output x + d (degree-deg polynomial). */
static void cheb_solve(const ocsr* M, double lmin, double lmax, int deg, const double* b, double* x, double* wk) {
  const int n = M->nrows;
  double* r = wk;
  double* d = wk + n;
  double* t = wk + 2 * (size_t)n;
  const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
  const double sigma = theta / delta;
  double rho = 1.0 / sigma;
#pragma omp parallel for schedule(static) if (n > 20000)
  for (int i = 0; i < n; ++i) {
    x[i] = 0.0;
    r[i] = b[i];
    d[i] = b[i] / theta;
  }
  for (int k = 0; k < deg; ++k) {
    spmv(M, d, t);
    const double rn = 1.0 / (2.0 * sigma - rho);
    const double a = rn * rho, cc = 2.0 * rn / delta;
#pragma omp parallel for schedule(static) if (n > 20000)
    for (int i = 0; i < n; ++i) {
      x[i] += d[i];
      r[i] -= t[i];
      d[i] = a * d[i] + cc * r[i];
    }
    rho = rn;
  }
#pragma omp parallel for schedule(static) if (n > 20000)
  for (int i = 0; i < n; ++i) x[i] += d[i];
}

void or_bmv(octx* c, const double* x, double* y) { spmv(&c->Bs, x, y); }
void or_apmv(octx* c, const double* x, double* y) { spmv(&c->Aps, x, y); }
void or_bsolve(octx* c, const double* b, double* x) {
  cheb_solve(&c->Bs, c->b_lmin, c->b_lmax, c->b_deg, b, x, c->wk + 8 * (size_t)c->n);
}
void or_apsolve(octx* c, const double* b, double* x) {
  cheb_solve(&c->Aps, c->ap_lmin, c->ap_lmax, c->ap_deg, b, x, c->wk + 8 * (size_t)c->n);
}

/* sparseAV / sparsefsAV */
void or_amv(octx* c, const double* v, double* w) {
  const int n = c->n, np = c->np;
  double* v0 = c->wk;
  double* w0 = c->wk + n;
#pragma omp parallel for schedule(static) if (n > 20000)
  for (int i = 0; i < n; ++i) v0[i] = v[i] * c->D[i];
  spmv(&c->A, v0, w0);
  if (!c->fs) {
#pragma omp parallel for schedule(static) if (n > 20000)
    for (int i = 0; i < n; ++i) w[i] = w0[i] * c->D[i];
    return;
  }
  double* x0 = c->wk + 2 * (size_t)n;
  double* y0 = x0 + np;
  double* w1 = c->wk + 3 * (size_t)n;
  spmv(&c->ET, v0, x0);
#pragma omp parallel for schedule(static) if (np > 20000)
  for (int i = 0; i < np; ++i) x0[i] = x0[i] * c->Dp[i];
  cheb_solve(&c->Aps, c->ap_lmin, c->ap_lmax, c->ap_deg, x0, y0, c->wk + 8 * (size_t)n);
#pragma omp parallel for schedule(static) if (np > 20000)
  for (int i = 0; i < np; ++i) y0[i] = y0[i] * c->Dp[i];
  spmv(&c->E, y0, w1);
#pragma omp parallel for schedule(static) if (n > 20000)
  for (int i = 0; i < n; ++i) w[i] = (w0[i] + w1[i]) * c->D[i];
}

/* Filter y = p(A B~^-1) v with p = sum_k mu_k T_k((X - cc)/dd). */
void or_chebav(octx* c, int m, const double* mu, double cc, double dd, const double* v, double* y) {
  const int n = c->n;
  double* vk = c->wk + 4 * (size_t)n;
  double* vkp1 = c->wk + 5 * (size_t)n;
  double* vkm1 = c->wk + 6 * (size_t)n;
  double* w2 = c->wk + 7 * (size_t)n;
#pragma omp parallel for schedule(static) if (n > 20000)
  for (int i = 0; i < n; ++i) {
    vk[i] = v[i];
    vkm1[i] = 0.0;
    y[i] = mu[0] * v[i];
  }
  for (int k = 1; k <= m; ++k) {
    or_bsolve(c, vk, w2);
    or_amv(c, w2, vkp1);
    const double s = (k == 1 ? 1.0 : 2.0) / dd;
    const double pm = k == 1 ? 0.0 : 1.0;
    const double muk = mu[k];
#pragma omp parallel for schedule(static) if (n > 20000)
    for (int i = 0; i < n; ++i) {
      double t = s * (vkp1[i] - cc * vk[i]) - pm * vkm1[i];
      vkp1[i] = t;
      y[i] += muk * t;
    }
    double* tmp = vkm1;
    vkm1 = vk;
    vk = vkp1;
    vkp1 = tmp;
  }
}

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void or_set_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}
