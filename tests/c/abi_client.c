/* A C client of libnmgpu, compiled and linked the way a NormalModes build
 * (or its Fortran bind(C) layer) would use the library: include nmgpu.h,
 * link -lnmgpu.  Checks the host-side entry points that need no GPU and,
 * given "nogpu", that nm_create fails loudly on a machine without one.
 * Prints "OK" and exits 0 when every check passes. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "nmgpu.h"

#define N 400
static double lam[N];

/* Y = diag(lam) X: an exact block operator for the moment recurrence */
static int diag_op(void* data, const double* X, double* Y, int ncols, int ld) {
  (void)data;
  for (int j = 0; j < ncols; ++j)
    for (int i = 0; i < N; ++i) Y[(size_t)j * ld + i] = lam[i] * X[(size_t)j * ld + i];
  return 0;
}

static int fails = 0;
#define CHECK(cond, msg)                                  \
  do {                                                    \
    if (!(cond)) {                                        \
      fprintf(stderr, "FAILED: %s (line %d)\n", msg, __LINE__); \
      ++fails;                                            \
    }                                                     \
  } while (0)

int main(int argc, char** argv) {
  for (int i = 0; i < N; ++i) lam[i] = i < 30 ? 0.0 : 2.0 * (i - 30) / (N - 31);
  /* moments of a diagonal operator are exact with Rademacher vectors */
  const int deg = 40;
  double mu[41];
  CHECK(nm_kpm_moments(diag_op, NULL, N, 0.0, 2.0, deg, 2, 7ull, mu) == NM_OK, "nm_kpm_moments");
  double err = 0.0, scale = 0.0;
  for (int k = 0; k <= deg; ++k) {
    double s = 0.0;
    for (int i = 0; i < N; ++i) s += cos(k * acos(lam[i] - 1.0)) * lam[i];
    s /= N;
    err = fmax(err, fabs(mu[k] - s));
    scale = fmax(scale, fabs(s));
  }
  CHECK(err <= 1e-12 * scale, "moments of a diagonal operator");
  nm_slice sl[3];
  double counts[3];
  CHECK(nm_kpm_slices(mu, deg, N, 0.0, 2.0, 10.0, 100.0, 3, sl, counts) == NM_OK, "nm_kpm_slices");
  CHECK(sl[0].f_lo_mhz == 10.0 && sl[2].f_hi_mhz == 100.0, "slice ends");
  CHECK(sl[0].f_hi_mhz == sl[1].f_lo_mhz && sl[1].f_hi_mhz == sl[2].f_lo_mhz, "slices are contiguous");
  CHECK(nm_kpm_slices(mu, deg, N, 0.0, 2.0, 0.0, 1.0, 3, sl, counts) == NM_ERR_ARG, "lower frequency 0");
  CHECK(nm_kpm_degree(0.0, 1.0, 0.5, 0.1, 4) == 0, "bad degree arguments");
  /* argument checks of the gravity adjoint terms */
  CHECK(nm_adjoint_gravity(NULL, 1, mu, N, NULL, 0, mu) == NM_ERR_ARG, "nm_adjoint_gravity(NULL)");
  nm_elem_model em;
  memset(&em, 0, sizeof(em));
  CHECK(nm_adjoint_gravity(&em, 1, mu, N, NULL, 0, mu) == NM_ERR_ARG, "nm_adjoint_gravity without g0");
  /* defaults */
  nm_opts o;
  nm_default_opts(&o);
  nm_solve_opts so;
  nm_default_solve_opts(&so);
  nm_kpm_opts ko;
  nm_default_kpm_opts(&ko);
  CHECK(ko.nvec == 16 && ko.degree == 0, "kpm defaults");
  if (argc > 1 && strcmp(argv[1], "nogpu") == 0) {
    /* no GPU: nm_create fails with NM_ERR_CUDA; the context it hands back
     * carries the message and is destroyed by the caller */
    const int rowptr[3] = {0, 1, 2}, col[2] = {0, 1};
    const double one[2] = {1.0, 1.0};
    nm_csr I2 = {2, 2, rowptr, col, one};
    nm_ctx* ctx = NULL;
    o.porder = 1;
    const int rc = nm_create(&ctx, &I2, &I2, NULL, NULL, NULL, &o);
    CHECK(rc == NM_ERR_CUDA, "nm_create without a GPU");
    CHECK(ctx != NULL && nm_last_error(ctx) != NULL && nm_last_error(ctx)[0] != '\0', "error message");
    nm_destroy(ctx);
    /* bad arguments are reported the same way */
    ctx = NULL;
    o.porder = 3;
    CHECK(nm_create(&ctx, &I2, &I2, NULL, NULL, NULL, &o) == NM_ERR_ARG, "porder 3 rejected");
    CHECK(ctx != NULL && strstr(nm_last_error(ctx), "porder") != NULL, "porder message");
    nm_destroy(ctx);
    CHECK(nm_create(NULL, &I2, &I2, NULL, NULL, NULL, &o) == NM_ERR_ARG, "NULL out");
  }
  if (fails) return 1;
  printf("OK\n");
  return 0;
}
