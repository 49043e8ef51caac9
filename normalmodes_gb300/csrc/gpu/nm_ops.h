// Operator-level routines shared by the context and solver translation units.
#pragma once

#include <functional>

#include "nm_internal.h"

namespace nmg {

int alloc_work(nm_ctx* c);
// Scaled operators on device vectors, enqueued on c->stream.
void amv64(nm_ctx* c, const double* x, double* y);     // sparseAV / sparsefsAV
void bsolve64(nm_ctx* c, const double* x, double* y);  // solveBV
// One filter degree step (B-solve + A-op + recurrence) on fixed buffers (timing).
void filter_step64(nm_ctx* c, const double* vk, double* vkm1, double* vkp1, double* yacc);
// y = p(A B~^-1) z, FP64 or FP32 (mixed) arithmetic
void chebav(nm_ctx* c, const Pol& pol, const double* z, double* y, bool mixed);

int lan_bounds_std(nm_ctx* c, int which, int msteps, double tol, double* lmin, double* lmax, int* steps);
int lan_bounds_gen(nm_ctx* c, int msteps, double tol, double* lmin, double* lmax, int* steps);

int ensure_basis(nm_ctx* c, Basis& b, int n, int ncols);
void free_basis(Basis& b);

}  // namespace nmg
