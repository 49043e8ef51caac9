// Eigensolve driver of libnmgpu: Lanczos bounds, the polynomial filter
// p(A B~^-1), polynomial-filtered non-restart Lanczos with full
// reorthogonalisation, Ritz vectors and the residual check.
//
// Restates pnm_apply_pevsl (src/mod_pevsl.f90:16-222) and the pEVSL routines
// it calls -- pEVSL_LANBOUNDS_F90 (:84), pEVSL_FINDPOL_F90 (:115),
// pEVSL_CHEBLANNR_F90 (:122), pEVSL_COPY_RESULT_F90 (:130) -- from the
// published EVSL methods; pEVSL itself is not part of the reference.
// Choices the reference leaves open are fixed to the same values as the CPU
// oracle: deterministic splitmix64 start vector, bounds checked every 10
// steps, Lanczos convergence tested at step 50 and every 50 steps after,
// two classical Gram-Schmidt passes, Jackson damping.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "nm_block.h"
#include "nm_internal.h"
#include "nm_ops.h"

namespace nmg {

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

constexpr int kT = 256;
inline int nb(long long n) { return (int)((n + kT - 1) / kT); }

// U(:, j) = V(:, 0..kdim-1) S(:, j) for j < nc; S column-major kdim x nc.
constexpr int kRitzCols = 16;
__global__ void __launch_bounds__(kT) k_ritz(double* const* __restrict__ chunks, size_t ld, int kdim,
                                             const double* __restrict__ S, int nc, double* __restrict__ U,
                                             size_t ldu, int n) {
  __shared__ double st[64][kRitzCols];
  const int i = blockIdx.x * kT + threadIdx.x;
  const int j0 = blockIdx.y * kRitzCols;
  const int ncol = min(kRitzCols, nc - j0);
  double acc[kRitzCols];
#pragma unroll
  for (int q = 0; q < kRitzCols; ++q) acc[q] = 0.0;
  for (int c0 = 0; c0 < kdim; c0 += 64) {
    const int cn = min(64, kdim - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < 64 * kRitzCols; t += kT) {
      const int cc = t / kRitzCols, q = t % kRitzCols;
      st[cc][q] = (cc < cn && q < ncol) ? S[(size_t)(j0 + q) * kdim + c0 + cc] : 0.0;
    }
    __syncthreads();
    if (i < n) {
      const double* base = chunks[c0 / Basis::kChunk] + i;
      for (int cc = 0; cc < cn; ++cc) {
        const double v = __ldg(base + (size_t)cc * ld);
#pragma unroll
        for (int q = 0; q < kRitzCols; ++q) acc[q] = fma(v, st[cc][q], acc[q]);
      }
    }
  }
  if (i < n)
    for (int q = 0; q < ncol; ++q) U[(size_t)(j0 + q) * ldu + i] = acc[q];
}

__global__ void k_resid(const double* __restrict__ w, const double* __restrict__ bw, double th, double* __restrict__ r,
                        int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) r[i] = fma(-th, bw[i], w[i]);
}

// Dot product brought back to the host.  A CUDA failure is recorded in the
// context (c->cuda_failed) and returns NaN, which every caller treats as an
// error.
double dot_sync(nm_ctx* c, const double* x, const double* y, int n) {
  dev_dot(x, y, n, c->red, c->scal, c->stream);
  cudaError_t e = cudaMemcpyAsync(c->h_scal, c->scal, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->h_scal + 8, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    c->cuda_failed = true;
    set_err(c, NM_ERR_CUDA, std::string("device error: ") + cudaGetErrorString(e));
    return std::nan("");
  }
  if (*(int*)(c->h_scal + 8) != 0) {
    c->cuda_failed = true;
    set_err(c, NM_ERR_TIMEOUT, "a grid barrier of the persistent Chebyshev kernel timed out");
    return std::nan("");
  }
  return c->h_scal[0];
}

// Ritz values and residual estimates of the extreme eigenpairs of T.
void tri_extremes(const std::vector<double>& d, const std::vector<double>& e, double beta, double& th0, double& th1,
                  double& r0, double& r1) {
  const int k = (int)d.size();
  th0 = tri_eig_index(d, e, 0);
  th1 = tri_eig_index(d, e, k - 1);
  std::vector<double> lam = {th0, th1}, S;
  if (k == 1) {
    r0 = r1 = std::fabs(beta);
    return;
  }
  tri_eigvecs(d, e, lam, S);
  r0 = std::fabs(beta * S[(size_t)0 * k + k - 1]);
  r1 = std::fabs(beta * S[(size_t)1 * k + k - 1]);
}

using Apply = std::function<void(const double*, double*)>;

// Lanczos with full reorthogonalisation for extreme-eigenvalue bounds.
// Standard form if solve is empty; generalized (B~^-1 A, B~^-1 inner
// product, z = B~ v carried) otherwise.
int lanczos_bounds(nm_ctx* c, int nn, const Apply& op, const Apply& solve, int msteps, double tol, double* lmin,
                   double* lmax, int* steps, double* znew, double* vnew) {
  msteps = std::min(std::min(msteps, nn), kMaxCols - 1);
  const bool gen = (bool)solve;
  Basis V, Zb;
  int rc;
  if ((rc = ensure_basis(c, V, nn, 1))) return rc;
  if (gen && (rc = ensure_basis(c, Zb, nn, 1))) return rc;
  Basis& Z = gen ? Zb : V;
  std::vector<double> h;
  start_vector(h, nn, kStartSeed);
  if (gen) {
    NM_CUDA(c, cudaMemcpyAsync(Z.col(0), h.data(), sizeof(double) * nn, cudaMemcpyHostToDevice, c->stream));
    solve(Z.col(0), V.col(0));
    const double t = 1.0 / std::sqrt(dot_sync(c, V.col(0), Z.col(0), nn));
    dev_scale(Z.col(0), Z.col(0), t, nn, c->stream);
    dev_scale(V.col(0), V.col(0), t, nn, c->stream);
  } else {
    double s = 0;
    for (double x : h) s += x * x;
    const double t = 1.0 / std::sqrt(s);
    for (double& x : h) x *= t;
    NM_CUDA(c, cudaMemcpyAsync(V.col(0), h.data(), sizeof(double) * nn, cudaMemcpyHostToDevice, c->stream));
  }
  std::vector<double> alpha, beta;
  double lo = 0, hi = 0;
  int k = 0;
  for (k = 0; k < msteps; ++k) {
    op(V.col(k), znew);
    if (k > 0) dev_axpy(znew, Z.col(k - 1), -beta[k - 1], nn, c->stream);
    const double a = dot_sync(c, V.col(k), znew, nn);
    alpha.push_back(a);
    dev_axpy(znew, Z.col(k), -a, nn, c->stream);
    for (int p = 0; p < 2; ++p) reorth_pass(V, Z, k + 1, znew, nn, c->red, c->hbuf, c->stream);
    double b;
    if (gen) {
      solve(znew, vnew);
      b = std::sqrt(std::max(dot_sync(c, vnew, znew, nn), 0.0));
    } else {
      b = std::sqrt(std::max(dot_sync(c, znew, znew, nn), 0.0));
    }
    if (!std::isfinite(a) || !std::isfinite(b)) {
      free_basis(V);
      free_basis(Zb);
      return c->cuda_failed ? (c->err.find("timed out") != std::string::npos ? NM_ERR_TIMEOUT : NM_ERR_CUDA)
                           : set_err(c, NM_ERR_NUMERIC, "non-finite value in Lanczos bounds");
    }
    beta.push_back(b);
    const bool last = (k == msteps - 1) || b == 0.0;
    if ((k + 1) % 10 == 0 || last) {
      std::vector<double> e(beta.begin(), beta.end() - 1);
      double th0, th1, r0, r1;
      tri_extremes(alpha, e, b, th0, th1, r0, r1);
      const double scale = std::max(std::fabs(th0), std::fabs(th1));
      lo = th0 - r0;
      hi = th1 + r1;
      if ((r0 <= tol * scale && r1 <= tol * scale) || last) break;
    }
    if ((rc = ensure_basis(c, V, nn, k + 2))) return rc;
    if (gen && (rc = ensure_basis(c, Zb, nn, k + 2))) return rc;
    if (gen) {
      dev_scale(V.col(k + 1), vnew, 1.0 / b, nn, c->stream);
      dev_scale(Zb.col(k + 1), znew, 1.0 / b, nn, c->stream);
    } else {
      dev_scale(V.col(k + 1), znew, 1.0 / b, nn, c->stream);
    }
  }
  free_basis(V);
  free_basis(Zb);
  *lmin = lo;
  *lmax = hi;
  *steps = k + 1;
  NM_CUDA(c, cudaGetLastError());
  return NM_OK;
}

template <typename VT, typename XT>
void chebav_t(nm_ctx* c, const Sell<VT>& A, const Sell<VT>& Bm, const Sell<VT>& Apm, const Sell<VT>& Em,
              const Sell<VT>& ETm, const Pol& pol, XT* vk, XT* vkm1, XT* vkp1, XT* w2, XT* bwork, XT* x0, XT* y0,
              XT* apwork, XT* y) {
  const int n = c->n;
  cudaStream_t s = c->stream;
  for (int k = 1; k <= pol.deg; ++k) {
    cheb_solve<VT, XT>(Bm, c->chebB, vk, w2, bwork, s);
    if (c->fs) {
      spmv<VT, XT>(ETm, w2, x0, s);
      if (c->coop_blocks > 0)
        cheb_solve_persistent<VT, XT>(Apm, c->chebAp, x0, y0, apwork, c->bar, c->d_status, c->coop_blocks, s);
      else
        cheb_solve<VT, XT>(Apm, c->chebAp, x0, y0, apwork, s);
    }
    FiltEpi ep;
    ep.mode = 1;
    ep.s = (k == 1 ? 1.0 : 2.0) / pol.dd;
    ep.cc = pol.cc;
    ep.pm = k == 1 ? 0.0 : 1.0;
    ep.mu = pol.mu[k];
    amv_fused<VT, XT>(A, c->fs ? &Em : nullptr, w2, y0, vkp1, vk, vkm1, y, ep, s);
    XT* t = vkm1;
    vkm1 = vk;
    vk = vkp1;
    vkp1 = t;
  }
  (void)n;
}

}  // namespace

// ---------------------------------------------------------------- basis
int ensure_basis(nm_ctx* c, Basis& b, int n, int ncols) {
  if (b.n == 0) {
    b.n = n;
    b.ld = ((size_t)n + 31) / 32 * 32;
  }
  const int need = (ncols + Basis::kChunk - 1) / Basis::kChunk;
  if ((int)b.chunks.size() >= need) return NM_OK;
  while ((int)b.chunks.size() < need) {
    double* p = nullptr;
    cudaError_t e = cudaMalloc(&p, b.ld * Basis::kChunk * sizeof(double));
    if (e != cudaSuccess) return set_err(c, NM_ERR_OOM, "Lanczos basis allocation failed");
    b.chunks.push_back(p);
    c->dev_bytes += b.ld * Basis::kChunk * sizeof(double);
  }
  if (b.d_chunks_cap < (int)b.chunks.size()) {
    if (b.d_chunks) cudaFree(b.d_chunks);
    b.d_chunks_cap = std::max(64, 2 * (int)b.chunks.size());
    NM_CUDA(c, cudaMalloc(&b.d_chunks, sizeof(double*) * b.d_chunks_cap));
  }
  NM_CUDA(c, cudaMemcpyAsync(b.d_chunks, b.chunks.data(), sizeof(double*) * b.chunks.size(), cudaMemcpyHostToDevice,
                             c->stream));
  NM_CUDA(c, cudaStreamSynchronize(c->stream));
  return NM_OK;
}

void free_basis(Basis& b) {
  for (double* p : b.chunks) cudaFree(p);
  if (b.d_chunks) cudaFree(b.d_chunks);
  b = Basis();
}

// ---------------------------------------------------------------- operators
void bsolve64(nm_ctx* c, const double* x, double* y) {
  cheb_solve<double, double>(c->B, c->chebB, x, y, c->w[4], c->stream);
  ++c->n_bsolve;
  c->n_spmv += c->chebB.deg;
}

void amv64(nm_ctx* c, const double* x, double* y) {
  FiltEpi ep;
  if (c->fs) {
    spmv<double, double>(c->ET, x, c->w[12], c->stream);
    if (c->coop_blocks > 0)
      cheb_solve_persistent<double, double>(c->Ap, c->chebAp, c->w[12], c->w[13], c->w[14], c->bar, c->d_status,
                                            c->coop_blocks, c->stream);
    else
      cheb_solve<double, double>(c->Ap, c->chebAp, c->w[12], c->w[13], c->w[14], c->stream);
    amv_fused<double, double>(c->A, &c->E, x, c->w[13], y, nullptr, nullptr, nullptr, ep, c->stream);
    c->n_spmv += 2 + c->chebAp.deg;
  } else {
    amv_fused<double, double>(c->A, nullptr, x, nullptr, y, nullptr, nullptr, nullptr, ep, c->stream);
    ++c->n_spmv;
  }
  ++c->n_amv;
}

void filter_step64(nm_ctx* c, const double* vk, double* vkm1, double* vkp1, double* yacc) {
  Pol p;
  p.deg = 2;
  p.mu = {0.0, 0.0, 0.5};
  p.cc = 0.5;
  p.dd = 0.5;
  // one degree step: solve, A-op, recurrence (k = 2 branch)
  cheb_solve<double, double>(c->B, c->chebB, vk, c->w[11], c->w[4], c->stream);
  if (c->fs) {
    spmv<double, double>(c->ET, c->w[11], c->w[12], c->stream);
    if (c->coop_blocks > 0)
      cheb_solve_persistent<double, double>(c->Ap, c->chebAp, c->w[12], c->w[13], c->w[14], c->bar, c->d_status,
                                            c->coop_blocks, c->stream);
    else
      cheb_solve<double, double>(c->Ap, c->chebAp, c->w[12], c->w[13], c->w[14], c->stream);
  }
  FiltEpi ep;
  ep.mode = 1;
  ep.s = 2.0 / p.dd;
  ep.cc = p.cc;
  ep.pm = 1.0;
  ep.mu = 0.5;
  amv_fused<double, double>(c->A, c->fs ? &c->E : nullptr, c->w[11], c->w[13], vkp1, vk, vkm1, yacc, ep, c->stream);
}

void chebav(nm_ctx* c, const Pol& pol, const double* z, double* y, bool mixed) {
  const int n = c->n;
  if (!mixed) {
    dev_init_filter(c->w[8], c->w[9], y, z, pol.mu[0], n, c->stream);
    chebav_t<double, double>(c, c->A, c->B, c->Ap, c->E, c->ET, pol, c->w[8], c->w[9], c->w[10], c->w[11], c->w[4],
                             c->w[12], c->w[13], c->w[14], y);
  } else {
    float* zf = c->w32[10];
    float* yf = c->w32[11];
    dev_d2f(zf, z, n, c->stream);
    dev_init_filter32(c->w32[3], c->w32[4], yf, zf, pol.mu[0], n, c->stream);
    chebav_t<float, float>(c, c->A32, c->B32, c->Ap32, c->E32, c->ET32, pol, c->w32[3], c->w32[4], c->w32[5],
                           c->w32[6], c->w32[2], c->w32[7], c->w32[8], c->w32[9], yf);
    dev_f2d(y, yf, n, c->stream);
  }
  c->n_amv += pol.deg;
  c->n_bsolve += pol.deg;
  c->n_spmv += (long long)pol.deg * (c->chebB.deg + (c->fs ? 2 + c->chebAp.deg : 1));
}

int lan_bounds_std(nm_ctx* c, int which, int msteps, double tol, double* lmin, double* lmax, int* steps) {
  const Sell<double>& M = which == 0 ? c->B : c->Ap;
  const int nn = which == 0 ? c->n : c->np;
  Apply op = [c, &M](const double* x, double* y) { spmv<double, double>(M, x, y, c->stream); };
  double* znew = which == 0 ? c->w[0] : c->w[12];
  double* vnew = which == 0 ? c->w[1] : c->w[13];
  return lanczos_bounds(c, nn, op, Apply(), msteps, tol, lmin, lmax, steps, znew, vnew);
}

int lan_bounds_gen(nm_ctx* c, int msteps, double tol, double* lmin, double* lmax, int* steps) {
  Apply op = [c](const double* x, double* y) { amv64(c, x, y); };
  Apply sv = [c](const double* x, double* y) { bsolve64(c, x, y); };
  return lanczos_bounds(c, c->n, op, sv, msteps, tol, lmin, lmax, steps, c->w[0], c->w[1]);
}

}  // namespace nmg

using namespace nmg;

extern "C" {

void nm_result_free(nm_result* r) {
  if (!r) return;
  free(r->lam);
  free(r->vec);
  free(r->err_ref);
  free(r->res2);
  std::memset(r, 0, sizeof(*r));
}

int nm_solve(nm_ctx* c, double f_lo, double f_hi, const nm_solve_opts* opts, nm_result* res) {
  if (!c || !res) return NM_ERR_ARG;
  std::memset(res, 0, sizeof(*res));
  if (!(f_lo < f_hi)) return set_err(c, NM_ERR_ARG, "lowfreq must be below upfreq");  // src/mod_para.f90:220-223
  nm_solve_opts o;
  if (opts) o = *opts;
  else nm_default_solve_opts(&o);
  const int n = c->n;
  const int maxit_def = 3 * std::max(4 * 802, 2000);
  int maxit = std::min(std::min(o.maxit > 0 ? o.maxit : maxit_def, n), kMaxCols - 1);
  c->cuda_failed = false;
  const double tol = o.tol > 0 ? o.tol : 1e-5;
  const double thr_int = o.thresh_int > 0 ? o.thresh_int : 0.8;
  const double thr_ext = o.thresh_ext > 0 ? o.thresh_ext : 0.7;
  const bool mixed = c->precision == NM_PREC_MIXED;
  const double t0 = now_s();
  const long long amv0 = c->n_amv, bs0 = c->n_bsolve, sp0 = c->n_spmv, k0 = launches();
  int rc;
  // the callback is the caller's for this call only
  struct ProgressScope {
    nm_ctx* c;
    ~ProgressScope() {
      c->progress = nullptr;
      c->progress_data = nullptr;
    }
  } pscope{c};
  c->progress = o.progress;
  c->progress_data = o.progress_data;
  // ---- bounds of B^-1 A (src/mod_pevsl.f90:84)
  double lmin, lmax;
  if (o.ab_bounds[1] > 0) {
    lmin = o.ab_bounds[0];
    lmax = o.ab_bounds[1];
  } else {
    int steps;
    if ((rc = lan_bounds_gen(c, o.mlan_bounds > 0 ? o.mlan_bounds : 3000, 1e-5, &lmin, &lmax, &steps))) return rc;
  }
  if (c->verbose) printf(" step 0: eigenvalue bounds for B^{-1}A: lmin %.15g lmax %.15g\n", lmin, lmax);
  progress(c, NM_PHASE_BOUNDS, 1, 1);
  const double t1 = now_s();
  // ---- interval (src/mod_pevsl.f90:93-103): frequencies are default REAL,
  //      PI the single-precision literal 3.14159265359 widened to real*8.
  const double PI = (double)3.14159265359f;
  const double lo = (double)(float)f_lo, hi = (double)(float)f_hi;
  double xintv[4] = {(2.0 * PI * lo) * (2.0 * PI * lo) * 1.0e-6, (2.0 * PI * hi) * (2.0 * PI * hi) * 1.0e-6, lmin, lmax};
  if (xintv[0] < 1.0e-10) xintv[0] = lmin;
  std::memcpy(res->xintv, xintv, sizeof(xintv));
  // ---- filter (src/mod_pevsl.f90:108-115)
  Pol pol = find_pol(xintv, thr_int, thr_ext, 2, 10000, o.damping);
  res->pol_deg = pol.deg;
  res->pol_gam = pol.gam;
  res->pol_bar = pol.bar;
  if (c->verbose) printf(" ** Cheb Poly of deg = %d, gam = %.15e, bar: %.15e\n", pol.deg, pol.gam, pol.bar);
  const double t2 = now_s();
  // ---- ChebLanNr (src/mod_pevsl.f90:116-122)
  Basis& V = c->V;
  Basis& Z = c->Z;
  double* U = nullptr;
  int nc = 0;
  double t3 = 0;
  bool converged = false;
  int kdim = 0;
  const double eps = 2.220446049250313e-16;
  if (o.block > 1) {
    converged = true;
    int steps = 0;
    // adaptive refinement of the mixed path: guard Ritz vectors of the modes
    // just outside [a, b] (filter value down to that at g b and a / g)
    const bool adaptive = mixed && o.polish == 0;
    const double gfac = o.refine_guard == 0.0 ? 1.5 : o.refine_guard;
    const bool guards = adaptive && gfac > 1.0;
    double guard_bar = -1.0;
    if (guards) {
      guard_bar = filter_value(pol, std::min(gfac * xintv[1], xintv[3]));
      if (xintv[0] > xintv[2]) guard_bar = std::min(guard_bar, filter_value(pol, std::max(xintv[0] / gfac, xintv[2])));
      if (!(guard_bar > 0.0)) guard_bar = -1.0;
    }
    if ((rc = block_lanczos(c, pol, maxit, o.use_graph != 0, &U, &nc, &steps, &res->t_filter, &res->t_orth,
                            &res->t_eig, guard_bar)))
      return rc;
    // FP32 filter: close Ritz pairs are mixed at the FP32 noise level; an
    // FP64 Rayleigh-Ritz over the Ritz block separates them.
    if (mixed && o.polish > 0) {
      // fixed refinement plan between two Rayleigh-Ritz passes (degree,
      // band: polish_plan)
      const PolishPlan plan = polish_plan(res->xintv, o.polish);
      const bool refine = plan.refine && nc > 0;
      std::vector<double> theta;
      // the first pass only feeds the refinement (FP32-accurate Ritz pairs
      // suffice, FP32 products); without refinement it is the FP64 pass
      if ((rc = rayleigh_ritz64(c, &U, nc, &theta, refine))) {
        cudaFree(U);
        return rc;
      }
      progress(c, NM_PHASE_RITZ, nc, nc);
      if (refine) {
        if ((rc = polish64(c, U, nc, theta, res->xintv[3], plan)) ||
            (rc = rayleigh_ritz64(c, &U, nc))) {
          cudaFree(U);
          return rc;
        }
      }
    } else if (mixed) {
      // adaptive refinement: passes of refine64 (degree per block from the
      // measured FP64 residuals), each closed by an FP64 Rayleigh-Ritz,
      // until every block is below the target (or the pass limit)
      const bool refine = o.polish == 0 && nc > 0;
      std::vector<double> theta;
      if ((rc = rayleigh_ritz64(c, &U, nc, &theta, refine))) {
        cudaFree(U);
        return rc;
      }
      progress(c, NM_PHASE_RITZ, nc, nc);
      // keep the Ritz vectors with quotients in [a / g, g b] (ascending
      // after each Rayleigh-Ritz): the filter's tail goes after the first,
      // and a column whose quotient left the window (a mixture drifting to
      // the null space or far up) after any later one
      auto keep_window = [&]() -> int {
        int i0 = 0, i1 = nc;
        window_range(theta.data(), nc, xintv[0] / gfac, gfac * xintv[1], &i0, &i1);
        if (i0 > 0)
          for (int j = i0; j < i1; ++j)
            NM_CUDA(c, cudaMemcpyAsync(U + (size_t)(j - i0) * n, U + (size_t)j * n, sizeof(double) * n,
                                       cudaMemcpyDeviceToDevice, c->stream));
        theta = std::vector<double>(theta.begin() + i0, theta.begin() + i1);
        nc = i1 - i0;
        return NM_OK;
      };
      if (refine && guards) {
        if ((rc = keep_window())) {
          cudaFree(U);
          return rc;
        }
        res->refine_guards = 0;
        for (double t : theta) res->refine_guards += t < xintv[0] || t > xintv[1];
      }
      RefineParams rp;
      // err_ref = res2 / sqrt(N); the passes aim at half the target, so the
      // closing Rayleigh-Ritz cannot lift a pair back over it
      rp.tol_res2 = 0.5 * (o.resid_tol > 0 ? o.resid_tol : 1e-10) * std::sqrt((double)n);
      if (o.refine_maxdeg > 0) rp.maxdeg = o.refine_maxdeg;
      if (o.refine_band > 1.0) rp.band = o.refine_band;
      rp.purge = o.refine_purge;
      if (o.refine_growth > 1.0) rp.max_growth = o.refine_growth;
      rp.want_lo = xintv[0];
      rp.want_hi = xintv[1];
      const double nearf = o.refine_near == 0.0 ? 1.05 : o.refine_near;
      // refine_sweeps 0: passes until every wanted Ritz vector meets the
      // target, at most 6, stopping early when a pass no longer halves the
      // largest wanted residual
      const int sweeps = o.refine_sweeps > 0 ? o.refine_sweeps : 6;
      double prev_want = 0.0;
      for (int sw = 0; refine && sw < sweeps; ++sw) {
        // the first pass damps from band x the block's top (the FP32
        // filter's noise far up the spectrum); the later ones from just above
        // the guarded set, so the out-of-set modes next to b are damped too
        rp.near_c = sw > 0 && nearf > 0.0 && !theta.empty() ? nearf * theta.back() : 0.0;
        rp.low_x = theta.empty() ? 0.0 : theta.front();
        RefineStats rs;
        if ((rc = refine64(c, U, nc, theta, res->xintv[3], rp, &rs))) {
          cudaFree(U);
          return rc;
        }
        res->refine_blocks += rs.blocks;
        res->refine_steps += rs.steps;
        res->refine_maxdeg = std::max(res->refine_maxdeg, rs.max_deg);
        if (sw == 0) res->res2_before_refine = rs.max_res2_before;
        if (c->verbose)
          printf(" refinement pass %d: %d blocks, %lld block degree steps (max degree %d), res2 before %.3e "
                 "(wanted %.3e, %d above the target)\n",
                 sw + 1, rs.blocks, rs.steps, rs.max_deg, rs.max_res2_before, rs.max_res2_want, rs.want_above);
        if (rs.blocks == 0) break;
        if ((rc = rayleigh_ritz64(c, &U, nc, &theta))) {
          cudaFree(U);
          return rc;
        }
        ++res->refine_passes;
        if (guards && (rc = keep_window())) {
          cudaFree(U);
          return rc;
        }
        // residuals measured before this pass against those before the last
        if (o.refine_sweeps <= 0 && sw >= 2 && !(rs.max_res2_want < 0.5 * prev_want)) break;
        prev_want = rs.max_res2_want;
      }
    }
    res->lanczos_steps = steps;
    res->nritz_above_bar = nc;
    t3 = now_s();
  } else {
  if ((rc = ensure_basis(c, V, n, 1)) || (rc = ensure_basis(c, Z, n, 1))) return rc;
  {
    std::vector<double> h;
    start_vector(h, n, kStartSeed);
    NM_CUDA(c, cudaMemcpyAsync(Z.col(0), h.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    bsolve64(c, Z.col(0), V.col(0));
    const double t = 1.0 / std::sqrt(dot_sync(c, V.col(0), Z.col(0), n));
    if (!std::isfinite(t)) return c->cuda_failed ? NM_ERR_CUDA : set_err(c, NM_ERR_NUMERIC, "B-norm of start vector");
    dev_scale(Z.col(0), Z.col(0), t, n, c->stream);
    dev_scale(V.col(0), V.col(0), t, n, c->stream);
  }
  long long graph_nodes = 0;
  double* fin = c->w[2];
  double* fout = c->w[3];
  cudaGraphExec_t gexec = nullptr;
  if (o.use_graph) {
    cudaGraph_t g;
    const long long l0 = launches();
    NM_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    chebav(c, pol, fin, fout, mixed);
    NM_CUDA(c, cudaStreamEndCapture(c->stream, &g));
    graph_nodes = launches() - l0;
    add_launches(-graph_nodes);  // captured, not executed
    NM_CUDA(c, cudaGraphInstantiate(&gexec, g, 0));
    cudaGraphDestroy(g);
    // the capture counted one application; undo so counters reflect launches
    c->n_amv -= pol.deg;
    c->n_bsolve -= pol.deg;
    c->n_spmv -= (long long)pol.deg * (c->chebB.deg + (c->fs ? 2 + c->chebAp.deg : 1));
  }
  std::vector<double> dT, eT;
  double beta = 0.0, tr0 = 0.0;
  for (int k = 0; k < maxit; ++k) {
    NM_CUDA(c, cudaMemcpyAsync(fin, Z.col(k), sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
    if (gexec) {
      NM_CUDA(c, cudaGraphLaunch(gexec, c->stream));
      add_launches(graph_nodes);
      c->n_amv += pol.deg;
      c->n_bsolve += pol.deg;
      c->n_spmv += (long long)pol.deg * (c->chebB.deg + (c->fs ? 2 + c->chebAp.deg : 1));
    } else {
      chebav(c, pol, fin, fout, mixed);
    }
    double* znew = fout;
    if (k > 0) dev_axpy(znew, Z.col(k - 1), -beta, n, c->stream);
    const double alpha = dot_sync(c, V.col(k), znew, n);
    dT.push_back(alpha);
    dev_axpy(znew, Z.col(k), -alpha, n, c->stream);
    for (int p = 0; p < 2; ++p) reorth_pass(V, Z, k + 1, znew, n, c->red, c->hbuf, c->stream);
    double* vnew = c->w[1];
    bsolve64(c, znew, vnew);
    beta = std::sqrt(std::max(dot_sync(c, vnew, znew, n), 0.0));
    if (!std::isfinite(alpha) || !std::isfinite(beta)) {
      if (gexec) cudaGraphExecDestroy(gexec);
      return c->cuda_failed ? (c->err.find("timed out") != std::string::npos ? NM_ERR_TIMEOUT : NM_ERR_CUDA)
                            : set_err(c, NM_ERR_NUMERIC, "non-finite Lanczos coefficient");
    }
    kdim = k + 1;
    if (beta == 0.0) {
      converged = true;
      break;
    }
    if ((rc = ensure_basis(c, V, n, k + 2)) || (rc = ensure_basis(c, Z, n, k + 2))) {
      if (gexec) cudaGraphExecDestroy(gexec);
      return rc;
    }
    dev_scale(V.col(k + 1), vnew, 1.0 / beta, n, c->stream);
    dev_scale(Z.col(k + 1), znew, 1.0 / beta, n, c->stream);
    eT.push_back(beta);
    progress(c, NM_PHASE_LANCZOS, kdim, maxit);  // dot_sync drained the stream
    if ((k < 50 || (k - 50) % 50 != 0) && k != maxit - 1) continue;
    std::vector<double> e(eT.begin(), eT.begin() + (kdim - 1));
    std::vector<double> ev = tri_eigs_above(dT, e, pol.bar - eps);
    double tr1 = 0.0;
    for (double x : ev) tr1 += x;
    if (c->verbose) printf(" k %4d:   nconv %4d  tr1 %21.15e\n", k, (int)ev.size(), tr1);
    if (std::fabs(tr1 - tr0) < 2e-12 || std::fabs(tr1) + std::fabs(tr0) < 1e-10) {
      converged = true;
      break;
    }
    tr0 = tr1;
  }
  if (gexec) cudaGraphExecDestroy(gexec);
  res->lanczos_steps = kdim;
  t3 = now_s();
  // ---- Ritz pairs with p(theta) >= bar
  std::vector<double> e(eT.begin(), eT.begin() + std::max(0, kdim - 1));
  std::vector<double> ritz = tri_eigs_above(dT, e, pol.bar);
  nc = (int)ritz.size();
  res->nritz_above_bar = nc;
  std::vector<double> S;
  tri_eigvecs(dT, e, ritz, S);
  if (nc > 0) {
    double* dS = nullptr;
    NM_CUDA(c, cudaMalloc(&U, sizeof(double) * (size_t)n * nc));
    NM_CUDA(c, cudaMalloc(&dS, sizeof(double) * (size_t)kdim * nc));
    NM_CUDA(c, cudaMemcpyAsync(dS, S.data(), sizeof(double) * (size_t)kdim * nc, cudaMemcpyHostToDevice, c->stream));
    dim3 g(nb(n), (nc + kRitzCols - 1) / kRitzCols);
    k_ritz<<<g, kT, 0, c->stream>>>(V.d_chunks, V.ld, kdim, dS, nc, U, (size_t)n, n);
    nmg::add_launches(1);
    NM_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(dS);
  }
  progress(c, NM_PHASE_RITZ, nc, nc);
  }  // single-vector path
  // ---- Rayleigh quotients, interval test and residuals of the Ritz vectors
  std::vector<double> lam, errv, res2v;
  std::vector<int> keep;
  if (nc > 0) {
    double* w2 = c->w[0];
    double* w = c->w[1];
    double* r = c->w[2];
    for (int j = 0; j < nc; ++j) {
      double* u = U + (size_t)j * n;
      spmv<double, double>(c->B, u, w2, c->stream);
      ++c->n_spmv;
      const double tn = std::sqrt(dot_sync(c, u, w2, n));
      if (tn == 0.0) continue;
      dev_scale(u, u, 1.0 / tn, n, c->stream);
      dev_scale(w2, w2, 1.0 / tn, n, c->stream);
      amv64(c, u, w);
      const double th = dot_sync(c, w, u, n);
      if (th < xintv[0] - eps || th > xintv[1] + eps) continue;
      k_resid<<<nb(n), kT, 0, c->stream>>>(w, w2, th, r, n);
      nmg::add_launches(1);
      const double rn = std::sqrt(dot_sync(c, r, r, n));
      if (!(rn < tol)) continue;
      lam.push_back(th);
      errv.push_back(std::sqrt(rn * rn / n) / std::fabs(th));  // src/mod_pevsl.f90:154-158
      res2v.push_back(rn / std::fabs(th));
      keep.push_back(j);
    }
  }
  // ---- sort ascending (ssort_real, src/mod_pevsl.f90:165-166) and copy out
  const int nev = (int)lam.size();
  std::vector<int> ord(nev);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return lam[a] < lam[b]; });
  res->nev = nev;
  res->n = n;
  res->lam = (double*)malloc(sizeof(double) * std::max(nev, 1));
  res->err_ref = (double*)malloc(sizeof(double) * std::max(nev, 1));
  res->res2 = (double*)malloc(sizeof(double) * std::max(nev, 1));
  for (int i = 0; i < nev; ++i) {
    res->lam[i] = lam[ord[i]];
    res->err_ref[i] = errv[ord[i]];
    res->res2[i] = res2v[ord[i]];
  }
  if (o.want_vectors && nev > 0) {
    res->vec = (double*)malloc(sizeof(double) * (size_t)n * nev);
    for (int i = 0; i < nev; ++i) {
      double* u = U + (size_t)keep[ord[i]] * n;
      if (o.unscale) dev_mul(u, u, c->D, n, c->stream);  // x = y .* D, src/mod_pevsl.f90:199
      NM_CUDA(c, cudaMemcpyAsync(res->vec + (size_t)i * n, u, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    }
  }
  NM_CUDA(c, cudaStreamSynchronize(c->stream));
  cudaFree(U);
  NM_CUDA(c, cudaGetLastError());
  if ((rc = check_status(c))) return rc;
  const double t4 = now_s();
  res->t_bounds = t1 - t0;
  res->t_filter_design = t2 - t1;
  res->t_lanczos = t3 - t2;
  res->t_ritz = t4 - t3;
  res->t_total = t4 - t0;
  res->n_amv = c->n_amv - amv0;
  res->n_bsolve = c->n_bsolve - bs0;
  res->n_spmv = c->n_spmv - sp0;
  res->n_kernels = launches() - k0;
  progress(c, NM_PHASE_DONE, nev, nev);
  if (c->verbose) {
    printf(" Relative errors: from the smallest to largest eigens:\n");
    for (int j = 0; j < nev; ++j) printf(" Row %d  relative err. %.6e\n", j + 1, res->err_ref[j]);
    printf(" Transform to frequencies (mHz), and periods (s)\n");
    for (int j = 0; j < nev; ++j) {
      const double l = res->lam[j];
      if (l > 1e-15) printf(" Row %d %.10f %.6f\n", j + 1, std::sqrt(l) / PI / 2.0 * 1e3, 2.0 * PI / std::sqrt(l));
      else printf(" Row %d %g ...too small...\n", j + 1, l);
    }
  }
  if (!converged && kdim >= maxit) return set_err(c, NM_ERR_NOCONV, "Lanczos reached MAXIT before convergence");
  return NM_OK;
}

int nm_solve_batched(nm_ctx* c, const nm_slice* slices, int nslices, const nm_solve_opts* opts, nm_result* results) {
  if (!c) return NM_ERR_ARG;
  if (!slices || !results || nslices < 0) return set_err(c, NM_ERR_ARG, "nm_solve_batched: bad arguments");
  for (int i = 0; i < nslices; ++i) std::memset(&results[i], 0, sizeof(nm_result));
  for (int i = 0; i < nslices; ++i) {
    if (!(slices[i].f_hi_mhz > slices[i].f_lo_mhz) || !(slices[i].f_lo_mhz >= 0.0))
      return set_err(c, NM_ERR_ARG, "nm_solve_batched: slice " + std::to_string(i) + " is not an interval");
  }
  int first_err = NM_OK;
  for (int i = 0; i < nslices; ++i) {
    const int rc = nm_solve(c, slices[i].f_lo_mhz, slices[i].f_hi_mhz, opts, &results[i]);
    if (rc == NM_ERR_NOCONV) {
      if (first_err == NM_OK) first_err = rc;
      continue;  // the slice's result holds what converged; the others still run
    }
    if (rc != NM_OK) return rc;
  }
  return first_err;
}

}  // extern "C"
