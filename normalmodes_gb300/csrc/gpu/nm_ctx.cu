// Context life cycle and the operator callbacks of libnmgpu.
//
// nm_create replaces setupmatvec (src/mod_matvec.f90:24-250): diagonal
// scaling (Bdiagscaling :252-342, Apdiagscaling :345-441, with Ap := -Ap of
// :137), Lanczos bounds of B_s and Ap_s (:83-86, :160-162) and the Chebyshev
// set-ups (:88-93, :167-174).  nm_amv / nm_bmv / nm_bsolve are the callbacks
// sparseAV or sparsefsAV, sparseBV and solveBV (:445-520).
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "nm_block.h"
#include "nm_internal.h"
#include "nm_ops.h"

namespace nmg {

int set_err(nm_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int check_csr(nm_ctx* c, const nm_csr* m, int nr, int nc, const char* name) {
  if (!m || !m->rowptr || (!m->col && m->rowptr[m->nrows] > 0) || (!m->val && m->rowptr[m->nrows] > 0))
    return set_err(c, NM_ERR_ARG, std::string("missing matrix ") + name);
  if (m->nrows != nr || m->ncols != nc) return set_err(c, NM_ERR_ARG, std::string("bad shape of ") + name);
  if (m->rowptr[0] != 0) return set_err(c, NM_ERR_ARG, std::string("rowptr[0] != 0 in ") + name);
  for (int i = 0; i < nr; ++i)
    if (m->rowptr[i + 1] < m->rowptr[i]) return set_err(c, NM_ERR_ARG, std::string("rowptr not monotone in ") + name);
  const long long nnz = m->rowptr[nr];
  for (long long q = 0; q < nnz; ++q)
    if (m->col[q] < 0 || m->col[q] >= nc) return set_err(c, NM_ERR_ARG, std::string("column out of range in ") + name);
  for (long long q = 0; q < nnz; ++q)
    if (!std::isfinite(m->val[q])) return set_err(c, NM_ERR_NUMERIC, std::string("non-finite value in ") + name);
  return NM_OK;
}

// 1/sqrt(sign * diag(m)); fails on a missing or non-positive diagonal.
int inv_sqrt_diag(nm_ctx* c, const nm_csr* m, double sign, std::vector<double>& d, const char* name) {
  d.assign(m->nrows, 0.0);
  for (int i = 0; i < m->nrows; ++i) {
    double v = 0.0;
    bool found = false;
    for (int q = m->rowptr[i]; q < m->rowptr[i + 1]; ++q)
      if (m->col[q] == i) {
        v = sign * m->val[q];
        found = true;
      }
    if (!found || !(v > 0.0) || !std::isfinite(v))
      return set_err(c, NM_ERR_NUMERIC, std::string("non-positive or missing diagonal in ") + name);
    d[i] = 1.0 / std::sqrt(v);
  }
  return NM_OK;
}

}  // namespace

int alloc_work(nm_ctx* c) {
  const size_t n = c->n, np = c->np > 0 ? c->np : 1;
  // 0..3 general, 4..7 B-solve work (4n contiguous), 8..11 filter vk, vkm1, vkp1, w2,
  // 12 x0 (np), 13 y0 (np), 14 Ap work (4np), 15 spare
  size_t sizes[16] = {n, n, n, n, 4 * n, 0, 0, 0, n, n, n, n, np, np, 4 * np, n};
  for (int i = 0; i < 16; ++i) {
    if (!sizes[i]) continue;
    NM_CUDA(c, cudaMalloc(&c->w[i], sizes[i] * sizeof(double)));
    c->dev_bytes += sizes[i] * sizeof(double);
  }
  c->w[5] = c->w[4] + n;
  c->w[6] = c->w[4] + 2 * n;
  c->w[7] = c->w[4] + 3 * n;
  if (c->precision == NM_PREC_MIXED) {
    size_t s32[12] = {n, n, 4 * n, n, n, n, n, np, np, 4 * np, n, n};
    for (int i = 0; i < 12; ++i) {
      NM_CUDA(c, cudaMalloc(&c->w32[i], s32[i] * sizeof(float)));
      c->dev_bytes += s32[i] * sizeof(float);
    }
  }
  c->red_cap = kMaxCols * kRedParts;
  NM_CUDA(c, cudaMalloc(&c->red, (size_t)c->red_cap * sizeof(double)));
  NM_CUDA(c, cudaMalloc(&c->hbuf, (size_t)kMaxCols * sizeof(double)));
  NM_CUDA(c, cudaMalloc(&c->scal, 64 * sizeof(double)));
  NM_CUDA(c, cudaMalloc(&c->bar, sizeof(GridBar)));
  NM_CUDA(c, cudaMalloc(&c->d_status, sizeof(int)));
  NM_CUDA(c, cudaMemset(c->bar, 0, sizeof(GridBar)));
  NM_CUDA(c, cudaMemset(c->d_status, 0, sizeof(int)));
  c->coop_blocks = coop_blocks_for_persistent();
  NM_CUDA(c, cudaMallocHost(&c->h_scal, 64 * sizeof(double)));
  c->dev_bytes += (size_t)c->red_cap * 8 + (size_t)kMaxCols * 8 + 512;
  return NM_OK;
}

int upload_cheb(nm_ctx* c, ChebSetup& ch) {
  cudaFree(ch.d_coef);
  ch.d_coef = nullptr;
  std::vector<double> buf(ch.a);
  buf.insert(buf.end(), ch.c.begin(), ch.c.end());
  if (buf.empty()) return NM_OK;
  NM_CUDA(c, cudaMalloc(&ch.d_coef, sizeof(double) * buf.size()));
  NM_CUDA(c, cudaMemcpy(ch.d_coef, buf.data(), sizeof(double) * buf.size(), cudaMemcpyHostToDevice));
  return NM_OK;
}

int check_status(nm_ctx* c) {
  int st = 0;
  NM_CUDA(c, cudaMemcpyAsync(&st, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  NM_CUDA(c, cudaStreamSynchronize(c->stream));
  if (st != 0) {
    c->cuda_failed = true;
    return set_err(c, NM_ERR_TIMEOUT, "a grid barrier of the persistent Chebyshev kernel timed out");
  }
  return NM_OK;
}

}  // namespace nmg

using namespace nmg;

extern "C" {

void nm_default_opts(nm_opts* o) {
  std::memset(o, 0, sizeof(*o));
  o->porder = 1;
  o->device = 0;
  o->precision = NM_PREC_FP64;
}

void nm_default_solve_opts(nm_solve_opts* o) {
  std::memset(o, 0, sizeof(*o));
  o->want_vectors = 1;
  o->use_graph = 1;
}

const char* nm_last_error(nm_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int nm_create(nm_ctx** out, const nm_csr* A, const nm_csr* B, const nm_csr* Ap, const nm_csr* E, const nm_csr* ET,
              const nm_opts* opts) {
  if (!out) return NM_ERR_ARG;
  *out = nullptr;
  nm_opts o;
  if (opts) o = *opts;
  else nm_default_opts(&o);
  auto* c = new nm_ctx();
  const double t0 = now_s();
  auto bail = [&](int rc) {
    *out = c;  // keep the context so nm_last_error can be read; caller destroys
    return rc;
  };
  if (o.porder != 1 && o.porder != 2) return bail(set_err(c, NM_ERR_ARG, "porder must be 1 or 2"));
  if (!A || !B) return bail(set_err(c, NM_ERR_ARG, "A and B are required"));
  c->fs = (Ap != nullptr);
  if (c->fs && (!E || !ET)) return bail(set_err(c, NM_ERR_ARG, "fluid-solid model needs Ap, E and ET"));
  c->n = B->nrows;
  c->np = c->fs ? Ap->nrows : 0;
  c->porder = o.porder;
  c->precision = o.precision;
  c->verbose = o.verbose;
  c->filter_form = o.filter_form;
  c->orth = o.orth;
  c->inner_tol = o.inner_tol;
  c->autotune = o.autotune;
  int rc;
  if ((rc = check_csr(c, B, c->n, c->n, "B"))) return bail(rc);
  if ((rc = check_csr(c, A, c->n, c->n, "A"))) return bail(rc);
  if (c->fs) {
    if ((rc = check_csr(c, Ap, c->np, c->np, "Ap"))) return bail(rc);
    if ((rc = check_csr(c, E, c->n, c->np, "E"))) return bail(rc);
    if ((rc = check_csr(c, ET, c->np, c->n, "ET"))) return bail(rc);
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= o.device)
    return bail(set_err(c, NM_ERR_CUDA, "no usable CUDA device"));
  c->device = o.device;
  if (cudaSetDevice(c->device) != cudaSuccess) return bail(set_err(c, NM_ERR_CUDA, "cudaSetDevice failed"));
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(set_err(c, NM_ERR_CUDA, "cudaStreamCreate failed"));
  // Diagonal scaling.
  if ((rc = inv_sqrt_diag(c, B, 1.0, c->hD, "B"))) return bail(rc);
  if (c->fs && (rc = inv_sqrt_diag(c, Ap, -1.0, c->hDp, "-Ap"))) return bail(rc);
  // Scaled SELL images, uploaded FP64 (and FP32 for the mixed filter).
  {
    SellHost hB = sell_from_csr(B, c->hD.data(), c->hD.data(), 1.0);
    if ((rc = upload(c, hB, c->B))) return bail(rc);
    if (c->precision == NM_PREC_MIXED && (rc = upload(c, hB, c->B32))) return bail(rc);
    c->h2d_bytes += (long long)B->rowptr[B->nrows] * 12 + (long long)(B->nrows + 1) * 4;
  }
  {
    SellHost hA = sell_from_csr(A, c->hD.data(), c->hD.data(), 1.0);
    if ((rc = upload(c, hA, c->A))) return bail(rc);
    if (c->precision == NM_PREC_MIXED && (rc = upload(c, hA, c->A32))) return bail(rc);
    c->h2d_bytes += (long long)A->rowptr[A->nrows] * 12 + (long long)(A->nrows + 1) * 4;
  }
  if (c->fs) {
    SellHost hAp = sell_from_csr(Ap, c->hDp.data(), c->hDp.data(), -1.0);
    SellHost hE = sell_from_csr(E, c->hD.data(), c->hDp.data(), 1.0);
    SellHost hET = sell_from_csr(ET, c->hDp.data(), c->hD.data(), 1.0);
    if ((rc = upload(c, hAp, c->Ap)) || (rc = upload(c, hE, c->E)) || (rc = upload(c, hET, c->ET))) return bail(rc);
    if (c->precision == NM_PREC_MIXED &&
        ((rc = upload(c, hAp, c->Ap32)) || (rc = upload(c, hE, c->E32)) || (rc = upload(c, hET, c->ET32))))
      return bail(rc);
    for (const nm_csr* m : {Ap, E, ET}) c->h2d_bytes += (long long)m->rowptr[m->nrows] * 12 + (long long)(m->nrows + 1) * 4;
  }
  if (cudaMalloc(&c->D, sizeof(double) * c->n) != cudaSuccess) return bail(set_err(c, NM_ERR_OOM, "alloc D"));
  cudaMemcpy(c->D, c->hD.data(), sizeof(double) * c->n, cudaMemcpyHostToDevice);
  if (c->fs) {
    if (cudaMalloc(&c->Dp, sizeof(double) * c->np) != cudaSuccess) return bail(set_err(c, NM_ERR_OOM, "alloc Dp"));
    cudaMemcpy(c->Dp, c->hDp.data(), sizeof(double) * c->np, cudaMemcpyHostToDevice);
  }
  if ((rc = alloc_work(c))) return bail(rc);
  if ((rc = block_build(c, A, B, Ap, E, ET))) return bail(rc);
  // Bounds and Chebyshev set-ups.
  c->chebB.deg = o.b_cheb_deg > 0 ? o.b_cheb_deg : (c->porder == 2 ? 45 : 25);
  if (o.b_bounds[1] > 0) {
    c->chebB.lmin = o.b_bounds[0];
    c->chebB.lmax = o.b_bounds[1];
  } else {
    int steps = 0;
    if ((rc = lan_bounds_std(c, 0, 1000, 1e-12, &c->chebB.lmin, &c->chebB.lmax, &steps))) return bail(rc);
    if (c->verbose) printf(" B cond. number %g %g %g\n", c->chebB.lmax / c->chebB.lmin, c->chebB.lmin, c->chebB.lmax);
  }
  cheb_coefs(c->chebB);
  if ((rc = upload_cheb(c, c->chebB))) return bail(rc);
  if (c->fs) {
    if (o.ap_bounds[1] > 0) {
      c->chebAp.lmin = o.ap_bounds[0];
      c->chebAp.lmax = o.ap_bounds[1];
    } else {
      int steps = 0;
      if ((rc = lan_bounds_std(c, 1, 2000, 1e-12, &c->chebAp.lmin, &c->chebAp.lmax, &steps))) return bail(rc);
      if (c->verbose)
        printf(" Ap cond. number %g %g %g\n", c->chebAp.lmax / c->chebAp.lmin, c->chebAp.lmin, c->chebAp.lmax);
    }
    if (o.ap_cheb_deg > 0) c->chebAp.deg = o.ap_cheb_deg;
    else if (c->porder == 2) c->chebAp.deg = std::max(std::min((int)(c->chebAp.lmax / c->chebAp.lmin), 15) * 3, 100);
    else c->chebAp.deg = 25;
    cheb_coefs(c->chebAp);
    if ((rc = upload_cheb(c, c->chebAp))) return bail(rc);
  }
  NM_CUDA(c, cudaStreamSynchronize(c->stream));
  c->t_setup = now_s() - t0;
  *out = c;
  return NM_OK;
}

void nm_destroy(nm_ctx* c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_basis(c->V);
  free_basis(c->Z);
  block_free(c);
  for (auto* m : {&c->A, &c->B, &c->Ap, &c->E, &c->ET}) free_sell(*m);
  for (auto* m : {&c->A32, &c->B32, &c->Ap32, &c->E32, &c->ET32}) free_sell(*m);
  for (int i = 0; i < 16; ++i)
    if (i < 5 || i > 7) cudaFree(c->w[i]);
  for (int i = 0; i < 12; ++i) cudaFree(c->w32[i]);
  cudaFree(c->D);
  cudaFree(c->Dp);
  cudaFree(c->red);
  cudaFree(c->hbuf);
  cudaFree(c->scal);
  cudaFree(c->bar);
  cudaFree(c->d_status);
  cudaFree(c->chebB.d_coef);
  cudaFree(c->chebAp.d_coef);
  if (c->h_scal) cudaFreeHost(c->h_scal);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int nm_get_info(nm_ctx* c, nm_info* info) {
  if (!c || !info) return NM_ERR_ARG;
  std::memset(info, 0, sizeof(*info));
  info->n = c->n;
  info->np = c->np;
  info->fs = c->fs;
  info->porder = c->porder;
  info->precision = c->precision;
  info->nnz_a = c->A.nnz;
  info->nnz_b = c->B.nnz;
  info->nnz_ap = c->Ap.nnz;
  info->nnz_e = c->E.nnz;
  info->nnz_et = c->ET.nnz;
  info->b_bounds[0] = c->chebB.lmin;
  info->b_bounds[1] = c->chebB.lmax;
  info->ap_bounds[0] = c->chebAp.lmin;
  info->ap_bounds[1] = c->chebAp.lmax;
  info->b_cheb_deg = c->chebB.deg;
  info->ap_cheb_deg = c->chebAp.deg;
  info->t_setup = c->t_setup;
  info->h2d_bytes = c->h2d_bytes;
  info->device_bytes = c->dev_bytes;
  info->mass_vec = info->mass_threads = info->ap_vec = info->ap_threads = -1;
  info->mass_sweep = info->ap_sweep = info->aop_threads = info->aop_sweep = -1;
  if (const nmg::BlockState* st = (const nmg::BlockState*)c->blk) {
    if (st->tuned) {
      const bool mixed = c->precision == NM_PREC_MIXED;
      const nmg::GatherCfg& gm = mixed ? st->gm32 : st->gm64;
      const nmg::GatherCfg& ga = mixed ? st->ga32 : st->ga64;
      info->mass_vec = gm.vec;
      info->mass_threads = gm.threads;
      info->ap_vec = ga.vec;
      info->ap_threads = ga.threads;
      const nmg::GatherCfg& gA = mixed ? st->gA32 : st->gA64;
      info->mass_sweep = gm.sweep;
      info->ap_sweep = ga.sweep;
      info->aop_threads = gA.threads;
      info->aop_sweep = gA.sweep;
    }
  }
  return NM_OK;
}

void* nm_get_stream(nm_ctx* c) { return c ? (void*)c->stream : nullptr; }

int nm_sync(nm_ctx* c) {
  if (!c) return NM_ERR_ARG;
  NM_CUDA(c, cudaStreamSynchronize(c->stream));
  return NM_OK;
}

int nm_amv_dev(nm_ctx* c, const double* x, double* y) {
  if (!c || !x || !y) return NM_ERR_ARG;
  amv64(c, x, y);
  return NM_OK;
}
int nm_bmv_dev(nm_ctx* c, const double* x, double* y) {
  if (!c || !x || !y) return NM_ERR_ARG;
  spmv(c->B, x, y, c->stream);
  ++c->n_spmv;
  return NM_OK;
}
int nm_bsolve_dev(nm_ctx* c, const double* x, double* y) {
  if (!c || !x || !y) return NM_ERR_ARG;
  bsolve64(c, x, y);
  return NM_OK;
}

static int host_call(nm_ctx* c, int which, const double* X, double* Y, int ncols, int ld) {
  if (!c || !X || !Y || ncols < 0 || ld < c->n) return c ? set_err(c, NM_ERR_ARG, "bad host call arguments") : NM_ERR_ARG;
  const size_t n = c->n;
  for (int j = 0; j < ncols; ++j) {
    NM_CUDA(c, cudaMemcpyAsync(c->w[0], X + (size_t)j * ld, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if (which == 0) amv64(c, c->w[0], c->w[1]);
    else if (which == 1) spmv(c->B, c->w[0], c->w[1], c->stream);
    else bsolve64(c, c->w[0], c->w[1]);
    NM_CUDA(c, cudaMemcpyAsync(Y + (size_t)j * ld, c->w[1], n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  }
  NM_CUDA(c, cudaStreamSynchronize(c->stream));
  NM_CUDA(c, cudaGetLastError());
  return check_status(c);
}

int nm_amv(nm_ctx* c, const double* x, double* y) { return host_call(c, 0, x, y, 1, c ? c->n : 0); }
int nm_bmv(nm_ctx* c, const double* x, double* y) { return host_call(c, 1, x, y, 1, c ? c->n : 0); }
int nm_bsolve(nm_ctx* c, const double* x, double* y) { return host_call(c, 2, x, y, 1, c ? c->n : 0); }
int nm_amv_block(nm_ctx* c, const double* X, double* Y, int ncols, int ld) { return host_call(c, 0, X, Y, ncols, ld); }
int nm_bmv_block(nm_ctx* c, const double* X, double* Y, int ncols, int ld) { return host_call(c, 1, X, Y, ncols, ld); }
int nm_bsolve_block(nm_ctx* c, const double* X, double* Y, int ncols, int ld) {
  return host_call(c, 2, X, Y, ncols, ld);
}

int nm_time_op(nm_ctx* c, int which, int reps, double* ms_per_op, double* bytes_per_op, int* launches_per_op) {
  if (!c || reps <= 0) return NM_ERR_ARG;
  if (which >= 4) {
    double ms = 0, by = 0;
    int la = 0;
    int rc = block_time_op(c, which, reps, &ms, &by, &la);
    if (rc) return rc;
    if (ms_per_op) *ms_per_op = ms;
    if (bytes_per_op) *bytes_per_op = by;
    if (launches_per_op) *launches_per_op = la;
    return NM_OK;
  }
  std::vector<double> hx;
  start_vector(hx, c->n, kStartSeed);
  NM_CUDA(c, cudaMemcpy(c->w[0], hx.data(), sizeof(double) * c->n, cudaMemcpyHostToDevice));
  const int dB = c->chebB.deg, dAp = c->chebAp.deg;
  double bytes = 0;
  int launches = 0;
  const double bsp = c->B.algo_bytes(8);
  const double asp = c->A.algo_bytes(8) + (c->fs ? c->E.algo_bytes(8) - (double)c->n * 8 : 0.0);
  const double apsp = c->fs ? c->Ap.algo_bytes(8) : 0.0;
  const double etsp = c->fs ? c->ET.algo_bytes(8) : 0.0;
  // Chebyshev step: one SpMV plus r, x, d updates (read r, x, d; write r, x, d')
  const double bcheb = dB * bsp + (double)dB * 5.0 * c->n * 8;
  const double apcheb = c->fs ? dAp * apsp + (double)dAp * 5.0 * c->np * 8 : 0.0;
  const double aop = asp + (c->fs ? etsp + apcheb : 0.0);
  auto run = [&]() {
    if (which == 0) amv64(c, c->w[0], c->w[1]);
    else if (which == 1) spmv(c->B, c->w[0], c->w[1], c->stream);
    else if (which == 2) bsolve64(c, c->w[0], c->w[1]);
    else filter_step64(c, c->w[0], c->w[1], c->w[2], c->w[3]);
  };
  switch (which) {
    case 0: bytes = aop; launches = c->fs ? 2 + dAp : 1; break;
    case 1: bytes = bsp; launches = 1; break;
    case 2: bytes = bcheb; launches = dB; break;
    default: bytes = bcheb + aop + 3.0 * c->n * 8; launches = dB + (c->fs ? 2 + dAp : 1); break;
  }
  for (int i = 0; i < 3; ++i) run();
  cudaEvent_t e0, e1;
  NM_CUDA(c, cudaEventCreate(&e0));
  NM_CUDA(c, cudaEventCreate(&e1));
  NM_CUDA(c, cudaStreamSynchronize(c->stream));
  NM_CUDA(c, cudaEventRecord(e0, c->stream));
  for (int i = 0; i < reps; ++i) run();
  NM_CUDA(c, cudaEventRecord(e1, c->stream));
  NM_CUDA(c, cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  NM_CUDA(c, cudaGetLastError());
  if (ms_per_op) *ms_per_op = ms / reps;
  if (bytes_per_op) *bytes_per_op = bytes;
  if (launches_per_op) *launches_per_op = launches;
  return NM_OK;
}

// Test hook of the failure detection: a grid-barrier wait that can never
// complete gives up after spin_limit polls; the host then reads the status
// word and reports NM_ERR_TIMEOUT, as for a persistent Chebyshev kernel.
int nm_test_barrier_timeout(nm_ctx* c, long long spin_limit) {
  if (!c || spin_limit <= 0 || spin_limit > kSpinLimit) return c ? set_err(c, NM_ERR_ARG, "bad spin limit") : NM_ERR_ARG;
  const int rc = barrier_timeout_probe(c, spin_limit);
  if (rc != NM_OK) return rc;
  return check_status(c);
}

}  // extern "C"
