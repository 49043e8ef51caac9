// Internal declarations of libnmgpu (GB300 / sm_103a eigensolver).
//
// Data layout in HBM
// ------------------
// Every sparse operator is stored as SELL-32: rows are grouped in slices of
// 32 consecutive rows, a slice is padded to its longest row and stored
// column-major (element k of row r of slice s at slice_ptr[s] + 32 k + r%32).
// One thread owns one row, so a warp reads 32 consecutive values / column
// indices per step (fully coalesced) and accumulates its row sequentially in
// CSR order: one FMA per stored non-zero and no cross-lane reduction.  On
// GB300 the FP64 pipe (about 1.2 TFLOP/s) rather than HBM bounds FP64 sparse
// products, so the layout avoids every FP64 instruction that is not the FMA.
// Matrices are stored pre-scaled (A_s = D A D, B_s = D B D, Ap_s, E_s =
// D E D_p, ET_s = D_p ET D), so each application is a single pass.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "nmgpu.h"

namespace nmg {

constexpr int kSlice = 32;

template <typename T>
struct Sell {
  int nrows = 0, ncols = 0, nslices = 0;
  long long nnz = 0;      // true non-zeros
  long long nstored = 0;  // padded elements
  long long* slice_ptr = nullptr;  // device, nslices + 1
  int* row_len = nullptr;          // device, nrows
  int* col = nullptr;              // device, nstored
  T* val = nullptr;                // device, nstored
  size_t bytes() const {
    return (size_t)(nslices + 1) * 8 + (size_t)nrows * 4 + (size_t)nstored * (4 + sizeof(T));
  }
  // algorithmic bytes of one product y = M x: values + indices + row offsets
  // + x once + y once
  double algo_bytes(size_t xs) const {
    return (double)nnz * (sizeof(T) + 4) + (double)(nrows + 1) * 4 + (double)ncols * xs + (double)nrows * xs;
  }
};

// Host-side SELL image built from CSR (scaled values), uploaded by upload().
struct SellHost {
  int nrows = 0, ncols = 0, nslices = 0;
  long long nnz = 0, nstored = 0;
  std::vector<long long> slice_ptr;
  std::vector<int> row_len, col;
  std::vector<double> val;
};

struct ChebSetup {
  double lmin = 0, lmax = 0;
  int deg = 0;
  std::vector<double> a, c;  // per-iteration recurrence coefficients
  double inv_theta = 0;
  double* d_coef = nullptr;  // device copy: a[0..deg-1], c[0..deg-1]
};

// State of the bounded software grid barrier of the persistent kernels.
struct GridBar {
  unsigned int count;
  unsigned int gen;
};
constexpr long long kSpinLimit = 1ll << 24;  // polls (~1 s) before a barrier wait gives up

// Basis of Lanczos vectors, allocated in chunks of kChunk columns.
struct Basis {
  static constexpr int kChunk = 64;
  int n = 0;
  size_t ld = 0;
  std::vector<double*> chunks;  // host copies of device chunk pointers
  double** d_chunks = nullptr;  // device array of chunk pointers
  int d_chunks_cap = 0;
  double* col(int j) const { return chunks[j / kChunk] + (size_t)(j % kChunk) * ld; }
};

}  // namespace nmg

struct nm_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int fs = 0, n = 0, np = 0, porder = 1, precision = 0, verbose = 0;
  // mixed block path options (nm_opts): filter form, FP64 Gram-Schmidt,
  // inner B~^-1 accuracy, autotuning
  int filter_form = 0, orth = 0, autotune = 0;
  double inner_tol = 0.0;
  nmg::Sell<double> A, B, Ap, E, ET;  // scaled, FP64
  nmg::Sell<float> A32, B32, Ap32, E32, ET32;
  double* D = nullptr;   // n
  double* Dp = nullptr;  // np
  std::vector<double> hD, hDp;
  nmg::ChebSetup chebB, chebAp;
  // work vectors (device)
  double* w[16] = {nullptr};
  float* w32[12] = {nullptr};
  double* red = nullptr;   // reduction scratch (kMaxCols * kRedParts doubles)
  double* hbuf = nullptr;  // Gram-Schmidt coefficients (kMaxCols doubles)
  double* scal = nullptr;  // device scalars (64 doubles)
  nmg::GridBar* bar = nullptr;  // grid barrier of the persistent Chebyshev kernel
  int* d_status = nullptr;      // sticky device error word (1 = barrier timeout)
  int coop_blocks = 0;          // co-resident blocks for the persistent kernel
  double* h_scal = nullptr;  // pinned host scalars (h_scal[8] holds the status word)
  int red_cap = 0;
  std::string err;
  bool cuda_failed = false;
  double t_setup = 0;
  long long h2d_bytes = 0;
  size_t dev_bytes = 0;
  long long n_amv = 0, n_bsolve = 0, n_spmv = 0;
  nmg::Basis V, Z;
  // block (batched) path: grouped operators and buffers, built on first use
  void* blk = nullptr;  // nmg::BlockState*
  const nm_csr* src[5] = {nullptr};  // not owned; only valid inside nm_create
  // progress callback of the solve in flight (nm_solve_opts.progress)
  nm_progress_fn progress = nullptr;
  void* progress_data = nullptr;
};

namespace nmg {

// Kernel launches enqueued by this library (CUDA-graph replays add the
// captured node count).  Read by nm_solve for nm_result.n_kernels.
long long launches();
void add_launches(long long k);

// Reports a phase boundary to the solve's progress callback, if any, after
// the context's stream has drained (so host timestamps taken in the callback
// cover the device work before it).
inline void progress(nm_ctx* c, int phase, int done, int total) {
  if (!c->progress) return;
  cudaStreamSynchronize(c->stream);
  c->progress(c->progress_data, phase, done, total);
}

// Entry (i, j) of the j-th Rademacher vector of length n for the KPM
// moments (+1 or -1 from splitmix64 of a per-entry counter): the host and
// the device moment routines use the same vectors.
inline double rademacher(unsigned long long seed, int j, int n, int i) {
  uint64_t x = seed * 0x100000001B3ull + (uint64_t)j * (uint64_t)n + (uint64_t)i;
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  x ^= x >> 31;
  return (x >> 63) ? 1.0 : -1.0;
}

// Runs f when the scope ends (device scratch released on every return path).
template <typename F>
struct OnExit {
  F f;
  ~OnExit() { f(); }
};
template <typename F>
OnExit<F> on_exit(F f) {
  return OnExit<F>{f};
}

// ---------------------------------------------------------------- status
int set_err(nm_ctx* c, int code, const std::string& msg);
#define NM_CUDA(c, call)                                                                 \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return nmg::set_err((c), e_ == cudaErrorMemoryAllocation ? NM_ERR_OOM : NM_ERR_CUDA, \
                          std::string(#call) + ": " + cudaGetErrorString(e_));           \
  } while (0)

// ---------------------------------------------------------------- host helpers (nm_host.cpp)
SellHost sell_from_csr(const nm_csr* m, const double* dl, const double* dr, double sign);
void cheb_coefs(ChebSetup& s);
void start_vector(std::vector<double>& v, int n, uint64_t seed);
constexpr uint64_t kStartSeed = 0x5EED5EEDull;

struct Pol {
  int deg = 0;
  std::vector<double> mu;
  double cc = 0, dd = 0, gam = 0, bar = 0;
  int kind = 0;  // 0 interior, 1 left, 2 right
};
Pol find_pol(const double xintv[4], double thresh_int, double thresh_ext, int min_deg, int max_deg, int damping);
// symmetric tridiagonal: eigenvalues >= lo (ascending) by Sturm bisection
std::vector<double> tri_eigs_above(const std::vector<double>& d, const std::vector<double>& e, double lo);
// all eigenvalues in [lo, hi]
std::vector<double> tri_eigs_range(const std::vector<double>& d, const std::vector<double>& e, double lo, double hi);
double tri_eig_index(const std::vector<double>& d, const std::vector<double>& e, int idx);
// eigenvectors for given eigenvalues (inverse iteration, clustered reorth), column-major k x m
void tri_eigvecs(const std::vector<double>& d, const std::vector<double>& e, const std::vector<double>& lam,
                 std::vector<double>& S);

// ---------------------------------------------------------------- kernels (nm_kernels.cu)
template <typename T>
int upload(nm_ctx* c, const SellHost& h, Sell<T>& d);
template <typename T>
void free_sell(Sell<T>& s);

// y = M x
template <typename VT, typename XT>
void spmv(const Sell<VT>& M, const XT* x, XT* y, cudaStream_t s);
// Chebyshev solve of M z = b with `ch` (deg products); work: 4 vectors of nrows
template <typename VT, typename XT>
void cheb_solve(const Sell<VT>& M, const ChebSetup& ch, const XT* b, XT* x, XT* work, cudaStream_t s);
// Same, all `deg` iterations in one cooperative launch with a bounded grid
// barrier between iterations (for the small pressure system).  On a barrier
// timeout the kernel sets *status = 1 and returns.
template <typename VT, typename XT>
void cheb_solve_persistent(const Sell<VT>& M, const ChebSetup& ch, const XT* b, XT* x, XT* work, GridBar* bar,
                           int* status, int blocks, cudaStream_t s);
int coop_blocks_for_persistent();
// Bring the sticky device status back (sync); returns NM_OK or NM_ERR_TIMEOUT.
int check_status(nm_ctx* c);
// Runs a one-block kernel whose grid-barrier wait can never complete and
// must give up after spin_limit polls (test hook of the bounded waits).
int barrier_timeout_probe(nm_ctx* c, long long spin_limit);
int upload_cheb(nm_ctx* c, ChebSetup& ch);
// w = A_s v (+ E_s y); epilogue modes
struct FiltEpi {
  int mode = 0;        // 0: out = w; 1: filter recurrence
  double s = 0, cc = 0, pm = 0, mu = 0;
  const void* fz = nullptr;  // block path, mode 1: forcing block (same precision as the vectors) or null
  double fco = 0;            // out += fco * fz before the accumulation
};
template <typename VT, typename XT>
void amv_fused(const Sell<VT>& A, const Sell<VT>* E, const XT* v, const XT* y, XT* out, const XT* vk,
               const XT* vkm1, XT* yacc, const FiltEpi& ep, cudaStream_t s);

// vector helpers
void dev_fill(double* x, double v, int n, cudaStream_t s);
void dev_axpy(double* y, const double* x, double a, int n, cudaStream_t s);           // y += a x
void dev_axpy_devscal(double* y, const double* x, const double* a, double sign, int n, cudaStream_t s);
void dev_scale_devscal_inv(double* y, const double* x, const double* a, int n, cudaStream_t s);  // y = x / a
void dev_scale(double* y, const double* x, double a, int n, cudaStream_t s);
void dev_mul(double* y, const double* x, const double* d, int n, cudaStream_t s);   // y = x .* d
void dev_copy(double* y, const double* x, int n, cudaStream_t s);
void dev_d2f(float* y, const double* x, int n, cudaStream_t s);
void dev_f2d(double* y, const float* x, int n, cudaStream_t s);
void dev_init_filter(double* vk, double* vkm1, double* y, const double* v, double mu0, int n, cudaStream_t s);
void dev_init_filter32(float* vk, float* vkm1, float* y, const float* v, double mu0, int n, cudaStream_t s);
// deterministic dot: out[0] = x . y  (red: scratch of >= kRedBlocks doubles)
constexpr int kRedBlocks = 1024;
void dev_dot(const double* x, const double* y, int n, double* red, double* out, cudaStream_t s);
void dev_sqrt_inplace(double* x, cudaStream_t s);
// reorth: h = V(:, 0..k)^T z ; z -= Z(:, 0..k) h     (red >= ncol * kRedParts)
constexpr int kRedParts = 64;
constexpr int kMaxCols = 16384;  // largest Krylov basis (MAXIT = 9624 in the reference)
void reorth_pass(const Basis& V, const Basis& Z, int ncol, double* z, int n, double* red, double* h, cudaStream_t s);

}  // namespace nmg
