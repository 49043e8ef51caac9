// Block (multi-vector) operators of libnmgpu: the grouped 3-component
// layouts and the SpMM kernels behind the batched filtered Lanczos.
//
// Layout: a block of S = 32 vectors is stored row-major (row i holds the 32
// column values contiguously), so a warp owns one matrix row and its 32 lanes
// own the 32 columns: every gathered neighbour row is one coalesced 128-byte
// (FP32) or 256-byte (FP64) load, and each matrix entry is a broadcast.
// The matrices use the displacement structure of the reference's assembly
// (3 DOFs per node copy, src/mod_cg_create_matrix.f90:1372-1389,1720-1736):
//   B  = M (x) I_3          -> scalar CSR M over 3-DOF groups
//   A, Ad                    -> CSR of 3x3 blocks over groups
//   E  (n x np)              -> CSR of 3x1 blocks, ET (np x n) -> 1x3 blocks
#pragma once

#include <cublas_v2.h>
#include <cusolverDn.h>

#include "nm_internal.h"

namespace nmg {

constexpr int kBlk = 32;

template <typename T>
struct GCsr {  // grouped CSR on the device
  int nrows = 0, ncols = 0, bs = 1;  // bs values per entry (1, 3 or 9)
  long long nnz = 0;                 // entries (blocks)
  int* rp = nullptr;
  int* ci = nullptr;
  T* v = nullptr;
  size_t bytes() const { return (size_t)(nrows + 1) * 4 + (size_t)nnz * (4 + bs * sizeof(T)); }
};

struct GCsrHost {
  int nrows = 0, ncols = 0, bs = 1;
  std::vector<int> rp, ci;
  std::vector<double> v;
};

// Host extraction from scaled DOF-level CSR; false if the structure is absent.
bool group_mass(const nm_csr* B, const std::vector<double>& D, GCsrHost& M);
bool group_bsr3(const nm_csr* A, const std::vector<double>& dl, const std::vector<double>& dr, GCsrHost& G);
bool group_e(const nm_csr* E, const std::vector<double>& D, const std::vector<double>& Dp, GCsrHost& G);
bool group_et(const nm_csr* ET, const std::vector<double>& Dp, const std::vector<double>& D, GCsrHost& G);
void scalar_csr(const nm_csr* m, const std::vector<double>& dl, const std::vector<double>& dr, double sign,
                GCsrHost& G);

template <typename T>
int upload_g(nm_ctx* c, const GCsrHost& h, GCsr<T>& d);
template <typename T>
void free_g(GCsr<T>& g);

// Launch shape of the gather Chebyshev kernels: vec 1 = 16-byte vector
// gathers (k_gcheb), 0 = one value per lane (k_mass_cheb, 4 gathers in
// flight per warp), 2 = the same with 8 in flight, -1 = the default for the
// component count; threads per CTA (one row per warp).  Picked per context
// by the autotuner (block_autotune).
struct GatherCfg {
  int vec = -1;
  int threads = 256;
  // 0: CTA b takes rows b*W .. b*W+W-1 (W = threads / 32, one per warp);
  // 1: sweep -- CTA b takes one contiguous range of about rows / grid rows
  //    and its warps walk it together, grid = the CTAs co-resident on the
  //    GPU, so the neighbour rows of nearby rows (space-filling-curve order)
  //    stay in that SM's L1
  int sweep = 0;
};

// Block kernels (S = kBlk columns, row-major blocks).
template <typename VT, typename XT>
void blk_mass_cheb(const GCsr<VT>& M, const ChebSetup& ch, const XT* b, XT* x, XT* work, cudaStream_t s,
                   const GatherCfg& cfg = GatherCfg());
template <typename VT, typename XT>
void blk_ap_cheb(const GCsr<VT>& Ap, const ChebSetup& ch, const XT* b, XT* x, XT* work, cudaStream_t s,
                 const GatherCfg& cfg = GatherCfg());
// Prefer L1 over shared memory for the gather kernels (once per context).
void blk_prefer_l1();
template <typename VT, typename XT>
void blk_et(const GCsr<VT>& ET, const XT* w, XT* x0, cudaStream_t s, const GatherCfg& cfg = GatherCfg());
template <typename VT, typename XT>
void blk_ap_cheb_persistent(const GCsr<VT>& Ap, const ChebSetup& ch, const XT* b, XT* x, XT* work, GridBar* bar,
                            int* status, int blocks, cudaStream_t s);
template <typename VT, typename XT>
void blk_amv(const GCsr<VT>& A, const GCsr<VT>* E, const XT* v, const XT* y, XT* out, const XT* vk, const XT* vkm1,
             XT* yacc, const FiltEpi& ep, cudaStream_t s, const GatherCfg& cfg = GatherCfg());
template <typename VT>
void blk_mass_spmv(const GCsr<VT>& M, const double* x, double* y, cudaStream_t s);
// Conversions between basis columns (FP64, column-major chunks) and row-major blocks.
template <typename XT>
void blk_gather_cols(const Basis& Z, int j0, int n, XT* blk, cudaStream_t s);   // blk = Z(:, j0:j0+S)^T
template <typename XT>
void blk_to_colmajor(const XT* blk, int n, double* out, size_t ld, cudaStream_t s);  // out(:, c) = blk(:, c)
template <typename XT>
void blk_init_filter(XT* vk, XT* vkm1, XT* y, const XT* v, double mu0, size_t len, cudaStream_t s);
// Range form of the filter: vk = a1 z, vkm1 = 0, y = mu1 vk.
template <typename XT>
void blk_init_range(XT* vk, XT* vkm1, XT* y, const XT* z, double a1, double mu1, size_t len, cudaStream_t s);
void blk_f2d_flat(const float* src, double* dst, size_t len, cudaStream_t s);
template <typename XT>
void blk_from_colmajor(const double* src, size_t ld, int n, XT* blk, cudaStream_t s);  // blk = src(:, 0:S)^T
int blk_coop_blocks();

// FP32 copy of a Lanczos basis (chunks of Basis::kChunk columns, ld = n
// rounded up to 32), the operand of the mixed path's Gram-Schmidt GEMMs.
struct Basis32 {
  int n = 0;
  size_t ld = 0;
  std::vector<float*> chunks;
  float* col(int j) const { return chunks[j / Basis::kChunk] + (size_t)(j % Basis::kChunk) * ld; }
};
// Column-major conversions of S-column blocks: dst = (float)src; W -= T.
void blk_d2f(const double* src, size_t lds, float* dst, size_t ldd, int n, int cols, cudaStream_t s);
void blk_sub_f32(double* W, size_t ldw, const float* T, size_t ldt, int n, int cols, cudaStream_t s);
void blk_f2d(const float* src, size_t lds, double* dst, size_t ldd, int n, int cols, cudaStream_t s);
// Polish helpers (row-major 32-column blocks): R = scale (AU - theta_col BU)
// in FP32; v += f_col R; U(:, col) += sc_col G(:, col) into column-major U.
void blk_resid_f32(const double* AU, const double* BU, const double* theta, float* R, float scale, size_t len,
                   cudaStream_t s);
void blk_force(float* v, const float* R, const float* f, size_t len, cudaStream_t s);
// Column sums of row-major 32-column FP64 blocks with `rows` rows: the 64
// doubles at scratch + blk_colres_scratch() - 64 receive sum_i (AU - theta_c
// BU)^2 (columns 0..31), then sum_i U BU (32..63); the summation order is
// fixed, so the result is the same on every run.
size_t blk_colres_scratch();
void blk_colres(const double* AU, const double* BU, const double* U, const double* theta, int rows, double* scratch,
                cudaStream_t s);
// KPM moment step over len elements: W0 <- alpha (T - c W1) - beta W0, then
// *out = V . W0 (double accumulation, fixed summation order; part holds
// blk_kpm_scratch() doubles).  T == nullptr: only *out = V . W0.
template <typename XT>
void blk_kpm_step(XT* W0, const XT* T, const XT* W1, const XT* V, double c, double alpha, double beta, size_t len,
                  double* part, double* out, cudaStream_t s);
size_t blk_kpm_scratch();
// KPM moments mu[0..degree] of the lambda-weighted density of B^-1 A on the
// device block path (nm_kpm_moments_ctx); nvec Rademacher vectors in blocks
// of 32, the same vectors and estimator as nm_kpm_moments.
int kpm_moments_block(nm_ctx* c, double lmin, double lmax, int degree, int nvec, unsigned long long seed,
                      double* mu);
// True when the context has no grouped (3-component) block operators.
bool block_path_missing(nm_ctx* c);

// Tensor-core Gram-Schmidt projection (nm_gs_tc.cu): H = V^T W for the FP32
// basis copy V (n x K, K a multiple of 32, chunks of 64 columns) and a
// 32-column FP32 block W, on tcgen05 (kind::tf32, 3xTF32 split).
// gs_tc_map encodes the TMA descriptor (CUtensorMap, gs_tc_map_bytes()
// bytes) of one 64-column chunk or of W (cols 32); base 16-byte aligned,
// ld a multiple of 4.  part holds gs_tc_part_floats(K, n) floats; status
// gets 2 if a bounded wait of the kernel ran out.  H is column-major with
// leading dimension ldh.
bool gs_tc_available();
size_t gs_tc_map_bytes();
int gs_tc_map(const float* base, int n, size_t ld, int cols, void* map_out);
size_t gs_tc_part_floats(int K, int n);
int gs_tc_project(const void* vmaps_dev, const void* wmap_dev, int K, int n, float* part, float* H, int ldh,
                  int* status, cudaStream_t s);
void blk_add_colmajor(const float* G, const double* sc, int n, double* U, size_t ld, cudaStream_t s);
// The same on the first ncol columns only (the others of U are not touched).
void blk_add_colmajor_cols(const float* G, const double* sc, int n, int ncol, double* U, size_t ld, cudaStream_t s);
// blk = src(:, 0:ncol)^T with columns ncol..31 of the row-major block zero.
void blk_from_colmajor_cols(const double* src, size_t ld, int n, int ncol, double* blk, cudaStream_t s);

// Grouped operators and buffers of the batched path.
struct BlockState {
  bool ok = false;
  GCsr<double> M64, A64, E64, ET64, Ap64;
  GCsr<float> M32, A32, E32, ET32, Ap32;
  float* f32 = nullptr;
  double* f64 = nullptr;
  Basis32 V32, Z32;  // FP32 copies of the basis (mixed path)
  // TMA descriptors of the V32 chunks for the tensor-core projection
  // (host copies, 64-byte aligned, and their device array)
  std::vector<uint8_t> vmaps;
  int vmaps_n = 0;
  void* d_vmaps = nullptr;
  // Chebyshev set-ups of the FP32 filter's inner solves (degrees matched to
  // FP32 accuracy; mixed path only, set by block_buffers)
  ChebSetup chB32, chAp32;
  // launch shapes of the gather solves chosen by block_autotune
  GatherCfg gm32, gm64, ga32, ga64;
  GatherCfg gA32, gA64;  // block A-op (k_et, k_amv3): threads and sweep
  bool tuned = false;
  size_t f32_len = 0, f64_len = 0;
  cublasHandle_t cublas = nullptr;
  cusolverDnHandle_t cusolver = nullptr;
  int coop = 0;
};
int block_buffers(nm_ctx* c);
// Times the gather-kernel variants of the mass and Ap Chebyshev solves on
// this context's matrices and keeps the fastest (once per context).
int block_autotune(nm_ctx* c);
int block_time_op(nm_ctx* c, int which, int reps, double* ms, double* bytes, int* launches_per_op);
int block_build(nm_ctx* c, const nm_csr* A, const nm_csr* B, const nm_csr* Ap, const nm_csr* E, const nm_csr* ET);
void block_free(nm_ctx* c);
// Block filtered Lanczos; on success U (n x nc, column-major, device, owned
// by the caller) holds the Ritz vectors with p(theta) >= bar, and, when
// 0 < guard_bar < bar, up to max_guard (-1: half the count above the bar
// plus 64) more with the largest filter values in [guard_bar, bar): the
// Ritz vectors of the modes just outside [a, b].
int block_lanczos(nm_ctx* c, const Pol& pol, int maxit, bool use_graph, double** U, int* nc, int* steps,
                  double* t_filter, double* t_orth, double* t_eig, double guard_bar = -1.0, int max_guard = -1);
// Value of the filter polynomial p at x (the Chebyshev series of pol).
double filter_value(const Pol& pol, double x);
// Index of the first Ritz value kept from the K ascending filter values
// evals: those >= bar, and when 0 < guard_bar < bar up to max_guard (-1:
// half the count above the bar plus 64) more in [guard_bar, bar).
int ritz_first(const double* evals, int K, double bar, double guard_bar, int max_guard);
// [i0, i1): the ascending theta[0..n) within [lo, hi].
void window_range(const double* theta, int n, double lo, double hi, int* i0, int* i1);
// FP64 Rayleigh-Ritz on the columns of U (n x nc): U <- U Q with
// (U^T A U) Q = (U^T B U) Q Theta.  Resolves the mixing of close Ritz pairs
// left by an FP32 filter.
// fp32_gemm: the three n x nc x nc products in FP32 (the pass before the
// refinement, which only needs FP32-accurate Ritz vectors and values).
int rayleigh_ritz64(nm_ctx* c, double** U, int nc, std::vector<double>* theta = nullptr, bool fp32_gemm = false);
// Plan of the mixed path's refinement for the interval xintv = [a, b,
// lmin, lmax] and a requested degree (0: default 80, < 0: off).  Any
// polynomial that damps the upper spectrum grows below theta: the
// components of a Ritz vector along the lower wanted modes and the zero
// modes are amplified by about exp(deg^2 (b - a) / (5 lmax)) when the band
// starts at c = 25 lmax / deg^2, so the degree is capped at
// 2 sqrt(lmax / (b - a)) (growth below ~2).  The band [c, lmax] is damped by
// ~1e4 (deg acosh(1 + 2 c / lmax) ~ 10) and starts above the interval with
// a margin (c >= 2 b = bfloor lmax), so every Ritz value lies below it.
struct PolishPlan {
  int deg = 0;          // degree for the lowest Ritz values (0: no refinement)
  double cfrac = 1.0;   // band start / lmax at that degree
  double bfloor = 1.0;  // lower limit of the band start: 2 b / lmax
  bool refine = false;
};
PolishPlan polish_plan(const double xintv[4], int requested);
// Degree of one block of Ritz values starting at theta (theta0 the lowest):
// deg sqrt(theta0 / theta), clamped to [min(20, deg), deg].
int polish_block_degree(const PolishPlan& p, double theta0, double theta);
// Band start / lmax for a block of degree d: max(25 / d^2, bfloor).
double polish_band(const PolishPlan& p, int d);
// Chebyshev degree reaching relative error eps on [lmin, lmax] of ref
// (2 sigma^d <= eps), never above ref.deg.
int cheb_degree_for(const ChebSetup& ref, double eps);
// p(0) of a filter polynomial: sum_k mu_k T_k(-cc / dd).
double filter_at_zero(const Pol& pol);

// Mixed path: refine the Ritz vectors U (n x nc, B-normalised, ascending
// Ritz values theta) towards FP64 accuracy: U <- U + B~^-1 D / tau, the
// part of q(A B~^-1) B U that differs from q(theta) B U, with q a Chebyshev
// polynomial of [c lmax, lmax] whose degree falls from deg for the lowest
// Ritz values to 20 as sqrt(theta_0 / theta) (c = max(25 / degree^2,
// bfloor); cfrac <= 0 disables the degree fall-off).  D follows the
// three-term recurrence driven by the FP64 residual A U - theta B U and runs
// in FP32 (it is small, so FP32 rounding stays at FP64 level relative to U).
int polish64(nm_ctx* c, double* U, int nc, const std::vector<double>& theta, double lmax, const PolishPlan& plan);

// Adaptive refinement of the mixed path (polish = 0): U <- h(B~^-1 A) U per
// Ritz vector with
//   h(x) = (x / theta) T_d(l(x)) / T_d(l(theta)),  l: [c, lmax] -> [-1, 1],
// applied in correction form, both factors driven by FP64 residuals
// R = A U - theta B U and computed in FP32 (the corrections are small, so
// their FP32 rounding stays far below FP64 level relative to U):
//  * T_d(l(.)) / T_d(l(theta)) damps the band [c, lmax], where FP32 rounding
//    of the filter left components of relative size ~1e-7 that the residual
//    weighs by lambda / theta (up to 1e6 for the lowest modes);
//  * x / theta is zero on the null space of A, the zero-frequency fluid
//    modes, whose FP32-level content (from the FP32 Ritz and Gram-Schmidt
//    products) no polynomial normalised at theta can damp.
// Any polynomial normalised at theta grows below it: with the band starting
// at c = band * (largest theta of the block), band = 8, the growth of the
// lower modes is about D^0.06 for a damping D, and the Rayleigh-Ritz over
// all Ritz vectors that closes each pass removes it along the other wanted
// modes.  The degree per block of 32 Ritz vectors is the smallest that
// brings every column's residual below tol_res2 with a margin `safety`,
// including the factor lmax / theta the purge multiplies the band by:
//   d = max_j acosh(safety (lmax/theta_j) res2_j / tol_res2)
//             / acosh(1 + 2 (c - theta_j) / (lmax - c)),
// clamped to [mindeg, maxdeg]; blocks already below tol_res2 are left alone.
// purge >= 0: h with the factor x / theta, applied as one three-term
// recurrence for (x T_d(l(x)) - theta T_d(l(theta))) / (x - theta), so no
// two large FP32 terms cancel; purge < 0: h = T_d(l(x)) / T_d(l(theta)).
struct RefineParams {
  double tol_res2 = 1e-7;  // target ||A u - theta B u||_2 / (|theta| ||u||_B)
  double band = 8.0;       // damped band from band x the block's largest Ritz value ...
  double near_c = 0.0;     // ... or, if > 0, from near_c, moved up as far as needed
  double max_growth = 1e3; // to keep the growth below the Ritz values under this,
  double low_x = 0.0;      // and that of modes in (0, low_x] (out of the set below
  double max_low_growth = 2.0;  // its lowest Ritz value), x / theta included, under this
  double safety = 4.0;
  int purge = 0;
  int mindeg = 8, maxdeg = 4000;
  // Ritz values outside [want_lo, want_hi] are guards: their target is
  // guard_tol x tol_res2
  double want_lo = 0.0, want_hi = 1e300, guard_tol = 100.0;
};
struct RefineStats {
  int blocks = 0, max_deg = 0;   // blocks refined, largest degree
  long long steps = 0;           // block degree steps spent
  double max_res2_before = 0.0;  // largest res2 measured before the pass
  double max_res2_want = 0.0;    // ... of the Ritz values in [want_lo, want_hi]
  int want_above = 0;            // of those, above the target
};
int refine_block_degree(const std::vector<double>& theta, const std::vector<double>& res2, double c0, double lmax,
                        const RefineParams& rp, bool purge);
// log of the largest growth factor T_d(l(x)) / T_d(l(theta_j)), x in [0,
// theta_j), of the block's refinement polynomial (degree from
// refine_block_degree) over its Ritz values theta_j
double refine_log_growth(const std::vector<double>& theta, const std::vector<double>& res2, double c0, double lmax,
                         const RefineParams& rp, bool purge);
// log of the largest gain (x / theta_j) T_d(l(x)) / T_d(l(theta_j)) of the
// block's refinement polynomial over x in (0, rp.low_x]: modes below the
// refined set, which no Rayleigh-Ritz removes (-inf without low_x)
double refine_low_growth(const std::vector<double>& theta, const std::vector<double>& res2, double c0, double lmax,
                         const RefineParams& rp, bool purge);
// start of the damped band of one block: band x thmax, or for a near pass
// the lowest c >= max(near_c, 1.05 thmax) with refine_log_growth <=
// log(max_growth) and refine_low_growth <= log(max_low_growth) (never above
// band x thmax), capped at lmax / 2
double refine_band_start(const std::vector<double>& theta, const std::vector<double>& res2, double thmax, double lmax,
                         const RefineParams& rp, bool purge);
int refine64(nm_ctx* c, double* U, int nc, const std::vector<double>& theta, double lmax, const RefineParams& rp,
             RefineStats* stats);

}  // namespace nmg
