// nm_bsolve_dev_noalloc: the B^-1 apply of nm_bsolve_dev (Chebyshev
// semi-iteration on the scaled mass matrix, deg SELL products) with its work
// vectors in a fixed scratch array compiled into this library, so a call
// allocates no device memory at all.
//
// Scratch
// -------
// g_scratch is a file-scope device array of kNoAllocBytes = 4 vectors of
// NM_NOALLOC_MAX_ROWS doubles (40 MiB): residual r, running sum x and the two
// ping-pong direction vectors d0/d1, each at a fixed offset that is a multiple
// of 256 bytes.  Nothing in it has to start at zero: the first iteration
// writes r, x and d0 for every row before any later iteration reads them, so
// a call never depends on what an earlier call left behind.  Every call on a
// device shares the one array (whatever the context), so two calls that
// overlap on the GPU (different streams, or contexts whose streams are not
// ordered) race on it and both results are undefined.
//
// Set-up
// ------
// The device address of g_scratch is looked up once per device with
// cudaGetSymbolAddress, with the context's device current, on the first call
// that targets that device; later calls reuse the cached pointer.  That first
// call on a device should come before any stream capture.  The address
// belongs to the device's primary context: cudaDeviceReset (or any other
// teardown of the primary context) leaves the cached pointer stale, so a
// process that resets a device must not call this entry point on it again.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "nm_internal.h"

namespace nmg {
namespace {

constexpr int kNoAllocMaxRows = NM_NOALLOC_MAX_ROWS;
constexpr size_t kNoAllocVecs = 4;
constexpr int kMaxDevices = 64;
constexpr int kThreadsNA = 256;
static_assert(((size_t)kNoAllocMaxRows * sizeof(double)) % 256 == 0, "scratch vectors must stay 256-byte aligned");

static __device__ __align__(256) double g_scratch[kNoAllocVecs * (size_t)kNoAllocMaxRows];

std::mutex g_setup_mu;
double* g_ptr[kMaxDevices] = {};

// Row product of one SELL-32 row in CSR order with two interleaved FMA
// chains combined at the end; the same summation order as the context's
// own B-solve, so both entry points give identical bits.
__device__ __forceinline__ double row_dot(const long long* __restrict__ slice_ptr, const int* __restrict__ row_len,
                                          const int* __restrict__ col, const double* __restrict__ val, int row,
                                          const double* __restrict__ x) {
  const long long base = slice_ptr[row >> 5] + (row & 31);
  const int len = row_len[row];
  double s0 = 0, s1 = 0;
  int k = 0;
  for (; k + 1 < len; k += 2) {
    const long long e0 = base + (long long)k * kSlice;
    const long long e1 = e0 + kSlice;
    s0 = fma(__ldg(val + e0), __ldg(x + __ldg(col + e0)), s0);
    s1 = fma(__ldg(val + e1), __ldg(x + __ldg(col + e1)), s1);
  }
  if (k < len) {
    const long long e0 = base + (long long)k * kSlice;
    s0 = fma(__ldg(val + e0), __ldg(x + __ldg(col + e0)), s0);
  }
  return s0 + s1;
}

// One iteration of the semi-iteration with x0 = 0:
//   t = M d;  r -= t;  x += d;  d' = a d + c r
// FIRST: d = b * inv_theta, r = b, x = 0 are implicit (nothing is read from
// the scratch).  LAST: writes only out = x + d + d'.
// scr points at the scratch: r at 0, x at ld, d0 at 2 ld, d1 at 3 ld.
template <bool FIRST, bool LAST>
__global__ void __launch_bounds__(kThreadsNA)
    k_cheb_scratch(int n, const long long* __restrict__ slice_ptr, const int* __restrict__ row_len,
                   const int* __restrict__ col, const double* __restrict__ val, const double* __restrict__ b,
                   double* __restrict__ out, double* __restrict__ scr, size_t ld, int it, double a, double c,
                   double inv_theta) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  double* r = scr;
  double* x = scr + ld;
  const double* dcur = scr + (2 + (it & 1)) * ld;
  double* dnext = scr + (2 + ((it + 1) & 1)) * ld;
  double dc, rr, xn;
  if (FIRST) {
    const double t = row_dot(slice_ptr, row_len, col, val, row, b) * inv_theta;
    const double bi = b[row];
    dc = bi * inv_theta;
    rr = bi - t;
    xn = dc;
  } else {
    const double t = row_dot(slice_ptr, row_len, col, val, row, dcur);
    dc = dcur[row];
    rr = r[row] - t;
    xn = x[row] + dc;
  }
  const double dn = fma(a, dc, c * rr);
  if (LAST) {
    out[row] = xn + dn;
  } else {
    r[row] = rr;
    x[row] = xn;
    dnext[row] = dn;
  }
}

// Cached device address of g_scratch on `dev`, looked up on first use with
// `dev` current (the caller's current device is restored afterwards).
int scratch_ptr(nm_ctx* c, int dev, double** out) {
  if (dev < 0 || dev >= kMaxDevices) return set_err(c, NM_ERR_ARG, "nm_bsolve_dev_noalloc: device index out of range");
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_ptr[dev]) {
    int prev = -1;
    NM_CUDA(c, cudaGetDevice(&prev));
    if (prev != dev) NM_CUDA(c, cudaSetDevice(dev));
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (prev != dev) cudaSetDevice(prev);
    if (e != cudaSuccess)
      return set_err(c, NM_ERR_CUDA, std::string("nm_bsolve_dev_noalloc: cudaGetSymbolAddress: ") +
                                         cudaGetErrorString(e));
    if (!p) return set_err(c, NM_ERR_CUDA, "nm_bsolve_dev_noalloc: scratch address is null");
    g_ptr[dev] = (double*)p;
  }
  *out = g_ptr[dev];
  return NM_OK;
}

}  // namespace
}  // namespace nmg

using namespace nmg;

int nm_bsolve_dev_noalloc(nm_ctx* c, const double* x, double* y) {
  if (!c || !x || !y) return c ? set_err(c, NM_ERR_ARG, "nm_bsolve_dev_noalloc: null argument") : NM_ERR_ARG;
  const int n = c->n;
  if (n > kNoAllocMaxRows)
    return set_err(c, NM_ERR_ARG, "nm_bsolve_dev_noalloc: n = " + std::to_string(n) +
                                      " rows exceeds the scratch maximum of " + std::to_string(kNoAllocMaxRows) +
                                      " rows (use nm_bsolve_dev)");
  double* scr = nullptr;
  const int rc = scratch_ptr(c, c->device, &scr);
  if (rc != NM_OK) return rc;
  if (n == 0) return NM_OK;
  const ChebSetup& ch = c->chebB;
  const Sell<double>& M = c->B;
  const size_t ld = (size_t)kNoAllocMaxRows;
  const int grid = (n + kThreadsNA - 1) / kThreadsNA;
  for (int k = 0; k < ch.deg; ++k) {
    const bool first = k == 0, last = k == ch.deg - 1;
    const double a = ch.a[k], cc = ch.c[k];
    if (first && last)
      k_cheb_scratch<true, true><<<grid, kThreadsNA, 0, c->stream>>>(n, M.slice_ptr, M.row_len, M.col, M.val, x, y,
                                                                      scr, ld, k, a, cc, ch.inv_theta);
    else if (first)
      k_cheb_scratch<true, false><<<grid, kThreadsNA, 0, c->stream>>>(n, M.slice_ptr, M.row_len, M.col, M.val, x, y,
                                                                       scr, ld, k, a, cc, ch.inv_theta);
    else if (last)
      k_cheb_scratch<false, true><<<grid, kThreadsNA, 0, c->stream>>>(n, M.slice_ptr, M.row_len, M.col, M.val, x, y,
                                                                       scr, ld, k, a, cc, ch.inv_theta);
    else
      k_cheb_scratch<false, false><<<grid, kThreadsNA, 0, c->stream>>>(n, M.slice_ptr, M.row_len, M.col, M.val, x,
                                                                        y, scr, ld, k, a, cc, ch.inv_theta);
  }
  add_launches(ch.deg);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return set_err(c, NM_ERR_CUDA, std::string("nm_bsolve_dev_noalloc: launch: ") + cudaGetErrorString(e));
  ++c->n_bsolve;
  c->n_spmv += ch.deg;
  return NM_OK;
}
