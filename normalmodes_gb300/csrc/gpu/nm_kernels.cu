// Device kernels of libnmgpu: SELL-32 sparse products, the fused Chebyshev
// semi-iteration, the fused operator + filter-recurrence kernel, and the
// FP64 vector / Gram-Schmidt kernels of the Lanczos process.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <type_traits>

#include "nm_internal.h"

namespace nmg {

static std::atomic<long long> g_launches{0};
long long launches() { return g_launches.load(); }
void add_launches(long long k) { g_launches += k; }
#define NM_COUNT(k) g_launches += (k)

namespace {

constexpr int kThreads = 256;

inline int nblk(long long n, int t = kThreads) { return (int)((n + t - 1) / t); }

template <typename T>
struct SellView {
  int nrows;
  const long long* __restrict__ slice_ptr;
  const int* __restrict__ row_len;
  const int* __restrict__ col;
  const T* __restrict__ val;
};

template <typename T>
SellView<T> view(const Sell<T>& m) {
  return SellView<T>{m.nrows, m.slice_ptr, m.row_len, m.col, m.val};
}

template <typename XT>
__device__ __forceinline__ XT fmaT(XT a, XT b, XT c);
template <>
__device__ __forceinline__ double fmaT<double>(double a, double b, double c) { return fma(a, b, c); }
template <>
__device__ __forceinline__ float fmaT<float>(float a, float b, float c) { return fmaf(a, b, c); }

// Row product of one SELL row in CSR order.  Two accumulators keep two
// independent FMA chains in flight; they are combined at the end so the
// result is deterministic.
// COHERENT_X: x was written earlier in the same launch by other blocks (the
// persistent kernel), so it must not go through the non-coherent read-only
// cache.
template <typename XT, bool COHERENT_X>
__device__ __forceinline__ XT ldx(const XT* p) {
  if (COHERENT_X) return *p;
  return __ldg(p);
}

template <typename VT, typename XT, bool COHERENT_X = false>
__device__ __forceinline__ XT sell_row(const SellView<VT>& M, int row, const XT* __restrict__ x) {
  const long long base = M.slice_ptr[row >> 5] + (row & 31);
  const int len = M.row_len[row];
  XT s0 = 0, s1 = 0;
  int k = 0;
  for (; k + 1 < len; k += 2) {
    const long long e0 = base + (long long)k * kSlice;
    const long long e1 = e0 + kSlice;
    const int c0 = __ldg(M.col + e0), c1 = __ldg(M.col + e1);
    const VT v0 = __ldg(M.val + e0), v1 = __ldg(M.val + e1);
    s0 = fmaT<XT>((XT)v0, ldx<XT, COHERENT_X>(x + c0), s0);
    s1 = fmaT<XT>((XT)v1, ldx<XT, COHERENT_X>(x + c1), s1);
  }
  if (k < len) {
    const long long e0 = base + (long long)k * kSlice;
    s0 = fmaT<XT>((XT)__ldg(M.val + e0), ldx<XT, COHERENT_X>(x + __ldg(M.col + e0)), s0);
  }
  return s0 + s1;
}

template <typename VT, typename XT>
__global__ void __launch_bounds__(kThreads) k_spmv(SellView<VT> M, const XT* __restrict__ x, XT* __restrict__ y) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= M.nrows) return;
  y[row] = sell_row<VT, XT>(M, row, x);
}

// One step of the Chebyshev semi-iteration (x0 = 0):
//   t = M d;  r -= t;  x += d;  d' = a d + c r
// FIRST: d = b * inv_theta, r = b, x = 0 are implicit.
// LAST : writes only xout = x + d + d'.
template <typename VT, typename XT, bool FIRST, bool LAST>
__global__ void __launch_bounds__(kThreads)
    k_cheb(SellView<VT> M, const XT* __restrict__ b, XT* __restrict__ x, XT* __restrict__ r,
           const XT* __restrict__ dcur, XT* __restrict__ dnext, XT* __restrict__ xout, XT a, XT c, XT inv_theta) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= M.nrows) return;
  XT dc, rr, xn;
  if (FIRST) {
    const XT t = sell_row<VT, XT>(M, row, b) * inv_theta;
    const XT bi = b[row];
    dc = bi * inv_theta;
    rr = bi - t;
    xn = dc;
  } else {
    const XT t = sell_row<VT, XT>(M, row, dcur);
    dc = dcur[row];
    rr = r[row] - t;
    xn = x[row] + dc;
  }
  const XT dn = fmaT<XT>(a, dc, c * rr);
  if (LAST) {
    xout[row] = xn + dn;
  } else {
    r[row] = rr;
    x[row] = xn;
    dnext[row] = dn;
  }
}

// Bounded grid barrier (sense by generation counter).  Thread 0 of each block
// arrives; the last arrival resets the counter and bumps the generation; the
// others poll the generation with a spin limit.  Returns false (and sets
// *status) if the wait gave up or another block already failed.
__device__ __forceinline__ bool grid_barrier(GridBar* bar, unsigned nblocks, int* status,
                                             long long spin_limit = kSpinLimit) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned g = *((volatile unsigned*)&bar->gen);
    __threadfence();
    const unsigned arrived = atomicAdd(&bar->count, 1u);
    if (arrived == nblocks - 1) {
      atomicExch(&bar->count, 0u);
      __threadfence();
      atomicAdd(&bar->gen, 1u);
    } else {
      long long spins = 0;
      while (*((volatile unsigned*)&bar->gen) == g) {
        if (*((volatile int*)status) != 0) {
          ok = 0;
          break;
        }
        if (++spins > spin_limit) {
          atomicExch(status, 1);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// All `deg` Chebyshev iterations in one launch; rows in a grid-stride loop,
// a grid barrier between iterations.  Same arithmetic per row as k_cheb.
constexpr int kThreadsP = 1024;  // persistent kernel: one CTA per SM
template <typename VT, typename XT>
__global__ void __launch_bounds__(kThreadsP)
    k_cheb_persist(SellView<VT> M, const XT* __restrict__ b, XT* xout, XT* r, XT* x, XT* d0, XT* d1,
                   const double* __restrict__ coef,
                   int deg, XT inv_theta, GridBar* bar, int* status) {
  const int stride = gridDim.x * blockDim.x;
  for (int k = 0; k < deg; ++k) {
    const XT a = (XT)coef[k], c = (XT)coef[deg + k];
    const XT* dcur = (k & 1) ? d1 : d0;
    XT* dnext = (k & 1) ? d0 : d1;
    const bool first = k == 0, last = k == deg - 1;
    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < M.nrows; row += stride) {
      XT dc, rr, xn;
      if (first) {
        const XT t = sell_row<VT, XT>(M, row, b) * inv_theta;
        const XT bi = b[row];
        dc = bi * inv_theta;
        rr = bi - t;
        xn = dc;
      } else {
        const XT t = sell_row<VT, XT, true>(M, row, dcur);
        dc = dcur[row];
        rr = r[row] - t;
        xn = x[row] + dc;
      }
      const XT dn = fmaT<XT>(a, dc, c * rr);
      if (last) {
        xout[row] = xn + dn;
      } else {
        r[row] = rr;
        x[row] = xn;
        dnext[row] = dn;
      }
    }
    if (!last && !grid_barrier(bar, gridDim.x, status)) return;
  }
}

// w = A v (+ E y) with epilogue.
// MODE 0: out = w
// MODE 1: t = s (w - cc vk) - pm vkm1;  out = t;  yacc += mu t
template <typename VT, typename XT, bool HAS_E, int MODE>
__global__ void __launch_bounds__(kThreads)
    k_amv(SellView<VT> A, SellView<VT> E, const XT* __restrict__ v, const XT* __restrict__ y, XT* __restrict__ out,
          const XT* __restrict__ vk, const XT* __restrict__ vkm1, XT* __restrict__ yacc, XT s, XT cc, XT pm, XT mu) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= A.nrows) return;
  XT w = sell_row<VT, XT>(A, row, v);
  if (HAS_E) w += sell_row<VT, XT>(E, row, y);
  if (MODE == 0) {
    out[row] = w;
  } else {
    const XT t = fmaT<XT>(s, fmaT<XT>(-cc, vk[row], w), -pm * vkm1[row]);
    out[row] = t;
    yacc[row] = fmaT<XT>(mu, t, yacc[row]);
  }
}

__global__ void k_fill(double* x, double v, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = v;
}
__global__ void k_axpy(double* y, const double* x, double a, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = fma(a, x[i], y[i]);
}
__global__ void k_axpy_ds(double* y, const double* x, const double* a, double sign, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = fma(sign * a[0], x[i], y[i]);
}
__global__ void k_scale_ds_inv(double* y, const double* x, const double* a, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[i] / a[0];
}
__global__ void k_scale(double* y, const double* x, double a, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i];
}
__global__ void k_mul(double* y, const double* x, const double* d, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[i] * d[i];
}
__global__ void k_copy(double* y, const double* x, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[i];
}
__global__ void k_d2f(float* y, const double* x, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = (float)x[i];
}
__global__ void k_f2d(double* y, const float* x, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = (double)x[i];
}
template <typename XT>
__global__ void k_init_filter(XT* vk, XT* vkm1, XT* y, const XT* v, XT mu0, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    XT vi = v[i];
    vk[i] = vi;
    vkm1[i] = 0;
    y[i] = mu0 * vi;
  }
}

// Deterministic two-stage dot product.
__global__ void __launch_bounds__(kThreads) k_dot1(const double* __restrict__ x, const double* __restrict__ y, int n,
                                                    double* __restrict__ red) {
  __shared__ double sh[kThreads];
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < n; i += (long long)gridDim.x * kThreads)
    s = fma(x[i], y[i], s);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) red[blockIdx.x] = sh[0];
}
__global__ void __launch_bounds__(kThreads) k_dot2(const double* __restrict__ red, int m, double* __restrict__ out) {
  __shared__ double sh[kThreads];
  double s = 0.0;
  for (int i = threadIdx.x; i < m; i += kThreads) s += red[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}
__global__ void k_sqrt(double* x) {
  if (threadIdx.x == 0 && blockIdx.x == 0) x[0] = sqrt(fmax(x[0], 0.0));
}

// Gram-Schmidt, pass 1: partial dots of 8 basis columns per block over one
// row partition.  red[j * kRedParts + part].
constexpr int kTC = 8;
__global__ void __launch_bounds__(kThreads)
    k_gs_dot(double* const* __restrict__ chunks, size_t ld, int ncol, const double* __restrict__ z, int n,
             double* __restrict__ red) {
  __shared__ double sh[kTC][kThreads];
  const int j0 = blockIdx.x * kTC;
  const int part = blockIdx.y;
  const int rows_per = (n + kRedParts - 1) / kRedParts;
  const int r0 = part * rows_per, r1 = min(n, r0 + rows_per);
  const double* cp[kTC];
  int nc = min(kTC, ncol - j0);
  for (int c = 0; c < kTC; ++c) {
    int j = j0 + (c < nc ? c : 0);
    cp[c] = chunks[j / Basis::kChunk] + (size_t)(j % Basis::kChunk) * ld;
  }
  double acc[kTC];
#pragma unroll
  for (int c = 0; c < kTC; ++c) acc[c] = 0.0;
  for (int i = r0 + threadIdx.x; i < r1; i += kThreads) {
    const double zi = z[i];
#pragma unroll
    for (int c = 0; c < kTC; ++c)
      if (c < nc) acc[c] = fma(__ldg(cp[c] + i), zi, acc[c]);
  }
#pragma unroll
  for (int c = 0; c < kTC; ++c) sh[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
#pragma unroll
      for (int c = 0; c < kTC; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < nc) red[(size_t)(j0 + threadIdx.x) * kRedParts + part] = sh[threadIdx.x][0];
}
__global__ void k_gs_sum(const double* __restrict__ red, int ncol, double* __restrict__ h) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ncol) return;
  double s = 0.0;
  for (int p = 0; p < kRedParts; ++p) s += red[(size_t)j * kRedParts + p];
  h[j] = s;
}
// Gram-Schmidt, pass 2: z -= Z h, one row per thread, h staged in shared memory.
__global__ void __launch_bounds__(kThreads)
    k_gs_update(double* const* __restrict__ chunks, size_t ld, int ncol, const double* __restrict__ h,
                double* __restrict__ z, int n) {
  __shared__ double hs[Basis::kChunk];
  const int i = blockIdx.x * kThreads + threadIdx.x;
  double acc0 = 0.0, acc1 = 0.0;
  for (int c0 = 0; c0 < ncol; c0 += Basis::kChunk) {
    const int nc = min(Basis::kChunk, ncol - c0);
    __syncthreads();
    if (threadIdx.x < nc) hs[threadIdx.x] = h[c0 + threadIdx.x];
    __syncthreads();
    if (i < n) {
      const double* base = chunks[c0 / Basis::kChunk] + i;
      int c = 0;
      for (; c + 1 < nc; c += 2) {
        acc0 = fma(__ldg(base + (size_t)c * ld), hs[c], acc0);
        acc1 = fma(__ldg(base + (size_t)(c + 1) * ld), hs[c + 1], acc1);
      }
      if (c < nc) acc0 = fma(__ldg(base + (size_t)c * ld), hs[c], acc0);
    }
  }
  if (i < n) z[i] -= acc0 + acc1;
}

}  // namespace

// ---------------------------------------------------------------- host wrappers
template <typename T>
int upload(nm_ctx* c, const SellHost& h, Sell<T>& d) {
  free_sell(d);
  d.nrows = h.nrows;
  d.ncols = h.ncols;
  d.nslices = h.nslices;
  d.nnz = h.nnz;
  d.nstored = h.nstored;
  NM_CUDA(c, cudaMalloc(&d.slice_ptr, sizeof(long long) * (h.nslices + 1)));
  NM_CUDA(c, cudaMalloc(&d.row_len, sizeof(int) * (h.nrows > 0 ? h.nrows : 1)));
  NM_CUDA(c, cudaMalloc(&d.col, sizeof(int) * (h.nstored > 0 ? h.nstored : 1)));
  NM_CUDA(c, cudaMalloc(&d.val, sizeof(T) * (h.nstored > 0 ? h.nstored : 1)));
  NM_CUDA(c, cudaMemcpy(d.slice_ptr, h.slice_ptr.data(), sizeof(long long) * (h.nslices + 1), cudaMemcpyHostToDevice));
  if (h.nrows) NM_CUDA(c, cudaMemcpy(d.row_len, h.row_len.data(), sizeof(int) * h.nrows, cudaMemcpyHostToDevice));
  if (h.nstored) {
    NM_CUDA(c, cudaMemcpy(d.col, h.col.data(), sizeof(int) * h.nstored, cudaMemcpyHostToDevice));
    if (std::is_same<T, double>::value) {
      NM_CUDA(c, cudaMemcpy(d.val, h.val.data(), sizeof(double) * h.nstored, cudaMemcpyHostToDevice));
    } else {
      std::vector<T> tmp(h.nstored);
      for (long long i = 0; i < h.nstored; ++i) tmp[i] = (T)h.val[i];
      NM_CUDA(c, cudaMemcpy(d.val, tmp.data(), sizeof(T) * h.nstored, cudaMemcpyHostToDevice));
    }
  }
  c->dev_bytes += d.bytes();
  return NM_OK;
}
template int upload<double>(nm_ctx*, const SellHost&, Sell<double>&);
template int upload<float>(nm_ctx*, const SellHost&, Sell<float>&);

template <typename T>
void free_sell(Sell<T>& s) {
  cudaFree(s.slice_ptr);
  cudaFree(s.row_len);
  cudaFree(s.col);
  cudaFree(s.val);
  s = Sell<T>();
}
template void free_sell<double>(Sell<double>&);
template void free_sell<float>(Sell<float>&);

template <typename VT, typename XT>
void spmv(const Sell<VT>& M, const XT* x, XT* y, cudaStream_t s) {
  if (M.nrows == 0) return;
  k_spmv<VT, XT><<<nblk(M.nrows), kThreads, 0, s>>>(view(M), x, y);
}
template void spmv<double, double>(const Sell<double>&, const double*, double*, cudaStream_t);
template void spmv<float, float>(const Sell<float>&, const float*, float*, cudaStream_t);

template <typename VT, typename XT>
void cheb_solve(const Sell<VT>& M, const ChebSetup& ch, const XT* b, XT* x, XT* work, cudaStream_t s) {
  const int n = M.nrows;
  if (n == 0) return;
  XT* r = work;
  XT* d0 = work + n;
  XT* d1 = work + 2 * (size_t)n;
  XT* xi = work + 3 * (size_t)n;
  const SellView<VT> v = view(M);
  const XT it = (XT)ch.inv_theta;
  for (int k = 0; k < ch.deg; ++k) {
    const XT a = (XT)ch.a[k], c = (XT)ch.c[k];
    const bool first = k == 0, last = k == ch.deg - 1;
    XT* dcur = (k & 1) ? d1 : d0;
    XT* dnext = (k & 1) ? d0 : d1;
    if (first && last)
      k_cheb<VT, XT, true, true><<<nblk(n), kThreads, 0, s>>>(v, b, xi, r, dcur, dnext, x, a, c, it);
    else if (first)
      k_cheb<VT, XT, true, false><<<nblk(n), kThreads, 0, s>>>(v, b, xi, r, dcur, dnext, x, a, c, it);
    else if (last)
      k_cheb<VT, XT, false, true><<<nblk(n), kThreads, 0, s>>>(v, b, xi, r, dcur, dnext, x, a, c, it);
    else
      k_cheb<VT, XT, false, false><<<nblk(n), kThreads, 0, s>>>(v, b, xi, r, dcur, dnext, x, a, c, it);
    NM_COUNT(1);
  }
}
template void cheb_solve<double, double>(const Sell<double>&, const ChebSetup&, const double*, double*, double*,
                                         cudaStream_t);
template void cheb_solve<float, float>(const Sell<float>&, const ChebSetup&, const float*, float*, float*,
                                       cudaStream_t);

template <typename VT, typename XT>
void cheb_solve_persistent(const Sell<VT>& M, const ChebSetup& ch, const XT* b, XT* x, XT* work, GridBar* bar,
                           int* status, int blocks, cudaStream_t s) {
  const int n = M.nrows;
  if (n == 0 || ch.deg == 0) return;
  XT* r = work;
  XT* d0 = work + n;
  XT* d1 = work + 2 * (size_t)n;
  XT* xi = work + 3 * (size_t)n;
  const SellView<VT> v = view(M);
  const XT it = (XT)ch.inv_theta;
  const double* coef = ch.d_coef;
  int deg = ch.deg;
  blocks = std::min(blocks, nblk(n, kThreadsP));
  if (blocks < 1) blocks = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(kThreadsP);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e = cudaMemsetAsync(bar, 0, sizeof(GridBar), s);
  if (e == cudaSuccess)
    e = cudaLaunchKernelEx(&cfg, k_cheb_persist<VT, XT>, v, b, x, r, xi, d0, d1, coef, deg, it, bar, status);
  if (e != cudaSuccess) {
    // A refused cooperative launch (more CTAs than can be co-resident, e.g.
    // under MPS or a partitioned GPU) is not sticky and would leave x
    // unwritten: clear it and run the same solve as separate launches, which
    // need no co-residency.  A sticky error resurfaces at the next launch.
    cudaGetLastError();
    cheb_solve<VT, XT>(M, ch, b, x, work, s);
    return;
  }
  NM_COUNT(1);
}
// Test hook for the bounded wait: one block waits at the grid barrier for
// `phantom` blocks that are never launched, so the wait runs out after
// `spin_limit` polls, the kernel sets the status word and returns.
__global__ void k_barrier_probe(GridBar* bar, int* status, unsigned phantom, long long spin_limit) {
  grid_barrier(bar, gridDim.x + phantom, status, spin_limit);
}

int barrier_timeout_probe(nm_ctx* c, long long spin_limit) {
  NM_CUDA(c, cudaMemsetAsync(c->bar, 0, sizeof(GridBar), c->stream));
  NM_CUDA(c, cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream));
  k_barrier_probe<<<1, 32, 0, c->stream>>>(c->bar, c->d_status, 1u, spin_limit);
  NM_COUNT(1);
  NM_CUDA(c, cudaGetLastError());
  NM_CUDA(c, cudaStreamSynchronize(c->stream));
  return NM_OK;
}

template void cheb_solve_persistent<double, double>(const Sell<double>&, const ChebSetup&, const double*, double*,
                                                    double*, GridBar*, int*, int, cudaStream_t);
template void cheb_solve_persistent<float, float>(const Sell<float>&, const ChebSetup&, const float*, float*, float*,
                                                  GridBar*, int*, int, cudaStream_t);

int coop_blocks_for_persistent() {
  int dev = 0, sms = 0, per = 0, coop = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  if (!coop) return 0;
  int p64 = 0, p32 = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p64, k_cheb_persist<double, double>, kThreadsP, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p32, k_cheb_persist<float, float>, kThreadsP, 0);
  per = std::min(1, std::min(p64, p32));
  return per * sms;
}

template <typename VT, typename XT>
void amv_fused(const Sell<VT>& A, const Sell<VT>* E, const XT* v, const XT* y, XT* out, const XT* vk, const XT* vkm1,
               XT* yacc, const FiltEpi& ep, cudaStream_t s) {
  const int n = A.nrows;
  const SellView<VT> av = view(A);
  const SellView<VT> ev = E ? view(*E) : SellView<VT>{0, nullptr, nullptr, nullptr, nullptr};
  const XT S = (XT)ep.s, CC = (XT)ep.cc, PM = (XT)ep.pm, MU = (XT)ep.mu;
  if (E) {
    if (ep.mode == 0)
      k_amv<VT, XT, true, 0><<<nblk(n), kThreads, 0, s>>>(av, ev, v, y, out, vk, vkm1, yacc, S, CC, PM, MU);
    else
      k_amv<VT, XT, true, 1><<<nblk(n), kThreads, 0, s>>>(av, ev, v, y, out, vk, vkm1, yacc, S, CC, PM, MU);
  } else {
    if (ep.mode == 0)
      k_amv<VT, XT, false, 0><<<nblk(n), kThreads, 0, s>>>(av, ev, v, y, out, vk, vkm1, yacc, S, CC, PM, MU);
    else
      k_amv<VT, XT, false, 1><<<nblk(n), kThreads, 0, s>>>(av, ev, v, y, out, vk, vkm1, yacc, S, CC, PM, MU);
  }
  NM_COUNT(1);
}
template void amv_fused<double, double>(const Sell<double>&, const Sell<double>*, const double*, const double*,
                                        double*, const double*, const double*, double*, const FiltEpi&, cudaStream_t);
template void amv_fused<float, float>(const Sell<float>&, const Sell<float>*, const float*, const float*, float*,
                                      const float*, const float*, float*, const FiltEpi&, cudaStream_t);

void dev_fill(double* x, double v, int n, cudaStream_t s) { k_fill<<<nblk(n), kThreads, 0, s>>>(x, v, n); }
void dev_axpy(double* y, const double* x, double a, int n, cudaStream_t s) {
  k_axpy<<<nblk(n), kThreads, 0, s>>>(y, x, a, n);
  NM_COUNT(1);
}
void dev_axpy_devscal(double* y, const double* x, const double* a, double sign, int n, cudaStream_t s) {
  k_axpy_ds<<<nblk(n), kThreads, 0, s>>>(y, x, a, sign, n);
  NM_COUNT(1);
}
void dev_scale_devscal_inv(double* y, const double* x, const double* a, int n, cudaStream_t s) {
  k_scale_ds_inv<<<nblk(n), kThreads, 0, s>>>(y, x, a, n);
  NM_COUNT(1);
}
void dev_scale(double* y, const double* x, double a, int n, cudaStream_t s) {
  k_scale<<<nblk(n), kThreads, 0, s>>>(y, x, a, n);
  NM_COUNT(1);
}
void dev_mul(double* y, const double* x, const double* d, int n, cudaStream_t s) {
  k_mul<<<nblk(n), kThreads, 0, s>>>(y, x, d, n);
  NM_COUNT(1);
}
void dev_copy(double* y, const double* x, int n, cudaStream_t s) { k_copy<<<nblk(n), kThreads, 0, s>>>(y, x, n); }
void dev_d2f(float* y, const double* x, int n, cudaStream_t s) { k_d2f<<<nblk(n), kThreads, 0, s>>>(y, x, n); }
void dev_f2d(double* y, const float* x, int n, cudaStream_t s) { k_f2d<<<nblk(n), kThreads, 0, s>>>(y, x, n); }
void dev_init_filter(double* vk, double* vkm1, double* y, const double* v, double mu0, int n, cudaStream_t s) {
  k_init_filter<double><<<nblk(n), kThreads, 0, s>>>(vk, vkm1, y, v, mu0, n);
  NM_COUNT(1);
}
void dev_init_filter32(float* vk, float* vkm1, float* y, const float* v, double mu0, int n, cudaStream_t s) {
  k_init_filter<float><<<nblk(n), kThreads, 0, s>>>(vk, vkm1, y, v, (float)mu0, n);
  NM_COUNT(1);
}
void dev_dot(const double* x, const double* y, int n, double* red, double* out, cudaStream_t s) {
  k_dot1<<<kRedBlocks, kThreads, 0, s>>>(x, y, n, red);
  NM_COUNT(1);
  k_dot2<<<1, kThreads, 0, s>>>(red, kRedBlocks, out);
  NM_COUNT(1);
}
void dev_sqrt_inplace(double* x, cudaStream_t s) { k_sqrt<<<1, 32, 0, s>>>(x); }

void reorth_pass(const Basis& V, const Basis& Z, int ncol, double* z, int n, double* red, double* h, cudaStream_t s) {
  // red holds ncol * kRedParts partial sums and h ncol coefficients; both are
  // sized for kMaxCols columns by the context.
  if (ncol > kMaxCols) return;
  dim3 g((ncol + kTC - 1) / kTC, kRedParts);
  k_gs_dot<<<g, kThreads, 0, s>>>(V.d_chunks, V.ld, ncol, z, n, red);
  NM_COUNT(1);
  k_gs_sum<<<nblk(ncol), kThreads, 0, s>>>(red, ncol, h);
  NM_COUNT(1);
  k_gs_update<<<nblk(n), kThreads, 0, s>>>(Z.d_chunks, Z.ld, ncol, h, z, n);
  NM_COUNT(1);
}

}  // namespace nmg
