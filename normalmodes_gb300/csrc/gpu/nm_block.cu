// Grouped 3-component operators and the block (32-column) SpMM kernels of
// the batched filtered Lanczos.  See nm_block.h for the layout.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <cmath>
#include <cstdlib>
#include <type_traits>

#include "nm_block.h"

namespace nmg {

// ---------------------------------------------------------------- host extraction
namespace {
inline bool same_row_pattern(const nm_csr* m, int r0, int r1, int colshift) {
  const int l0 = m->rowptr[r0 + 1] - m->rowptr[r0], l1 = m->rowptr[r1 + 1] - m->rowptr[r1];
  if (l0 != l1) return false;
  for (int k = 0; k < l0; ++k)
    if (m->col[m->rowptr[r1] + k] != m->col[m->rowptr[r0] + k] + colshift) return false;
  return true;
}
}  // namespace

bool group_mass(const nm_csr* B, const std::vector<double>& D, GCsrHost& M) {
  if (B->nrows % 3) return false;
  const int ng = B->nrows / 3;
  M = GCsrHost();
  M.nrows = M.ncols = ng;
  M.bs = 1;
  M.rp.assign(ng + 1, 0);
  for (int g = 0; g < ng; ++g) {
    for (int p = 1; p < 3; ++p) {
      if (!same_row_pattern(B, 3 * g, 3 * g + p, p)) return false;
      if (D[3 * g + p] != D[3 * g]) return false;
      for (int k = 0; k < B->rowptr[3 * g + 1] - B->rowptr[3 * g]; ++k)
        if (B->val[B->rowptr[3 * g + p] + k] != B->val[B->rowptr[3 * g] + k]) return false;
    }
    for (int q = B->rowptr[3 * g]; q < B->rowptr[3 * g + 1]; ++q) {
      const int c = B->col[q];
      if (c % 3) return false;
      M.ci.push_back(c / 3);
      M.v.push_back(B->val[q] * D[c] * D[3 * g]);
    }
    M.rp[g + 1] = (int)M.ci.size();
  }
  return true;
}

bool group_bsr3(const nm_csr* A, const std::vector<double>& dl, const std::vector<double>& dr, GCsrHost& G) {
  if (A->nrows % 3 || A->ncols % 3) return false;
  const int ng = A->nrows / 3;
  G = GCsrHost();
  G.nrows = ng;
  G.ncols = A->ncols / 3;
  G.bs = 9;
  G.rp.assign(ng + 1, 0);
  for (int g = 0; g < ng; ++g) {
    for (int p = 1; p < 3; ++p)
      if (!same_row_pattern(A, 3 * g, 3 * g + p, 0)) return false;
    const int q0 = A->rowptr[3 * g], len = A->rowptr[3 * g + 1] - q0;
    if (len % 3) return false;
    for (int k = 0; k < len; k += 3) {
      const int c = A->col[q0 + k];
      if (c % 3 || A->col[q0 + k + 1] != c + 1 || A->col[q0 + k + 2] != c + 2) return false;
      G.ci.push_back(c / 3);
      for (int p = 0; p < 3; ++p)
        for (int q = 0; q < 3; ++q) {
          const int r = 3 * g + p;
          G.v.push_back(A->val[A->rowptr[r] + k + q] * dr[c + q] * dl[r]);
        }
    }
    G.rp[g + 1] = (int)G.ci.size();
  }
  return true;
}

bool group_e(const nm_csr* E, const std::vector<double>& D, const std::vector<double>& Dp, GCsrHost& G) {
  if (E->nrows % 3) return false;
  const int ng = E->nrows / 3;
  G = GCsrHost();
  G.nrows = ng;
  G.ncols = E->ncols;
  G.bs = 3;
  G.rp.assign(ng + 1, 0);
  for (int g = 0; g < ng; ++g) {
    for (int p = 1; p < 3; ++p)
      if (!same_row_pattern(E, 3 * g, 3 * g + p, 0)) return false;
    const int len = E->rowptr[3 * g + 1] - E->rowptr[3 * g];
    for (int k = 0; k < len; ++k) {
      const int c = E->col[E->rowptr[3 * g] + k];
      G.ci.push_back(c);
      for (int p = 0; p < 3; ++p) {
        const int r = 3 * g + p;
        G.v.push_back(E->val[E->rowptr[r] + k] * Dp[c] * D[r]);
      }
    }
    G.rp[g + 1] = (int)G.ci.size();
  }
  return true;
}

bool group_et(const nm_csr* ET, const std::vector<double>& Dp, const std::vector<double>& D, GCsrHost& G) {
  if (ET->ncols % 3) return false;
  G = GCsrHost();
  G.nrows = ET->nrows;
  G.ncols = ET->ncols / 3;
  G.bs = 3;
  G.rp.assign(ET->nrows + 1, 0);
  for (int r = 0; r < ET->nrows; ++r) {
    const int q0 = ET->rowptr[r], len = ET->rowptr[r + 1] - q0;
    if (len % 3) return false;
    for (int k = 0; k < len; k += 3) {
      const int c = ET->col[q0 + k];
      if (c % 3 || ET->col[q0 + k + 1] != c + 1 || ET->col[q0 + k + 2] != c + 2) return false;
      G.ci.push_back(c / 3);
      for (int q = 0; q < 3; ++q) G.v.push_back(ET->val[q0 + k + q] * D[c + q] * Dp[r]);
    }
    G.rp[r + 1] = (int)G.ci.size();
  }
  return true;
}

void scalar_csr(const nm_csr* m, const std::vector<double>& dl, const std::vector<double>& dr, double sign,
                GCsrHost& G) {
  G = GCsrHost();
  G.nrows = m->nrows;
  G.ncols = m->ncols;
  G.bs = 1;
  G.rp.assign(m->rowptr, m->rowptr + m->nrows + 1);
  G.ci.assign(m->col, m->col + m->rowptr[m->nrows]);
  G.v.resize(G.ci.size());
  for (int r = 0; r < m->nrows; ++r)
    for (int q = m->rowptr[r]; q < m->rowptr[r + 1]; ++q) G.v[q] = sign * m->val[q] * dr[m->col[q]] * dl[r];
}

template <typename T>
int upload_g(nm_ctx* c, const GCsrHost& h, GCsr<T>& d) {
  free_g(d);
  d.nrows = h.nrows;
  d.ncols = h.ncols;
  d.bs = h.bs;
  d.nnz = (long long)h.ci.size();
  NM_CUDA(c, cudaMalloc(&d.rp, sizeof(int) * (h.nrows + 1)));
  NM_CUDA(c, cudaMalloc(&d.ci, sizeof(int) * std::max<long long>(d.nnz, 1)));
  NM_CUDA(c, cudaMalloc(&d.v, sizeof(T) * std::max<size_t>(h.v.size(), 1)));
  NM_CUDA(c, cudaMemcpy(d.rp, h.rp.data(), sizeof(int) * (h.nrows + 1), cudaMemcpyHostToDevice));
  if (d.nnz) NM_CUDA(c, cudaMemcpy(d.ci, h.ci.data(), sizeof(int) * d.nnz, cudaMemcpyHostToDevice));
  if (!h.v.empty()) {
    if (std::is_same<T, double>::value) {
      NM_CUDA(c, cudaMemcpy(d.v, h.v.data(), sizeof(double) * h.v.size(), cudaMemcpyHostToDevice));
    } else {
      std::vector<T> tmp(h.v.begin(), h.v.end());
      NM_CUDA(c, cudaMemcpy(d.v, tmp.data(), sizeof(T) * tmp.size(), cudaMemcpyHostToDevice));
    }
  }
  c->dev_bytes += d.bytes();
  return NM_OK;
}
template int upload_g<double>(nm_ctx*, const GCsrHost&, GCsr<double>&);
template int upload_g<float>(nm_ctx*, const GCsrHost&, GCsr<float>&);

template <typename T>
void free_g(GCsr<T>& g) {
  cudaFree(g.rp);
  cudaFree(g.ci);
  cudaFree(g.v);
  g = GCsr<T>();
}
template void free_g<double>(GCsr<double>&);
template void free_g<float>(GCsr<float>&);

// ---------------------------------------------------------------- kernels
namespace {

constexpr int kT = 256;             // threads per block = 8 rows of 32 lanes
constexpr int kRowsPerBlock = kT / kBlk;
inline int nrb(long long rows) { return (int)((rows + kRowsPerBlock - 1) / kRowsPerBlock); }
constexpr int kTMax = 1024;  // largest CTA of the row kernels (sweep launches)

// Rows a warp computes.  Plain (sweep == 0): CTA b takes rows b*W .. b*W+W-1
// with W warps, one row per warp.  Sweep: CTA b takes the contiguous range
// [b*chunk, (b+1)*chunk) and its W warps walk it together (warp w: rows
// start+w, start+w+W, ...), so the rows in flight on one SM are neighbours
// along the space-filling curve and their gathered neighbour rows are shared
// in that SM's L1.  The loop bound is warp-uniform, so shuffles stay legal.
struct RowRange {
  int r, end, step;
};
__device__ __forceinline__ RowRange row_range(int nrows, int sweep) {
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  RowRange rr;
  if (sweep) {
    const int chunk = (nrows + gridDim.x - 1) / gridDim.x;
    const long long start = (long long)blockIdx.x * chunk;
    rr.r = (int)min((long long)nrows, start + w);
    rr.end = (int)min((long long)nrows, start + chunk);
    rr.step = nw;
  } else {
    rr.r = blockIdx.x * nw + w;
    rr.end = min(nrows, rr.r + 1);
    rr.step = 1;
  }
  return rr;
}

template <typename XT>
__device__ __forceinline__ XT fm(XT a, XT b, XT c) {
  return fma(a, b, c);
}

template <typename XT, bool COH>
__device__ __forceinline__ XT ld(const XT* p) {
  if (COH) return *p;
  return __ldg(p);
}

// One Chebyshev iteration of the mass solve on a block, three-term form.
// With x_0 = 0 and x_1 = b / theta, the semi-iteration
//   x_{j+1} = x_j + a_{j-1} (x_j - x_{j-1}) + c_{j-1} (b - M x_j)
// is the same polynomial in M as the residual / direction form
// (x += d, r -= M d, d = a d + c r) with the same a, c, but it streams four
// blocks per step (gather x_j, own x_{j-1}, own b, write x_{j+1}) instead of
// six.  MODE 0: j = 1 (x_j = b / theta, x_{j-1} = 0); MODE 1: j = 2
// (x_{j-1} = b / theta); MODE 2: general.  xprev and xout may alias: each
// row is read and then written by the thread that owns it, and no thread
// gathers from that buffer in the same step.
// Rows are 3-DOF groups, t_p = sum_h M_gh x(3h+p, lane); one warp per group
// row (lane = block column).  The warp loads up to 32 (column, value)
// entries of its row at once, one per lane, and broadcasts them with
// shuffles, so the gathers of consecutive entries have no load dependency
// between them and can be in flight together.  CTAs take consecutive rows;
// rows are numbered along a space-filling curve, so the rows in flight at
// any time form a compact piece of the mesh whose neighbour rows stay in L2.
template <typename VT, typename XT, int NC, int MODE, int MAXT, int UNR = 4>
__global__ void __launch_bounds__(MAXT, 1)
    k_mass_cheb(int ng, const int* __restrict__ rp, const int* __restrict__ ci, const VT* __restrict__ mv,
                const XT* __restrict__ b, const XT* __restrict__ xcur, const XT* xprev, XT* xout, XT a, XT c,
                XT inv_theta, int sweep) {
  // UNR gathers in flight per warp; a batch's last group is padded with
  // zero-weight entries on the warp's own row (exact: adds +0), so no
  // neighbour is gathered alone
  const int lane = threadIdx.x & (kBlk - 1);
  const RowRange rr = row_range(ng, sweep);
  for (int g = rr.r; g < rr.end; g += rr.step) {
  const XT* src = MODE == 0 ? b : xcur;
  XT bo[NC], xc[NC], xp[NC];
  const size_t i0 = (size_t)NC * g * kBlk + lane;
  // own-row state, loaded before the gathers so the loads overlap
#pragma unroll
  for (int p = 0; p < NC; ++p) {
    bo[p] = b[i0 + p * kBlk];
    xc[p] = MODE == 0 ? bo[p] * inv_theta : xcur[i0 + p * kBlk];
    xp[p] = MODE == 0 ? (XT)0 : MODE == 1 ? bo[p] * inv_theta : xprev[i0 + p * kBlk];
  }
  XT t[NC];
#pragma unroll
  for (int p = 0; p < NC; ++p) t[p] = 0;
  const int e0 = rp[g], e1 = rp[g + 1];
  for (int base = e0; base < e1; base += kBlk) {
    const int cnt = min(kBlk, e1 - base);
    const int myh = lane < cnt ? __ldg(ci + base + lane) : 0;
    const XT mym = lane < cnt ? (XT)__ldg(mv + base + lane) : (XT)0;
    for (int k = 0; k < cnt; k += UNR) {
      const XT* xs[UNR];
      XT m[UNR];
#pragma unroll
      for (int u = 0; u < UNR; ++u) {
        const int q = (k + u) & 31;
        const int h = __shfl_sync(0xffffffffu, myh, q);
        const XT mq = __shfl_sync(0xffffffffu, mym, q);
        const bool in = k + u < cnt;
        xs[u] = src + (size_t)NC * (in ? h : g) * kBlk + lane;
        m[u] = in ? mq : (XT)0;
      }
      XT v[UNR][NC];
#pragma unroll
      for (int u = 0; u < UNR; ++u)
#pragma unroll
        for (int p = 0; p < NC; ++p) v[u][p] = __ldg(xs[u] + p * kBlk);
#pragma unroll
      for (int u = 0; u < UNR; ++u)
#pragma unroll
        for (int p = 0; p < NC; ++p) t[p] = fm<XT>(m[u], v[u][p], t[p]);
    }
  }
#pragma unroll
  for (int p = 0; p < NC; ++p) {
    const XT tt = MODE == 0 ? t[p] * inv_theta : t[p];
    // x_{j+1} = x_j + a (x_j - x_{j-1}) + c (b - M x_j)
    xout[i0 + p * kBlk] = fm<XT>(c, bo[p] - tt, fm<XT>(a, xc[p] - xp[p], xc[p]));
  }
  }  // rows
}

// Vector-load variant of the gather Chebyshev step (same recurrence, MODE
// convention and results up to rounding).  A warp still owns one row, but
// each neighbour row of the block (NC * 32 values) is read with 16-byte
// loads by LPN = 32 / V lanes (V values per load), so one warp instruction
// fetches SLOTS = V neighbour rows at once: lane (q, i) accumulates columns
// V*i .. V*i+V-1 over the neighbours k with k % SLOTS == q, and the SLOTS
// partial sums are combined with shuffles at the end.  Four times fewer load
// instructions than the scalar-lane kernel for FP32.
template <typename XT>
struct Vec16;
template <>
struct Vec16<float> {
  using T = float4;
  static constexpr int V = 4;
};
template <>
struct Vec16<double> {
  using T = double2;
  static constexpr int V = 2;
};
template <typename VT4, typename XT>
__device__ __forceinline__ void vfma(XT m, const VT4& x, XT* acc);
template <>
__device__ __forceinline__ void vfma<float4, float>(float m, const float4& x, float* acc) {
  acc[0] = fmaf(m, x.x, acc[0]);
  acc[1] = fmaf(m, x.y, acc[1]);
  acc[2] = fmaf(m, x.z, acc[2]);
  acc[3] = fmaf(m, x.w, acc[3]);
}
template <>
__device__ __forceinline__ void vfma<double2, double>(double m, const double2& x, double* acc) {
  acc[0] = fma(m, x.x, acc[0]);
  acc[1] = fma(m, x.y, acc[1]);
}
template <typename VT4>
__device__ __forceinline__ VT4 ldv(const VT4* p) {
  return __ldg(p);
}

template <typename VT, typename XT, int NC, int MODE, int MAXT>
__global__ void __launch_bounds__(MAXT, 1)
    k_gcheb(int ng, const int* __restrict__ rp, const int* __restrict__ ci, const VT* __restrict__ mv,
            const XT* __restrict__ b, const XT* __restrict__ xcur, const XT* xprev, XT* xout, XT a, XT c,
            XT inv_theta, int sweep) {
  using V4 = typename Vec16<XT>::T;
  constexpr int V = Vec16<XT>::V;
  constexpr int LPN = kBlk / V;      // lanes per neighbour row (per component)
  constexpr int SLOTS = 32 / LPN;    // neighbour rows per warp instruction
  constexpr int RW = NC * kBlk;      // values per block row
  const int lane = threadIdx.x & 31;
  const int q = lane / LPN, i = lane % LPN;
  const RowRange rr = row_range(ng, sweep);
  for (int g = rr.r; g < rr.end; g += rr.step) {
  const XT* src = MODE == 0 ? b : xcur;
  XT acc[NC][V];
#pragma unroll
  for (int p = 0; p < NC; ++p)
#pragma unroll
    for (int v = 0; v < V; ++v) acc[p][v] = 0;
  const int e0 = rp[g], e1 = rp[g + 1];
  for (int base = e0; base < e1; base += 32) {
    const int cnt = min(32, e1 - base);
    const int myh = lane < cnt ? __ldg(ci + base + lane) : g;
    const XT mym = lane < cnt ? (XT)__ldg(mv + base + lane) : (XT)0;
    for (int k = 0; k < cnt; k += 2 * SLOTS) {
      // two rounds of SLOTS neighbours in flight; entries past cnt carry m = 0
      const int k0 = k + q, k1 = k + SLOTS + q;
      const int h0 = __shfl_sync(0xffffffffu, myh, k0 & 31), h1 = __shfl_sync(0xffffffffu, myh, k1 & 31);
      const XT m0 = __shfl_sync(0xffffffffu, mym, k0 & 31), m1 = __shfl_sync(0xffffffffu, mym, k1 & 31);
      const XT w0 = k0 < cnt ? m0 : (XT)0, w1 = k1 < cnt ? m1 : (XT)0;
      const V4* p0 = reinterpret_cast<const V4*>(src + (size_t)(k0 < cnt ? h0 : g) * RW) + i;
      const V4* p1 = reinterpret_cast<const V4*>(src + (size_t)(k1 < cnt ? h1 : g) * RW) + i;
      V4 x0[NC], x1[NC];
#pragma unroll
      for (int p = 0; p < NC; ++p) {
        x0[p] = ldv(p0 + p * LPN);
        x1[p] = ldv(p1 + p * LPN);
      }
#pragma unroll
      for (int p = 0; p < NC; ++p) {
        vfma<V4, XT>(w0, x0[p], acc[p]);
        vfma<V4, XT>(w1, x1[p], acc[p]);
      }
    }
  }
  // combine the SLOTS partial sums (butterfly: every lane gets the total)
#pragma unroll
  for (int o = LPN; o < 32; o <<= 1)
#pragma unroll
    for (int p = 0; p < NC; ++p)
#pragma unroll
      for (int v = 0; v < V; ++v) acc[p][v] += __shfl_xor_sync(0xffffffffu, acc[p][v], o);
  // epilogue: lane (q, i) writes components q, q + SLOTS, ..., columns V*i ..
#pragma unroll
  for (int pq = 0; pq < NC; pq += SLOTS) {
    const int cq = pq + q;
    if (cq >= NC) break;
    XT t[V];
#pragma unroll
    for (int p = 0; p < NC; ++p)
      if (p == cq) {
#pragma unroll
        for (int v = 0; v < V; ++v) t[v] = acc[p][v];
      }
    const size_t o = (size_t)g * RW + (size_t)cq * kBlk + (size_t)i * V;
    const V4 bo = *reinterpret_cast<const V4*>(b + o);
    const XT* bs = reinterpret_cast<const XT*>(&bo);
    V4 xc4, xp4;
    if (MODE != 0) xc4 = *reinterpret_cast<const V4*>(xcur + o);
    if (MODE == 2) xp4 = *reinterpret_cast<const V4*>(xprev + o);
    const XT* xcs = reinterpret_cast<const XT*>(&xc4);
    const XT* xps = reinterpret_cast<const XT*>(&xp4);
    V4 out;
    XT* os = reinterpret_cast<XT*>(&out);
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const XT xc = MODE == 0 ? bs[v] * inv_theta : xcs[v];
      const XT xp = MODE == 0 ? (XT)0 : MODE == 1 ? bs[v] * inv_theta : xps[v];
      const XT tt = MODE == 0 ? t[v] * inv_theta : t[v];
      os[v] = fm<XT>(c, bs[v] - tt, fm<XT>(a, xc - xp, xc));
    }
    *reinterpret_cast<V4*>(xout + o) = out;
  }
  }  // rows
}

template <typename VT>
__global__ void __launch_bounds__(kT) k_mass_spmv(int ng, const int* __restrict__ rp, const int* __restrict__ ci,
                                                  const VT* __restrict__ mv, const double* __restrict__ x,
                                                  double* __restrict__ y) {
  const int lane = threadIdx.x & (kBlk - 1);
  const int g = blockIdx.x * kRowsPerBlock + (threadIdx.x >> 5);
  if (g >= ng) return;
  double t0 = 0, t1 = 0, t2 = 0;
  for (int e = rp[g]; e < rp[g + 1]; ++e) {
    const int h = __ldg(ci + e);
    const double m = (double)__ldg(mv + e);
    const double* xs = x + (size_t)3 * h * kBlk + lane;
    t0 = fma(m, __ldg(xs), t0);
    t1 = fma(m, __ldg(xs + kBlk), t1);
    t2 = fma(m, __ldg(xs + 2 * kBlk), t2);
  }
  y[((size_t)3 * g) * kBlk + lane] = t0;
  y[((size_t)3 * g + 1) * kBlk + lane] = t1;
  y[((size_t)3 * g + 2) * kBlk + lane] = t2;
}

// x0(k, lane) = sum_entries sum_q et_q w(3h+q, lane)   (pressure rows)
template <typename VT, typename XT, int MAXT>
__global__ void __launch_bounds__(MAXT, 1) k_et(int np, const int* __restrict__ rp, const int* __restrict__ ci,
                                              const VT* __restrict__ v3, const XT* __restrict__ w,
                                              XT* __restrict__ x0, int sweep) {
  const int lane = threadIdx.x & (kBlk - 1);
  const RowRange rr = row_range(np, sweep);
  for (int k = rr.r; k < rr.end; k += rr.step) {
  XT s = 0;
  const int e0 = rp[k], e1 = rp[k + 1];
  for (int base = e0; base < e1; base += kBlk) {
    const int cnt = min(kBlk, e1 - base);
    const int myh = lane < cnt ? __ldg(ci + base + lane) : 0;
    int q = 0;
    for (; q + 2 <= cnt; q += 2) {
      XT w_[2][3];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const XT* ws = w + (size_t)3 * __shfl_sync(0xffffffffu, myh, q + u) * kBlk + lane;
        w_[u][0] = __ldg(ws);
        w_[u][1] = __ldg(ws + kBlk);
        w_[u][2] = __ldg(ws + 2 * kBlk);
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const VT* e3 = v3 + 3 * (size_t)(base + q + u);
        s = fm<XT>((XT)__ldg(e3), w_[u][0], s);
        s = fm<XT>((XT)__ldg(e3 + 1), w_[u][1], s);
        s = fm<XT>((XT)__ldg(e3 + 2), w_[u][2], s);
      }
    }
    for (; q < cnt; ++q) {
      const XT* ws = w + (size_t)3 * __shfl_sync(0xffffffffu, myh, q) * kBlk + lane;
      const VT* e3 = v3 + 3 * (size_t)(base + q);
      s = fm<XT>((XT)__ldg(e3), __ldg(ws), s);
      s = fm<XT>((XT)__ldg(e3 + 1), __ldg(ws + kBlk), s);
      s = fm<XT>((XT)__ldg(e3 + 2), __ldg(ws + 2 * kBlk), s);
    }
  }
  x0[(size_t)k * kBlk + lane] = s;
  }  // rows
}

__device__ __forceinline__ bool gbar(GridBar* bar, unsigned nblocks, int* status) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned g = *((volatile unsigned*)&bar->gen);
    __threadfence();
    if (atomicAdd(&bar->count, 1u) == nblocks - 1) {
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
        if (++spins > kSpinLimit) {
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

// Persistent Chebyshev solve on the pressure block: all iterations in one
// cooperative launch, rows in a grid-stride loop, bounded grid barriers.
constexpr int kTP = 1024;  // threads of the persistent kernel (one CTA per SM)
constexpr int kRowsP = kTP / kBlk;
template <typename VT, typename XT>
__global__ void __launch_bounds__(kTP)
    k_ap_cheb(int np, const int* __restrict__ rp, const int* __restrict__ ci, const VT* __restrict__ av,
              const XT* __restrict__ b, XT* xout, XT* r, XT* x, XT* d0, XT* d1, const double* __restrict__ coef,
              int deg, XT inv_theta, GridBar* bar, int* status) {
  const int lane = threadIdx.x & (kBlk - 1);
  const int rstride = gridDim.x * kRowsP;
  for (int k = 0; k < deg; ++k) {
    const XT a = (XT)coef[k], c = (XT)coef[deg + k];
    const XT* dcur = (k & 1) ? d1 : d0;
    XT* dnext = (k & 1) ? d0 : d1;
    const bool first = k == 0, last = k == deg - 1;
    for (int row = blockIdx.x * kRowsP + (threadIdx.x >> 5); row < np; row += rstride) {
      const XT* src = first ? b : dcur;
      XT t = 0;
      const int e0 = rp[row], e1 = rp[row + 1];
      for (int base = e0; base < e1; base += kBlk) {
        const int cnt = min(kBlk, e1 - base);
        const int myh = lane < cnt ? __ldg(ci + base + lane) : 0;
        const XT mya = lane < cnt ? (XT)__ldg(av + base + lane) : (XT)0;
        int q = 0;
        for (; q + 4 <= cnt; q += 4) {
          XT xv[4], m[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const XT* xp = src + (size_t)__shfl_sync(0xffffffffu, myh, q + u) * kBlk + lane;
            xv[u] = first ? __ldg(xp) : *xp;  // written by other blocks in this launch: coherent load
            m[u] = __shfl_sync(0xffffffffu, mya, q + u);
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) t = fm<XT>(m[u], xv[u], t);
        }
        for (; q < cnt; ++q) {
          const XT* xp = src + (size_t)__shfl_sync(0xffffffffu, myh, q) * kBlk + lane;
          t = fm<XT>(__shfl_sync(0xffffffffu, mya, q), first ? __ldg(xp) : *xp, t);
        }
      }
      const size_t idx = (size_t)row * kBlk + lane;
      XT dc, rr, xn;
      if (first) {
        const XT bi = b[idx];
        dc = bi * inv_theta;
        rr = bi - t * inv_theta;
        xn = dc;
      } else {
        dc = dcur[idx];
        rr = r[idx] - t;
        xn = x[idx] + dc;
      }
      const XT dn = fm<XT>(a, dc, c * rr);
      if (last) {
        xout[idx] = xn + dn;
      } else {
        r[idx] = rr;
        x[idx] = xn;
        dnext[idx] = dn;
      }
    }
    if (!last && !gbar(bar, gridDim.x, status)) return;
  }
}

// w(3g+p) = sum_h A_gh(p, :) v(3h + :) [+ sum_k E_gk(p) y(k)]; epilogue as k_amv.
template <typename VT, typename XT, bool HAS_E, int MODE, int MAXT>
__global__ void __launch_bounds__(MAXT, 1)
    k_amv3(int ng, const int* __restrict__ arp, const int* __restrict__ aci, const VT* __restrict__ av,
           const int* __restrict__ erp, const int* __restrict__ eci, const VT* __restrict__ ev,
           const XT* __restrict__ v, const XT* __restrict__ y, XT* __restrict__ out, const XT* __restrict__ vk,
           const XT* __restrict__ vkm1, XT* __restrict__ yacc, XT s, XT cc, XT pm, XT mu,
           const XT* __restrict__ fz, XT fco, int sweep) {
  const int lane = threadIdx.x & (kBlk - 1);
  const RowRange rr = row_range(ng, sweep);
  for (int g = rr.r; g < rr.end; g += rr.step) {
  XT w0 = 0, w1 = 0, w2 = 0;
  const int a0 = arp[g], a1 = arp[g + 1];
  for (int base = a0; base < a1; base += kBlk) {
    const int cnt = min(kBlk, a1 - base);
    const int myh = lane < cnt ? __ldg(aci + base + lane) : 0;
    int k = 0;
    for (; k + 2 <= cnt; k += 2) {
      XT xv[2][3];
      const VT* a9[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const XT* vs = v + (size_t)3 * __shfl_sync(0xffffffffu, myh, k + u) * kBlk + lane;
        xv[u][0] = __ldg(vs);
        xv[u][1] = __ldg(vs + kBlk);
        xv[u][2] = __ldg(vs + 2 * kBlk);
        a9[u] = av + 9 * (size_t)(base + k + u);
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        w0 = fm<XT>((XT)__ldg(a9[u] + 0), xv[u][0], w0);
        w0 = fm<XT>((XT)__ldg(a9[u] + 1), xv[u][1], w0);
        w0 = fm<XT>((XT)__ldg(a9[u] + 2), xv[u][2], w0);
        w1 = fm<XT>((XT)__ldg(a9[u] + 3), xv[u][0], w1);
        w1 = fm<XT>((XT)__ldg(a9[u] + 4), xv[u][1], w1);
        w1 = fm<XT>((XT)__ldg(a9[u] + 5), xv[u][2], w1);
        w2 = fm<XT>((XT)__ldg(a9[u] + 6), xv[u][0], w2);
        w2 = fm<XT>((XT)__ldg(a9[u] + 7), xv[u][1], w2);
        w2 = fm<XT>((XT)__ldg(a9[u] + 8), xv[u][2], w2);
      }
    }
    for (; k < cnt; ++k) {
      const XT* vs = v + (size_t)3 * __shfl_sync(0xffffffffu, myh, k) * kBlk + lane;
      const XT x0 = __ldg(vs), x1 = __ldg(vs + kBlk), x2 = __ldg(vs + 2 * kBlk);
      const VT* a9 = av + 9 * (size_t)(base + k);
      w0 = fm<XT>((XT)__ldg(a9 + 0), x0, w0);
      w0 = fm<XT>((XT)__ldg(a9 + 1), x1, w0);
      w0 = fm<XT>((XT)__ldg(a9 + 2), x2, w0);
      w1 = fm<XT>((XT)__ldg(a9 + 3), x0, w1);
      w1 = fm<XT>((XT)__ldg(a9 + 4), x1, w1);
      w1 = fm<XT>((XT)__ldg(a9 + 5), x2, w1);
      w2 = fm<XT>((XT)__ldg(a9 + 6), x0, w2);
      w2 = fm<XT>((XT)__ldg(a9 + 7), x1, w2);
      w2 = fm<XT>((XT)__ldg(a9 + 8), x2, w2);
    }
  }
  if (HAS_E) {
    for (int e = erp[g]; e < erp[g + 1]; ++e) {
      const XT yk = __ldg(y + (size_t)__ldg(eci + e) * kBlk + lane);
      const VT* e3 = ev + 3 * (size_t)e;
      w0 = fm<XT>((XT)__ldg(e3 + 0), yk, w0);
      w1 = fm<XT>((XT)__ldg(e3 + 1), yk, w1);
      w2 = fm<XT>((XT)__ldg(e3 + 2), yk, w2);
    }
  }
  const XT ww[3] = {w0, w1, w2};
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    const size_t idx = ((size_t)3 * g + p) * kBlk + lane;
    if (MODE == 0) {
      out[idx] = ww[p];
    } else {
      XT t = fm<XT>(s, fm<XT>(-cc, vk[idx], ww[p]), -pm * vkm1[idx]);
      if (fz) t = fm<XT>(fco, fz[idx], t);
      out[idx] = t;
      yacc[idx] = fm<XT>(mu, t, yacc[idx]);
    }
  }
  }  // rows
}

// blk(i, c) = Z(:, j0 + c)(i) through a 32 x 32 shared-memory tile.
template <typename XT>
__global__ void k_gather_cols(double* const* __restrict__ chunks, size_t ld, int j0, int n, XT* __restrict__ blk) {
  __shared__ double tile[kBlk][kBlk + 1];
  const int i0 = blockIdx.x * kBlk;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int c = ty; c < kBlk; c += 8) {
    const int j = j0 + c;
    const double* col = chunks[j / Basis::kChunk] + (size_t)(j % Basis::kChunk) * ld;
    const int i = i0 + tx;
    tile[c][tx] = i < n ? col[i] : 0.0;
  }
  __syncthreads();
  for (int r = ty; r < kBlk; r += 8) {
    const int i = i0 + r;
    if (i < n) blk[(size_t)i * kBlk + tx] = (XT)tile[tx][r];
  }
}

template <typename XT>
__global__ void k_to_colmajor(const XT* __restrict__ blk, int n, double* __restrict__ out, size_t ld) {
  __shared__ double tile[kBlk][kBlk + 1];
  const int i0 = blockIdx.x * kBlk;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int r = ty; r < kBlk; r += 8) {
    const int i = i0 + r;
    tile[r][tx] = i < n ? (double)blk[(size_t)i * kBlk + tx] : 0.0;
  }
  __syncthreads();
  for (int c = ty; c < kBlk; c += 8) {
    const int i = i0 + tx;
    if (i < n) out[(size_t)c * ld + i] = tile[tx][c];
  }
}

template <typename XT>
__global__ void k_from_colmajor(const double* __restrict__ src, size_t ld, int n, int ncol, XT* __restrict__ blk) {
  __shared__ double tile[kBlk][kBlk + 1];
  const int i0 = blockIdx.x * kBlk;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int c = ty; c < kBlk; c += 8) {
    const int i = i0 + tx;
    tile[c][tx] = i < n && c < ncol ? src[(size_t)c * ld + i] : 0.0;  // columns >= ncol read as zero
  }
  __syncthreads();
  for (int r = ty; r < kBlk; r += 8) {
    const int i = i0 + r;
    if (i < n) blk[(size_t)i * kBlk + tx] = (XT)tile[tx][r];
  }
}

// Range form of the filter: vk = a1 z, vkm1 = 0, y = mu1 vk.
template <typename XT>
__global__ void k_init_range_blk(XT* vk, XT* vkm1, XT* y, const XT* z, XT a1, XT mu1, size_t len) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= len) return;
  const XT v = a1 * z[i];
  vk[i] = v;
  vkm1[i] = (XT)0;
  y[i] = mu1 * v;
}
// dst (row-major FP64 block) = (double) src (row-major FP32 block)
__global__ void k_f2d_flat(const float* __restrict__ src, double* __restrict__ dst, size_t len) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < len) dst[i] = (double)src[i];
}

template <typename XT>
__global__ void k_init_filter_blk(XT* vk, XT* vkm1, XT* y, const XT* v, XT mu0, size_t len) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < len) {
    const XT vi = v[i];
    vk[i] = vi;
    vkm1[i] = 0;
    y[i] = mu0 * vi;
  }
}

}  // namespace

// Default gather kernel per component count when the autotuner has not
// run: the 16-byte vector-load kernel (k_gcheb) for one-component rows (Ap,
// 128-byte rows), the one-value-per-lane kernel (k_mass_cheb) for the
// three-component mass rows.
bool gather_vec(int nc) { return nc == 1; }

// Grid of a launch with `thr` threads per CTA over `nrows` rows: one row per
// warp (plain), or for a sweep the CTAs of `fn` that fit on the GPU at once
// (occupancy API, cached per kernel and CTA size), each taking one
// contiguous range of rows.
int row_grid(const void* fn, int thr, int nrows, int sweep) {
  const int rows = thr / 32;
  const int plain = (nrows + rows - 1) / rows;
  if (!sweep) return std::max(1, plain);
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> cache;
  int per_gpu = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find({fn, thr});
    if (it != cache.end()) {
      per_gpu = it->second;
    } else {
      int dev = 0, sms = 0, per = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, thr, 0) != cudaSuccess || per < 1) {
        cudaGetLastError();
        per = 1;
      }
      per_gpu = std::max(1, sms) * per;
      cache[{fn, thr}] = per_gpu;
    }
  }
  return std::max(1, std::min(per_gpu, plain));
}

int launch_threads(const GatherCfg& cfg) {
  const int cap = cfg.sweep ? kTMax : kT;
  return std::min(cap, std::max(32, cfg.threads / 32 * 32));
}

template <typename VT, typename XT, int NC>
void gather_cheb(const GCsr<VT>& M, const ChebSetup& ch, const XT* b, XT* x, XT* work, cudaStream_t s,
                 const GatherCfg& cfg) {
  const int ng = M.nrows;
  if (ng == 0 || ch.deg == 0) return;
  const size_t len = (size_t)NC * ng * kBlk;
  XT* buf[2] = {work, work + len};  // x_j lives in buf[j & 1]
  const XT it = (XT)ch.inv_theta;
  // kernel: 0 one value per lane, 4 gathers in flight; 1 16-byte vector
  // gathers (k_gcheb); 2 one value per lane, 8 gathers in flight (CTAs of
  // at most 256 threads)
  const int kind = cfg.vec < 0 ? (gather_vec(NC) ? 1 : 0) : cfg.vec;
  const bool vec = kind == 1, deep = kind == 2;
  const int thr = deep ? std::min(kT, launch_threads(cfg)) : launch_threads(cfg);
  const int sw = deep ? 0 : cfg.sweep;
  const bool big = thr > kT;  // CTAs above 256 threads use the kernels compiled for 1024
  const void* fn = deep ? (const void*)k_mass_cheb<VT, XT, NC, 2, kT, 8>
                   : vec ? (big ? (const void*)k_gcheb<VT, XT, NC, 2, kTMax> : (const void*)k_gcheb<VT, XT, NC, 2, kT>)
                         : (big ? (const void*)k_mass_cheb<VT, XT, NC, 2, kTMax>
                                : (const void*)k_mass_cheb<VT, XT, NC, 2, kT>);
  const int grid = row_grid(fn, thr, ng, sw);
  for (int j = 1; j <= ch.deg; ++j) {
    const XT a = (XT)ch.a[j - 1], c = (XT)ch.c[j - 1];
    XT* out = j == ch.deg ? x : buf[(j + 1) & 1];
    const XT* cur = buf[j & 1];
    const XT* prev = buf[(j + 1) & 1];
#define NM_MV(MODE)                                                                                            \
  do {                                                                                                         \
    if (big)                                                                                                   \
      k_gcheb<VT, XT, NC, MODE, kTMax><<<grid, thr, 0, s>>>(ng, M.rp, M.ci, M.v, b, cur, prev, out, a, c, it, sw); \
    else                                                                                                       \
      k_gcheb<VT, XT, NC, MODE, kT><<<grid, thr, 0, s>>>(ng, M.rp, M.ci, M.v, b, cur, prev, out, a, c, it, sw);    \
  } while (0)
#define NM_MC(MODE)                                                                                           \
  do {                                                                                                        \
    if (big)                                                                                                  \
      k_mass_cheb<VT, XT, NC, MODE, kTMax><<<grid, thr, 0, s>>>(ng, M.rp, M.ci, M.v, b, cur, prev, out, a, c, it, \
                                                                 sw);                                         \
    else                                                                                                      \
      k_mass_cheb<VT, XT, NC, MODE, kT><<<grid, thr, 0, s>>>(ng, M.rp, M.ci, M.v, b, cur, prev, out, a, c, it, sw); \
  } while (0)
#define NM_MD(MODE) \
  k_mass_cheb<VT, XT, NC, MODE, kT, 8><<<grid, thr, 0, s>>>(ng, M.rp, M.ci, M.v, b, cur, prev, out, a, c, it, 0)
    if (deep) {
      if (j == 1) NM_MD(0);
      else if (j == 2) NM_MD(1);
      else NM_MD(2);
    } else if (vec) {
      if (j == 1) NM_MV(0);
      else if (j == 2) NM_MV(1);
      else NM_MV(2);
    } else {
      if (j == 1) NM_MC(0);
      else if (j == 2) NM_MC(1);
      else NM_MC(2);
    }
#undef NM_MC
#undef NM_MV
#undef NM_MD
    nmg::add_launches(1);
  }
}

template <typename VT, typename XT>
void blk_mass_cheb(const GCsr<VT>& M, const ChebSetup& ch, const XT* b, XT* x, XT* work, cudaStream_t s,
                   const GatherCfg& cfg) {
  gather_cheb<VT, XT, 3>(M, ch, b, x, work, s, cfg);
}

template <typename VT, typename XT>
void blk_ap_cheb(const GCsr<VT>& Ap, const ChebSetup& ch, const XT* b, XT* x, XT* work, cudaStream_t s,
                 const GatherCfg& cfg) {
  gather_cheb<VT, XT, 1>(Ap, ch, b, x, work, s, cfg);
}

// Largest L1 (no shared-memory carve-out) for every gather kernel: their
// neighbour rows are reused from L1, and they use no shared memory but the
// few bytes of k_colres_part.
template <typename VT, typename XT, int MAXT>
void prefer_l1_set() {
  const void* fs[] = {(const void*)k_mass_cheb<VT, XT, 3, 0, MAXT>, (const void*)k_mass_cheb<VT, XT, 3, 1, MAXT>,
                      (const void*)k_mass_cheb<VT, XT, 3, 2, MAXT>, (const void*)k_mass_cheb<VT, XT, 1, 0, MAXT>,
                      (const void*)k_mass_cheb<VT, XT, 1, 1, MAXT>, (const void*)k_mass_cheb<VT, XT, 1, 2, MAXT>,
                      (const void*)k_gcheb<VT, XT, 3, 0, MAXT>,     (const void*)k_gcheb<VT, XT, 3, 1, MAXT>,
                      (const void*)k_gcheb<VT, XT, 3, 2, MAXT>,     (const void*)k_gcheb<VT, XT, 1, 0, MAXT>,
                      (const void*)k_gcheb<VT, XT, 1, 1, MAXT>,     (const void*)k_gcheb<VT, XT, 1, 2, MAXT>,
                      (const void*)k_amv3<VT, XT, true, 0, MAXT>,   (const void*)k_amv3<VT, XT, true, 1, MAXT>,
                      (const void*)k_amv3<VT, XT, false, 0, MAXT>,  (const void*)k_amv3<VT, XT, false, 1, MAXT>,
                      (const void*)k_et<VT, XT, MAXT>};
  for (const void* f : fs) cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
  if (MAXT == kT)
    for (const void* f : {(const void*)k_mass_cheb<VT, XT, 3, 0, kT, 8>, (const void*)k_mass_cheb<VT, XT, 3, 1, kT, 8>,
                          (const void*)k_mass_cheb<VT, XT, 3, 2, kT, 8>, (const void*)k_mass_cheb<VT, XT, 1, 0, kT, 8>,
                          (const void*)k_mass_cheb<VT, XT, 1, 1, kT, 8>, (const void*)k_mass_cheb<VT, XT, 1, 2, kT, 8>})
      cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
}

void blk_prefer_l1() {
  prefer_l1_set<float, float, kT>();
  prefer_l1_set<float, float, kTMax>();
  prefer_l1_set<double, double, kT>();
  prefer_l1_set<double, double, kTMax>();
  cudaGetLastError();
}

template <typename VT>
void blk_mass_spmv(const GCsr<VT>& M, const double* x, double* y, cudaStream_t s) {
  k_mass_spmv<VT><<<nrb(M.nrows), kT, 0, s>>>(M.nrows, M.rp, M.ci, M.v, x, y);
  nmg::add_launches(1);
}

template <typename VT, typename XT>
void blk_et(const GCsr<VT>& ET, const XT* w, XT* x0, cudaStream_t s, const GatherCfg& cfg) {
  const int thr = launch_threads(cfg);
  if (thr > kT) {
    const int grid = row_grid((const void*)k_et<VT, XT, kTMax>, thr, ET.nrows, cfg.sweep);
    k_et<VT, XT, kTMax><<<grid, thr, 0, s>>>(ET.nrows, ET.rp, ET.ci, ET.v, w, x0, cfg.sweep);
  } else {
    const int grid = row_grid((const void*)k_et<VT, XT, kT>, thr, ET.nrows, cfg.sweep);
    k_et<VT, XT, kT><<<grid, thr, 0, s>>>(ET.nrows, ET.rp, ET.ci, ET.v, w, x0, cfg.sweep);
  }
  nmg::add_launches(1);
}

template <typename VT, typename XT>
void blk_ap_cheb_persistent(const GCsr<VT>& Ap, const ChebSetup& ch, const XT* b, XT* x, XT* work, GridBar* bar,
                            int* status, int blocks, cudaStream_t s) {
  const int np = Ap.nrows;
  if (np == 0 || ch.deg == 0) return;
  const size_t len = (size_t)np * kBlk;
  XT* r = work;
  XT* d0 = work + len;
  XT* d1 = work + 2 * len;
  XT* xi = work + 3 * len;
  blocks = std::max(1, std::min(blocks, (np + kRowsP - 1) / kRowsP));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(kTP);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const XT it = (XT)ch.inv_theta;
  int deg = ch.deg;
  cudaError_t e = cudaMemsetAsync(bar, 0, sizeof(GridBar), s);
  if (e == cudaSuccess)
    e = cudaLaunchKernelEx(&cfg, k_ap_cheb<VT, XT>, np, (const int*)Ap.rp, (const int*)Ap.ci, (const VT*)Ap.v, b, x,
                           r, xi, d0, d1, (const double*)ch.d_coef, deg, it, bar, status);
  if (e != cudaSuccess) {
    // refused cooperative launch (not sticky): clear it and run the gather
    // form of the same solve, which needs no co-resident CTAs
    cudaGetLastError();
    blk_ap_cheb<VT, XT>(Ap, ch, b, x, work, s);
    return;
  }
  nmg::add_launches(1);
}

int blk_coop_blocks() {
  int dev = 0, sms = 0, coop = 0, p64 = 0, p32 = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  if (!coop) return 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p64, k_ap_cheb<double, double>, kTP, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p32, k_ap_cheb<float, float>, kTP, 0);
  // one CTA per SM keeps the barrier to one arrival per SM
  return std::min(1, std::min(p64, p32)) * sms;
}

template <typename VT, typename XT>
void blk_amv(const GCsr<VT>& A, const GCsr<VT>* E, const XT* v, const XT* y, XT* out, const XT* vk, const XT* vkm1,
             XT* yacc, const FiltEpi& ep, cudaStream_t s, const GatherCfg& cfg) {
  const int ng = A.nrows;
  const int thr = launch_threads(cfg), sw = cfg.sweep;
  const bool big = thr > kT;
  const int grid = row_grid(big ? (const void*)k_amv3<VT, XT, true, 1, kTMax> : (const void*)k_amv3<VT, XT, true, 1, kT>,
                            thr, ng, sw);
  const XT S = (XT)ep.s, CC = (XT)ep.cc, PM = (XT)ep.pm, MU = (XT)ep.mu, FC = (XT)ep.fco;
  const XT* FZ = (const XT*)ep.fz;
  const int* erp = E ? E->rp : nullptr;
  const int* eci = E ? E->ci : nullptr;
  const VT* ev = E ? E->v : nullptr;
#define NM_AMV(HE, MO)                                                                                            \
  do {                                                                                                            \
    if (big)                                                                                                      \
      k_amv3<VT, XT, HE, MO, kTMax><<<grid, thr, 0, s>>>(ng, A.rp, A.ci, A.v, erp, eci, ev, v, y, out, vk, vkm1,    \
                                                         yacc, S, CC, PM, MU, FZ, FC, sw);                         \
    else                                                                                                          \
      k_amv3<VT, XT, HE, MO, kT><<<grid, thr, 0, s>>>(ng, A.rp, A.ci, A.v, erp, eci, ev, v, y, out, vk, vkm1, yacc, \
                                                      S, CC, PM, MU, FZ, FC, sw);                                  \
  } while (0)
  if (E) {
    if (ep.mode == 0) NM_AMV(true, 0);
    else NM_AMV(true, 1);
  } else {
    if (ep.mode == 0) NM_AMV(false, 0);
    else NM_AMV(false, 1);
  }
#undef NM_AMV
  nmg::add_launches(1);
}

template <typename XT>
void blk_gather_cols(const Basis& Z, int j0, int n, XT* blk, cudaStream_t s) {
  k_gather_cols<XT><<<(n + kBlk - 1) / kBlk, dim3(kBlk, 8), 0, s>>>(Z.d_chunks, Z.ld, j0, n, blk);
  nmg::add_launches(1);
}
namespace {
__global__ void k_d2f(const double* __restrict__ src, size_t lds, float* __restrict__ dst, size_t ldd, int n,
                      int cols) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * cols) return;
  const int c = (int)(t / n), i = (int)(t % n);
  dst[(size_t)c * ldd + i] = (float)src[(size_t)c * lds + i];
}
__global__ void k_f2d(const float* __restrict__ src, size_t lds, double* __restrict__ dst, size_t ldd, int n,
                      int cols) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * cols) return;
  const int c = (int)(t / n), i = (int)(t % n);
  dst[(size_t)c * ldd + i] = (double)src[(size_t)c * lds + i];
}
__global__ void k_sub_f32(double* __restrict__ W, size_t ldw, const float* __restrict__ T, size_t ldt, int n,
                          int cols) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * cols) return;
  const int c = (int)(t / n), i = (int)(t % n);
  W[(size_t)c * ldw + i] -= (double)T[(size_t)c * ldt + i];
}
}  // namespace

namespace {
// R = (float)(AU - theta_col BU) on row-major 32-column blocks
__global__ void k_resid_f32(const double* __restrict__ AU, const double* __restrict__ BU,
                            const double* __restrict__ theta, float* __restrict__ R, float scale, size_t len) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= len) return;
  R[i] = (float)(AU[i] - theta[i & (kBlk - 1)] * BU[i]) * scale;
}
// v += f_col R
__global__ void k_force(float* __restrict__ v, const float* __restrict__ R, const float* __restrict__ f, size_t len) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= len) return;
  v[i] = fmaf(f[i & (kBlk - 1)], R[i], v[i]);
}
// U(:, col) += sc_col G(:, col): G row-major 32-column block, U column-major
__global__ void k_add_colmajor(const float* __restrict__ G, const double* __restrict__ sc, int n, int ncol,
                               double* __restrict__ U, size_t ld) {
  __shared__ float tile[kBlk][kBlk + 1];
  const int i0 = blockIdx.x * kBlk;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int r = ty; r < kBlk; r += 8) {
    const int i = i0 + r;
    tile[r][tx] = i < n ? G[(size_t)i * kBlk + tx] : 0.0f;
  }
  __syncthreads();
  for (int c = ty; c < ncol; c += 8) {
    const int i = i0 + tx;
    if (i < n) U[(size_t)c * ld + i] += sc[c] * (double)tile[tx][c];
  }
}
}  // namespace

namespace {
// Per-column sums of a row-major 32-column FP64 block pair, in a fixed order:
// stage 1, CTA b sums rows b, b + G, b + 2G, ... (one warp per row, lane =
// column) into part[b][0:32] = sum (AU - theta BU)^2, part[b][32:64] =
// sum U BU; stage 2 adds the G partial sums in CTA order.
constexpr int kColRedCtas = 512;
__global__ void __launch_bounds__(256) k_colres_part(const double* __restrict__ AU, const double* __restrict__ BU,
                                                     const double* __restrict__ U, const double* __restrict__ theta,
                                                     int rows, double* __restrict__ part) {
  __shared__ double sr[8][kBlk], su[8][kBlk];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const double th = theta[lane];
  double r2 = 0.0, ub = 0.0;
  for (int i = blockIdx.x * 8 + w; i < rows; i += gridDim.x * 8) {
    const size_t o = (size_t)i * kBlk + lane;
    const double bu = BU[o];
    const double r = fma(-th, bu, AU[o]);
    r2 = fma(r, r, r2);
    ub = fma(U[o], bu, ub);
  }
  sr[w][lane] = r2;
  su[w][lane] = ub;
  __syncthreads();
  if (w == 0) {
    double a = 0.0, b = 0.0;
    for (int q = 0; q < 8; ++q) {
      a += sr[q][lane];
      b += su[q][lane];
    }
    part[(size_t)blockIdx.x * 2 * kBlk + lane] = a;
    part[(size_t)blockIdx.x * 2 * kBlk + kBlk + lane] = b;
  }
}
__global__ void k_colres_sum(const double* __restrict__ part, int nparts, double* __restrict__ out) {
  const int t = threadIdx.x;  // 64 threads: 32 residual sums, 32 B-norms
  double a = 0.0;
  for (int b = 0; b < nparts; ++b) a += part[(size_t)b * 2 * kBlk + t];
  out[t] = a;
}
}  // namespace

size_t blk_colres_scratch() { return (size_t)kColRedCtas * 2 * kBlk + 2 * kBlk; }

namespace {
// One KPM step on row-major blocks: W0 <- alpha (T - c W1) - beta W0 (alpha
// = 2/e, beta = 1 for the three-term step; alpha = 1/e, beta = 0 for T_1),
// and the per-CTA partial sums of V . W0 (in a fixed order: CTA b sums the
// grid-stride elements it owns, a tree within the CTA).
template <typename XT>
__global__ void __launch_bounds__(256) k_kpm_step(XT* __restrict__ W0, const XT* __restrict__ T,
                                                  const XT* __restrict__ W1, const XT* __restrict__ V, double c,
                                                  double alpha, double beta, size_t len, double* __restrict__ part) {
  __shared__ double red[256];
  double acc = 0.0;
  for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < len; i += (size_t)gridDim.x * 256) {
    const double w = alpha * ((double)T[i] - c * (double)W1[i]) - beta * (double)W0[i];
    const XT wx = (XT)w;
    W0[i] = wx;
    acc = fma((double)V[i], (double)wx, acc);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}
template <typename XT>
__global__ void __launch_bounds__(256) k_vdot_part(const XT* __restrict__ V, const XT* __restrict__ W, size_t len,
                                                   double* __restrict__ part) {
  __shared__ double red[256];
  double acc = 0.0;
  for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < len; i += (size_t)gridDim.x * 256)
    acc = fma((double)V[i], (double)W[i], acc);
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}
__global__ void k_sum_parts(const double* __restrict__ part, int nparts, double* __restrict__ out) {
  double s = 0.0;
  for (int b = 0; b < nparts; ++b) s += part[b];
  *out = s;
}
constexpr int kKpmCtas = 1024;
}  // namespace

template <typename XT>
void blk_kpm_step(XT* W0, const XT* T, const XT* W1, const XT* V, double c, double alpha, double beta, size_t len,
                  double* part, double* out, cudaStream_t s) {
  const int g = (int)std::max<size_t>(1, std::min<size_t>(kKpmCtas, (len + 255) / 256));
  if (T) k_kpm_step<XT><<<g, 256, 0, s>>>(W0, T, W1, V, c, alpha, beta, len, part);
  else k_vdot_part<XT><<<g, 256, 0, s>>>(V, W0, len, part);
  k_sum_parts<<<1, 1, 0, s>>>(part, g, out);
  nmg::add_launches(2);
}
template void blk_kpm_step<float>(float*, const float*, const float*, const float*, double, double, double, size_t,
                                  double*, double*, cudaStream_t);
template void blk_kpm_step<double>(double*, const double*, const double*, const double*, double, double, double,
                                   size_t, double*, double*, cudaStream_t);
size_t blk_kpm_scratch() { return kKpmCtas; }

void blk_colres(const double* AU, const double* BU, const double* U, const double* theta, int rows, double* scratch,
                cudaStream_t s) {
  const int g = std::max(1, std::min(kColRedCtas, (rows + 7) / 8));
  k_colres_part<<<g, 256, 0, s>>>(AU, BU, U, theta, rows, scratch);
  k_colres_sum<<<1, 2 * kBlk, 0, s>>>(scratch, g, scratch + (size_t)kColRedCtas * 2 * kBlk);
  nmg::add_launches(2);
}

void blk_resid_f32(const double* AU, const double* BU, const double* theta, float* R, float scale, size_t len,
                   cudaStream_t s) {
  k_resid_f32<<<(int)((len + 255) / 256), 256, 0, s>>>(AU, BU, theta, R, scale, len);
  nmg::add_launches(1);
}
void blk_force(float* v, const float* R, const float* f, size_t len, cudaStream_t s) {
  k_force<<<(int)((len + 255) / 256), 256, 0, s>>>(v, R, f, len);
  nmg::add_launches(1);
}
void blk_add_colmajor(const float* G, const double* sc, int n, double* U, size_t ld, cudaStream_t s) {
  blk_add_colmajor_cols(G, sc, n, kBlk, U, ld, s);
}
void blk_add_colmajor_cols(const float* G, const double* sc, int n, int ncol, double* U, size_t ld, cudaStream_t s) {
  k_add_colmajor<<<(n + kBlk - 1) / kBlk, dim3(kBlk, 8), 0, s>>>(G, sc, n, std::min(ncol, kBlk), U, ld);
  nmg::add_launches(1);
}

void blk_d2f(const double* src, size_t lds, float* dst, size_t ldd, int n, int cols, cudaStream_t s) {
  const long long tot = (long long)n * cols;
  k_d2f<<<(int)((tot + 255) / 256), 256, 0, s>>>(src, lds, dst, ldd, n, cols);
  nmg::add_launches(1);
}
void blk_f2d(const float* src, size_t lds, double* dst, size_t ldd, int n, int cols, cudaStream_t s) {
  const long long tot = (long long)n * cols;
  k_f2d<<<(int)((tot + 255) / 256), 256, 0, s>>>(src, lds, dst, ldd, n, cols);
  nmg::add_launches(1);
}
void blk_sub_f32(double* W, size_t ldw, const float* T, size_t ldt, int n, int cols, cudaStream_t s) {
  const long long tot = (long long)n * cols;
  k_sub_f32<<<(int)((tot + 255) / 256), 256, 0, s>>>(W, ldw, T, ldt, n, cols);
  nmg::add_launches(1);
}

template <typename XT>
void blk_to_colmajor(const XT* blk, int n, double* out, size_t ld, cudaStream_t s) {
  k_to_colmajor<XT><<<(n + kBlk - 1) / kBlk, dim3(kBlk, 8), 0, s>>>(blk, n, out, ld);
  nmg::add_launches(1);
}
template <typename XT>
void blk_from_colmajor(const double* src, size_t ld, int n, XT* blk, cudaStream_t s) {
  k_from_colmajor<XT><<<(n + kBlk - 1) / kBlk, dim3(kBlk, 8), 0, s>>>(src, ld, n, kBlk, blk);
  nmg::add_launches(1);
}
template void blk_from_colmajor<float>(const double*, size_t, int, float*, cudaStream_t);
template void blk_from_colmajor<double>(const double*, size_t, int, double*, cudaStream_t);
void blk_from_colmajor_cols(const double* src, size_t ld, int n, int ncol, double* blk, cudaStream_t s) {
  k_from_colmajor<double><<<(n + kBlk - 1) / kBlk, dim3(kBlk, 8), 0, s>>>(src, ld, n, std::min(ncol, kBlk), blk);
  nmg::add_launches(1);
}

template <typename XT>
void blk_init_range(XT* vk, XT* vkm1, XT* y, const XT* z, double a1, double mu1, size_t len, cudaStream_t s) {
  k_init_range_blk<XT><<<(int)((len + 255) / 256), 256, 0, s>>>(vk, vkm1, y, z, (XT)a1, (XT)mu1, len);
  nmg::add_launches(1);
}
template void blk_init_range<float>(float*, float*, float*, const float*, double, double, size_t, cudaStream_t);
void blk_f2d_flat(const float* src, double* dst, size_t len, cudaStream_t s) {
  k_f2d_flat<<<(int)((len + 255) / 256), 256, 0, s>>>(src, dst, len);
  nmg::add_launches(1);
}

template <typename XT>
void blk_init_filter(XT* vk, XT* vkm1, XT* y, const XT* v, double mu0, size_t len, cudaStream_t s) {
  k_init_filter_blk<XT><<<(int)((len + 255) / 256), 256, 0, s>>>(vk, vkm1, y, v, (XT)mu0, len);
  nmg::add_launches(1);
}

#define NM_INST(VT, XT)                                                                                              \
  template void blk_mass_cheb<VT, XT>(const GCsr<VT>&, const ChebSetup&, const XT*, XT*, XT*, cudaStream_t,          \
                                      const GatherCfg&);                                                           \
  template void blk_ap_cheb<VT, XT>(const GCsr<VT>&, const ChebSetup&, const XT*, XT*, XT*, cudaStream_t,            \
                                    const GatherCfg&);                                                             \
  template void blk_et<VT, XT>(const GCsr<VT>&, const XT*, XT*, cudaStream_t, const GatherCfg&);                   \
  template void blk_ap_cheb_persistent<VT, XT>(const GCsr<VT>&, const ChebSetup&, const XT*, XT*, XT*, GridBar*,   \
                                               int*, int, cudaStream_t);                                           \
  template void blk_amv<VT, XT>(const GCsr<VT>&, const GCsr<VT>*, const XT*, const XT*, XT*, const XT*, const XT*, \
                                XT*, const FiltEpi&, cudaStream_t, const GatherCfg&);
NM_INST(double, double)
NM_INST(float, float)
#undef NM_INST
template void blk_mass_spmv<double>(const GCsr<double>&, const double*, double*, cudaStream_t);
template void blk_gather_cols<float>(const Basis&, int, int, float*, cudaStream_t);
template void blk_gather_cols<double>(const Basis&, int, int, double*, cudaStream_t);
template void blk_to_colmajor<float>(const float*, int, double*, size_t, cudaStream_t);
template void blk_to_colmajor<double>(const double*, int, double*, size_t, cudaStream_t);
template void blk_init_filter<float>(float*, float*, float*, const float*, double, size_t, cudaStream_t);
template void blk_init_filter<double>(double*, double*, double*, const double*, double, size_t, cudaStream_t);

}  // namespace nmg
