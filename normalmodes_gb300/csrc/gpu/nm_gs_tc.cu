// Block Gram-Schmidt projection on the 5th-generation tensor cores
// (tcgen05, sm_103a): H = V^T W for the FP32 copy V of the Krylov basis
// (n x K, chunks of 64 columns) and a 32-column block W (n x 32), the
// dense contraction of the full reorthogonalisation inside pEVSL's
// ChebLanNr (src/mod_pevsl.f90:122) on the mixed-precision block path.
//
// Shape and data flow.  The reduction runs over the n rows, so the grid is
// (K / 128 basis tiles) x (row splits); each CTA accumulates one 128 x 32
// tile of H over its row range in tensor memory and writes it as a partial
// sum, and a second kernel adds the partials of all splits in a fixed order
// (FP64 accumulation).  Per stage of 32 rows:
//   * warp 0 (one lane) loads the 128 x 32 slice of V (two 64-column chunk
//     boxes) and the 32 x 32 slice of W with TMA (cp.async.bulk.tensor,
//     128-byte swizzle) onto an mbarrier with the expected byte count;
//   * warps 2-5 split every value into a TF32 head and an FP32 tail
//     (x = hi + lo, hi = x rounded to TF32) in place / beside it;
//   * warp 1 (one lane) issues tcgen05.mma kind::tf32, M = 128, N = 32,
//     K = 8, for hi*hi + hi*lo + lo*hi (the "3xTF32" product, relative error
//     ~2^-21 instead of TF32's 2^-11) and commits to the stage's empty
//     barrier;
// then warps 2-5 read the accumulator back with tcgen05.ld (each warp its
// 32 TMEM lanes) and store the partial tile.  Both operands are K-major
// (consecutive rows of V and W are contiguous in memory).
//
// Every wait is bounded (about 2 s of %globaltimer): on a timeout the kernel
// sets the status word, skips the rest of its work, waits (bounded) for the
// MMAs it issued, frees its tensor memory and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "nm_block.h"
#include "nm_internal.h"

namespace nmg {
namespace {

constexpr int kTcM = 128;        // basis vectors per CTA tile (two 64-column chunks)
constexpr int kTcN = 32;         // block columns
constexpr int kTcK = 32;         // rows per stage: 32 FP32 = one 128-byte swizzle row
constexpr int kTcStages = 4;
constexpr int kTcThreads = 192;  // warp 0 TMA, warp 1 MMA, warps 2-5 split and epilogue
constexpr uint32_t kABytes = kTcM * kTcK * 4;  // 16 KB
constexpr uint32_t kBBytes = kTcN * kTcK * 4;  // 4 KB
constexpr uint32_t kStageBytes = 2 * (kABytes + kBBytes);
constexpr size_t kTcSmem = 1024 + (size_t)kTcStages * kStageBytes + 256;
constexpr unsigned long long kTcTimeoutNs = 2000000000ull;
constexpr int kTmemCols = 32;

// Instruction descriptor of tcgen05.mma kind::tf32: D FP32 (bits 4-5 = 1),
// A and B TF32 (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0),
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                            ((uint32_t)(kTcM >> 4) << 24);

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("{ .reg .b64 st; mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1; }" ::"r"(saddr(b)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("{ .reg .b64 st; mbarrier.arrive.shared::cta.b64 st, [%0]; }" ::"r"(saddr(b)) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
      : "=r"(ok)
      : "r"(saddr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase with the given parity to complete.  false if
// another thread of the CTA gave up (*err set) or the time ran out (then
// sets *err and the kernel's status word).
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, volatile int* err, int* status) {
  const unsigned long long t0 = now_ns();
  while (!mbar_test(b, parity)) {
    if (*err) return false;
    if (now_ns() - t0 > kTcTimeoutNs) {
      *err = 1;
      atomicExch(status, 2);
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          saddr(dst)),
      "l"(map), "r"(x), "r"(y), "r"(saddr(bar))
      : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row core
// groups 1024 bytes apart (stride byte offset), descriptor version 1 (bits
// 46-47), layout type 2 = SWIZZLE_128B (bits 61-63).
__device__ __forceinline__ uint64_t sdesc(uint32_t a) {
  uint64_t d = (uint64_t)((a >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{ .reg .pred p; setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p; }" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
               : "memory");
}

// x = hi + lo with hi = x rounded to TF32 (low 13 mantissa bits zero) and lo
// the exact FP32 remainder.
__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo) {
  uint32_t h;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
  hi = __uint_as_float(h);
  lo = x - hi;
}

__global__ void __launch_bounds__(kTcThreads, 1)
    k_gs_tc(const CUtensorMap* __restrict__ vmaps, const CUtensorMap* __restrict__ wmap, int K, int n,
            int rows_per_split, float* __restrict__ part, int kpad, int* status) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* stage = sm;
  uint64_t* bars = (uint64_t*)(sm + (size_t)kTcStages * kStageBytes);
  uint64_t* full = bars;
  uint64_t* conv = bars + kTcStages;
  uint64_t* empty = bars + 2 * kTcStages;
  uint64_t* done = bars + 3 * kTcStages;
  volatile int* err = (volatile int*)(bars + 3 * kTcStages + 1);
  uint32_t* tmem_slot = (uint32_t*)(bars + 3 * kTcStages + 2);
  auto a_hi = [&](int s) { return stage + (size_t)s * kStageBytes; };
  auto a_lo = [&](int s) { return stage + (size_t)s * kStageBytes + kABytes; };
  auto b_hi = [&](int s) { return stage + (size_t)s * kStageBytes + 2 * kABytes; };
  auto b_lo = [&](int s) { return stage + (size_t)s * kStageBytes + 2 * kABytes + kBBytes; };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kTcM;
  const int split = blockIdx.y;
  const int i0 = split * rows_per_split;
  const int i1 = min(n, i0 + rows_per_split);
  const int niter = i1 > i0 ? (i1 - i0 + kTcK - 1) / kTcK : 0;
  const int chunk0 = m0 / 64;
  const bool two = m0 + 64 < K;
  const uint32_t tx = (two ? 2u : 1u) * (kABytes / 2) + kBBytes;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kTcStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&conv[s], 128);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *err = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {  // TMA producer
      for (int it = 0; it < niter && !*err; ++it) {
        const int s = it % kTcStages;
        if (it >= kTcStages && !mbar_wait(&empty[s], ((it / kTcStages) - 1) & 1, err, status)) break;
        mbar_expect_tx(&full[s], tx);
        const int x = i0 + it * kTcK;
        tma_load_2d(a_hi(s), vmaps + chunk0, x, 0, &full[s]);
        if (two) tma_load_2d(a_hi(s) + kABytes / 2, vmaps + chunk0 + 1, x, 0, &full[s]);
        tma_load_2d(b_hi(s), wmap, x, 0, &full[s]);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      int issued = 0;
      for (int it = 0; it < niter; ++it) {
        const int s = it % kTcStages;
        if (!mbar_wait(&conv[s], (it / kTcStages) & 1, err, status)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t ah = saddr(a_hi(s)), al = saddr(a_lo(s)), bh = saddr(b_hi(s)), bl = saddr(b_lo(s));
#pragma unroll
        for (int k = 0; k < kTcK / 8; ++k) {  // K = 8 TF32 = 32 bytes per instruction
          const uint32_t off = (uint32_t)k * 32u;
          mma_tf32(tmem, sdesc(ah + off), sdesc(bh + off), (it > 0 || k > 0) ? 1u : 0u);
          mma_tf32(tmem, sdesc(ah + off), sdesc(bl + off), 1u);
          mma_tf32(tmem, sdesc(al + off), sdesc(bh + off), 1u);
        }
        mma_commit(&empty[s]);
        ++issued;
      }
      // arrives once every MMA issued above has completed (also when none was)
      mma_commit(done);
      (void)issued;
    }
  } else {  // warps 2-5: TF32 split, then the epilogue
    const int t = threadIdx.x - 64;  // 0..127
    for (int it = 0; it < niter; ++it) {
      const int s = it % kTcStages;
      if (!mbar_wait(&full[s], (it / kTcStages) & 1, err, status)) break;
      float4* ah = (float4*)a_hi(s);
      float4* al = (float4*)a_lo(s);
      for (int q = t; q < (int)(kABytes / 16); q += 128) {
        const float4 v = ah[q];
        float4 h, l;
        split_tf32(v.x, h.x, l.x);
        split_tf32(v.y, h.y, l.y);
        split_tf32(v.z, h.z, l.z);
        split_tf32(v.w, h.w, l.w);
        ah[q] = h;
        al[q] = l;
      }
      float4* bh = (float4*)b_hi(s);
      float4* bl = (float4*)b_lo(s);
      for (int q = t; q < (int)(kBBytes / 16); q += 128) {
        const float4 v = bh[q];
        float4 h, l;
        split_tf32(v.x, h.x, l.x);
        split_tf32(v.y, h.y, l.y);
        split_tf32(v.z, h.z, l.z);
        split_tf32(v.w, h.w, l.w);
        bh[q] = h;
        bl[q] = l;
      }
      // make the generic-proxy stores visible to the tensor cores' reads
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(&conv[s]);
    }
    // epilogue: accumulator rows 32 * (warp % 4) + lane, 32 columns
    const bool ok = mbar_wait(done, 0, err, status);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok && !*err) {
      const int sub = warp & 3;
      const int row = sub * 32 + lane;
      uint32_t r[32];
      const uint32_t taddr = tmem + ((uint32_t)(sub * 32) << 16);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
          "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
            "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
            "=r"(r[30]), "=r"(r[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (m0 + row < K) {
        float4* dst = (float4*)(part + ((size_t)split * kpad + m0 + row) * kTcN);
        if (niter == 0) {
          for (int c = 0; c < kTcN / 4; ++c) dst[c] = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
          for (int c = 0; c < kTcN / 4; ++c)
            dst[c] = make_float4(__uint_as_float(r[4 * c]), __uint_as_float(r[4 * c + 1]),
                                 __uint_as_float(r[4 * c + 2]), __uint_as_float(r[4 * c + 3]));
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

// H(k, c) = sum over splits of part[split][k][c] (FP64 sum in split order),
// stored FP32 column-major with leading dimension ldh.
__global__ void k_gs_tc_reduce(const float* __restrict__ part, int nsplit, int kpad, int K, float* __restrict__ H,
                               int ldh) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= K * kTcN) return;
  const int k = t / kTcN, c = t % kTcN;
  double s = 0.0;
  for (int p = 0; p < nsplit; ++p) s += (double)part[((size_t)p * kpad + k) * kTcN + c];
  H[(size_t)c * ldh + k] = (float)s;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    cudaGetLastError();
  });
  return fn;
}

}  // namespace

bool gs_tc_available() {
  int dev = 0, major = 0, minor = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  cudaGetLastError();
  return major == 10 && minor == 3 && encode_fn() != nullptr;
}

int gs_tc_map(const float* base, int n, size_t ld, int cols, void* map_out) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc) return NM_ERR_CUDA;
  if (((uintptr_t)base & 15) || (ld * 4) % 16 != 0 || (cols != 32 && cols != 64)) return NM_ERR_ARG;
  const cuuint64_t gdim[2] = {(cuuint64_t)n, (cuuint64_t)cols};
  const cuuint64_t gstride[1] = {(cuuint64_t)ld * 4};
  const cuuint32_t box[2] = {(cuuint32_t)kTcK, (cuuint32_t)(cols == 64 ? 64 : 32)};
  const cuuint32_t estride[2] = {1, 1};
  const CUresult r = enc((CUtensorMap*)map_out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, gdim, gstride, box,
                         estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? NM_OK : NM_ERR_ARG;
}

size_t gs_tc_map_bytes() { return sizeof(CUtensorMap); }

int gs_tc_splits(int K, int n) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int tiles = (K + kTcM - 1) / kTcM;
  const int want = std::max(1, (2 * std::max(sms, 1) + tiles - 1) / tiles);  // ~2 CTAs per SM
  const int most = std::max(1, (n + 4095) / 4096);                           // at least 4096 rows per split
  return std::min(want, most);
}

// Floats of the partial-sum buffer for every K up to Kmax (the split count
// falls as K grows, so the product is not monotone in K).
size_t gs_tc_part_floats(int Kmax, int n) {
  size_t most = 0;
  for (int K = 32; K <= std::max(Kmax, 32); K += 32) {
    const size_t kpad = (size_t)(K + kTcM - 1) / kTcM * kTcM;
    most = std::max(most, (size_t)gs_tc_splits(K, n) * kpad * kTcN);
  }
  return most;
}

int gs_tc_project(const void* vmaps_dev, const void* wmap_dev, int K, int n, float* part, float* H, int ldh,
                  int* status, cudaStream_t s) {
  if (K <= 0 || n <= 0 || K % 32 != 0) return NM_ERR_ARG;
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(k_gs_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
  });
  if (attr != cudaSuccess) return NM_ERR_CUDA;
  const int tiles = (K + kTcM - 1) / kTcM;
  const int kpad = tiles * kTcM;
  const int nsplit = gs_tc_splits(K, n);
  const int rows = ((n + nsplit - 1) / nsplit + kTcK - 1) / kTcK * kTcK;
  k_gs_tc<<<dim3(tiles, nsplit), kTcThreads, kTcSmem, s>>>((const CUtensorMap*)vmaps_dev,
                                                          (const CUtensorMap*)wmap_dev, K, n, rows, part, kpad,
                                                          status);
  k_gs_tc_reduce<<<(K * kTcN + 255) / 256, 256, 0, s>>>(part, nsplit, kpad, K, H, ldh);
  add_launches(2);
  return cudaGetLastError() == cudaSuccess ? NM_OK : NM_ERR_CUDA;
}

}  // namespace nmg

// ---------------------------------------------------------------- test hook
// H = V^T W on the tensor cores for device arrays V (n x K, column-major,
// leading dimension ldv, taken as chunks of 64 columns like the basis) and W
// (n x 32, leading dimension ldw); H column-major with leading dimension
// ldh.  Returns NM_OK, NM_ERR_ARG (shapes the kernel does not take),
// NM_ERR_CUDA (no tcgen05 device) or NM_ERR_TIMEOUT (a bounded wait ran out).
extern "C" int nm_test_gs_tc(const float* V, int ldv, int n, int K, const float* W, int ldw, float* H, int ldh) {
  using namespace nmg;
  if (!V || !W || !H || n <= 0 || K <= 0 || K % 64 != 0 || ldv < n || ldw < n || ldh < K) return NM_ERR_ARG;
  if (!gs_tc_available()) return NM_ERR_CUDA;
  const int nch = K / 64;
  std::vector<uint8_t> maps((size_t)(nch + 1) * gs_tc_map_bytes() + 64);
  uint8_t* m = (uint8_t*)(((uintptr_t)maps.data() + 63) & ~(uintptr_t)63);
  for (int c = 0; c < nch; ++c)
    if (gs_tc_map(V + (size_t)c * 64 * ldv, n, (size_t)ldv, 64, m + (size_t)c * gs_tc_map_bytes()) != NM_OK)
      return NM_ERR_ARG;
  if (gs_tc_map(W, n, (size_t)ldw, 32, m + (size_t)nch * gs_tc_map_bytes()) != NM_OK) return NM_ERR_ARG;
  void* dmaps = nullptr;
  float* part = nullptr;
  int* status = nullptr;
  int rc = NM_OK;
  if (cudaMalloc(&dmaps, (size_t)(nch + 1) * gs_tc_map_bytes()) != cudaSuccess ||
      cudaMalloc(&part, sizeof(float) * gs_tc_part_floats(K, n)) != cudaSuccess ||
      cudaMalloc(&status, sizeof(int)) != cudaSuccess) {
    rc = NM_ERR_OOM;
  } else {
    cudaMemcpy(dmaps, m, (size_t)(nch + 1) * gs_tc_map_bytes(), cudaMemcpyHostToDevice);
    cudaMemset(status, 0, sizeof(int));
    rc = gs_tc_project(dmaps, (uint8_t*)dmaps + (size_t)nch * gs_tc_map_bytes(), K, n, part, H, ldh, status, 0);
    int st = 0;
    if (cudaMemcpy(&st, status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) rc = NM_ERR_CUDA;
    else if (rc == NM_OK && st != 0) rc = NM_ERR_TIMEOUT;
  }
  cudaFree(dmaps);
  cudaFree(part);
  cudaFree(status);
  return rc;
}
