// lu_tc.cu -- complex FP32 trailing-update GEMM of the precision-form LU on the
// fifth-generation tensor cores (tcgen05, kind::tf32, accumulator in TMEM).
//
//   C (M x N complex, column-major) -= A (M x K complex) * B (K x N complex)
//
// Complex -> real: with A' the M x 2K real matrix whose rows interleave (re, im)
// and B' the 2K x 2N real matrix whose column pair (2n, 2n+1) is
// ([Br, -Bi], [Bi, Br]) interleaved along K, A' B' = [Cr, Ci] interleaved along
// the columns, which is exactly the float2 layout of a row of C.
//
// Precision: every operand is split into a TF32 head and a TF32 tail (both
// rounded to nearest), and the accumulator receives lo*hi + hi*lo + hi*hi ("3xTF32"),
// which keeps the product close to FP32 accuracy; the FP64 refinement of the
// solver then removes the remaining FP32-level error.
//
// Kernel: one CTA (4 warps) per 128 x 128 real output tile (128 rows, 64 complex
// columns).  Thread 0 streams K in chunks of 32 FP32 (one 128-byte swizzle row)
// with TMA into a 2-stage ring (head and tail planes of A' and B'), waits on the
// stage's mbarrier and issues 3 x 4 tcgen05.mma (M=128, N=128, K=8) per chunk;
// tcgen05.commit releases the stage.  After the last commit the 4 warps read
// their 32-lane quarter of the accumulator with tcgen05.ld and subtract it from C
// with coalesced float2 accesses.  All waits are bounded; on timeout the kernel
// records an error, skips the rest and still frees its TMEM.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <mutex>
#include <vector>

#include "lu_common.cuh"
#include "solve_internal.h"
#include "stats.h"

namespace wmom {
namespace tc {

constexpr int BM = 128;  // accumulator lanes = rows of C per CTA
constexpr int BN = 128;  // accumulator FP32 columns = 64 complex columns of C
constexpr int KC = 32;   // FP32 elements of K per chunk (128 bytes)
constexpr int STAGES = 2;
constexpr int A_BYTES = BM * KC * 4;  // 16 KB per plane
constexpr int B_BYTES = BN * KC * 4;  // 16 KB per plane
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 128;
constexpr int NTHREADS = 128;
constexpr unsigned long long kWaitNs = 1000000000ull;  // 1 s per wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred P1;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, P1;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// Bounded wait on an mbarrier phase; false on timeout or when another CTA of the
// launch has already recorded one (err != 0).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, const int* err) {
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (*reinterpret_cast<const volatile int*>(err)) return false;
    if (global_ns() - t0 > kWaitNs) return false;
  }
  return true;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B
// apart (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(16u >> 4) << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor: D = F32, A = B = TF32, both K-major, N = BN, M = BM.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) |
                            ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// ---------------------------------------------------------------- pack ----
// A (M x K complex, col-major) -> hi/lo planes, row-major M x K2p FP32 (re, im
// interleaved along K, zero padding up to K2p).
__global__ void pack_a_kernel(const float2* __restrict__ A, long long lda, int M, int K, int K2p,
                              float* __restrict__ hi, float* __restrict__ lo) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;  // complex column, K2p/2 of them
  if (m >= M) return;
  float2 v = make_float2(0.f, 0.f);
  if (k < K) v = A[(size_t)k * lda + m];
  const float hr = tf32_rna(v.x), hi_ = tf32_rna(v.y);
  const size_t o = (size_t)m * K2p + 2 * k;
  hi[o] = hr;
  hi[o + 1] = hi_;
  lo[o] = tf32_rna(v.x - hr);
  lo[o + 1] = tf32_rna(v.y - hi_);
}

// B (K x N complex, col-major) -> hi/lo planes of B'^T, row-major 2N x K2p FP32:
// row 2n = (Br, -Bi) pairs, row 2n+1 = (Bi, Br) pairs along K.
__global__ void pack_b_kernel(const float2* __restrict__ B, long long ldb, int K, int N, int K2p,
                              float* __restrict__ hi, float* __restrict__ lo) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;  // complex row of B, K2p/2 of them
  const int n = blockIdx.y;
  if (2 * k >= K2p) return;
  float2 v = make_float2(0.f, 0.f);
  if (k < K) v = B[(size_t)n * ldb + k];
  const float hr = tf32_rna(v.x), hi_ = tf32_rna(v.y);
  const float lr = tf32_rna(v.x - hr), li = tf32_rna(v.y - hi_);
  const size_t r0 = (size_t)(2 * n) * K2p + 2 * k;
  const size_t r1 = (size_t)(2 * n + 1) * K2p + 2 * k;
  hi[r0] = hr;
  hi[r0 + 1] = -hi_;
  hi[r1] = hi_;
  hi[r1 + 1] = hr;
  lo[r0] = lr;
  lo[r0 + 1] = -li;
  lo[r1] = li;
  lo[r1 + 1] = lr;
}

// ---------------------------------------------------------------- gemm ----
__global__ void __launch_bounds__(NTHREADS, 1)
    cgemm_sub_tc_kernel(const __grid_constant__ CUtensorMap mapAhi, const __grid_constant__ CUtensorMap mapAlo,
                        const __grid_constant__ CUtensorMap mapBhi, const __grid_constant__ CUtensorMap mapBlo,
                        float2* __restrict__ C, long long ldc, int M, int N, int nchunks, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + STAGES * STAGE_BYTES);  // full[2], done[2]
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail;

  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int m0 = blockIdx.x * BM;
  const int j0 = blockIdx.y * BN;  // real column of the accumulator = row of B'^T

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int i = 0; i < 2 * STAGES; ++i) mbar_init(smem_u32(&bars[i]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_fail = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (tid == 0) {
    bool ok = *reinterpret_cast<const volatile int*>(err) == 0;
    int issued_last = -1;
    int tma_pending = -1;  // chunk whose copies were issued but not yet seen complete
    for (int c = 0; c < nchunks && ok; ++c) {
      const int s = c % STAGES;
      const uint32_t full = smem_u32(&bars[s]);
      const uint32_t done = smem_u32(&bars[STAGES + s]);
      if (c >= STAGES) ok = mbar_wait(done, ((c - STAGES) / STAGES) & 1, err);
      if (!ok) break;
      unsigned char* st = base + s * STAGE_BYTES;
      const uint32_t a_hi = smem_u32(st), a_lo = a_hi + A_BYTES;
      const uint32_t b_hi = a_hi + 2 * A_BYTES, b_lo = b_hi + B_BYTES;
      mbar_expect_tx(full, STAGE_BYTES);
      tma_load_2d(a_hi, &mapAhi, c * KC, m0, full);
      tma_load_2d(a_lo, &mapAlo, c * KC, m0, full);
      tma_load_2d(b_hi, &mapBhi, c * KC, j0, full);
      tma_load_2d(b_lo, &mapBlo, c * KC, j0, full);
      tma_pending = c;
      ok = mbar_wait(full, (c / STAGES) & 1, err);
      if (!ok) break;
      tma_pending = -1;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // tail terms first, head product last
      const uint32_t as[3] = {a_lo, a_hi, a_hi};
      const uint32_t bs[3] = {b_hi, b_lo, b_hi};
#pragma unroll
      for (int sp = 0; sp < 3; ++sp)
#pragma unroll
        for (int kk = 0; kk < KC / 8; ++kk)
          mma_tf32(tmem, sdesc(as[sp] + kk * 32), sdesc(bs[sp] + kk * 32), (c | sp | kk) != 0 ? 1u : 0u);
      mma_commit(done);
      issued_last = c;
    }
    if (ok && issued_last >= 0) {
      const int s = issued_last % STAGES;
      ok = mbar_wait(smem_u32(&bars[STAGES + s]), (issued_last / STAGES) & 1, err);
    }
    if (!ok) {
      s_fail = 1;
      atomicExch(err, 1);
      // before leaving, give this CTA's own copies and MMAs in flight a bounded
      // chance to land, so nothing writes shared memory or TMEM after release
      const int zero = 0;
      if (tma_pending >= 0) mbar_wait(smem_u32(&bars[tma_pending % STAGES]), (tma_pending / STAGES) & 1, &zero);
      if (issued_last >= 0)
        mbar_wait(smem_u32(&bars[STAGES + issued_last % STAGES]), (issued_last / STAGES) & 1, &zero);
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  if (!s_fail) {
    const int row = m0 + warp * 32 + (tid & 31);
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
#pragma unroll 1
    for (int cc = 0; cc < BN / 32; ++cc) {
      uint32_t r[32];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
          "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
            "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(tmem + lane_base + (uint32_t)(cc * 32))
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < M) {
        const int n0 = (j0 >> 1) + cc * 16;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int n = n0 + j;
          if (n < N) {
            float2* p = C + (size_t)n * ldc + row;
            float2 v = *p;
            v.x -= __uint_as_float(r[2 * j]);
            v.y -= __uint_as_float(r[2 * j + 1]);
            *p = v;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
  }
}

// ----------------------------------------------------------- host side ----
namespace {

using EncodeFn = PFN_cuTensorMapEncodeTiled_v12000;

EncodeFn encode_fn() {
  static EncodeFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeFn>(p);
  });
  return fn;
}

bool make_map(CUtensorMap* map, const float* ptr, int rows, int k2p) {
  EncodeFn enc = encode_fn();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)k2p, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)k2p * sizeof(float)};
  cuuint32_t box[2] = {(cuuint32_t)KC, (cuuint32_t)BM};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(ptr), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

struct TcWorkspace {
  float* buf = nullptr;
  size_t cap = 0;  // floats
  int* err = nullptr;
};

std::mutex g_mu;
std::vector<TcWorkspace> g_ws;

cudaError_t get_ws(size_t floats, TcWorkspace** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if ((int)g_ws.size() <= dev) g_ws.resize(dev + 1);
  TcWorkspace& w = g_ws[dev];
  if (!w.err) {
    e = cudaMalloc(&w.err, sizeof(int));
    if (e != cudaSuccess) return e;
    e = cudaMemset(w.err, 0, sizeof(int));
    if (e != cudaSuccess) return e;
  }
  if (w.cap < floats) {
    if (w.buf) {
      cudaDeviceSynchronize();
      cudaFree(w.buf);
      w.buf = nullptr;
    }
    e = cudaMalloc(&w.buf, floats * sizeof(float));
    if (e != cudaSuccess) {
      w.cap = 0;
      return e;
    }
    w.cap = floats;
  }
  *out = &w;
  return cudaSuccess;
}

}  // namespace

cudaError_t cgemm_sub_tc(const float2* A, long long lda, const float2* B, long long ldb, float2* C, long long ldc,
                         int M, int N, int K, cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
  const int K2p = ((2 * K + KC - 1) / KC) * KC;
  const size_t a_pl = (size_t)M * K2p, b_pl = (size_t)2 * N * K2p;
  std::lock_guard<std::mutex> lk(g_mu);
  TcWorkspace* w = nullptr;
  cudaError_t e = get_ws(2 * a_pl + 2 * b_pl, &w);
  if (e != cudaSuccess) return e;
  float* ahi = w->buf;
  float* alo = ahi + a_pl;
  float* bhi = alo + a_pl;
  float* blo = bhi + b_pl;
  stats::count(stats::kMisc, 2);
  pack_a_kernel<<<dim3((M + 127) / 128, K2p / 2), 128, 0, s>>>(A, lda, M, K, K2p, ahi, alo);
  pack_b_kernel<<<dim3((K2p / 2 + 127) / 128, N), 128, 0, s>>>(B, ldb, K, N, K2p, bhi, blo);
  CUtensorMap mah, mal, mbh, mbl;
  if (!make_map(&mah, ahi, M, K2p) || !make_map(&mal, alo, M, K2p) || !make_map(&mbh, bhi, 2 * N, K2p) ||
      !make_map(&mbl, blo, 2 * N, K2p))
    return cudaErrorInvalidValue;
  static bool attr_set = false;
  if (!attr_set) {
    e = cudaFuncSetAttribute(cgemm_sub_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  dim3 grid((M + BM - 1) / BM, (2 * N + BN - 1) / BN);
  stats::Scope sc(stats::kTcGemm, s, 8.0 * M * (double)N * K);
  cgemm_sub_tc_kernel<<<grid, NTHREADS, SMEM_BYTES, s>>>(mah, mal, mbh, mbl, C, ldc, M, N, K2p / KC, w->err);
  return cudaGetLastError();
}

int read_and_clear_error() {
  std::lock_guard<std::mutex> lk(g_mu);
  int dev = 0;
  cudaGetDevice(&dev);
  if ((int)g_ws.size() <= dev || !g_ws[dev].err) return 0;
  int h = 0;
  cudaMemcpy(&h, g_ws[dev].err, sizeof(int), cudaMemcpyDeviceToHost);
  if (h) cudaMemset(g_ws[dev].err, 0, sizeof(int));
  return h;
}

}  // namespace tc

GemmHook<float2> tc_gemm_hook() {
  if (std::getenv("WMOM_NO_TC")) return nullptr;
  int dev = 0, major = 0, minor = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  if (major != 10) return nullptr;
  return &tc::cgemm_sub_tc;
}

}  // namespace wmom

extern "C" wmom_status wmom_cgemm_sub_tc(int m, int n, int k, const void* a_dev, long long lda, const void* b_dev,
                                         long long ldb, void* c_dev, long long ldc, void* stream) {
  if (m < 0 || n < 0 || k < 0 || (m && (!a_dev || !c_dev || lda < m || ldc < m)) || (n && (!b_dev || ldb < k)))
    return WMOM_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = wmom::tc::cgemm_sub_tc(reinterpret_cast<const float2*>(a_dev), lda,
                                         reinterpret_cast<const float2*>(b_dev), ldb, reinterpret_cast<float2*>(c_dev),
                                         ldc, m, n, k, s);
  if (e != cudaSuccess) return wmom_fail_cuda(e, "cgemm_sub_tc");
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return wmom_fail_cuda(e, "cgemm_sub_tc sync");
  if (wmom::tc::read_and_clear_error()) return WMOM_ERR_TIMEOUT;
  return WMOM_OK;
}
