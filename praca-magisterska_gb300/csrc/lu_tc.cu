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
// Kernel: persistent, one CTA (6 warps) per SM, each walking 128 x 256 real output
// tiles (128 rows, 128 complex columns; measured against 128 x 128 tiles on one large
// update: 176 vs 167 TFLOP/s at K = 96, 235 vs 209 at K = 192, as each stage's four
// operand planes then feed twice the MMA work).  The narrow 128 x 128 tile is the
// other instantiation: a factorisation's late trailing matrices have few wide tiles
// for 152 SMs, so the autotuner times both per order (LuWorkspace::tile_n).  A producer thread streams K in chunks of 32
// FP32 (one 128-byte swizzle row) with TMA into a 2-stage ring (head and tail
// planes of A' and B'); an MMA thread issues 3 x 4 tcgen05.mma (M=128, N=256, K=8)
// per chunk into one of two TMEM accumulators; four epilogue warps read their
// 32-lane quarter of a finished accumulator with tcgen05.ld and subtract it from C
// with coalesced float2 accesses while the next tile is being multiplied.  All
// waits are bounded; on timeout the kernel records an error, skips the rest and
// still frees its TMEM.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "lu_common.cuh"
#include "solve_internal.h"
#include "stats.h"
#include "tcgen05_util.cuh"

namespace wmom {
namespace tc {

constexpr int BM = 128;  // accumulator lanes = rows of C per CTA
// accumulator FP32 columns per tile (BN: 256 = 128 complex columns of C, or 128 = 64;
// the factorisation's autotuner picks one per order, LuWorkspace::tile_n)
constexpr int kTileWide = 256, kTileNarrow = 128;
constexpr int KC = 32;   // FP32 elements of K per chunk (128 bytes)
constexpr int KC16 = 64; // FP16 elements of K per chunk (128 bytes)
constexpr int STAGES = 2;
constexpr int A_BYTES = BM * 128;  // 16 KB per plane (one 128-byte row of K per row)
__host__ __device__ constexpr int b_bytes(int bn) { return bn * 128; }  // 32 or 16 KB per plane
__host__ __device__ constexpr int stage_bytes(int bn) { return 2 * A_BYTES + 2 * b_bytes(bn); }
__host__ __device__ constexpr int smem_bytes(int bn) { return STAGES * stage_bytes(bn) + 1024 + 128; }
constexpr int NTHREADS = 192;         // producer warp, MMA warp, 4 epilogue warps
// Shared-memory matrix descriptor: K-major, 128-byte swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) { return sdesc_sw<128>(addr); }

// Instruction descriptor: D = F32, A = B = TF32, both K-major, N = bn, M = BM.
__host__ __device__ constexpr uint32_t idesc_tf32(int bn) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(bn >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

template <int BN>
__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
  constexpr uint32_t kIdesc = idesc_tf32(BN);
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

// Instruction descriptor of the FP16-plane variant: D = F32, A = B = F16, both K-major.
__host__ __device__ constexpr uint32_t idesc_f16(int bn) {
  return (1u << 4) | ((uint32_t)(bn >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

template <int BN>
__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
  constexpr uint32_t kIdescF16 = idesc_f16(BN);
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(kIdescF16), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// ---------------------------------------------------------------- pack ----
// A (M x K complex, col-major) -> hi/lo planes, row-major M x K2p FP32 (re, im
// interleaved along K, zero padding up to K2p).  A block transposes a tile of 32 rows
// x 32 complex columns through shared memory: column reads and plane writes are both
// coalesced.
__global__ void __launch_bounds__(256) pack_a_kernel(const float2* __restrict__ A, long long lda, int M, int K,
                                                     int K2p, float* __restrict__ hi, float* __restrict__ lo,
                                                     long long astride) {
  __shared__ float2 tile[32][33];  // [complex column][row]
  // batch: blockIdx.z selects the matrix; its planes follow each other
  A += (size_t)blockIdx.z * astride;
  hi += (size_t)blockIdx.z * M * K2p;
  lo += (size_t)blockIdx.z * M * K2p;
  const int m0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int k = k0 + ty + 8 * i, m = m0 + tx;
    tile[ty + 8 * i][tx] = (k < K && m < M) ? A[(size_t)k * lda + m] : make_float2(0.f, 0.f);
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = ty + 8 * i, m = m0 + r, k = k0 + tx;
    if (m >= M || 2 * k >= K2p) continue;
    const float2 v = tile[tx][r];
    const float hr = tf32_rna(v.x), hi_ = tf32_rna(v.y);
    const size_t o = (size_t)m * K2p + 2 * k;
    *reinterpret_cast<float2*>(hi + o) = make_float2(hr, hi_);
    *reinterpret_cast<float2*>(lo + o) = make_float2(tf32_rna(v.x - hr), tf32_rna(v.y - hi_));
  }
}

// B (K x N complex, col-major) -> hi/lo planes of B'^T, row-major 2N x K2p FP32:
// row 2n = (Br, -Bi) pairs, row 2n+1 = (Bi, Br) pairs along K.
__global__ void pack_b_kernel(const float2* __restrict__ B, long long ldb, int K, int N, int K2p,
                              float* __restrict__ hi, float* __restrict__ lo, long long bstride) {
  B += (size_t)blockIdx.z * bstride;
  hi += (size_t)blockIdx.z * 2 * N * K2p;
  lo += (size_t)blockIdx.z * 2 * N * K2p;
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

// ------------------------------------------------------- FP16 planes ----
// The FP16-plane variant scales every row of A' and every complex column of B by a
// power of two that brings its largest |re| or |im| into [2^14, 2^15) -- inside the
// FP16 range (65504) with room for the rounding of the head -- and splits each scaled
// value x into an FP16 head and tail, hi = fp16(x), lo = fp16(x - hi) (x - hi is exact
// in FP32): 22 significant bits, as the TF32 head and tail.  Entries far below their
// row's or column's maximum lose relative bits in the FP16 subnormal range, never more
// than 2^-39 of that maximum, i.e. the split is accurate normwise.  The epilogue
// multiplies each accumulator by 2^-(e_row + e_col).

__device__ __forceinline__ int fp16_scale_exp(float mx) {
  if (!(mx > 0.f) || !(mx < 3.0e38f)) return 0;  // zero (or not finite): no scaling
  int e;
  frexpf(mx, &e);  // mx in [2^(e-1), 2^e)
  return 15 - e;
}

// ea[m] for the rows of A (M x K complex, column-major): one thread per row.
__global__ void rowexp_a_kernel(const float2* __restrict__ A, long long lda, int M, int K, int* __restrict__ ea,
                                long long astride) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  A += (size_t)blockIdx.y * astride;
  float mx = 0.f;
  for (int k = 0; k < K; ++k) {
    const float2 v = A[(size_t)k * lda + m];
    mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
  }
  ea[(size_t)blockIdx.y * M + m] = fp16_scale_exp(mx);
}

// eb[n] for the columns of B (K x N complex, column-major): one warp per column.
__global__ void colexp_b_kernel(const float2* __restrict__ B, long long ldb, int K, int N, int* __restrict__ eb,
                                long long bstride) {
  const int n = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (n >= N) return;
  B += (size_t)blockIdx.y * bstride + (size_t)n * ldb;
  float mx = 0.f;
  for (int k = lane; k < K; k += 32) mx = fmaxf(mx, fmaxf(fabsf(B[k].x), fabsf(B[k].y)));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) eb[(size_t)blockIdx.y * N + n] = fp16_scale_exp(mx);
}

// 2^k as a float, exactly: built from its exponent field where that is normal
__device__ __forceinline__ float pow2f(int k) {
  return (k >= -126 && k <= 127) ? __int_as_float((k + 127) << 23) : ldexpf(1.0f, k);
}

__device__ __forceinline__ void split_f16(float x, __half* hi, __half* lo) {
  const __half h = __float2half_rn(x);
  *hi = h;
  *lo = __float2half_rn(x - __half2float(h));
}

// pack_a_kernel's transpose with FP16 planes of the scaled rows.
__global__ void __launch_bounds__(256) pack_a_f16_kernel(const float2* __restrict__ A, long long lda, int M, int K,
                                                         int K2p, __half* __restrict__ hi, __half* __restrict__ lo,
                                                         const int* __restrict__ ea, long long astride) {
  __shared__ float2 tile[32][33];  // [complex column][row]
  A += (size_t)blockIdx.z * astride;
  hi += (size_t)blockIdx.z * M * K2p;
  lo += (size_t)blockIdx.z * M * K2p;
  ea += (size_t)blockIdx.z * M;
  const int m0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int k = k0 + ty + 8 * i, m = m0 + tx;
    tile[ty + 8 * i][tx] = (k < K && m < M) ? A[(size_t)k * lda + m] : make_float2(0.f, 0.f);
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = ty + 8 * i, m = m0 + r, k = k0 + tx;
    if (m >= M || 2 * k >= K2p) continue;
    const float2 v = tile[tx][r];
    const int e = ea[m];
    __half2 h, l;
    split_f16(ldexpf(v.x, e), &h.x, &l.x);
    split_f16(ldexpf(v.y, e), &h.y, &l.y);
    const size_t o = (size_t)m * K2p + 2 * k;
    *reinterpret_cast<__half2*>(hi + o) = h;
    *reinterpret_cast<__half2*>(lo + o) = l;
  }
}

// pack_b_kernel with FP16 planes of the scaled columns.
__global__ void pack_b_f16_kernel(const float2* __restrict__ B, long long ldb, int K, int N, int K2p,
                                  __half* __restrict__ hi, __half* __restrict__ lo, const int* __restrict__ eb,
                                  long long bstride) {
  B += (size_t)blockIdx.z * bstride;
  hi += (size_t)blockIdx.z * 2 * N * K2p;
  lo += (size_t)blockIdx.z * 2 * N * K2p;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;  // complex row of B, K2p/2 of them
  const int n = blockIdx.y;
  if (2 * k >= K2p) return;
  const int e = eb[(size_t)blockIdx.z * N + n];
  float2 v = make_float2(0.f, 0.f);
  if (k < K) v = B[(size_t)n * ldb + k];
  __half hr, lr, hi_, li;
  split_f16(ldexpf(v.x, e), &hr, &lr);
  split_f16(ldexpf(v.y, e), &hi_, &li);
  const size_t r0 = (size_t)(2 * n) * K2p + 2 * k;
  const size_t r1 = (size_t)(2 * n + 1) * K2p + 2 * k;
  hi[r0] = hr;
  hi[r0 + 1] = __hneg(hi_);
  hi[r1] = hi_;
  hi[r1 + 1] = hr;
  lo[r0] = lr;
  lo[r0 + 1] = __hneg(li);
  lo[r1] = li;
  lo[r1 + 1] = lr;
}

// ---------------------------------------------------------------- gemm ----
// Persistent, warp-specialised: CTA b takes output tiles b, b + grid, ... (tiles
// ordered rows fastest, then columns, then matrices of the batch).
//   warp 0 (one thread): TMA producer, K chunks of successive tiles into the
//                        STAGES-deep ring (full[s] completes when a stage lands);
//   warp 1 (one thread): MMA issuer, 3 x 4 tcgen05.mma per chunk into accumulator
//                        tl % 2 of TMEM; commit to empty[s] frees the stage, commit
//                        to tfull[b] hands a finished tile to the epilogue;
//   warps 2-5:           epilogue, C -= accumulator b (TMEM lane quarter warp % 4,
//                        one row of C per thread), then arrive on tempty[b].
// The two accumulators let the tensor cores work on tile i + 1 while tile i's C
// traffic is in flight.  Every wait is bounded (kWaitNs) and also gives up once
// another role or CTA has recorded a failure; a role that gives up lets its own
// copies and MMAs in flight land (bounded) before the CTA frees its TMEM.
struct TileCoord {
  int mat, m0, j0;
};

template <int BN>
__device__ __forceinline__ TileCoord tile_coord(int t, int tiles_m, int tiles_n) {
  const int per_mat = tiles_m * tiles_n;
  const int mat = t / per_mat;
  const int r = t - mat * per_mat;
  const int tn = r / tiles_m;
  return TileCoord{mat, (r - tn * tiles_m) * BM, tn * BN};
}

// F16: FP16 planes of scaled operands (kind::f16, 64 elements of K per chunk; ea / eb
// hold the rows' and columns' exponents), else TF32 planes (kind::tf32, 32 per chunk).
// BN: FP32 columns of an output tile (256 or 128).
template <bool F16, int BN>
__global__ void __launch_bounds__(NTHREADS, 1)
    cgemm_sub_tc_kernel(const __grid_constant__ CUtensorMap mapAhi, const __grid_constant__ CUtensorMap mapAlo,
                        const __grid_constant__ CUtensorMap mapBhi, const __grid_constant__ CUtensorMap mapBlo,
                        float2* __restrict__ C, long long ldc, int M, int N, int nchunks, int tiles_m,
                        int tiles_n, int ntiles, int* __restrict__ err, long long cstride,
                        const int* __restrict__ ea, const int* __restrict__ eb) {
  constexpr int kChunk = F16 ? KC16 : KC;  // K elements per chunk (128 bytes)
  constexpr int B_BYTES = b_bytes(BN), STAGE_BYTES = stage_bytes(BN);
  constexpr int TMEM_COLS = 2 * BN;  // two accumulators
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + STAGES * STAGE_BYTES);
  // bars: full[STAGES], empty[STAGES], tfull[2], tempty[2]
  __shared__ uint32_t tmem_base;
  __shared__ volatile int s_fail;
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  auto full_bar = [&](int s) { return smem_u32(&bars[s]); };
  auto empty_bar = [&](int s) { return smem_u32(&bars[STAGES + s]); };
  auto tfull_bar = [&](int b) { return smem_u32(&bars[2 * STAGES + b]); };
  auto tempty_bar = [&](int b) { return smem_u32(&bars[2 * STAGES + 2 + b]); };

  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full_bar(s), 1);
      mbar_init(empty_bar(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(tfull_bar(b), 1);
      mbar_init(tempty_bar(b), NTHREADS / 32 - 2);  // one arrival per epilogue warp
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_fail = *reinterpret_cast<const volatile int*>(err) != 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (warp == 0) {
    if (lane == 0) {
      // ------------------------------------------------------ TMA producer
      int it = 0;  // chunks issued
      bool ok = !s_fail;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const TileCoord tc = tile_coord<BN>(t, tiles_m, tiles_n);
        for (int c = 0; c < nchunks; ++c) {
          const int s = it % STAGES, use = it / STAGES;
          if (use > 0 && !(ok = role_wait(empty_bar(s), (use - 1) & 1, err, &s_fail))) break;
          const uint32_t a_hi = smem_u32(base + s * STAGE_BYTES), a_lo = a_hi + A_BYTES;
          const uint32_t b_hi = a_hi + 2 * A_BYTES, b_lo = b_hi + B_BYTES;
          mbar_expect_tx(full_bar(s), STAGE_BYTES);
          tma_load_3d(a_hi, &mapAhi, c * kChunk, tc.m0, tc.mat, full_bar(s));
          tma_load_3d(a_lo, &mapAlo, c * kChunk, tc.m0, tc.mat, full_bar(s));
          tma_load_3d(b_hi, &mapBhi, c * kChunk, tc.j0, tc.mat, full_bar(s));
          tma_load_3d(b_lo, &mapBlo, c * kChunk, tc.j0, tc.mat, full_bar(s));
          ++it;
        }
      }
      if (!ok) {
        s_fail = 1;
        atomicExch(err, 1);
        // the copies of the last STAGES chunks may still be landing
        const int zero = 0;
        const volatile int no_fail = 0;
        for (int i = it > STAGES ? it - STAGES : 0; i < it; ++i)
          role_wait(full_bar(i % STAGES), (i / STAGES) & 1, &zero, &no_fail);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ------------------------------------------------------- MMA issuer
      int it = 0, tl = 0;
      bool ok = !s_fail;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++tl) {
        const int b = tl & 1, use = tl >> 1;
        if (use > 0 && !(ok = role_wait(tempty_bar(b), (use - 1) & 1, err, &s_fail))) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t acc = tmem + (uint32_t)(b * BN);
        for (int c = 0; c < nchunks; ++c) {
          const int s = it % STAGES;
          if (!(ok = role_wait(full_bar(s), (it / STAGES) & 1, err, &s_fail))) break;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t a_hi = smem_u32(base + s * STAGE_BYTES), a_lo = a_hi + A_BYTES;
          const uint32_t b_hi = a_hi + 2 * A_BYTES, b_lo = b_hi + B_BYTES;
          // tail terms first, head product last
          const uint32_t as[3] = {a_lo, a_hi, a_hi};
          const uint32_t bs[3] = {b_hi, b_lo, b_hi};
          // 4 MMAs of 32 bytes of K each per plane product (K = 8 TF32 or 16 FP16)
#pragma unroll
          for (int sp = 0; sp < 3; ++sp)
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const uint32_t accum = (c | sp | kk) != 0 ? 1u : 0u;
              if constexpr (F16)
                mma_f16<BN>(acc, sdesc(as[sp] + kk * 32), sdesc(bs[sp] + kk * 32), accum);
              else
                mma_tf32<BN>(acc, sdesc(as[sp] + kk * 32), sdesc(bs[sp] + kk * 32), accum);
            }
          mma_commit(empty_bar(s));
          ++it;
        }
        if (!ok) break;
        mma_commit(tfull_bar(b));
      }
      if (!ok) {
        s_fail = 1;
        atomicExch(err, 1);
        // the last commit covers every MMA this thread issued
        if (it > 0) {
          const int zero = 0;
          const volatile int no_fail = 0;
          role_wait(empty_bar((it - 1) % STAGES), ((it - 1) / STAGES) & 1, &zero, &no_fail);
        }
      }
    }
  } else {
    // ----------------------------------------------------------- epilogue
    const int q = warp & 3;  // TMEM lanes 32q..32q+31 are the ones this warp may read
    int tl = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++tl) {
      const TileCoord tc = tile_coord<BN>(t, tiles_m, tiles_n);
      float2* Cm = C + (size_t)tc.mat * cstride;
      const int row = tc.m0 + q * 32 + lane;
      const bool row_ok = row < M;
      // FP16 planes: the row's scale (the columns' are read per chunk)
      const float srow = F16 && row_ok ? pow2f(-ea[(size_t)tc.mat * M + row]) : 1.0f;
      auto load_c_chunk = [&](int cc, float2* dst) {
        const int n0 = (tc.j0 >> 1) + cc * 16;
#pragma unroll
        for (int j = 0; j < 16; ++j)
          dst[j] = (row_ok && n0 + j < N) ? Cm[(size_t)(n0 + j) * ldc + row] : make_float2(0.f, 0.f);
      };
      float2 cbuf[16], nxt[16];
      load_c_chunk(0, cbuf);  // in flight while the accumulator is being computed
      const int b = tl & 1, use = tl >> 1;
      int ok = 0;
      if (lane == 0) ok = role_wait(tfull_bar(b), use & 1, err, &s_fail) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);  // warp-uniform from here on
      if (!ok) {
        if (lane == 0) {
          s_fail = 1;
          atomicExch(err, 1);
        }
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * BN);
#pragma unroll
      for (int cc = 0; cc < BN / 32; ++cc) {
        if (cc + 1 < BN / 32) load_c_chunk(cc + 1, nxt);
        uint32_t r[32];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
            "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
              "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
              "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
              "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr + (uint32_t)(cc * 32)));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (row_ok) {
          const int n0 = (tc.j0 >> 1) + cc * 16;
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            if (n0 + j < N) {
              float2 v = cbuf[j];
              float pr = __uint_as_float(r[2 * j]), pi = __uint_as_float(r[2 * j + 1]);
              if constexpr (F16) {
                // the scaled product times 2^-e_row, then 2^-e_col: exact unless the
                // true product is below FP32's normal range
                const float scol = pow2f(-eb[(size_t)tc.mat * N + n0 + j]);
                pr = (pr * srow) * scol;
                pi = (pi * srow) * scol;
              }
              v.x -= pr;
              v.y -= pi;
              Cm[(size_t)(n0 + j) * ldc + row] = v;
            }
          }
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) cbuf[j] = nxt[j];
      }
      // accumulator b read out: the MMA issuer may overwrite it
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(tempty_bar(b));
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 1) {
    __syncwarp();  // lane 0 ran the MMA loop alone: converge before the .aligned op
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// ----------------------------------------------------------- host side ----
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

namespace {

// 3-D map over `batch` planes of rows x k2p elements (row-major; FP32 or FP16),
// boxes of one 128-byte row of K x box_rows.
bool make_map(CUtensorMap* map, const void* ptr, int rows, int k2p, int batch, int box_rows, bool f16) {
  EncodeFn enc = encode_fn();
  if (!enc) return false;
  const size_t elem = f16 ? 2 : 4;
  cuuint64_t dims[3] = {(cuuint64_t)k2p, (cuuint64_t)rows, (cuuint64_t)batch};
  cuuint64_t strides[2] = {(cuuint64_t)k2p * elem, (cuuint64_t)rows * k2p * elem};
  cuuint32_t box[3] = {(cuuint32_t)(f16 ? KC16 : KC), (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(map, f16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                   const_cast<void*>(ptr), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// Operand planes of the tensor-core update: FP16 (scaled, kind::f16) when
// WMOM_TC_PLANES=f16, TF32 when tf32 (the default).
bool f16_planes() {
  static const bool on = [] {
    const char* e = std::getenv("WMOM_TC_PLANES");
    return e && std::strcmp(e, "f16") == 0;
  }();
  return on;
}

}  // namespace

// Grows ws->tc_buf to `floats`.  Inside a stream capture it refuses (the capture
// then fails and the caller launches directly, which grows the buffer); otherwise
// the old buffer is released only after the work queued on `s` has finished (in
// stream order for a pooled workspace, else by waiting for `s`).
cudaError_t tc_scratch(LuWorkspace* ws, size_t floats, cudaStream_t s) {
  if (!ws->tc_err) {
    cudaError_t e = cudaMalloc(&ws->tc_err, sizeof(int));
    if (e != cudaSuccess) return e;
    e = cudaMemset(ws->tc_err, 0, sizeof(int));
    if (e != cudaSuccess) return e;
  }
  if (ws->tc_cap >= floats) return cudaSuccess;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(s, &cs);
  if (e != cudaSuccess) return e;
  if (cs != cudaStreamCaptureStatusNone) return cudaErrorStreamCaptureUnsupported;
  if (ws->tc_buf) {
    if (ws->pooled) {
      e = cudaFreeAsync(ws->tc_buf, s);
    } else {
      e = cudaStreamSynchronize(s);
      if (e == cudaSuccess) e = cudaFree(ws->tc_buf);
    }
    ws->tc_buf = nullptr;
    ws->tc_cap = 0;
    if (e != cudaSuccess) return e;
  }
  e = ws->pooled ? cudaMallocAsync(reinterpret_cast<void**>(&ws->tc_buf), floats * sizeof(float), s)
                 : cudaMalloc(&ws->tc_buf, floats * sizeof(float));
  if (e != cudaSuccess) {
    ws->tc_buf = nullptr;
    return e;
  }
  ws->tc_cap = floats;
  ++ws->tc_gen;
  return cudaSuccess;
}

namespace {

// Scratch of the stand-alone entry point wmom_cgemm_sub_tc: one per device,
// serialised by a mutex (that entry point synchronises before returning).
std::mutex g_mu;
std::vector<LuWorkspace> g_ws;

}  // namespace

cudaError_t cgemm_sub_tc(LuWorkspace* ws, const float2* A, long long lda, const float2* B, long long ldb,
                         float2* C, long long ldc, int M, int N, int K, cudaStream_t s, int batch,
                         long long bstride) {
  if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
  if (!ws || batch < 1 || batch > 65535 || N > 65535) return cudaErrorInvalidValue;
  const bool f16 = f16_planes();
  const int kc = f16 ? KC16 : KC;
  const int K2p = ((2 * K + kc - 1) / kc) * kc;
  // planes in elements; the FP16 variant's row and column exponents follow its planes
  const size_t a_pl = (size_t)M * K2p * batch, b_pl = (size_t)2 * N * K2p * batch;
  const size_t plane_floats = f16 ? (a_pl + b_pl) : 2 * a_pl + 2 * b_pl;
  const size_t exp_ints = f16 ? ((size_t)M + (size_t)N) * batch : 0;
  cudaError_t e = tc_scratch(ws, plane_floats + exp_ints, s);
  if (e != cudaSuccess) return e;
  CUtensorMap mah, mal, mbh, mbl;
  // tile width: the one the factorisation's tuner chose for this workspace (the
  // FP16-plane variant always runs the wide tile)
  const int bn = (!f16 && ws->tile_n == kTileNarrow) ? kTileNarrow : kTileWide;
  const void* kern = f16 ? (const void*)cgemm_sub_tc_kernel<true, kTileWide>
                         : (bn == kTileNarrow ? (const void*)cgemm_sub_tc_kernel<false, kTileNarrow>
                                              : (const void*)cgemm_sub_tc_kernel<false, kTileWide>);
  int* ea = nullptr;
  int* eb = nullptr;
  if (f16) {
    __half* ahi = reinterpret_cast<__half*>(ws->tc_buf);
    __half* alo = ahi + a_pl;
    __half* bhi = alo + a_pl;
    __half* blo = bhi + b_pl;
    ea = reinterpret_cast<int*>(ws->tc_buf + plane_floats);
    eb = ea + (size_t)M * batch;
    stats::count(stats::kMisc, 4);
    rowexp_a_kernel<<<dim3((M + 255) / 256, batch), 256, 0, s>>>(A, lda, M, K, ea, bstride);
    colexp_b_kernel<<<dim3((N + 7) / 8, batch), 256, 0, s>>>(B, ldb, K, N, eb, bstride);
    pack_a_f16_kernel<<<dim3((M + 31) / 32, (K2p / 2 + 31) / 32, batch), 256, 0, s>>>(A, lda, M, K, K2p, ahi, alo,
                                                                                      ea, bstride);
    pack_b_f16_kernel<<<dim3((K2p / 2 + 127) / 128, N, batch), 128, 0, s>>>(B, ldb, K, N, K2p, bhi, blo, eb,
                                                                           bstride);
    if (!make_map(&mah, ahi, M, K2p, batch, BM, true) || !make_map(&mal, alo, M, K2p, batch, BM, true) ||
        !make_map(&mbh, bhi, 2 * N, K2p, batch, bn, true) || !make_map(&mbl, blo, 2 * N, K2p, batch, bn, true))
      return cudaErrorInvalidValue;
  } else {
    float* ahi = ws->tc_buf;
    float* alo = ahi + a_pl;
    float* bhi = alo + a_pl;
    float* blo = bhi + b_pl;
    stats::count(stats::kMisc, 2);
    pack_a_kernel<<<dim3((M + 31) / 32, (K2p / 2 + 31) / 32, batch), 256, 0, s>>>(A, lda, M, K, K2p, ahi, alo,
                                                                                  bstride);
    pack_b_kernel<<<dim3((K2p / 2 + 127) / 128, N, batch), 128, 0, s>>>(B, ldb, K, N, K2p, bhi, blo, bstride);
    if (!make_map(&mah, ahi, M, K2p, batch, BM, false) || !make_map(&mal, alo, M, K2p, batch, BM, false) ||
        !make_map(&mbh, bhi, 2 * N, K2p, batch, bn, false) || !make_map(&mbl, blo, 2 * N, K2p, batch, bn, false))
      return cudaErrorInvalidValue;
  }
  const int smem = smem_bytes(bn);
  e = allow_dynamic_smem(kern, smem);
  if (e != cudaSuccess) return e;
  const int tiles_m = (M + BM - 1) / BM, tiles_n = (2 * N + bn - 1) / bn;
  const long long ntiles = (long long)tiles_m * tiles_n * batch;
  if (ntiles > 0x7fffffffLL) return cudaErrorInvalidValue;
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
  }
  const int grid = (int)std::min<long long>(ntiles, nsm);
  stats::Scope sc(stats::kTcGemm, s, 8.0 * M * (double)N * K * batch);
  if (f16)
    cgemm_sub_tc_kernel<true, kTileWide><<<grid, NTHREADS, smem, s>>>(mah, mal, mbh, mbl, C, ldc, M, N, K2p / kc,
                                                                      tiles_m, tiles_n, (int)ntiles, ws->tc_err,
                                                                      bstride, ea, eb);
  else if (bn == kTileNarrow)
    cgemm_sub_tc_kernel<false, kTileNarrow><<<grid, NTHREADS, smem, s>>>(mah, mal, mbh, mbl, C, ldc, M, N,
                                                                         K2p / kc, tiles_m, tiles_n, (int)ntiles,
                                                                         ws->tc_err, bstride, nullptr, nullptr);
  else
    cgemm_sub_tc_kernel<false, kTileWide><<<grid, NTHREADS, smem, s>>>(mah, mal, mbh, mbl, C, ldc, M, N, K2p / kc,
                                                                       tiles_m, tiles_n, (int)ntiles, ws->tc_err,
                                                                       bstride, nullptr, nullptr);
  return cudaGetLastError();
}

int read_and_clear_error(LuWorkspace* ws, cudaStream_t s) {
  if (!ws || !ws->tc_err) return 0;
  int h = 0;
  if (cudaMemcpyAsync(&h, ws->tc_err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return 1;
  if (h) {
    cudaMemsetAsync(ws->tc_err, 0, sizeof(int), s);
    cudaStreamSynchronize(s);
  }
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
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return wmom_fail_cuda(e, "cgemm_sub_tc device");
  std::lock_guard<std::mutex> lk(wmom::tc::g_mu);
  if ((int)wmom::tc::g_ws.size() <= dev) wmom::tc::g_ws.resize(dev + 1);
  wmom::LuWorkspace* ws = &wmom::tc::g_ws[dev];
  e = wmom::tc::cgemm_sub_tc(ws, reinterpret_cast<const float2*>(a_dev), lda, reinterpret_cast<const float2*>(b_dev),
                             ldb, reinterpret_cast<float2*>(c_dev), ldc, m, n, k, s, 1, 0);
  if (e != cudaSuccess) return wmom_fail_cuda(e, "cgemm_sub_tc");
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return wmom_fail_cuda(e, "cgemm_sub_tc sync");
  if (wmom::tc::read_and_clear_error(ws, s)) return WMOM_ERR_TIMEOUT;
  return WMOM_OK;
}
