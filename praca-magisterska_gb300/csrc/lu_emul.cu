// lu_emul.cu -- FP64-grade complex trailing update of the LU on the bf16 tensor
// cores (tcgen05 kind::f16), the second tier of the precision form:
//
//   C (M x N complex128, column-major) -= A (M x K complex) * B (K x N complex)
//
// Method: error-free splitting in the manner of Ozaki, Ogita, Oishi and Rump
// ("Error-free transformations of matrix multiplication by using fast routines of
// matrix multiplication and its applications", Numer. Algorithms 59, 2012),
// arranged for FP32 tensor-core accumulation:
//   * complex -> real as in lu_tc.cu: A' (M x 2K) interleaves (re, im) along K,
//     B'^T (2N x 2K) has rows 2n = (Br, -Bi) and 2n+1 = (Bi, Br);
//   * row m of A' is scaled by 2^-ea[m] (ea = the exponent of its largest entry,
//     so the scaled entries lie in (-1, 1)), column n of B by 2^-eb[n];
//   * a scaled entry x is rounded once to the 48-bit fixed-point integer
//     X = rint(x 2^48) and written as NS = 6 balanced base-256 digits,
//       x = sum_t d_t 2^(-8(t+1)) + rest,  |rest| <= 2^-49,
//     |d_0| <= 256, d_t in [-128, 127] for t > 0; plane t stores d_t 2^(-8t), exact
//     in bf16;
//   * the product of planes i and j has weight 2^(-8(i+j)) ("level" i + j); the
//     levels 0, 1 and 2 each go to their own TMEM accumulator, where their sums
//     are exact in FP32 as long as 2K <= 192 (|level-2 sum| <= 192 (2*256*128 +
//     128^2) 2^-16 < 2^24 2^-16); levels 3..NS-1 go to further accumulators (one
//     shared, or one each, by tile shape), whose FP32 rounding is below 2^-48 of
//     the leading term;
//   * the epilogue adds the levels beyond 2 in FP32 and then levels 2, 1 and 0
//     error-free (a float pair), scales the pair by 2^(ea + eb - 16) with integer
//     operations on the exponent and subtracts it from C with two FP64 additions.
// Dropped levels (i + j >= NS) and the digit remainder are about 2^-45 of
// K * max|A| * max|B|, so the factorisation this update serves is FP64-grade
// (backward error near FP64 LU's); the FP64 refinement checks every solution.
//
// Kernel: persistent, one CTA (10 warps) per SM, 128 x BN real output tiles
// (BN / 2 complex columns; BN = 64 or 32).  A producer thread streams K in chunks of
// 32 bf16 (one 64-byte swizzle row) of all 2 x NS planes with 4-D TMA into a 3-stage
// ring; an MMA thread issues the 21 plane products (2 K-steps each) of a chunk into
// the NLEV accumulators of one of two accumulator sets, products of consecutive
// levels merged into one wide MMA (EmulShape); eight epilogue warps (two per TMEM
// lane quarter) prefetch their entries of C while the tile is multiplied, then read
// the accumulators with tcgen05.ld and update C while the next tile is multiplied.
// Every wait is bounded; on timeout the kernel records an error, skips the rest and
// still frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "lu_common.cuh"
#include "solve_internal.h"
#include "stats.h"
#include "tcgen05_util.cuh"

namespace wmom {
namespace emul {

using namespace tc;

constexpr int BM = 128;                             // accumulator lanes = rows of C per tile
constexpr int KC = 32;                              // bf16 of K per chunk (64 bytes)
constexpr int NS = 6;                               // digit planes per operand
constexpr int NBUF = 2;                             // accumulator sets (tile i's epilogue || i+1's MMAs)
constexpr int STAGES = 3;
constexpr int A_TILE = BM * KC * 2;                 // one plane's tile of A' (8 KB)
constexpr int EPI_WARPS = 8;                        // two per TMEM lane quarter, one column half each
constexpr int NTHREADS = 64 + 32 * EPI_WARPS;       // producer warp, MMA warp, epilogue warps
constexpr int kMaxK = 96;                           // complex K per launch (2K <= 192)

static_assert(NS * (NS + 1) / 2 == 21, "plane products per chunk");

// Tile shape: BN real columns of C per tile and NLEV accumulators per tile (levels
// 0 .. NLEV-2 each in its own, levels NLEV-1 .. NS-1 sharing the last).  The NLEV
// accumulators of one set lie side by side in TMEM (level L at column L * BN), and the
// NS planes of B'^T side by side in shared memory (plane j at row j * BN), so that
// the products of A plane i with B planes 0 .. NLEV-1-i, whose levels i .. NLEV-1
// are consecutive accumulators, are ONE MMA of N = (NLEV - i) * BN; only products
// whose level lies beyond the last accumulator are issued one plane at a time.
//   64 x 4: 15 MMAs per K step (N = 256, 192, 128, 64 and eleven of 64) instead of the
//           21 plane products; two sets fill TMEM.
//   32 x 6: every level in its own accumulator, 6 MMAs per K step (N = 192 .. 32)
//           for a tile half as wide; A is streamed twice as often per output.
template <int BN_, int NLEV_>
struct EmulShape {
  static constexpr int BN = BN_;
  static constexpr int NLEV = NLEV_;
  static constexpr int B_TILE = BN * KC * 2;                    // one plane's tile of B'^T
  static constexpr int STAGE_BYTES = NS * (A_TILE + B_TILE);
  static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 128;
  static constexpr int TMEM_USED = NBUF * NLEV * BN;
  static constexpr int TMEM_COLS = TMEM_USED <= 256 ? 256 : 512;  // a power of two
  static_assert(BN % 32 == 0 && NLEV * BN <= 256 && TMEM_USED <= 512, "tile shape");
  static_assert(NLEV >= 4 && NLEV <= NS, "levels 0, 1, 2 stay exact in their own accumulators");
  static_assert(STAGE_BYTES % 1024 == 0 && B_TILE % 512 == 0, "swizzle atoms stay aligned");
  static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");
};
using ShapeWide = EmulShape<64, 4>;
using ShapeNarrow = EmulShape<32, 6>;

// Instruction descriptor: D = F32, A = B = BF16, both K-major, M = BM, N = n.
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

// 2^e as a double (exact; ldexp outside the normal range).
__device__ __forceinline__ double pow2(int e) {
  if (e >= -1022 && e <= 1023) return __hiloint2double((e + 1023) << 20, 0);
  return ldexp(1.0, e);
}

// Plane values p[t] = d_t 2^(-8t) of x = v 2^-e in (-1, 1) (sc48 = 2^(48-e)): x is
// rounded once to the 48-bit fixed-point integer X = rint(x 2^48) (one exact FP64
// scaling and one conversion), whose balanced base-256 digits follow by integer
// operations: d_5..d_1 in [-128, 127], d_0 = what is left, |d_0| <= 256.  Then
// x = sum_t d_t 2^(-8(t+1)) to within 2^-49.
__device__ __forceinline__ void digit_planes(double v, double sc48, float p[NS]) {
  long long X = __double2ll_rn(v * sc48);
  int d[NS];
#pragma unroll
  for (int t = NS - 1; t > 0; --t) {
    d[t] = (int)((X + 128) & 255) - 128;
    X = (X - d[t]) >> 8;
  }
  d[0] = (int)X;
  float w = 1.0f;
#pragma unroll
  for (int t = 0; t < NS; ++t) {
    p[t] = (float)d[t] * w;
    w *= 0x1p-8f;
  }
}

// 16 consecutive 32-bit TMEM columns of this warp's lane quarter.
__device__ __forceinline__ void tmem_ld16(uint32_t addr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(addr));
}

// Error-free sum of two floats: s + e = a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// 2^k x as a double for a float x that is zero or normal, by integer operations on
// the bit fields (exact; the caller keeps k within [-900, 900], so that the result
// is a normal double for every accumulator value).
__device__ __forceinline__ double f32_scaled(float x, int k) {
  const uint32_t u = __float_as_uint(x);
  const uint32_t mag = u & 0x7fffffffu;
  const uint32_t sign = u & 0x80000000u;
  const uint32_t hi = sign | ((mag >> 3) + ((uint32_t)(896 + k) << 20));
  return __hiloint2double((int)(mag ? hi : sign), (int)(mag ? (u << 29) : 0u));
}

// 2^k x for a float x that is zero or normal, by an integer add to its exponent field;
// ok when the result is zero or a normal float as well.
__device__ __forceinline__ bool f32_scale_ok(float x, int k) {
  const int e = (int)((__float_as_uint(x) >> 23) & 255u);
  return x == 0.f || (e > 0 && e + k >= 1 && e + k <= 254);
}
__device__ __forceinline__ float f32_scale(float x, int k) {
  return x == 0.f ? x : __uint_as_float(__float_as_uint(x) + ((unsigned)k << 23));
}

// c - (s + e) for a float-float c = (ch, cl) and the unnormalised float pair (s, e):
// one error-free sum of the heads and the tails added, about 2^-48 relative
__device__ __forceinline__ void ff_sub_pair(float& ch, float& cl, float s, float e) {
  float h, t;
  two_sum(ch, -s, h, t);
  t = __fadd_rn(t, __fsub_rn(cl, e));
  ch = __fadd_rn(h, t);
  cl = __fsub_rn(t, __fsub_rn(ch, h));
}

__device__ __forceinline__ uint32_t bf16x2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// ---------------------------------------------------------------- pack ----
// A (M x K complex, column-major) -> NS planes of A' (row-major M x K2p bf16,
// zero beyond 2K) and the row exponents ea.  A block of 4 warps covers 32 rows:
// lane = row (coalesced column reads), warp = a quarter of the K2p/2 complex
// columns; the quarters' row maxima meet in shared memory.
// An entry of an operand held as complex128, or (FFS) as float-float (float4: hi.re,
// hi.im, lo.re, lo.im in the same 16 bytes; hi + lo is exact in FP64).
template <bool FFS>
__device__ __forceinline__ double2 ld_operand(const double2* p) {
  if constexpr (FFS) {
    const float4 f = *reinterpret_cast<const float4*>(p);
    return make_double2((double)f.x + (double)f.z, (double)f.y + (double)f.w);
  } else {
    return *p;
  }
}

template <bool FFS>
__global__ void __launch_bounds__(128) emul_pack_a_kernel(const double2* __restrict__ A, long long lda, int M, int K,
                                                         int K2p, __nv_bfloat16* __restrict__ planes,
                                                         size_t plane_elems, int* __restrict__ ea,
                                                         long long astride) {
  __shared__ double smax[4][32];
  const int b = blockIdx.y;
  const int lane = threadIdx.x & 31, part = threadIdx.x >> 5;
  const int m = blockIdx.x * 32 + lane;
  const int kq = K2p / 8;  // complex columns per quarter (a multiple of 4)
  const int k0 = part * kq;
  A += (size_t)b * astride;
  double mx = 0.0;
  if (m < M)
    for (int k = k0; k < min(K, k0 + kq); ++k) {
      const double2 v = ld_operand<FFS>(&A[(size_t)k * lda + m]);
      mx = fmax(mx, fmax(fabs(v.x), fabs(v.y)));
    }
  smax[part][lane] = mx;
  __syncthreads();
  mx = fmax(fmax(smax[0][lane], smax[1][lane]), fmax(smax[2][lane], smax[3][lane]));
  if (m >= M) return;
  int e = 0;
  frexp(mx, &e);  // mx < 2^e; e = 0 for a zero row
  if (part == 0) ea[(size_t)b * M + m] = e;
  const double sc48 = pow2(48 - e);
  __nv_bfloat16* row = planes + ((size_t)b * M + m) * K2p;
  for (int kc = k0; kc < k0 + kq; kc += 4) {  // 4 complex = 8 bf16 = 16 bytes per plane
    float pr[4][NS], pi[4][NS];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      double2 v = make_double2(0.0, 0.0);
      if (kc + u < K) v = ld_operand<FFS>(&A[(size_t)(kc + u) * lda + m]);
      digit_planes(v.x, sc48, pr[u]);
      digit_planes(v.y, sc48, pi[u]);
    }
#pragma unroll
    for (int t = 0; t < NS; ++t) {
      uint4 q;
      q.x = bf16x2(pr[0][t], pi[0][t]);
      q.y = bf16x2(pr[1][t], pi[1][t]);
      q.z = bf16x2(pr[2][t], pi[2][t]);
      q.w = bf16x2(pr[3][t], pi[3][t]);
      *reinterpret_cast<uint4*>(row + (size_t)t * plane_elems + 2 * kc) = q;
    }
  }
}

// B (K x N complex, column-major) -> NS planes of B'^T (row-major 2N x K2p bf16)
// and the column exponents eb.  One warp per column (lanes along K).
template <bool FFS>
__global__ void emul_pack_b_kernel(const double2* __restrict__ B, long long ldb, int K, int N, int K2p,
                                   __nv_bfloat16* __restrict__ planes, size_t plane_elems,
                                   int* __restrict__ eb, long long bstride) {
  const int b = blockIdx.y;
  const int lane = threadIdx.x & 31;
  const int n = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (n >= N) return;  // warp-uniform
  B += (size_t)b * bstride + (size_t)n * ldb;
  double mx = 0.0;
  for (int k = lane; k < K; k += 32) {
    const double2 v = ld_operand<FFS>(&B[k]);
    mx = fmax(mx, fmax(fabs(v.x), fabs(v.y)));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  int e = 0;
  frexp(mx, &e);
  if (lane == 0) eb[(size_t)b * N + n] = e;
  const double sc48 = pow2(48 - e);
  __nv_bfloat16* r0 = planes + ((size_t)b * 2 * N + 2 * (size_t)n) * K2p;
  __nv_bfloat16* r1 = r0 + K2p;
  for (int k = lane; k < K2p / 2; k += 32) {
    double2 v = make_double2(0.0, 0.0);
    if (k < K) v = ld_operand<FFS>(&B[k]);
    float pr[NS], pi[NS];
    digit_planes(v.x, sc48, pr);
    digit_planes(v.y, sc48, pi);
#pragma unroll
    for (int t = 0; t < NS; ++t) {
      *reinterpret_cast<uint32_t*>(r0 + (size_t)t * plane_elems + 2 * k) = bf16x2(pr[t], -pi[t]);
      *reinterpret_cast<uint32_t*>(r1 + (size_t)t * plane_elems + 2 * k) = bf16x2(pi[t], pr[t]);
    }
  }
}

// ---------------------------------------------------------------- gemm ----
struct TileCoord {
  int mat, m0, j0;
};

__device__ __forceinline__ TileCoord tile_coord(int t, int tiles_m, int tiles_n, int bn) {
  const int per_mat = tiles_m * tiles_n;
  const int mat = t / per_mat;
  const int r = t - mat * per_mat;
  const int tn = r / tiles_m;
  return TileCoord{mat, (r - tn * tiles_m) * BM, tn * bn};
}

// FFS: C holds float-float values (float4 hi.re, hi.im, lo.re, lo.im per entry), which
// the epilogue updates in float-float arithmetic on the FP32 pipe; else complex128,
// updated with two FP64 additions per real entry.  SH: the tile shape (EmulShape).
template <bool FFS, class SH>
__global__ void __launch_bounds__(NTHREADS, 1)
    zgemm_sub_emul_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                          const int* __restrict__ ea, const int* __restrict__ eb, double2* __restrict__ C,
                          long long ldc, int M, int N, int nchunks, int tiles_m, int tiles_n, int ntiles,
                          int* __restrict__ err, long long cstride) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  constexpr int BN = SH::BN, NLEV = SH::NLEV, B_TILE = SH::B_TILE, STAGE_BYTES = SH::STAGE_BYTES;
  constexpr int TMEM_COLS = SH::TMEM_COLS;
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + STAGES * STAGE_BYTES);
  // bars: full[STAGES], empty[STAGES], tfull[NBUF], tempty[NBUF]
  __shared__ uint32_t tmem_base;
  __shared__ volatile int s_fail;
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  auto full_bar = [&](int s) { return smem_u32(&bars[s]); };
  auto empty_bar = [&](int s) { return smem_u32(&bars[STAGES + s]); };
  auto tfull_bar = [&](int b) { return smem_u32(&bars[2 * STAGES + b]); };
  auto tempty_bar = [&](int b) { return smem_u32(&bars[2 * STAGES + NBUF + b]); };

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
    for (int b = 0; b < NBUF; ++b) {
      mbar_init(tfull_bar(b), 1);
      mbar_init(tempty_bar(b), EPI_WARPS);  // one arrival per epilogue warp
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
      int it = 0;
      bool ok = !s_fail;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const TileCoord tc = tile_coord(t, tiles_m, tiles_n, BN);
        for (int c = 0; c < nchunks; ++c) {
          const int s = it % STAGES, use = it / STAGES;
          if (use > 0 && !(ok = role_wait(empty_bar(s), (use - 1) & 1, err, &s_fail))) break;
          const uint32_t a0 = smem_u32(base + s * STAGE_BYTES);
          const uint32_t b0 = a0 + NS * A_TILE;
          mbar_expect_tx(full_bar(s), STAGE_BYTES);
#pragma unroll
          for (int p = 0; p < NS; ++p) {
            tma_load_4d(a0 + p * A_TILE, &mapA, c * KC, tc.m0, tc.mat, p, full_bar(s));
            tma_load_4d(b0 + p * B_TILE, &mapB, c * KC, tc.j0, tc.mat, p, full_bar(s));
          }
          ++it;
        }
      }
      if (!ok) {
        s_fail = 1;
        atomicExch(err, 1);
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
        const int b = tl % NBUF, use = tl / NBUF;
        if (use > 0 && !(ok = role_wait(tempty_bar(b), (use - 1) & 1, err, &s_fail))) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t accb = tmem + (uint32_t)(b * NLEV * BN);
        for (int c = 0; c < nchunks; ++c) {
          const int s = it % STAGES;
          if (!(ok = role_wait(full_bar(s), (it / STAGES) & 1, err, &s_fail))) break;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t a0 = smem_u32(base + s * STAGE_BYTES);
          const uint32_t b0 = a0 + NS * A_TILE;
#pragma unroll
          for (int kk = 0; kk < KC / 16; ++kk) {
            const uint64_t bd0 = sdesc_sw<64>(b0 + kk * 32);  // B planes 0, 1, ... side by side
#pragma unroll
            for (int i = 0; i < NS; ++i) {
              const uint64_t ad = sdesc_sw<64>(a0 + i * A_TILE + kk * 32);
              // B planes 0 .. NLEV-1-i: levels i .. NLEV-1, consecutive accumulators,
              // one MMA; the tile's first one (i = 0, all NLEV accumulators) overwrites
              if (i < NLEV)
                mma_bf16(accb + (uint32_t)(i * BN), ad, bd0, idesc_bf16((NLEV - i) * BN),
                         (c == 0 && kk == 0 && i == 0) ? 0u : 1u);
              // B planes whose level lies beyond the last accumulator: into it, one each
#pragma unroll
              for (int j = (i < NLEV ? NLEV - i : 0); j <= NS - 1 - i; ++j)
                mma_bf16(accb + (uint32_t)((NLEV - 1) * BN), ad, sdesc_sw<64>(b0 + j * B_TILE + kk * 32),
                         idesc_bf16(BN), 1u);
            }
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
        if (it > 0) {
          const int zero = 0;
          const volatile int no_fail = 0;
          role_wait(empty_bar((it - 1) % STAGES), ((it - 1) / STAGES) & 1, &zero, &no_fail);
        }
      }
    }
  } else {
    // ----------------------------------------------------------- epilogue
    // warp w >= 2: TMEM lanes 32 (w % 4) .. +31 (the quarter it may read), complex
    // columns h*CW .. h*CW+CW-1 of the tile (CW = BN / 4)
    constexpr int CW = BN / 4;
    const int q = warp & 3, h = (warp - 2) >> 2;
    int tl = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++tl) {
      const TileCoord tc = tile_coord(t, tiles_m, tiles_n, BN);
      double2* Cm = C + (size_t)tc.mat * cstride;
      const int* ebm = eb + (size_t)tc.mat * N;
      const int row = tc.m0 + q * 32 + lane;
      const bool row_ok = row < M;
      const int erow = row_ok ? ea[(size_t)tc.mat * M + row] - 16 : 0;
      const int n0 = (tc.j0 >> 1) + h * CW;
      // this thread's CW entries of C, in flight while the tile is multiplied
      double2 cv[CW];
#pragma unroll
      for (int j = 0; j < CW; ++j)
        cv[j] = (row_ok && n0 + j < N) ? Cm[(size_t)(n0 + j) * ldc + row] : make_double2(0.0, 0.0);
      const int b = tl % NBUF, use = tl / NBUF;
      int ok = 0;
      if (lane == 0) ok = role_wait(tfull_bar(b), use & 1, err, &s_fail) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) {
        if (lane == 0) {
          s_fail = 1;
          atomicExch(err, 1);
        }
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * NLEV * BN + h * (BN / 2));
#pragma unroll
      for (int cc = 0; cc < BN / 32; ++cc) {
        // the levels of 16 real entries (8 complex) summed into float pairs (s, e),
        // highest level first, one accumulator read at a time: the accumulators beyond
        // level 2 (2^-24 and less of the leading term) in plain FP32, then levels 2, 1
        // and 0 error-free
        float sp[16], ep[16];
        {
          uint32_t rt[16], r2[16];
          tmem_ld16(taddr + (uint32_t)((NLEV - 1) * BN + cc * 16), rt);
          tmem_ld16(taddr + (uint32_t)(2 * BN + cc * 16), r2);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          float tail[16];
#pragma unroll
          for (int x = 0; x < 16; ++x) tail[x] = __uint_as_float(rt[x]);
#pragma unroll
          for (int L = NLEV - 2; L >= 3; --L) {
            tmem_ld16(taddr + (uint32_t)(L * BN + cc * 16), rt);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int x = 0; x < 16; ++x) tail[x] = __fadd_rn(tail[x], __uint_as_float(rt[x]));
          }
#pragma unroll
          for (int x = 0; x < 16; ++x) two_sum(__uint_as_float(r2[x]), tail[x], sp[x], ep[x]);
        }
#pragma unroll
        for (int L = 1; L >= 0; --L) {
          uint32_t rl[16];
          tmem_ld16(taddr + (uint32_t)(L * BN + cc * 16), rl);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int x = 0; x < 16; ++x) {
            float e2;
            two_sum(__uint_as_float(rl[x]), sp[x], sp[x], e2);
            ep[x] = __fadd_rn(ep[x], e2);
          }
        }
        if (row_ok) {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int n = n0 + cc * 8 + j;
            if (n < N) {
              // scaled and subtracted with two FP64 additions per real entry (the
              // SM's FP64 pipe is the epilogue's arithmetic bound; the rest is FP32
              // and integer work)
              const int k = erow + ebm[n];
              double2 v = cv[cc * 8 + j];
              if constexpr (FFS) {
                const float s0 = sp[2 * j], e0 = ep[2 * j], s1 = sp[2 * j + 1], e1 = ep[2 * j + 1];
                float4 f = *reinterpret_cast<const float4*>(&v);  // hi.re, hi.im, lo.re, lo.im
                if (f32_scale_ok(s0, k) && f32_scale_ok(e0, k) && f32_scale_ok(s1, k) && f32_scale_ok(e1, k)) {
                  ff_sub_pair(f.x, f.z, f32_scale(s0, k), f32_scale(e0, k));
                  ff_sub_pair(f.y, f.w, f32_scale(s1, k), f32_scale(e1, k));
                } else {
                  // out of FP32's exponent range after scaling: through FP64
                  const double sc = pow2(k);
                  const double re = ((double)f.x + (double)f.z - (double)s0 * sc) - (double)e0 * sc;
                  const double im = ((double)f.y + (double)f.w - (double)s1 * sc) - (double)e1 * sc;
                  const float rh = __double2float_rn(re), ih = __double2float_rn(im);
                  f = make_float4(rh, ih, __double2float_rn(re - (double)rh), __double2float_rn(im - (double)ih));
                }
                *reinterpret_cast<float4*>(&Cm[(size_t)n * ldc + row]) = f;
                continue;
              }
              if (k >= -900 && k <= 900) {
                v.x = __dsub_rn(__dsub_rn(v.x, f32_scaled(sp[2 * j], k)), f32_scaled(ep[2 * j], k));
                v.y = __dsub_rn(__dsub_rn(v.y, f32_scaled(sp[2 * j + 1], k)), f32_scaled(ep[2 * j + 1], k));
              } else {
                const double sc = pow2(k);
                v.x = __dsub_rn(__dsub_rn(v.x, (double)sp[2 * j] * sc), (double)ep[2 * j] * sc);
                v.y = __dsub_rn(__dsub_rn(v.y, (double)sp[2 * j + 1] * sc), (double)ep[2 * j + 1] * sc);
              }
              Cm[(size_t)n * ldc + row] = v;
            }
          }
        }
      }
      // accumulator set b read out: the MMA issuer may overwrite it
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(tempty_bar(b));
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 1) {
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// ----------------------------------------------------------- host side ----
namespace {

// 4-D map over NS planes of `batch` matrices of rows x k2p bf16 (row-major),
// 32 x box_rows boxes with 64-byte swizzle.
bool make_map(CUtensorMap* map, const __nv_bfloat16* ptr, int rows, int k2p, int batch, int box_rows) {
  EncodeFn enc = encode_fn();
  if (!enc) return false;
  cuuint64_t dims[4] = {(cuuint64_t)k2p, (cuuint64_t)rows, (cuuint64_t)batch, (cuuint64_t)NS};
  cuuint64_t strides[3] = {(cuuint64_t)k2p * 2, (cuuint64_t)rows * k2p * 2, (cuuint64_t)batch * rows * k2p * 2};
  cuuint32_t box[4] = {(cuuint32_t)KC, (cuuint32_t)box_rows, 1, 1};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16*>(ptr), dims, strides, box,
                   estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

std::mutex g_mu;
std::vector<LuWorkspace> g_ws;

// Tile width of the update: 32 (ShapeNarrow) unless WMOM_EMUL_TILE=64 (ShapeWide).
// Measured on 8192 x 8192 x 96: 1.04 ms per call narrow, 1.09 ms wide; both shapes
// keep the tensor pipe near 45% busy, and the narrow tile's shorter epilogue hides
// better behind its MMAs.  The shape changes only the FP32 rounding of the levels
// beyond 2, about 2^-48 of the leading term.
int emul_tile() {
  const char* v = std::getenv("WMOM_EMUL_TILE");
  return (v && std::atoi(v) == 64) ? 64 : 32;
}

template <class SH>
cudaError_t launch_gemm(bool ffs, const __nv_bfloat16* pa, const __nv_bfloat16* pb, const int* ea, const int* eb,
                        double2* C, long long ldc, int M, int N, int K2p, int batch, long long bstride, int* err,
                        int nsm, cudaStream_t s) {
  CUtensorMap ma, mb;
  if (!make_map(&ma, pa, M, K2p, batch, BM) || !make_map(&mb, pb, 2 * N, K2p, batch, SH::BN))
    return cudaErrorInvalidValue;
  const void* kern =
      ffs ? (const void*)zgemm_sub_emul_kernel<true, SH> : (const void*)zgemm_sub_emul_kernel<false, SH>;
  cudaError_t e = allow_dynamic_smem(kern, SH::SMEM_BYTES);
  if (e != cudaSuccess) return e;
  const int tiles_m = (M + BM - 1) / BM, tiles_n = (2 * N + SH::BN - 1) / SH::BN;
  const long long ntiles = (long long)tiles_m * tiles_n * batch;
  if (ntiles > 0x7fffffffLL) return cudaErrorInvalidValue;
  const int grid = (int)std::min<long long>(ntiles, nsm);
  if (ffs)
    zgemm_sub_emul_kernel<true, SH><<<grid, NTHREADS, SH::SMEM_BYTES, s>>>(
        ma, mb, ea, eb, C, ldc, M, N, K2p / KC, tiles_m, tiles_n, (int)ntiles, err, bstride);
  else
    zgemm_sub_emul_kernel<false, SH><<<grid, NTHREADS, SH::SMEM_BYTES, s>>>(
        ma, mb, ea, eb, C, ldc, M, N, K2p / KC, tiles_m, tiles_n, (int)ntiles, err, bstride);
  return cudaGetLastError();
}

}  // namespace

cudaError_t zgemm_sub_emul(LuWorkspace* ws, const double2* A, long long lda, const double2* B, long long ldb,
                           double2* C, long long ldc, int M, int N, int K, cudaStream_t s, int batch,
                           long long bstride) {
  if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
  if (!ws || batch < 1 || batch > 65535) return cudaErrorInvalidValue;
  if (K > kMaxK) {
    // K slabs of at most kMaxK, one after another on C (keeps levels 0-2 exact)
    for (int k0 = 0; k0 < K; k0 += kMaxK) {
      const int kk = std::min(kMaxK, K - k0);
      const cudaError_t e = zgemm_sub_emul(ws, A + (size_t)k0 * lda, lda, B + k0, ldb, C, ldc, M, N, kk, s, batch,
                                           bstride);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  const int K2p = ((2 * K + KC - 1) / KC) * KC;
  const size_t a_pl = (size_t)M * K2p * batch, b_pl = (size_t)2 * N * K2p * batch;  // bf16 per plane
  const size_t plane_bytes = 2 * (size_t)NS * (a_pl + b_pl);
  const size_t exp_bytes = sizeof(int) * ((size_t)M + N) * batch;
  cudaError_t e = tc_scratch(ws, (plane_bytes + exp_bytes) / sizeof(float) + 64, s);
  if (e != cudaSuccess) return e;
  __nv_bfloat16* pa = reinterpret_cast<__nv_bfloat16*>(ws->tc_buf);
  __nv_bfloat16* pb = pa + NS * a_pl;
  int* ea = reinterpret_cast<int*>(pb + NS * b_pl);
  int* eb = ea + (size_t)M * batch;
  stats::count(stats::kMisc, 2);
  const bool ffs = ws->ff_storage;
  if (ffs) {
    emul_pack_a_kernel<true><<<dim3((M + 31) / 32, batch), 128, 0, s>>>(A, lda, M, K, K2p, pa, a_pl, ea, bstride);
    emul_pack_b_kernel<true><<<dim3((N + 7) / 8, batch), 256, 0, s>>>(B, ldb, K, N, K2p, pb, b_pl, eb, bstride);
  } else {
    emul_pack_a_kernel<false><<<dim3((M + 31) / 32, batch), 128, 0, s>>>(A, lda, M, K, K2p, pa, a_pl, ea, bstride);
    emul_pack_b_kernel<false><<<dim3((N + 7) / 8, batch), 256, 0, s>>>(B, ldb, K, N, K2p, pb, b_pl, eb, bstride);
  }
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
  }
  stats::Scope sc(stats::kEmulGemm, s, 8.0 * M * (double)N * K * batch);
  if (emul_tile() == 32)
    return launch_gemm<ShapeNarrow>(ffs, pa, pb, ea, eb, C, ldc, M, N, K2p, batch, bstride, ws->tc_err, nsm, s);
  return launch_gemm<ShapeWide>(ffs, pa, pb, ea, eb, C, ldc, M, N, K2p, batch, bstride, ws->tc_err, nsm, s);
}

}  // namespace emul

GemmHook<double2> emul_gemm_hook() {
  if (std::getenv("WMOM_NO_EMUL")) return nullptr;
  int dev = 0, major = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  if (major != 10) return nullptr;
  return &emul::zgemm_sub_emul;
}

}  // namespace wmom

extern "C" wmom_status wmom_zgemm_sub_emul(int m, int n, int k, const void* a_dev, long long lda, const void* b_dev,
                                           long long ldb, void* c_dev, long long ldc, void* stream) {
  if (m < 0 || n < 0 || k < 0 || (m && (!a_dev || !c_dev || lda < m || ldc < m)) || (n && (!b_dev || ldb < k)))
    return WMOM_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return wmom_fail_cuda(e, "zgemm_sub_emul device");
  std::lock_guard<std::mutex> lk(wmom::emul::g_mu);
  if ((int)wmom::emul::g_ws.size() <= dev) wmom::emul::g_ws.resize(dev + 1);
  wmom::LuWorkspace* ws = &wmom::emul::g_ws[dev];
  e = wmom::emul::zgemm_sub_emul(ws, reinterpret_cast<const double2*>(a_dev), lda,
                                 reinterpret_cast<const double2*>(b_dev), ldb, reinterpret_cast<double2*>(c_dev), ldc,
                                 m, n, k, s, 1, 0);
  if (e != cudaSuccess) return wmom_fail_cuda(e, "zgemm_sub_emul");
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return wmom_fail_cuda(e, "zgemm_sub_emul sync");
  if (wmom::tc::read_and_clear_error(ws, s)) return WMOM_ERR_TIMEOUT;
  return WMOM_OK;
}
