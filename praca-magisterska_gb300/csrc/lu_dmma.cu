// lu_dmma.cu -- the plain FP64 form's trailing update on the FP64 tensor pipe.
//
// C (M x N) -= A (M x K) * B (K x N) for complex FP64 column-major operands, as
// warp-level DMMA: mma.sync.m8n8k4.row.col.f64 (8 x 8 real tile, k = 4), four real
// products per complex product (Cr -= Ar Br - Ai Bi, Ci -= Ar Bi + Ai Br) into
// separate real and imaginary accumulators.  The reference factors with MKL's
// zgetrf on the CPU and cuBLAS zgetrfBatched on the GPU ("wersja referencyjna/
// Wire_MoM.cu":372, "wersja gpu/Wire_MoM.cu":468); this is the FP64 tensor-pipe
// counterpart of the SIMT gemm_sub_kernel<double2> of lu.cu, kept beside it so
// that the two can be timed on the same shapes (bench.py --workload gemm_dmma /
// gemm_simt) and the faster one used.
//
// CTA: 64 x 64 complex outputs, four warps of 32 x 32 (4 x 4 MMA tiles); K staged in
// shared memory 8 complex columns at a time, double-buffered (34 KB of static shared
// memory), the next stage's global loads issued before the current stage's MMAs.  Fragment layout of
// m8n8k4.f64 (PTX ISA): lane l, g = l >> 2, t = l & 3: A[g][t] (row-major 8 x 4),
// B[t][g] (column-major 4 x 8), C[g][2t], C[g][2t + 1].
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>

#include "lu_common.cuh"
#include "lu_internal.h"
#include "stats.h"
#include "wmom_internal.h"

namespace wmom {

namespace {

constexpr int kDmBM = 64, kDmBN = 64, kDmBK = 8;
constexpr int kDmLd = kDmBM + 2;  // padded row of the staged tiles: fragment reads are conflict-free
constexpr int kDmThreads = 128;

__device__ __forceinline__ void dmma(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(kDmThreads) zgemm_sub_dmma_kernel(const double2* __restrict__ Am, long long lda,
                                                                   const double2* __restrict__ Bm, long long ldb,
                                                                   double2* __restrict__ Cm, long long ldc, int M,
                                                                   int N, int K, long long bstride) {
  __shared__ double2 As[2][kDmBK][kDmLd];  // [k][m]
  __shared__ double2 Bs[2][kDmBK][kDmLd];  // [k][n]
  Am += (size_t)blockIdx.z * bstride;
  Bm += (size_t)blockIdx.z * bstride;
  Cm += (size_t)blockIdx.z * bstride;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
  const int m0 = blockIdx.x * kDmBM, n0 = blockIdx.y * kDmBN;

  // this thread's share of a stage: 4 entries of A (consecutive rows across the
  // threads) and 4 of B (consecutive k across the threads)
  constexpr int kPer = kDmBK * kDmBM / kDmThreads;
  double2 ra[kPer], rb[kPer];
  auto load_stage = [&](int k0) {
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
      const int idx = tid + q * kDmThreads;
      const int kk = idx / kDmBM, r = idx - kk * kDmBM;
      const int gr = m0 + r, gk = k0 + kk;
      ra[q] = (gr < M && gk < K) ? Am[(size_t)gk * lda + gr] : make_double2(0.0, 0.0);
      const int c = idx / kDmBK, kb = idx - c * kDmBK;
      const int gc = n0 + c, gkb = k0 + kb;
      rb[q] = (gc < N && gkb < K) ? Bm[(size_t)gc * ldb + gkb] : make_double2(0.0, 0.0);
    }
  };
  auto store_stage = [&](int buf) {
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
      const int idx = tid + q * kDmThreads;
      const int kk = idx / kDmBM, r = idx - kk * kDmBM;
      As[buf][kk][r] = ra[q];
      const int c = idx / kDmBK, kb = idx - c * kDmBK;
      Bs[buf][kb][c] = rb[q];
    }
  };

  double cr[4][4][2], ci[4][4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) cr[i][j][0] = cr[i][j][1] = ci[i][j][0] = ci[i][j][1] = 0.0;

  const int nst = (K + kDmBK - 1) / kDmBK;
  if (nst > 0) {
    load_stage(0);
    store_stage(0);
  }
  __syncthreads();
  for (int st = 0; st < nst; ++st) {
    const int buf = st & 1;
    if (st + 1 < nst) load_stage((st + 1) * kDmBK);  // in flight during the MMAs below
#pragma unroll
    for (int kk = 0; kk < kDmBK; kk += 4) {
      double ar[4], ai[4], nai[4], br[4], bi[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const double2 a = As[buf][kk + t][wm + 8 * i + g];
        ar[i] = a.x;
        ai[i] = a.y;
        nai[i] = -a.y;
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const double2 b = Bs[buf][kk + t][wn + 8 * j + g];
        br[j] = b.x;
        bi[j] = b.y;
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          dmma(cr[i][j][0], cr[i][j][1], ar[i], br[j]);
          dmma(cr[i][j][0], cr[i][j][1], nai[i], bi[j]);
          dmma(ci[i][j][0], ci[i][j][1], ar[i], bi[j]);
          dmma(ci[i][j][0], ci[i][j][1], ai[i], br[j]);
        }
    }
    if (st + 1 < nst) store_stage(buf ^ 1);
    __syncthreads();
  }
  // C -= the accumulated product: entry (wm + 8i + g, wn + 8j + 2t + h)
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int gc = n0 + wn + 8 * j + 2 * t + h;
      if (gc >= N) continue;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int gr = m0 + wm + 8 * i + g;
        if (gr >= M) continue;
        double2* p = &Cm[(size_t)gc * ldc + gr];
        double2 v = *p;
        v.x -= cr[i][j][h];
        v.y -= ci[i][j][h];
        *p = v;
      }
    }
}

}  // namespace

cudaError_t zgemm_sub_dmma(const double2* Am, long long lda, const double2* Bm, long long ldb, double2* Cm,
                           long long ldc, int M, int N, int K, cudaStream_t s, int batch, long long bstride) {
  if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
  stats::Scope sc(stats::kGemm, s, 8.0 * M * (double)N * K * batch);
  dim3 grid((M + kDmBM - 1) / kDmBM, (N + kDmBN - 1) / kDmBN, batch);
  zgemm_sub_dmma_kernel<<<grid, kDmThreads, 0, s>>>(Am, lda, Bm, ldb, Cm, ldc, M, N, K, bstride);
  return cudaGetLastError();
}

bool fp64_update_dmma() {
  static const bool on = [] {
    const char* e = std::getenv("WMOM_FP64_UPDATE");
    return e && std::strcmp(e, "dmma") == 0;
  }();
  return on;
}

}  // namespace wmom

using namespace wmom;

extern "C" wmom_status wmom_zgemm_sub_fp64(int m, int n, int k, const void* a_dev, long long lda, const void* b_dev,
                                           long long ldb, void* c_dev, long long ldc, int variant, void* stream) {
  if (m < 0 || n < 0 || k < 0 || (m && (!a_dev || !c_dev || lda < m || ldc < m)) || (n && (!b_dev || ldb < k)) ||
      (variant != 0 && variant != 1))
    return WMOM_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const double2* A = reinterpret_cast<const double2*>(a_dev);
  const double2* B = reinterpret_cast<const double2*>(b_dev);
  double2* C = reinterpret_cast<double2*>(c_dev);
  cudaError_t e = variant == 1 ? zgemm_sub_dmma(A, lda, B, ldb, C, ldc, m, n, k, s, 1, 0)
                               : zgemm_sub_simt(A, lda, B, ldb, C, ldc, m, n, k, s, 1, 0);
  if (e != cudaSuccess) return wmom_fail_cuda(e, "zgemm_sub_fp64");
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return wmom_fail_cuda(e, "zgemm_sub_fp64 sync");
  return WMOM_OK;
}
