// lu.cu -- blocked right-looking complex LU with partial pivoting, and the
// triangular solves, on one GPU (FP64 plain form; the same templates run in FP32
// for the precision form, whose trailing update is the tensor-core GEMM in
// lu_tc.cu).
//
// Replaces the reference's LAPACKE_zgetrf / LAPACKE_zgetrs pair
// ("wersja referencyjna/Wire_MoM.cu":372,382) and the cublasZgetrfBatched /
// cublasZgetrsBatched path of "wersja gpu/Wire_MoM.cu":417-504.  Semantics are
// LAPACK's: the pivot of column j is the first row of largest |re|+|im| on or
// below the diagonal, rows are interchanged across the full width, L is unit lower
// triangular, ipiv is 1-based, info = first exactly-zero pivot column.
//
// Per panel of NB columns:
//   1. panel_kernel   -- cooperative launch; the panel rows are spread over the
//                        CTAs' shared memory and each column costs ONE grid-wide
//                        barrier (pivot candidates, the candidate rows and the
//                        diagonal row are published before it, so the winner, the
//                        swap and the rank-1 update follow without another one);
//   2. laswp_kernel   -- the NB interchanges applied to the columns left and right;
//   3. trsm_kernel    -- U12 = L11^-1 A12;
//   4. gemm_kernel    -- A22 -= L21 U12.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <mutex>
#include <vector>

#include "lu_common.cuh"
#include "lu_internal.h"
#include "stats.h"
#include "wmom_internal.h"

namespace wmom {

// ------------------------------------------------------------- panel ----
template <typename C, int NB>
struct PanelStage {
  decltype(C{}.x) cand_val[2][kMaxPanelBlocks];
  int cand_row[2][kMaxPanelBlocks];
  C cand_data[2][kMaxPanelBlocks][NB];
  C diag_data[2][NB];
};

template <typename C, int NB, int NT>
__global__ void __launch_bounds__(NT) panel_kernel(C* __restrict__ A, long long lda, int n, int j0,
                                                   int nb, int rpc, int* __restrict__ ipiv,
                                                   PanelStage<C, NB>* __restrict__ st,
                                                   GridBarrier* __restrict__ gb) {
  using R = decltype(C{}.x);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tile = reinterpret_cast<C*>(smem_raw);  // column-major rpc x nb
  C* prow = tile + (size_t)rpc * NB;          // pivot row, nb entries
  __shared__ R red_v[NT / 32];
  __shared__ int red_r[NT / 32];
  __shared__ int red_b[NT / 32];
  __shared__ unsigned int gen_local;

  const int tid = threadIdx.x;
  const int b = blockIdx.x;
  const int P = gridDim.x;
  const int base = j0 + b * rpc;
  const int cnt = max(0, min(rpc, n - base));
  if (tid == 0) gen_local = ld_acquire_u32(&gb->gen);

  for (int c = 0; c < nb; ++c)
    for (int r = tid; r < cnt; r += NT) tile[(size_t)c * rpc + r] = A[(size_t)(j0 + c) * lda + base + r];
  __syncthreads();

  for (int j = 0; j < nb; ++j) {
    const int gj = j0 + j;
    const int par = j & 1;
    // 1. local candidate: largest |re|+|im| in column j on rows >= gj, first on ties
    R best = R(-1);
    int brow = INT_MAX;
    for (int r = tid; r < cnt; r += NT) {
      const int g = base + r;
      if (g >= gj) {
        const R v = cabs1(tile[(size_t)j * rpc + r]);
        if (v > best || (v == best && g < brow)) {
          best = v;
          brow = g;
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const R ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int orow = __shfl_xor_sync(0xffffffffu, brow, o);
      if (ov > best || (ov == best && orow < brow)) {
        best = ov;
        brow = orow;
      }
    }
    if ((tid & 31) == 0) {
      red_v[tid >> 5] = best;
      red_r[tid >> 5] = brow;
    }
    __syncthreads();
    if (tid < 32) {
      best = tid < NT / 32 ? red_v[tid] : R(-1);
      brow = tid < NT / 32 ? red_r[tid] : INT_MAX;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const R ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int orow = __shfl_xor_sync(0xffffffffu, brow, o);
        if (ov > best || (ov == best && orow < brow)) {
          best = ov;
          brow = orow;
        }
      }
      if (tid == 0) {
        red_v[0] = best;
        red_r[0] = brow;
      }
    }
    __syncthreads();
    best = red_v[0];
    brow = red_r[0];
    // 2. publish the candidate row and, from its owner, the diagonal row
    if (tid == 0) {
      st->cand_val[par][b] = best;
      st->cand_row[par][b] = brow;
    }
    if (best >= R(0))
      for (int c = tid; c < nb; c += NT) st->cand_data[par][b][c] = tile[(size_t)c * rpc + (brow - base)];
    if (gj >= base && gj < base + cnt)
      for (int c = tid; c < nb; c += NT) st->diag_data[par][c] = tile[(size_t)c * rpc + (gj - base)];
    __syncthreads();  // red_* reuse below
    // 3. one grid-wide barrier per column
    if (!grid_barrier(gb, (unsigned)P, &gen_local)) return;
    // 4. winner over all blocks (deterministic: largest value, then smallest row)
    best = R(-1);
    brow = INT_MAX;
    int bblk = -1;
    for (int q = tid; q < P; q += NT) {
      const R v = *reinterpret_cast<volatile R*>(&st->cand_val[par][q]);
      const int rr = *reinterpret_cast<volatile int*>(&st->cand_row[par][q]);
      if (v > best || (v == best && rr < brow)) {
        best = v;
        brow = rr;
        bblk = q;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const R ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int orow = __shfl_xor_sync(0xffffffffu, brow, o);
      const int ob = __shfl_xor_sync(0xffffffffu, bblk, o);
      if (ov > best || (ov == best && orow < brow)) {
        best = ov;
        brow = orow;
        bblk = ob;
      }
    }
    if ((tid & 31) == 0) {
      red_v[tid >> 5] = best;
      red_r[tid >> 5] = brow;
      red_b[tid >> 5] = bblk;
    }
    __syncthreads();
    if (tid < 32) {
      best = tid < NT / 32 ? red_v[tid] : R(-1);
      brow = tid < NT / 32 ? red_r[tid] : INT_MAX;
      bblk = tid < NT / 32 ? red_b[tid] : -1;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const R ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int orow = __shfl_xor_sync(0xffffffffu, brow, o);
        const int ob = __shfl_xor_sync(0xffffffffu, bblk, o);
        if (ov > best || (ov == best && orow < brow)) {
          best = ov;
          brow = orow;
          bblk = ob;
        }
      }
      if (tid == 0) {
        red_v[0] = best;
        red_r[0] = brow;
        red_b[0] = bblk;
      }
    }
    __syncthreads();
    const int prw = red_r[0];
    const int pblk = red_b[0];
    if (b == 0 && tid == 0) ipiv[gj] = prw + 1;
    // 5. pivot row into shared memory; 6. interchange rows gj and prw
    for (int c = tid; c < nb; c += NT) {
      const C* src = &st->cand_data[par][pblk][c];
      C v;
      v.x = *reinterpret_cast<const volatile R*>(&src->x);
      v.y = *reinterpret_cast<const volatile R*>(&src->y);
      prow[c] = v;
    }
    __syncthreads();
    if (prw != gj) {
      if (prw >= base && prw < base + cnt)
        for (int c = tid; c < nb; c += NT) {
          const C* src = &st->diag_data[par][c];
          C v;
          v.x = *reinterpret_cast<const volatile R*>(&src->x);
          v.y = *reinterpret_cast<const volatile R*>(&src->y);
          tile[(size_t)c * rpc + (prw - base)] = v;
        }
      if (gj >= base && gj < base + cnt)
        for (int c = tid; c < nb; c += NT) tile[(size_t)c * rpc + (gj - base)] = prow[c];
    }
    __syncthreads();
    // 7. scale the column below the diagonal, then the rank-1 update of the panel
    const C piv = prow[j];
    const bool zero = piv.x == R(0) && piv.y == R(0);
    if (zero) {
      if (b == 0 && tid == 0) atomicCAS(&gb->info, 0, gj + 1);
    } else {
      const C inv = crecip(piv);
      for (int r = tid; r < cnt; r += NT)
        if (base + r > gj) tile[(size_t)j * rpc + r] = cmul(tile[(size_t)j * rpc + r], inv);
    }
    __syncthreads();
    const int ncol = nb - j - 1;
    if (ncol > 0 && cnt > 0) {
      const int total = cnt * ncol;
      for (int idx = tid; idx < total; idx += NT) {
        const int cc = idx / cnt;
        const int r = idx - cc * cnt;
        if (base + r > gj) {
          const int c = j + 1 + cc;
          tile[(size_t)c * rpc + r] = cfms(tile[(size_t)c * rpc + r], tile[(size_t)j * rpc + r], prow[c]);
        }
      }
    }
    __syncthreads();
  }
  for (int c = 0; c < nb; ++c)
    for (int r = tid; r < cnt; r += NT) A[(size_t)(j0 + c) * lda + base + r] = tile[(size_t)c * rpc + r];
}

// ------------------------------------------------------------- laswp ----
// Interchanges of pivots [k0, k0+kn) applied to the columns [0, j_skip0) and
// [j_skip1, ncols) of A: one thread per column, interchanges in order.
template <typename C>
__global__ void laswp_kernel(C* __restrict__ A, long long lda, int ncols, int j_skip0, int j_skip1,
                             int k0, int kn, const int* __restrict__ ipiv) {
  __shared__ int piv[256];
  for (int i = threadIdx.x; i < kn && i < 256; i += blockDim.x) piv[i] = ipiv[k0 + i] - 1;
  __syncthreads();
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int left = j_skip0;
  if (c >= left) c += (j_skip1 - j_skip0);
  if (c >= ncols) return;
  C* col = A + (size_t)c * lda;
  for (int i = 0; i < kn; ++i) {
    const int p = piv[i];
    if (p != k0 + i) {
      const C t = col[k0 + i];
      col[k0 + i] = col[p];
      col[p] = t;
    }
  }
}

// -------------------------------------------------------------- trsm ----
// B (nb x ncols, at column offset of a strided matrix) <- T^-1 B for a triangular
// nb x nb T held in the same kind of storage.  UPPER=false: unit lower (forward
// substitution); UPPER=true: non-unit upper (back substitution).  One CTA per
// TRSM_COLS columns; T and the B block are staged in shared memory.
constexpr int kTrsmCols = 16;

template <typename C, bool UPPER>
__global__ void __launch_bounds__(256) trsm_kernel(const C* __restrict__ T, long long ldt, C* __restrict__ B,
                                                   long long ldb, int nb, int ncols) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* Ts = reinterpret_cast<C*>(smem_raw);  // nb x nb, column-major
  C* Bs = Ts + (size_t)nb * nb;            // nb x kTrsmCols, column-major
  const int tid = threadIdx.x;
  const int c0 = blockIdx.x * kTrsmCols;
  const int nc = min(kTrsmCols, ncols - c0);
  for (int idx = tid; idx < nb * nb; idx += blockDim.x) {
    const int c = idx / nb, r = idx - c * nb;
    Ts[idx] = T[(size_t)c * ldt + r];
  }
  for (int idx = tid; idx < nb * nc; idx += blockDim.x) {
    const int c = idx / nb, r = idx - c * nb;
    Bs[idx] = B[(size_t)(c0 + c) * ldb + r];
  }
  __syncthreads();
  const int total = nb * nc;
  if (!UPPER) {
    for (int k = 0; k < nb - 1; ++k) {
      for (int idx = tid; idx < total; idx += blockDim.x) {
        const int c = idx / nb, r = idx - c * nb;
        if (r > k) Bs[c * nb + r] = cfms(Bs[c * nb + r], Ts[(size_t)k * nb + r], Bs[c * nb + k]);
      }
      __syncthreads();
    }
  } else {
    for (int k = nb - 1; k >= 0; --k) {
      for (int c = tid; c < nc; c += blockDim.x) Bs[c * nb + k] = cdiv(Bs[c * nb + k], Ts[(size_t)k * nb + k]);
      __syncthreads();
      for (int idx = tid; idx < total; idx += blockDim.x) {
        const int c = idx / nb, r = idx - c * nb;
        if (r < k) Bs[c * nb + r] = cfms(Bs[c * nb + r], Ts[(size_t)k * nb + r], Bs[c * nb + k]);
      }
      __syncthreads();
    }
  }
  for (int idx = tid; idx < total; idx += blockDim.x) {
    const int c = idx / nb, r = idx - c * nb;
    B[(size_t)(c0 + c) * ldb + r] = Bs[idx];
  }
}

// -------------------------------------------------------------- gemm ----
// Cm (M x N) -= Am (M x K) * Bm (K x N), complex, column-major strided operands.
// 64 x 64 output tile per CTA, 256 threads, 4 x 4 complex accumulators per thread
// in registers, K staged through shared memory 16 at a time.  SIMT FMA: for FP64
// this is bound by the FP64 pipe, which the FP64 tensor instructions of this GPU
// do not exceed.
constexpr int kGemmBM = 64, kGemmBN = 64, kGemmBK = 16;

template <typename C>
__global__ void __launch_bounds__(256) gemm_sub_kernel(const C* __restrict__ Am, long long lda,
                                                       const C* __restrict__ Bm, long long ldb,
                                                       C* __restrict__ Cm, long long ldc, int M, int N,
                                                       int K) {
  __shared__ C As[kGemmBK][kGemmBM + 1];
  __shared__ C Bs[kGemmBK][kGemmBN + 1];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.x * kGemmBM, n0 = blockIdx.y * kGemmBN;
  C acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = cmake<C>(0, 0);
  for (int k0 = 0; k0 < K; k0 += kGemmBK) {
    for (int idx = tid; idx < kGemmBK * kGemmBM; idx += 256) {
      const int kk = idx / kGemmBM, r = idx - kk * kGemmBM;
      const int gr = m0 + r, gk = k0 + kk;
      As[kk][r] = (gr < M && gk < K) ? Am[(size_t)gk * lda + gr] : cmake<C>(0, 0);
    }
    for (int idx = tid; idx < kGemmBK * kGemmBN; idx += 256) {
      const int c = idx / kGemmBK, kk = idx - c * kGemmBK;
      const int gc = n0 + c, gk = k0 + kk;
      Bs[kk][c] = (gc < N && gk < K) ? Bm[(size_t)gc * ldb + gk] : cmake<C>(0, 0);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kGemmBK; ++kk) {
      C a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          acc[i][j].x = fma(a[i].x, b[j].x, fma(-a[i].y, b[j].y, acc[i][j].x));
          acc[i][j].y = fma(a[i].x, b[j].y, fma(a[i].y, b[j].x, acc[i][j].y));
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int gc = n0 + ty + 16 * j;
    if (gc >= N) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int gr = m0 + tx + 16 * i;
      if (gr < M) {
        C* p = &Cm[(size_t)gc * ldc + gr];
        C v = *p;
        v.x -= acc[i][j].x;
        v.y -= acc[i][j].y;
        *p = v;
      }
    }
  }
}

// ------------------------------------------------------- permutation ----
// perm[i] = original row that ends up in row i after the interchanges ipiv[0..n).
__global__ void pivots_to_perm_kernel(const int* __restrict__ ipiv, int n, int* __restrict__ perm) {
  extern __shared__ int sp[];
  for (int i = threadIdx.x; i < n; i += blockDim.x) sp[i] = i;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < n; ++i) {
      const int p = ipiv[i] - 1;
      if (p != i && p >= 0 && p < n) {
        const int t = sp[i];
        sp[i] = sp[p];
        sp[p] = t;
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = sp[i];
}

template <typename C>
__global__ void gather_rows_kernel(const C* __restrict__ src, long long lds, C* __restrict__ dst,
                                   long long ldd, const int* __restrict__ perm, int n, int nrhs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i < n && c < nrhs) dst[(size_t)c * ldd + i] = src[(size_t)c * lds + perm[i]];
}

// ----------------------------------------------------------- host side ----
namespace {

template <typename C>
struct PanelCfg;
template <>
struct PanelCfg<double2> {
  static constexpr int NB = 64;
  static constexpr int NT = 256;
};
template <>
struct PanelCfg<float2> {
  static constexpr int NB = 64;
  static constexpr int NT = 256;
};

struct DeviceLimits {
  int sms = 0;
  int smem_optin = 0;
};

DeviceLimits device_limits() {
  static std::mutex mu;
  static std::vector<DeviceLimits> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  if ((int)cache.size() <= dev) cache.resize(dev + 1);
  if (cache[dev].sms == 0) {
    cudaDeviceGetAttribute(&cache[dev].sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&cache[dev].smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  }
  return cache[dev];
}

}  // namespace

size_t lu_workspace_bytes(int elem_bytes) {
  // barrier + stage for the larger (FP64) configuration
  (void)elem_bytes;
  return sizeof(GridBarrier) + 256 + sizeof(PanelStage<double2, 64>) + 256;
}

template <typename C>
cudaError_t lu_factor_t(C* A, long long lda, int n, int* ipiv, LuWorkspace* ws, cudaStream_t s,
                        GemmHook<C> gemm_hook) {
  constexpr int NB = PanelCfg<C>::NB;
  constexpr int NT = PanelCfg<C>::NT;
  using Stage = PanelStage<C, NB>;
  const DeviceLimits lim = device_limits();
  GridBarrier* gb = ws->barrier;
  Stage* st = reinterpret_cast<Stage*>(ws->stage);
  cudaError_t e;
  for (int j0 = 0; j0 < n; j0 += NB) {
    const int nb = std::min(NB, n - j0);
    const int m = n - j0;
    // panel: enough blocks that each holds a modest slice of rows
    int P = std::min({lim.sms, kMaxPanelBlocks, (m + 15) / 16});
    P = std::max(P, 1);
    int rpc = (m + P - 1) / P;
    size_t smem = (size_t)rpc * NB * sizeof(C) + NB * sizeof(C);
    while (smem > (size_t)lim.smem_optin - 4096 && P < std::min(lim.sms, kMaxPanelBlocks)) {
      ++P;
      rpc = (m + P - 1) / P;
      smem = (size_t)rpc * NB * sizeof(C) + NB * sizeof(C);
    }
    P = (m + rpc - 1) / rpc;
    auto kern = panel_kernel<C, NB, NT>;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem);
    if (e != cudaSuccess) return e;
    if (per_sm * lim.sms < P) return cudaErrorCooperativeLaunchTooLarge;
    C* Ap = A;
    long long ldap = lda;
    int np = n, j0p = j0, nbp = nb, rpcp = rpc;
    int* ipivp = ipiv;
    void* args[] = {&Ap, &ldap, &np, &j0p, &nbp, &rpcp, &ipivp, &st, &gb};
    {
      stats::Scope sc(stats::kPanel, s, 8.0 * m * (double)nb * nb / 2.0);
      e = cudaLaunchCooperativeKernel((const void*)kern, dim3(P), dim3(NT), args, smem, s);
    }
    if (e != cudaSuccess) return e;
    // interchanges on the other columns
    const int other = n - nb;
    if (other > 0) {
      stats::Scope sc(stats::kLaswp, s, 2.0 * nb * other * sizeof(C));
      laswp_kernel<C><<<(other + 127) / 128, 128, 0, s>>>(A, lda, n, j0, j0 + nb, j0, nb, ipiv);
      e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    const int rest = n - j0 - nb;
    if (rest > 0) {
      C* A11 = A + (size_t)j0 * lda + j0;
      C* A12 = A + (size_t)(j0 + nb) * lda + j0;
      C* A21 = A + (size_t)j0 * lda + j0 + nb;
      C* A22 = A + (size_t)(j0 + nb) * lda + j0 + nb;
      const size_t tsmem = ((size_t)nb * nb + (size_t)nb * kTrsmCols) * sizeof(C);
      e = cudaFuncSetAttribute(trsm_kernel<C, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)tsmem);
      if (e != cudaSuccess) return e;
      {
        stats::Scope sc(stats::kTrsm, s, 4.0 * nb * (double)nb * rest);
        trsm_kernel<C, false><<<(rest + kTrsmCols - 1) / kTrsmCols, 256, tsmem, s>>>(A11, lda, A12, lda, nb, rest);
      }
      e = cudaGetLastError();
      if (e != cudaSuccess) return e;
      if (gemm_hook) {
        e = gemm_hook(A21, lda, A12, lda, A22, lda, rest, rest, nb, s);
      } else {
        stats::Scope sc(stats::kGemm, s, 8.0 * rest * (double)rest * nb);
        dim3 grid((rest + kGemmBM - 1) / kGemmBM, (rest + kGemmBN - 1) / kGemmBN);
        gemm_sub_kernel<C><<<grid, 256, 0, s>>>(A21, lda, A12, lda, A22, lda, rest, rest, nb);
        e = cudaGetLastError();
      }
      if (e != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

template <typename C>
cudaError_t lu_solve_t(const C* A, long long lda, int n, const int* ipiv, C* B, long long ldb, int nrhs,
                       LuWorkspace* ws, cudaStream_t s) {
  constexpr int NB = PanelCfg<C>::NB;
  cudaError_t e;
  // row interchanges: B <- P B through a permutation gather into the scratch copy
  if ((size_t)n * sizeof(int) > 200 * 1024) return cudaErrorInvalidValue;
  e = cudaFuncSetAttribute(pivots_to_perm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(n * sizeof(int)));
  if (e != cudaSuccess) return e;
  stats::count(stats::kMisc, 2);
  pivots_to_perm_kernel<<<1, 256, n * sizeof(int), s>>>(ipiv, n, ws->perm);
  C* tmp = reinterpret_cast<C*>(ws->rhs);
  if ((size_t)n * nrhs * sizeof(C) > ws->rhs_bytes) return cudaErrorInvalidValue;
  e = cudaMemcpy2DAsync(tmp, (size_t)n * sizeof(C), B, (size_t)ldb * sizeof(C), (size_t)n * sizeof(C), nrhs,
                        cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return e;
  gather_rows_kernel<C><<<dim3((n + 255) / 256, nrhs), 256, 0, s>>>(tmp, n, B, ldb, ws->perm, n, nrhs);
  const size_t tsmem = ((size_t)NB * NB + (size_t)NB * kTrsmCols) * sizeof(C);
  e = cudaFuncSetAttribute(trsm_kernel<C, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsmem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(trsm_kernel<C, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsmem);
  if (e != cudaSuccess) return e;
  // forward: L unit lower
  const int nblocks = (n + NB - 1) / NB;
  stats::Scope sc(stats::kTrsm, s, 8.0 * n * (double)n * nrhs, 4 * nblocks - 2);
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int kb = std::min(NB, n - k0);
    const size_t sm = ((size_t)kb * kb + (size_t)kb * kTrsmCols) * sizeof(C);
    trsm_kernel<C, false><<<(nrhs + kTrsmCols - 1) / kTrsmCols, 256, sm, s>>>(
        A + (size_t)k0 * lda + k0, lda, B + k0, ldb, kb, nrhs);
    const int below = n - k0 - kb;
    if (below > 0) {
      dim3 grid((below + kGemmBM - 1) / kGemmBM, (nrhs + kGemmBN - 1) / kGemmBN);
      gemm_sub_kernel<C><<<grid, 256, 0, s>>>(A + (size_t)k0 * lda + k0 + kb, lda, B + k0, ldb, B + k0 + kb,
                                              ldb, below, nrhs, kb);
    }
  }
  // backward: U non-unit upper
  const int nblk = (n + NB - 1) / NB;
  for (int bi = nblk - 1; bi >= 0; --bi) {
    const int k0 = bi * NB;
    const int kb = std::min(NB, n - k0);
    const size_t sm = ((size_t)kb * kb + (size_t)kb * kTrsmCols) * sizeof(C);
    trsm_kernel<C, true><<<(nrhs + kTrsmCols - 1) / kTrsmCols, 256, sm, s>>>(
        A + (size_t)k0 * lda + k0, lda, B + k0, ldb, kb, nrhs);
    if (k0 > 0) {
      dim3 grid((k0 + kGemmBM - 1) / kGemmBM, (nrhs + kGemmBN - 1) / kGemmBN);
      gemm_sub_kernel<C><<<grid, 256, 0, s>>>(A + (size_t)k0 * lda, lda, B + k0, ldb, B, ldb, k0, nrhs, kb);
    }
  }
  return cudaGetLastError();
}

template cudaError_t lu_factor_t<double2>(double2*, long long, int, int*, LuWorkspace*, cudaStream_t,
                                          GemmHook<double2>);
template cudaError_t lu_factor_t<float2>(float2*, long long, int, int*, LuWorkspace*, cudaStream_t,
                                         GemmHook<float2>);
template cudaError_t lu_solve_t<double2>(const double2*, long long, int, const int*, double2*, long long, int,
                                         LuWorkspace*, cudaStream_t);
template cudaError_t lu_solve_t<float2>(const float2*, long long, int, const int*, float2*, long long, int,
                                        LuWorkspace*, cudaStream_t);

}  // namespace wmom
