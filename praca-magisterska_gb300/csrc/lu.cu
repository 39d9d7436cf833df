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
#include <atomic>
#include <climits>
#include <cstddef>
#include <cstdlib>
#include <cstdint>
#include <map>
#include <tuple>
#include <mutex>
#include <type_traits>
#include <vector>

#include "lu_common.cuh"
#include "lu_internal.h"
#include "stats.h"
#include "wmom_internal.h"

namespace wmom {

// Test hook (wmom_debug_panel_missing_arrivals): extra arrivals every cooperative
// panel's grid barrier waits for and never gets, so that its bounded wait runs out.
std::atomic<unsigned int> g_panel_missing_arrivals{0};

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
                                                   GridBarrier* __restrict__ gb, unsigned int bar_base,
                                                   long long astride) {
  using R = decltype(C{}.x);
  // FP32 panels gather every block's candidate into shared memory after the barrier
  // (one parallel round trip); FP64 panels read the winner's row only
  constexpr bool kGather = sizeof(R) == 4;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tile = reinterpret_cast<C*>(smem_raw);  // column-major rpc x nb
  C* prow = tile + (size_t)rpc * NB;          // pivot row, nb entries
  C* cdat = prow + NB;                        // gather: candidate rows, P x NB
  C* dgr = cdat + (kGather ? (size_t)gridDim.x * NB : 0);  // gather: diagonal row
  R* cval = reinterpret_cast<R*>(dgr + NB);                // gather: candidate values
  int* crow = reinterpret_cast<int*>(cval + (kGather ? gridDim.x : 0));
  __shared__ R red_v[NT / 32];
  __shared__ int red_r[NT / 32];
  __shared__ int red_b[NT / 32];

  // batch: blockIdx.y selects the matrix, its pivots, staging and barrier
  A += (size_t)blockIdx.y * astride;
  ipiv += (size_t)blockIdx.y * n;
  st += blockIdx.y;
  gb += blockIdx.y;
  const int tid = threadIdx.x;
  const int b = blockIdx.x;
  const int P = gridDim.x;
  const int base = j0 + b * rpc;
  const int cnt = max(0, min(rpc, n - base));

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
    if (!grid_barrier_count(gb, bar_base + (unsigned)P * (unsigned)(j + 1))) return;
    // 4. winner over all blocks (deterministic: largest value, then smallest row)
    if constexpr (kGather) {
      for (int q = tid; q < P; q += NT) {
        cval[q] = __ldcg(&st->cand_val[par][q]);
        crow[q] = __ldcg(&st->cand_row[par][q]);
      }
      for (int c = tid; c < nb; c += NT) dgr[c] = __ldcg(&st->diag_data[par][c]);
      // the P candidate rows are one contiguous P x NB block of the staging area;
      // kGatherILP independent loads per thread are in flight before any is stored
      // (entries c >= nb of a narrow last panel are copied but never used)
      {
        constexpr int kGatherILP = 8;
        const C* src = &st->cand_data[par][0][0];
        const int tot = P * NB;
        for (int i0 = tid; i0 < tot; i0 += NT * kGatherILP) {
          C v[kGatherILP];
#pragma unroll
          for (int u = 0; u < kGatherILP; ++u)
            if (i0 + u * NT < tot) v[u] = __ldcg(src + i0 + u * NT);
#pragma unroll
          for (int u = 0; u < kGatherILP; ++u)
            if (i0 + u * NT < tot) cdat[i0 + u * NT] = v[u];
        }
      }
      __syncthreads();
      if (tid < 32) {
        best = R(-1);
        brow = INT_MAX;
        int bblk = -1;
        for (int q = tid; q < P; q += 32) {
          if (cval[q] > best || (cval[q] == best && crow[q] < brow)) {
            best = cval[q];
            brow = crow[q];
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
        if (tid == 0) {
          red_r[0] = brow;
          red_b[0] = bblk;
        }
      }
      __syncthreads();
    }
    if constexpr (!kGather) {
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
    }  // FP64 candidate scan
    const int prw = red_r[0];
    const int pblk = red_b[0];
    if (b == 0 && tid == 0) ipiv[gj] = prw + 1;
    // 5. pivot row into shared memory; 6. interchange rows gj and prw
    for (int c = tid; c < nb; c += NT) {
      if constexpr (kGather) {
        prow[c] = cdat[(size_t)pblk * NB + c];
      } else {
        const C* src = &st->cand_data[par][pblk][c];
        C v;
        v.x = *reinterpret_cast<const volatile R*>(&src->x);
        v.y = *reinterpret_cast<const volatile R*>(&src->y);
        prow[c] = v;
      }
    }
    __syncthreads();
    if (prw != gj) {
      if (prw >= base && prw < base + cnt)
        for (int c = tid; c < nb; c += NT) {
          if constexpr (kGather) {
            tile[(size_t)c * rpc + (prw - base)] = dgr[c];
          } else {
            const C* src = &st->diag_data[par][c];
            C v;
            v.x = *reinterpret_cast<const volatile R*>(&src->x);
            v.y = *reinterpret_cast<const volatile R*>(&src->y);
            tile[(size_t)c * rpc + (prw - base)] = v;
          }
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

// Row-owner panel (FP32 precision form).  Each thread owns one row of the block's
// slab (rpc <= NT) for the whole column loop: it finds its own candidate, swaps,
// scales and updates its own row, so a column needs only two block barriers (the
// pivot reduction and the candidate gather) besides the grid-wide one.  Same
// pivot rule and order of operations per row as panel_kernel.
template <typename C, int NB, int NT>
__global__ void __launch_bounds__(NT) panel_rows_kernel(C* __restrict__ A, long long lda, int n, int j0, int nb,
                                                        int rpc, int* __restrict__ ipiv,
                                                        PanelStage<C, NB>* __restrict__ st,
                                                        GridBarrier* __restrict__ gb, unsigned int bar_base,
                                                        long long astride) {
  using R = decltype(C{}.x);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tile = reinterpret_cast<C*>(smem_raw);          // column-major rpc x NB
  C* cdat = tile + (size_t)rpc * NB;                  // candidate rows, P x NB
  C* dgr = cdat + (size_t)gridDim.x * NB;             // diagonal row, NB
  R* cval = reinterpret_cast<R*>(dgr + NB);           // candidate values, P
  int* crow = reinterpret_cast<int*>(cval + gridDim.x);  // candidate rows, P
  __shared__ R red_v[2][NT / 32];
  __shared__ int red_r[2][NT / 32];

  A += (size_t)blockIdx.y * astride;
  ipiv += (size_t)blockIdx.y * n;
  st += blockIdx.y;
  gb += blockIdx.y;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int b = blockIdx.x;
  const int P = gridDim.x;
  const int base = j0 + b * rpc;
  const int cnt = max(0, min(rpc, n - base));
  const bool own = t < cnt;  // this thread's row: base + t
  const int gr = base + t;

  if (own) {
    // the row, 16 loads in flight at a time
    for (int c0 = 0; c0 < nb; c0 += 16) {
      C v[16];
#pragma unroll
      for (int u = 0; u < 16; ++u)
        if (c0 + u < nb) v[u] = A[(size_t)(j0 + c0 + u) * lda + gr];
#pragma unroll
      for (int u = 0; u < 16; ++u)
        if (c0 + u < nb) tile[(size_t)(c0 + u) * rpc + t] = v[u];
    }
  }
  __syncthreads();

  for (int j = 0; j < nb; ++j) {
    const int gj = j0 + j;
    const int par = j & 1;
    // 1. candidate: largest |re|+|im| in column j on rows >= gj, first row on ties
    R best = R(-1);
    int brow = INT_MAX;
    if (own && gr >= gj) {
      best = cabs1(tile[(size_t)j * rpc + t]);
      brow = gr;
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
    if (lane == 0) {
      red_v[par][warp] = best;
      red_r[par][warp] = brow;
    }
    __syncthreads();
    // every thread reduces the per-warp results itself (no second barrier)
    best = R(-1);
    brow = INT_MAX;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) {
      const R v = red_v[par][w];
      const int r = red_r[par][w];
      if (v > best || (v == best && r < brow)) {
        best = v;
        brow = r;
      }
    }
    // 2. publish the candidate and, from its owner, the diagonal row
    if (t == 0) {
      st->cand_val[par][b] = best;
      st->cand_row[par][b] = brow;
    }
    if (t < nb) {
      if (best >= R(0)) st->cand_data[par][b][t] = tile[(size_t)t * rpc + (brow - base)];
      if (gj >= base && gj < base + cnt) st->diag_data[par][t] = tile[(size_t)t * rpc + (gj - base)];
    }
    // 3. one grid-wide barrier per column
    if (!grid_barrier_count(gb, bar_base + (unsigned)P * (unsigned)(j + 1))) return;
    // 4. gather every block's candidate (one round trip, kILP loads in flight)
    for (int q = t; q < P; q += NT) {
      cval[q] = __ldcg(&st->cand_val[par][q]);
      crow[q] = __ldcg(&st->cand_row[par][q]);
    }
    if (t < nb) dgr[t] = __ldcg(&st->diag_data[par][t]);
    {
      constexpr int kILP = 8;
      const C* src = &st->cand_data[par][0][0];
      const int tot = P * NB;
      for (int i0 = t; i0 < tot; i0 += NT * kILP) {
        C v[kILP];
#pragma unroll
        for (int u = 0; u < kILP; ++u)
          if (i0 + u * NT < tot) v[u] = __ldcg(src + i0 + u * NT);
#pragma unroll
        for (int u = 0; u < kILP; ++u)
          if (i0 + u * NT < tot) cdat[i0 + u * NT] = v[u];
      }
    }
    __syncthreads();
    // winner over all blocks, computed by every warp (deterministic: largest value,
    // then smallest row)
    best = R(-1);
    brow = INT_MAX;
    int bblk = -1;
    for (int q = lane; q < P; q += 32) {
      if (cval[q] > best || (cval[q] == best && crow[q] < brow)) {
        best = cval[q];
        brow = crow[q];
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
    const int prw = brow;
    const C* prow = cdat + (size_t)bblk * NB;  // the pivot row
    if (b == 0 && t == 0) ipiv[gj] = prw + 1;
    const C piv = prow[j];
    const bool zero = piv.x == R(0) && piv.y == R(0);
    if (zero && b == 0 && t == 0) atomicCAS(&gb->info, 0, gj + 1);
    // 5. this thread's row: interchange, then scale and rank-1 update below gj
    if (own) {
      if (prw != gj) {
        if (gr == prw)
          for (int c = 0; c < nb; ++c) tile[(size_t)c * rpc + t] = dgr[c];
        else if (gr == gj)
          for (int c = 0; c < nb; ++c) tile[(size_t)c * rpc + t] = prow[c];
      }
      if (gr > gj) {
        C l = tile[(size_t)j * rpc + t];
        if (!zero) {
          l = cmul(l, crecip(piv));
          tile[(size_t)j * rpc + t] = l;
        }
        for (int c = j + 1; c < nb; ++c) tile[(size_t)c * rpc + t] = cfms(tile[(size_t)c * rpc + t], l, prow[c]);
      }
    }
  }
  __syncthreads();
  if (own)
    for (int c = 0; c < nb; ++c) A[(size_t)(j0 + c) * lda + gr] = tile[(size_t)c * rpc + t];
}

// Cluster panel (FP32 precision form).  One thread-block cluster of CS CTAs per
// matrix holds the panel (m rows x w columns) in the CTAs' shared memory, one row per
// thread.  Per column: each CTA reduces its candidate, publishes it (value, row and
// the candidate row) in its own shared memory, and the cluster meets at the hardware
// cluster barrier; every CTA then reads the CS candidates and the winning row through
// distributed shared memory.  No global memory and no software barrier on the
// column path, and clusters do not depend on one another.  Same pivot rule and order
// of operations per row as panel_kernel / panel_rows_kernel.
constexpr int kClusterMax = 16;
constexpr int kClusterThreads = 512;

template <typename C>
struct ClusterPub {
  using R = decltype(C{}.x);
  R val;
  int row;
  int pad[sizeof(R) == 8 ? 1 : 2];  // cand starts 16-byte aligned
  C cand[64];
  C diag[64];
};

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t map_rank(const void* p, unsigned rank) {
  uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(p)), r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ float ld_cluster_f32(uint32_t a) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ int ld_cluster_s32(uint32_t a) {
  int v;
  asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ float2 ld_cluster_f2(uint32_t a) {
  float2 v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ double ld_cluster_f64(uint32_t a) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ double2 ld_cluster_d2(uint32_t a) {
  double2 v;
  asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ float ld_cluster_r(const float*, uint32_t a) { return ld_cluster_f32(a); }
__device__ __forceinline__ double ld_cluster_r(const double*, uint32_t a) { return ld_cluster_f64(a); }
__device__ __forceinline__ float2 ld_cluster_c(const float2*, uint32_t a) { return ld_cluster_f2(a); }
__device__ __forceinline__ double2 ld_cluster_c(const double2*, uint32_t a) { return ld_cluster_d2(a); }

// RPT rows per thread (1, or 2 for panels whose rows would otherwise need a cluster
// wider than the GPU can hold for a whole batch at once): thread t owns rows t and
// t + kClusterThreads of its CTA's slab.  C = float2 (precision form) or double2
// (plain form and the precision form's FP64-grade tiers).
template <typename C, int RPT>
__global__ void __launch_bounds__(kClusterThreads, 1) panel_cluster_kernel(C* __restrict__ A, long long lda, int n,
                                                                           int j0, int w, int rpc,
                                                                           int* __restrict__ ipiv,
                                                                           GridBarrier* __restrict__ gb,
                                                                           long long astride) {
  using R = decltype(C{}.x);
  using Pub = ClusterPub<C>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Pub* pub = reinterpret_cast<Pub*>(smem_raw);  // [2]
  C* prow = reinterpret_cast<C*>(pub + 2);      // winner row, 64
  C* dgr = prow + 64;                           // diagonal row, 64
  C* tile = dgr + 64;                           // column-major rpc x w
  __shared__ R red_v[2][kClusterThreads / 32];
  __shared__ int red_r[2][kClusterThreads / 32];
  __shared__ C s_inv;  // 1 / pivot of the current column, computed once per CTA

  A += (size_t)blockIdx.y * astride;
  ipiv += (size_t)blockIdx.y * n;
  gb += blockIdx.y;
  const unsigned cs = gridDim.x;  // the cluster spans blockIdx.x
  const unsigned rank = cluster_rank();
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int base = j0 + (int)rank * rpc;
  const int cnt = max(0, min(rpc, n - base));

#pragma unroll
  for (int rr = 0; rr < RPT; ++rr) {
    const int lr = t + rr * kClusterThreads;  // local row
    if (lr < cnt) {
      const int gr = base + lr;
      for (int c0 = 0; c0 < w; c0 += 16) {
        C v[16];
#pragma unroll
        for (int u = 0; u < 16; ++u)
          if (c0 + u < w) v[u] = A[(size_t)(j0 + c0 + u) * lda + gr];
#pragma unroll
        for (int u = 0; u < 16; ++u)
          if (c0 + u < w) tile[(size_t)(c0 + u) * rpc + lr] = v[u];
      }
    }
  }
  __syncthreads();

  for (int j = 0; j < w; ++j) {
    const int gj = j0 + j;
    const int par = j & 1;
    // 1. this CTA's candidate (the thread's rows in increasing order: first on ties)
    R best = R(-1);
    int brow = INT_MAX;
#pragma unroll
    for (int rr = 0; rr < RPT; ++rr) {
      const int lr = t + rr * kClusterThreads;
      if (lr < cnt && base + lr >= gj) {
        const R v = cabs1(tile[(size_t)j * rpc + lr]);
        if (v > best) {
          best = v;
          brow = base + lr;
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
    if (lane == 0) {
      red_v[par][warp] = best;
      red_r[par][warp] = brow;
    }
    __syncthreads();
    best = R(-1);
    brow = INT_MAX;
#pragma unroll
    for (int q = 0; q < kClusterThreads / 32; ++q) {
      const R v = red_v[par][q];
      const int r = red_r[par][q];
      if (v > best || (v == best && r < brow)) {
        best = v;
        brow = r;
      }
    }
    // 2. publish it in this CTA's shared memory
    Pub& my = pub[par];
    if (t == 0) {
      my.val = best;
      my.row = brow;
    }
    if (t < w) {
      if (best >= R(0)) my.cand[t] = tile[(size_t)t * rpc + (brow - base)];
      if (gj >= base && gj < base + cnt) my.diag[t] = tile[(size_t)t * rpc + (gj - base)];
    }
    // 3. the cluster meets (also orders this CTA's own threads)
    cluster_sync_all();
    // 4. winner over the cluster, computed by every warp from the CTAs' shared memory
    R v = R(-1);
    int r = INT_MAX, q = -1;
    if (lane < (int)cs) {
      v = ld_cluster_r(&pub[par].val, map_rank(&pub[par].val, lane));
      r = ld_cluster_s32(map_rank(&pub[par].row, lane));
      q = lane;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const R ov = __shfl_xor_sync(0xffffffffu, v, o);
      const int orow = __shfl_xor_sync(0xffffffffu, r, o);
      const int oq = __shfl_xor_sync(0xffffffffu, q, o);
      if (ov > v || (ov == v && orow < r)) {
        v = ov;
        r = orow;
        q = oq;
      }
    }
    const int prw = r;
    const unsigned owner_gj = (unsigned)((gj - j0) / rpc);  // the CTA holding row gj
    if (t < w) {
      const C pv = ld_cluster_c(prow, map_rank(&pub[par].cand[t], (unsigned)q));
      prow[t] = pv;
      if (t == j) s_inv = (pv.x == R(0) && pv.y == R(0)) ? pv : crecip(pv);
      if (prw != gj) dgr[t] = ld_cluster_c(prow, map_rank(&pub[par].diag[t], owner_gj));
    }
    __syncthreads();
    if (rank == 0 && t == 0) ipiv[gj] = prw + 1;
    const C piv = prow[j];
    const bool zero = piv.x == R(0) && piv.y == R(0);
    if (zero && rank == 0 && t == 0) atomicCAS(&gb->info, 0, gj + 1);
    // 5. this thread's rows: interchange, then scale and rank-1 update below gj
#pragma unroll
    for (int rr = 0; rr < RPT; ++rr) {
      const int lr = t + rr * kClusterThreads;
      if (lr >= cnt) continue;
      const int gr = base + lr;
      if (prw != gj) {
        if (gr == prw)
          for (int c = 0; c < w; ++c) tile[(size_t)c * rpc + lr] = dgr[c];
        else if (gr == gj)
          for (int c = 0; c < w; ++c) tile[(size_t)c * rpc + lr] = prow[c];
      }
      if (gr > gj) {
        C l = tile[(size_t)j * rpc + lr];
        if (!zero) {
          l = cmul(l, s_inv);
          tile[(size_t)j * rpc + lr] = l;
        }
        for (int c = j + 1; c < w; ++c) tile[(size_t)c * rpc + lr] = cfms(tile[(size_t)c * rpc + lr], l, prow[c]);
      }
    }
  }
  // no CTA leaves while another may still read its shared memory
  cluster_sync_all();
#pragma unroll
  for (int rr = 0; rr < RPT; ++rr) {
    const int lr = t + rr * kClusterThreads;
    if (lr < cnt)
      for (int c = 0; c < w; ++c) A[(size_t)(j0 + c) * lda + base + lr] = tile[(size_t)c * rpc + lr];
  }
}

// Order keys of non-negative floating-point values (and of -1, below them all):
// the IEEE bits as a signed integer order like the values.
__device__ __forceinline__ long long order_key(float v) { return (long long)__float_as_int(v); }
__device__ __forceinline__ long long order_key(double v) { return __double_as_longlong(v); }
template <typename R>
__device__ __forceinline__ R key_value(long long k);
template <>
__device__ __forceinline__ float key_value<float>(long long k) {
  return __int_as_float((int)k);
}
template <>
__device__ __forceinline__ double key_value<double>(long long k) {
  return __longlong_as_double(k);
}

// The same panel with a one-column look-ahead.  After the pivot of column j is
// known, each thread updates column j + 1 of its rows first; the CTA then finds and
// publishes its candidate for column j + 1 and arrives at the cluster barrier, and
// only then updates the rest of its rows (columns j + 2 ..) while the barrier
// completes.  The published candidate row and diagonal row therefore lag one update
// behind in their columns j + 2 ..; each CTA that reads them applies that update
// itself (c - l * p, with the row's own multiplier l and the previous pivot row p,
// the same cfms the owner applies), so the factors are bit-identical to
// panel_cluster_kernel's.
template <typename C, int RPT>
__global__ void __launch_bounds__(kClusterThreads, 1) panel_cluster_la_kernel(C* __restrict__ A, long long lda,
                                                                              int n, int j0, int w, int rpc,
                                                                              int* __restrict__ ipiv,
                                                                              GridBarrier* __restrict__ gb,
                                                                              long long astride) {
  using R = decltype(C{}.x);
  using Pub = ClusterPub<C>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Pub* pub = reinterpret_cast<Pub*>(smem_raw);  // [2]
  C* prw_buf = reinterpret_cast<C*>(pub + 2);   // pivot rows of columns j - 1 and j, 2 x 64
  C* dgr = prw_buf + 128;                       // diagonal row, 64
  C* tile = dgr + 64;                           // column-major rpc x w
  // candidates are compared through order keys: for the values compared here
  // (|re| + |im| >= 0, and -1 for no candidate) the IEEE bits as a signed integer
  // order like the values, so the pivot search runs on the integer pipe instead of
  // GB300's narrow FP64 pipe; the pivot chosen is the same
  __shared__ long long red_k[2][kClusterThreads / 32];
  __shared__ int red_r[2][kClusterThreads / 32];
  __shared__ C s_inv;  // 1 / pivot of the current column, computed once per CTA
  __shared__ int s_prw;  // pivot row of the current column

  A += (size_t)blockIdx.y * astride;
  ipiv += (size_t)blockIdx.y * n;
  gb += blockIdx.y;
  const unsigned cs = gridDim.x;  // the cluster spans blockIdx.x
  const unsigned rank = cluster_rank();
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int base = j0 + (int)rank * rpc;
  const int cnt = max(0, min(rpc, n - base));

#pragma unroll
  for (int rr = 0; rr < RPT; ++rr) {
    const int lr = t + rr * kClusterThreads;  // local row
    if (lr < cnt) {
      const int gr = base + lr;
      for (int c0 = 0; c0 < w; c0 += 16) {
        C v[16];
#pragma unroll
        for (int u = 0; u < 16; ++u)
          if (c0 + u < w) v[u] = A[(size_t)(j0 + c0 + u) * lda + gr];
#pragma unroll
        for (int u = 0; u < 16; ++u)
          if (c0 + u < w) tile[(size_t)(c0 + u) * rpc + lr] = v[u];
      }
    }
  }
  __syncthreads();

  // this CTA's candidate for column jc among its rows >= j0 + jc (first on ties),
  // published with the candidate row and, from its owner, row j0 + jc
  auto publish = [&](int jc) {
    const int gjc = j0 + jc;
    const int pc = jc & 1;
    long long best = order_key(R(-1));
    int brow = INT_MAX;
#pragma unroll
    for (int rr = 0; rr < RPT; ++rr) {
      const int lr = t + rr * kClusterThreads;
      if (lr < cnt && base + lr >= gjc) {
        const long long v = order_key(cabs1(tile[(size_t)jc * rpc + lr]));
        if (v > best) {
          best = v;
          brow = base + lr;
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int orow = __shfl_xor_sync(0xffffffffu, brow, o);
      if (ov > best || (ov == best && orow < brow)) {
        best = ov;
        brow = orow;
      }
    }
    if (lane == 0) {
      red_k[pc][warp] = best;
      red_r[pc][warp] = brow;
    }
    __syncthreads();
    if (t < w) {  // only these threads publish
      best = order_key(R(-1));
      brow = INT_MAX;
#pragma unroll
      for (int q = 0; q < kClusterThreads / 32; ++q) {
        const long long v = red_k[pc][q];
        const int r = red_r[pc][q];
        if (v > best || (v == best && r < brow)) {
          best = v;
          brow = r;
        }
      }
      Pub& my = pub[pc];
      if (t == 0) {
        my.val = key_value<R>(best);
        my.row = brow;
      }
      if (best >= 0) my.cand[t] = tile[(size_t)t * rpc + (brow - base)];
      if (gjc >= base && gjc < base + cnt) my.diag[t] = tile[(size_t)t * rpc + (gjc - base)];
    }
    // every read of the tile for the publication is done before the rows change
    __syncthreads();
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
  };

  publish(0);
  C lr_l[RPT];  // the rows' multipliers of the current column
  for (int j = 0; j < w; ++j) {
    const int gj = j0 + j;
    const int par = j & 1;
    C* prow = prw_buf + 64 * par;               // pivot row of column j
    const C* pprev = prw_buf + 64 * (par ^ 1);  // pivot row of column j - 1
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    // winner over the cluster, from the CTAs' shared memory, by the warps that
    // fetch the pivot and diagonal rows (the others learn the pivot row below)
    const unsigned owner_gj = (unsigned)((gj - j0) / rpc);  // the CTA holding row gj
    int r = INT_MAX, q = -1;
    if (warp * 32 < w) {
      long long v = order_key(R(-1));
      if (lane < (int)cs) {
        v = order_key(ld_cluster_r(&pub[par].val, map_rank(&pub[par].val, lane)));
        r = ld_cluster_s32(map_rank(&pub[par].row, lane));
        q = lane;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const long long ov = __shfl_xor_sync(0xffffffffu, v, o);
        const int orow = __shfl_xor_sync(0xffffffffu, r, o);
        const int oq = __shfl_xor_sync(0xffffffffu, q, o);
        if (ov > v || (ov == v && orow < r)) {
          v = ov;
          r = orow;
          q = oq;
        }
      }
      if (t == 0) s_prw = r;
    }
    if (t < w) {
      const int prw = r;
      // the published rows lag the update of column j - 1 in their columns > j
      C pv = ld_cluster_c(prow, map_rank(&pub[par].cand[t], (unsigned)q));
      if (j > 0 && t > j) pv = cfms(pv, ld_cluster_c(prow, map_rank(&pub[par].cand[j - 1], (unsigned)q)), pprev[t]);
      prow[t] = pv;
      // the pivot's reciprocal once for the CTA (Smith's formula divides: costly in FP64)
      if (t == j) s_inv = (pv.x == R(0) && pv.y == R(0)) ? pv : crecip(pv);
      if (prw != gj) {
        C dv = ld_cluster_c(prow, map_rank(&pub[par].diag[t], owner_gj));
        if (j > 0 && t > j) dv = cfms(dv, ld_cluster_c(prow, map_rank(&pub[par].diag[j - 1], owner_gj)), pprev[t]);
        dgr[t] = dv;
      }
    }
    __syncthreads();
    const int prw = s_prw;
    if (rank == 0 && t == 0) ipiv[gj] = prw + 1;
    const C piv = prow[j];
    const bool zero = piv.x == R(0) && piv.y == R(0);
    if (zero && rank == 0 && t == 0) atomicCAS(&gb->info, 0, gj + 1);
    // this thread's rows: interchange, scale, then column j + 1 only
#pragma unroll
    for (int rr = 0; rr < RPT; ++rr) {
      const int lr = t + rr * kClusterThreads;
      lr_l[rr] = cmake<C>(0, 0);
      if (lr >= cnt) continue;
      const int gr = base + lr;
      if (prw != gj) {
        if (gr == prw)
          for (int c = 0; c < w; ++c) tile[(size_t)c * rpc + lr] = dgr[c];
        else if (gr == gj)
          for (int c = 0; c < w; ++c) tile[(size_t)c * rpc + lr] = prow[c];
      }
      if (gr > gj) {
        C l = tile[(size_t)j * rpc + lr];
        if (!zero) {
          l = cmul(l, s_inv);
          tile[(size_t)j * rpc + lr] = l;
        }
        lr_l[rr] = l;
        if (j + 1 < w) tile[(size_t)(j + 1) * rpc + lr] = cfms(tile[(size_t)(j + 1) * rpc + lr], l, prow[j + 1]);
      }
    }
    if (j + 1 < w) {
      __syncthreads();  // column j + 1 of every row is current
      publish(j + 1);
      // the rest of this thread's rows while the cluster meets
#pragma unroll
      for (int rr = 0; rr < RPT; ++rr) {
        const int lr = t + rr * kClusterThreads;
        if (lr >= cnt || base + lr <= gj) continue;
        const C l = lr_l[rr];
        for (int c = j + 2; c < w; ++c) tile[(size_t)c * rpc + lr] = cfms(tile[(size_t)c * rpc + lr], l, prow[c]);
      }
    }
  }
  // no CTA leaves while another may still read its shared memory
  cluster_sync_all();
#pragma unroll
  for (int rr = 0; rr < RPT; ++rr) {
    const int lr = t + rr * kClusterThreads;
    if (lr < cnt)
      for (int c = 0; c < w; ++c) A[(size_t)(j0 + c) * lda + base + lr] = tile[(size_t)c * rpc + lr];
  }
}

// ------------------------------------------------------------- laswp ----
// Interchanges of pivots [k0, k0+kn) applied to the columns [0, j_skip0) and
// [j_skip1, ncols) of A: one thread per column, interchanges in order.
template <typename C>
__global__ void laswp_kernel(C* __restrict__ A, long long lda, int ncols, int j_skip0, int j_skip1,
                             int k0, int kn, const int* __restrict__ ipiv, long long astride, int n) {
  __shared__ int piv[256];
  A += (size_t)blockIdx.y * astride;
  ipiv += (size_t)blockIdx.y * n;
  for (int i = threadIdx.x; i < kn && i < 256; i += blockDim.x) piv[i] = ipiv[k0 + i] - 1;
  __syncthreads();
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int left = j_skip0;
  if (c >= left) c += (j_skip1 - j_skip0);
  if (c >= ncols) return;
  C* col = A + (size_t)c * lda;
  for (int i = 0; i < kn; ++i) {
    const int p = piv[i];
    // a pivot outside the matrix is left alone: after a panel gave up on a timed-out
    // wait its later pivots were never written and hold what the buffer held
    if (p != k0 + i && p >= 0 && p < n) {
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
                                                   long long ldb, int nb, int ncols, long long tstride,
                                                   long long bstride) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T += (size_t)blockIdx.y * tstride;
  B += (size_t)blockIdx.y * bstride;
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

// FP64 unit-lower TRSM of the second tier's narrow panels, B <- L^-1 B for an NB x NB
// unit lower L (NB = 8, 16, 24, 32: the FP64 cluster panels' widths), one thread per
// column of B holding the whole column in registers, one warp per block.  Every
// element receives its updates in increasing k, as in trsm_kernel, so the results are
// identical; but no barrier separates the rows, and no padded row costs FP64 work.
// The FP64 pipe bounds it (4 NB (NB - 1) / 2 FP64 FMAs per column).  trsm_kernel, with
// a barrier per row of the triangle, ran at about a third of that rate.
template <typename C, int NB>
__global__ void __launch_bounds__(32) trsm_lower_reg_kernel(const C* __restrict__ T, long long ldt,
                                                            C* __restrict__ B, long long ldb, int ncols,
                                                            long long tstride, long long bstride) {
  __shared__ C Ls[NB * NB];  // column-major, strictly lower part (the rest zero, never read)
  T += (size_t)blockIdx.y * tstride;
  B += (size_t)blockIdx.y * bstride;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < NB * NB; idx += 32) {
    const int k = idx / NB, r = idx - k * NB;
    Ls[idx] = r > k ? T[(size_t)k * ldt + r] : cmake<C>(0, 0);
  }
  __syncthreads();
  const int c = blockIdx.x * 32 + tid;
  if (c >= ncols) return;
  C* col = B + (size_t)c * ldb;
  C x[NB];
#pragma unroll
  for (int r = 0; r < NB; ++r) x[r] = col[r];
#pragma unroll
  for (int k = 0; k < NB - 1; ++k)
#pragma unroll
    for (int r = k + 1; r < NB; ++r) x[r] = cfms(x[r], Ls[k * NB + r], x[k]);
#pragma unroll
  for (int r = 0; r < NB; ++r) col[r] = x[r];
}

template <typename C>
cudaError_t trsm_lower_reg(const C* T, long long ldt, C* B, long long ldb, int nb, int ncols, long long tstride,
                           long long bstride, int batch, cudaStream_t s, bool* done) {
  *done = true;
  const dim3 grid((ncols + 31) / 32, batch);
  switch (nb) {
    case 8: trsm_lower_reg_kernel<C, 8><<<grid, 32, 0, s>>>(T, ldt, B, ldb, ncols, tstride, bstride); break;
    case 16: trsm_lower_reg_kernel<C, 16><<<grid, 32, 0, s>>>(T, ldt, B, ldb, ncols, tstride, bstride); break;
    case 24: trsm_lower_reg_kernel<C, 24><<<grid, 32, 0, s>>>(T, ldt, B, ldb, ncols, tstride, bstride); break;
    case 32: trsm_lower_reg_kernel<C, 32><<<grid, 32, 0, s>>>(T, ldt, B, ldb, ncols, tstride, bstride); break;
    default: *done = false; return cudaSuccess;
  }
  return cudaGetLastError();
}

// FP32 unit-lower TRSM of the factorisation, B <- L^-1 B for an nb x nb unit lower L
// (nb <= 64), one thread per column of B.  L and the B block are staged once per
// block in shared memory (loads batched, kILP in flight per thread); L is read by
// broadcast.  Rows are solved in four blocks of 16 whose unknowns live in registers:
// the block's own triangle, then its contribution to every row below.  For each row
// the updates come in increasing k, i.e. in trsm_kernel's order of operations, so
// both kernels give identical results.  Rows and columns of L beyond nb are zero.
constexpr int kTrsmColThreads = 128;

template <typename C>
__global__ void __launch_bounds__(kTrsmColThreads) trsm_lower_cols_kernel(const C* __restrict__ T, long long ldt,
                                                                         C* __restrict__ B, long long ldb, int nb,
                                                                         int ncols, long long tstride,
                                                                         long long bstride) {
  constexpr int kILP = 8;
  constexpr int ldbs = kTrsmColThreads + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* Ls = reinterpret_cast<C*>(smem_raw);  // [64][64] column-major: Ls[k*64 + r] = l_rk
  C* Bs = Ls + 64 * 64;                     // [64][ldbs]: Bs[r*ldbs + c]
  T += (size_t)blockIdx.y * tstride;
  B += (size_t)blockIdx.y * bstride;
  const int tid = threadIdx.x;
  const int c0 = blockIdx.x * kTrsmColThreads;
  const int nc = min(kTrsmColThreads, ncols - c0);
  for (int i0 = tid; i0 < 64 * 64; i0 += kTrsmColThreads * kILP) {
    C v[kILP];
#pragma unroll
    for (int u = 0; u < kILP; ++u) {
      const int idx = i0 + u * kTrsmColThreads, k = idx >> 6, r = idx & 63;
      v[u] = (idx < 64 * 64 && r < nb && k < nb && r > k) ? T[(size_t)k * ldt + r] : cmake<C>(0, 0);
    }
#pragma unroll
    for (int u = 0; u < kILP; ++u)
      if (i0 + u * kTrsmColThreads < 64 * 64) Ls[i0 + u * kTrsmColThreads] = v[u];
  }
  for (int i0 = tid; i0 < 64 * nc; i0 += kTrsmColThreads * kILP) {
    C v[kILP];
#pragma unroll
    for (int u = 0; u < kILP; ++u) {
      const int idx = i0 + u * kTrsmColThreads, c = idx >> 6, r = idx & 63;
      v[u] = (idx < 64 * nc && r < nb) ? B[(size_t)(c0 + c) * ldb + r] : cmake<C>(0, 0);
    }
#pragma unroll
    for (int u = 0; u < kILP; ++u) {
      const int idx = i0 + u * kTrsmColThreads;
      if (idx < 64 * nc) Bs[(idx & 63) * ldbs + (idx >> 6)] = v[u];
    }
  }
  __syncthreads();
  if (tid < nc) {
#pragma unroll 1
    for (int r0 = 0; r0 < 64; r0 += 16) {
      C x[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) x[i] = Bs[(r0 + i) * ldbs + tid];
#pragma unroll
      for (int k = 0; k < 15; ++k)
#pragma unroll
        for (int i = k + 1; i < 16; ++i) x[i] = cfms(x[i], Ls[(r0 + k) * 64 + r0 + i], x[k]);
#pragma unroll
      for (int i = 0; i < 16; ++i) Bs[(r0 + i) * ldbs + tid] = x[i];
#pragma unroll 1
      for (int r = r0 + 16; r < 64; ++r) {
        C b = Bs[r * ldbs + tid];
#pragma unroll
        for (int k = 0; k < 16; ++k) b = cfms(b, Ls[(r0 + k) * 64 + r], x[k]);
        Bs[r * ldbs + tid] = b;
      }
    }
  }
  __syncthreads();
  for (int idx = tid; idx < 64 * nc; idx += kTrsmColThreads) {
    const int c = idx >> 6, r = idx & 63;
    if (r < nb) B[(size_t)(c0 + c) * ldb + r] = Bs[r * ldbs + c];
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
                                                       int K, long long bstride) {
  __shared__ C As[kGemmBK][kGemmBM + 1];
  __shared__ C Bs[kGemmBK][kGemmBN + 1];
  // batch: blockIdx.z selects the matrix (all three operands live in it)
  Am += (size_t)blockIdx.z * bstride;
  Bm += (size_t)blockIdx.z * bstride;
  Cm += (size_t)blockIdx.z * bstride;
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

cudaError_t zgemm_sub_simt(const double2* Am, long long lda, const double2* Bm, long long ldb, double2* Cm,
                           long long ldc, int M, int N, int K, cudaStream_t s, int batch, long long bstride) {
  if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
  stats::Scope sc(stats::kGemm, s, 8.0 * M * (double)N * K * batch);
  dim3 grid((M + kGemmBM - 1) / kGemmBM, (N + kGemmBN - 1) / kGemmBN, batch);
  gemm_sub_kernel<double2><<<grid, 256, 0, s>>>(Am, lda, Bm, ldb, Cm, ldc, M, N, K, bstride);
  return cudaGetLastError();
}

// --------------------------------------------------------------- trsv ----
// One right-hand side, the whole triangular solve in ONE launch.  Each CTA owns a
// block of 64 rows; it takes a ticket (atomicAdd) that fixes its block in
// dependency order (forward for L, backward for U), so a CTA only ever waits on
// CTAs that were scheduled before it.  It subtracts the contributions of the
// finished blocks as their "ready" flags appear (release/acquire on a flag word
// holding the call's epoch), solves its 64 x 64 diagonal block in one warp with
// shuffles, publishes its part of x and raises its flag.  Waits are bounded.
constexpr int kTrsvB = 64;
constexpr unsigned long long kTrsvWaitNs = 1000000000ull;

__device__ __forceinline__ int ld_acquire_i32(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_i32(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// inv (optional): the inverses of the factors' kTrsvB x kTrsvB diagonal blocks
// (lu_block_inverses); each block's solution is then one parallel product with its
// inverse instead of a kTrsvB-step substitution by one warp, the chain's critical path.
template <typename C, bool UPPER>
__global__ void __launch_bounds__(256) trsv_kernel(const C* __restrict__ A, long long lda, int n, C* x,
                                                   int* flags, unsigned int* ticket, int epoch, int* err,
                                                   long long astride, int flag_stride, const int* __restrict__ sel,
                                                   const C* __restrict__ inv) {
  using R = decltype(C{}.x);
  __shared__ C xs[kTrsvB];
  __shared__ C part[4][kTrsvB];
  __shared__ int s_b, s_m, s_ok;
  const int tid = threadIdx.x;
  const int nblk = (n + kTrsvB - 1) / kTrsvB;
  const int batch = (int)gridDim.x / nblk;  // the grid holds nblk blocks of each matrix
  // One ticket counter per launch orders the CTAs: ticket t is block t / batch (in
  // dependency order) of matrix t % batch.  The chains of all matrices of a batch
  // advance together, and a CTA only waits on CTAs that took smaller tickets.
  if (tid == 0) {
    const unsigned t = atomicAdd(ticket, 1u);
    const int bi = (int)(t / (unsigned)batch);
    s_m = (int)(t % (unsigned)batch);
    s_b = UPPER ? nblk - 1 - bi : bi;
    s_ok = 1;
  }
  __syncthreads();
  const int b = s_b;
  if (b < 0 || b >= nblk) return;
  // the matrix, its right-hand side (sel: slot s_m of the batch is matrix sel[s_m])
  // and the slot's flags
  const int mat = sel ? sel[s_m] : s_m;
  A += (size_t)mat * astride;
  x += (size_t)mat * n;
  flags += (size_t)s_m * flag_stride;
  const int r0 = b * kTrsvB;
  const int rows = min(kTrsvB, n - r0);
  const int r = tid & (kTrsvB - 1), g = tid >> 6;
  // the diagonal block goes to shared memory first: its loads overlap the waits
  extern __shared__ __align__(16) unsigned char trsv_smem[];
  C* Ds = reinterpret_cast<C*>(trsv_smem);  // kTrsvB x kTrsvB, column-major
  const C* Ib = inv ? inv + (((size_t)mat * nblk + b) * 2 + (UPPER ? 1 : 0)) * kTrsvB * kTrsvB : nullptr;
  for (int idx = tid; idx < kTrsvB * kTrsvB; idx += blockDim.x) {
    const int c = idx / kTrsvB, q = idx - c * kTrsvB;
    if (Ib)
      Ds[idx] = Ib[idx];
    else
      Ds[idx] = (c < rows && q < rows) ? A[(size_t)(r0 + c) * lda + r0 + q] : cmake<C>(0, 0);
  }
  // back substitution divides by the diagonal: Smith's ratio and the reciprocal of
  // its denominator for every diagonal entry, in parallel and before the waits, so
  // that the dependent chain below multiplies instead of dividing
  __shared__ R dg_r[kTrsvB], dg_inv[kTrsvB];
  __shared__ int dg_sw[kTrsvB];
  if (UPPER && !Ib && tid < kTrsvB) {
    const int c = tid;
    const C d = (c < rows) ? A[(size_t)(r0 + c) * lda + r0 + c] : cmake<C>(1, 0);
    if (fabs(d.x) >= fabs(d.y)) {
      const R q = d.y / d.x;
      dg_r[c] = q;
      dg_inv[c] = R(1) / (d.x + d.y * q);
      dg_sw[c] = 0;
    } else {
      const R q = d.x / d.y;
      dg_r[c] = q;
      dg_inv[c] = R(1) / (d.y + d.x * q);
      dg_sw[c] = 1;
    }
  }
  C acc = cmake<C>(0, 0);
  const int nsteps = UPPER ? nblk - 1 - b : b;
  // this thread's 16 entries of an off-diagonal 64 x 64 tile: row r, columns g + 4i;
  // the next tile is loaded (independent loads) before the wait for its x
  constexpr int kPer = kTrsvB / 4;
  auto load_tile = [&](int j, C* dst) {
    const int c0 = j * kTrsvB;
    const int cols = min(kTrsvB, n - c0);
    const C* col = A + (size_t)c0 * lda + r0 + r;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int c = g + 4 * i;
      dst[i] = (r < rows && c < cols) ? col[(size_t)c * lda] : cmake<C>(0, 0);
    }
  };
  C a_cur[kPer];
  if (nsteps > 0) load_tile(UPPER ? nblk - 1 : 0, a_cur);
  for (int step = 0; step < nsteps; ++step) {
    const int j = UPPER ? nblk - 1 - step : step;
    if (tid == 0) {
      const unsigned long long t0 = global_ns();
      while (ld_acquire_i32(&flags[j]) != epoch) {
        if (ld_volatile_i32(err) || global_ns() - t0 > kTrsvWaitNs) {
          atomicExch(err, 1);
          s_ok = 0;
          break;
        }
        __nanosleep(20);
      }
    }
    __syncthreads();
    if (!s_ok) return;
    const int c0 = j * kTrsvB;
    const int cols = min(kTrsvB, n - c0);
    if (tid < cols) xs[tid] = __ldcg(&x[c0 + tid]);
    __syncthreads();
    C a_next[kPer];
    if (step + 1 < nsteps) load_tile(UPPER ? j - 1 : j + 1, a_next);
    if (r < rows) {
#pragma unroll
      for (int i = 0; i < kPer; ++i)
        if (g + 4 * i < cols) acc = cfms(acc, a_cur[i], xs[g + 4 * i]);
    }
#pragma unroll
    for (int i = 0; i < kPer; ++i) a_cur[i] = a_next[i];
    __syncthreads();
  }
  part[g][r] = acc;
  __syncthreads();
  if (Ib) {
    // s = x_blk - sum(T x) in xs, then x_blk = Inv s: thread (r, g) sums the columns
    // g + 4i of row r, the four partial sums meet in part[]
    if (tid < kTrsvB) {
      C v = cmake<C>(0, 0);
      if (tid < rows) {
        const C b0 = x[r0 + tid];
        v = cmake<C>(b0.x + (part[0][tid].x + part[1][tid].x + part[2][tid].x + part[3][tid].x),
                     b0.y + (part[0][tid].y + part[1][tid].y + part[2][tid].y + part[3][tid].y));
      }
      xs[tid] = v;
    }
    __syncthreads();
    C y = cmake<C>(0, 0);  // -sum(Inv s)
#pragma unroll
    for (int i = 0; i < kPer; ++i) y = cfms(y, Ds[(size_t)(g + 4 * i) * kTrsvB + r], xs[g + 4 * i]);
    part[g][r] = y;
    __syncthreads();
    if (tid < rows)
      x[r0 + tid] = cmake<C>(-((part[0][tid].x + part[1][tid].x) + (part[2][tid].x + part[3][tid].x)),
                             -((part[0][tid].y + part[1][tid].y) + (part[2][tid].y + part[3][tid].y)));
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release_i32(&flags[b], epoch);
    return;
  }
  if (tid < 32) {
    // lane l holds rows l and l + 32 of the block; part[] already holds -sum(T x)
    C s0 = cmake<C>(0, 0), s1 = cmake<C>(0, 0);
    if (tid < rows) {
      const C b0 = x[r0 + tid];
      s0 = cmake<C>(b0.x + (part[0][tid].x + part[1][tid].x + part[2][tid].x + part[3][tid].x),
                    b0.y + (part[0][tid].y + part[1][tid].y + part[2][tid].y + part[3][tid].y));
    }
    if (tid + 32 < rows) {
      const int q = tid + 32;
      const C b1 = x[r0 + q];
      s1 = cmake<C>(b1.x + (part[0][q].x + part[1][q].x + part[2][q].x + part[3][q].x),
                    b1.y + (part[0][q].y + part[1][q].y + part[2][q].y + part[3][q].y));
    }
    const C* D = Ds;  // diagonal block (leading dimension kTrsvB)
    constexpr long long lda = kTrsvB;
    if (!UPPER) {
      for (int c = 0; c < rows; ++c) {
        const R xr = __shfl_sync(0xffffffffu, c < 32 ? s0.x : s1.x, c & 31);
        const R xi = __shfl_sync(0xffffffffu, c < 32 ? s0.y : s1.y, c & 31);
        const C xc = cmake<C>(xr, xi);
        if (tid > c && tid < rows) s0 = cfms(s0, D[(size_t)c * lda + tid], xc);
        if (tid + 32 > c && tid + 32 < rows) s1 = cfms(s1, D[(size_t)c * lda + tid + 32], xc);
      }
    } else {
      // a / d_c by Smith's formula with the precomputed ratio and reciprocal
      auto div_diag = [&](C a, int c) -> C {
        const R q = dg_r[c], inv = dg_inv[c];
        return dg_sw[c] ? cmake<C>((a.x * q + a.y) * inv, (a.y * q - a.x) * inv)
                        : cmake<C>((a.x + a.y * q) * inv, (a.y - a.x * q) * inv);
      };
      for (int c = rows - 1; c >= 0; --c) {
        if (c < 32) {
          if (tid == c) s0 = div_diag(s0, c);
        } else {
          if (tid + 32 == c) s1 = div_diag(s1, c);
        }
        const R xr = __shfl_sync(0xffffffffu, c < 32 ? s0.x : s1.x, c & 31);
        const R xi = __shfl_sync(0xffffffffu, c < 32 ? s0.y : s1.y, c & 31);
        const C xc = cmake<C>(xr, xi);
        if (tid < c && tid < rows) s0 = cfms(s0, D[(size_t)c * lda + tid], xc);
        if (tid + 32 < c && tid + 32 < rows) s1 = cfms(s1, D[(size_t)c * lda + tid + 32], xc);
      }
    }
    if (tid < rows) x[r0 + tid] = s0;
    if (tid + 32 < rows) x[r0 + tid + 32] = s1;
    __threadfence();
  }
  __syncthreads();
  if (tid == 0) st_release_i32(&flags[b], epoch);
}

// ------------------------------------------------- float-float trsv ----
// The second tier's corrections solve with FP64-grade factors held as float-float
// values: every entry of the factors is hi + lo, two complex64 values with |lo| at
// most half an FP32 ulp of hi, stored as one float4 (hi.re, hi.im, lo.re, lo.im) in
// place of the complex128 entry (split_ff_inplace; the same 16 bytes, so the factors'
// layout and strides are unchanged).  The arithmetic is compensated FP32 (Dekker's and Knuth's error-free
// products and sums), about 2^-48 relative per operation, on the FP32 pipe, which
// GB300 runs 64 times as fast as its FP64 pipe.  Inside iterative refinement with
// FP64 residuals that accuracy is enough: it is below the second tier's own
// factorisation error (about 2^-45), so the corrections contract as fast as with FP64
// solves, and the FP64 residual still sets the final accuracy.  Block structure,
// ticket order, ready flags and bounded waits are trsv_kernel's.
struct Ff {
  float h, l;
};
struct __align__(16) Ffc {
  Ff re, im;
};

__device__ __forceinline__ void ff_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// acc - a * b
__device__ __forceinline__ Ff ff_fms(Ff acc, Ff a, Ff b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);  // the head product's rounding error, exactly
  e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, e));
  float s, t;
  ff_two_sum(acc.h, -p, s, t);
  t = __fadd_rn(t, __fsub_rn(acc.l, e));
  const float h = __fadd_rn(s, t);
  return Ff{h, __fsub_rn(t, __fsub_rn(h, s))};
}

__device__ __forceinline__ Ff ff_add(Ff a, Ff b) {
  float s, e;
  ff_two_sum(a.h, b.h, s, e);
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  const float h = __fadd_rn(s, e);
  return Ff{h, __fsub_rn(e, __fsub_rn(h, s))};
}

__device__ __forceinline__ Ff ff_neg(Ff a) { return Ff{-a.h, -a.l}; }

// acc - a * b, complex
__device__ __forceinline__ Ffc ffc_fms(Ffc acc, const Ffc& a, const Ffc& b) {
  acc.re = ff_fms(acc.re, a.re, b.re);
  acc.re = ff_fms(acc.re, ff_neg(a.im), b.im);
  acc.im = ff_fms(acc.im, a.re, b.im);
  acc.im = ff_fms(acc.im, a.im, b.re);
  return acc;
}

__device__ __forceinline__ Ffc ffc_add(const Ffc& a, const Ffc& b) { return Ffc{ff_add(a.re, b.re), ff_add(a.im, b.im)}; }

// a * b, complex: 0 - (-a) * b
__device__ __forceinline__ Ffc ffc_mul(const Ffc& a, const Ffc& b) {
  return ffc_fms(Ffc{Ff{0.f, 0.f}, Ff{0.f, 0.f}}, Ffc{ff_neg(a.re), ff_neg(a.im)}, b);
}

__device__ __forceinline__ Ff ff_of(double v) {
  const float h = __double2float_rn(v);
  return Ff{h, __double2float_rn(v - (double)h)};
}
__device__ __forceinline__ double ff_dbl(Ff a) { return (double)a.h + (double)a.l; }
__device__ __forceinline__ Ffc ffc_of(double2 v) { return Ffc{ff_of(v.x), ff_of(v.y)}; }
__device__ __forceinline__ double2 ffc_dbl(const Ffc& a) { return make_double2(ff_dbl(a.re), ff_dbl(a.im)); }
__device__ __forceinline__ Ffc ffc_ld(const float4* a, size_t i) {
  const float4 v = a[i];
  return Ffc{Ff{v.x, v.z}, Ff{v.y, v.w}};
}

// inv (optional): the inverses of the factors' kTrsvB x kTrsvB diagonal blocks
// (ff_block_inverses); the block's solution is then one parallel product with the
// inverse instead of a kTrsvB-step substitution by one warp, which was the chain's
// critical path.
template <bool UPPER>
__global__ void __launch_bounds__(256) trsv_ff_kernel(const float4* __restrict__ A, long long lda, int n,
                                                      double2* x, int* flags,
                                                      unsigned int* ticket, int epoch, int* err, long long astride,
                                                      int flag_stride, const int* __restrict__ sel,
                                                      const float4* __restrict__ inv) {
  __shared__ Ffc xs[kTrsvB];
  __shared__ Ffc part[4][kTrsvB];
  __shared__ Ffc dinv[kTrsvB];  // 1 / u_cc (back substitution)
  __shared__ int s_b, s_m, s_ok;
  const int tid = threadIdx.x;
  const int nblk = (n + kTrsvB - 1) / kTrsvB;
  const int batch = (int)gridDim.x / nblk;
  if (tid == 0) {
    const unsigned t = atomicAdd(ticket, 1u);
    const int bi = (int)(t / (unsigned)batch);
    s_m = (int)(t % (unsigned)batch);
    s_b = UPPER ? nblk - 1 - bi : bi;
    s_ok = 1;
  }
  __syncthreads();
  const int b = s_b;
  if (b < 0 || b >= nblk) return;
  const int mat = sel ? sel[s_m] : s_m;
  A += (size_t)mat * astride;
  x += (size_t)mat * n;
  flags += (size_t)s_m * flag_stride;
  const int r0 = b * kTrsvB;
  const int rows = min(kTrsvB, n - r0);
  const int r = tid & (kTrsvB - 1), g = tid >> 6;
  // the diagonal block in shared memory, and (back substitution) the reciprocals of
  // its diagonal, in FP64 once per entry, before the waits
  extern __shared__ __align__(16) unsigned char trsv_ff_smem[];
  Ffc* Ds = reinterpret_cast<Ffc*>(trsv_ff_smem);  // kTrsvB x kTrsvB, column-major
  const float4* Ib = inv ? inv + (((size_t)mat * nblk + b) * 2 + (UPPER ? 1 : 0)) * kTrsvB * kTrsvB : nullptr;
  for (int idx = tid; idx < kTrsvB * kTrsvB; idx += blockDim.x) {
    const int c = idx / kTrsvB, q = idx - c * kTrsvB;
    if (Ib)
      Ds[idx] = ffc_ld(Ib, idx);
    else
      Ds[idx] = (c < rows && q < rows) ? ffc_ld(A, (size_t)(r0 + c) * lda + r0 + q)
                                       : Ffc{Ff{0.f, 0.f}, Ff{0.f, 0.f}};
  }
  if (UPPER && !Ib && tid < kTrsvB) {
    const int c = tid;
    double2 d = make_double2(1.0, 0.0);
    if (c < rows) {
      const Ffc dd = ffc_ld(A, (size_t)(r0 + c) * lda + r0 + c);
      d = ffc_dbl(dd);
    }
    dinv[c] = ffc_of(crecip(d));
  }
  Ffc acc{Ff{0.f, 0.f}, Ff{0.f, 0.f}};
  const int nsteps = UPPER ? nblk - 1 - b : b;
  constexpr int kPer = kTrsvB / 4;
  auto load_tile = [&](int j, Ffc* dst) {
    const int c0 = j * kTrsvB;
    const int cols = min(kTrsvB, n - c0);
    const size_t base = (size_t)c0 * lda + r0 + r;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int c = g + 4 * i;
      dst[i] = (r < rows && c < cols) ? ffc_ld(A, base + (size_t)c * lda) : Ffc{Ff{0.f, 0.f}, Ff{0.f, 0.f}};
    }
  };
  Ffc a_cur[kPer];
  if (nsteps > 0) load_tile(UPPER ? nblk - 1 : 0, a_cur);
  for (int step = 0; step < nsteps; ++step) {
    const int j = UPPER ? nblk - 1 - step : step;
    if (tid == 0) {
      const unsigned long long t0 = global_ns();
      while (ld_acquire_i32(&flags[j]) != epoch) {
        if (ld_volatile_i32(err) || global_ns() - t0 > kTrsvWaitNs) {
          atomicExch(err, 1);
          s_ok = 0;
          break;
        }
        __nanosleep(20);
      }
    }
    __syncthreads();
    if (!s_ok) return;
    const int c0 = j * kTrsvB;
    const int cols = min(kTrsvB, n - c0);
    if (tid < cols) xs[tid] = ffc_of(__ldcg(&x[c0 + tid]));
    __syncthreads();
    Ffc a_next[kPer];
    if (step + 1 < nsteps) load_tile(UPPER ? j - 1 : j + 1, a_next);
    if (r < rows) {
#pragma unroll
      for (int i = 0; i < kPer; ++i)
        if (g + 4 * i < cols) acc = ffc_fms(acc, a_cur[i], xs[g + 4 * i]);
    }
#pragma unroll
    for (int i = 0; i < kPer; ++i) a_cur[i] = a_next[i];
    __syncthreads();
  }
  part[g][r] = acc;
  __syncthreads();
  if (Ib) {
    // s = x_blk - sum(T x) in xs, then x_blk = Inv s: thread (r, g) sums the columns
    // g + 4i of row r, the four partial sums meet in part[]
    if (tid < kTrsvB)
      xs[tid] = tid < rows ? ffc_add(ffc_add(ffc_of(x[r0 + tid]), ffc_add(part[0][tid], part[1][tid])),
                                     ffc_add(part[2][tid], part[3][tid]))
                           : Ffc{Ff{0.f, 0.f}, Ff{0.f, 0.f}};
    __syncthreads();
    Ffc y{Ff{0.f, 0.f}, Ff{0.f, 0.f}};  // -sum(Inv s)
#pragma unroll
    for (int i = 0; i < kPer; ++i) y = ffc_fms(y, Ds[(size_t)(g + 4 * i) * kTrsvB + r], xs[g + 4 * i]);
    part[g][r] = y;
    __syncthreads();
    if (tid < rows) {
      const Ffc v = ffc_add(ffc_add(part[0][tid], part[1][tid]), ffc_add(part[2][tid], part[3][tid]));
      x[r0 + tid] = make_double2(-ff_dbl(v.re), -ff_dbl(v.im));
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) st_release_i32(&flags[b], epoch);
    return;
  }
  if (tid < 32) {
    // lane l holds rows l and l + 32 of the block; part[] holds -sum(T x) per group
    Ffc s0{Ff{0.f, 0.f}, Ff{0.f, 0.f}}, s1 = s0;
    if (tid < rows)
      s0 = ffc_add(ffc_add(ffc_of(x[r0 + tid]), ffc_add(part[0][tid], part[1][tid])),
                   ffc_add(part[2][tid], part[3][tid]));
    if (tid + 32 < rows) {
      const int q = tid + 32;
      s1 = ffc_add(ffc_add(ffc_of(x[r0 + q]), ffc_add(part[0][q], part[1][q])), ffc_add(part[2][q], part[3][q]));
    }
    const Ffc* D = Ds;
    constexpr int ld = kTrsvB;
    auto shfl = [&](const Ffc& v, int src) {
      return Ffc{Ff{__shfl_sync(0xffffffffu, v.re.h, src), __shfl_sync(0xffffffffu, v.re.l, src)},
                 Ff{__shfl_sync(0xffffffffu, v.im.h, src), __shfl_sync(0xffffffffu, v.im.l, src)}};
    };
    if (!UPPER) {
      for (int c = 0; c < rows; ++c) {
        const Ffc xc = shfl(c < 32 ? s0 : s1, c & 31);
        if (tid > c && tid < rows) s0 = ffc_fms(s0, D[(size_t)c * ld + tid], xc);
        if (tid + 32 > c && tid + 32 < rows) s1 = ffc_fms(s1, D[(size_t)c * ld + tid + 32], xc);
      }
    } else {
      for (int c = rows - 1; c >= 0; --c) {
        // x_c = s_c / u_cc = s_c * (1 / u_cc), by its owner lane
        if (c < 32) {
          if (tid == c) s0 = ffc_mul(s0, dinv[c]);
        } else {
          if (tid + 32 == c) s1 = ffc_mul(s1, dinv[c]);
        }
        const Ffc xc = shfl(c < 32 ? s0 : s1, c & 31);
        if (tid < c && tid < rows) s0 = ffc_fms(s0, D[(size_t)c * ld + tid], xc);
        if (tid + 32 < c && tid + 32 < rows) s1 = ffc_fms(s1, D[(size_t)c * ld + tid + 32], xc);
      }
    }
    if (tid < rows) x[r0 + tid] = ffc_dbl(s0);
    if (tid + 32 < rows) x[r0 + tid + 32] = ffc_dbl(s1);
    __threadfence();
  }
  __syncthreads();
  if (tid == 0) st_release_i32(&flags[b], epoch);
}

// The inverses of the float-float factors' kTrsvB x kTrsvB diagonal blocks, for
// trsv_ff_kernel: grid (blocks, matrices, 2), z = 0 the unit lower L block, z = 1 the
// upper U block; inv holds per matrix and block the two inverses, column-major, with
// an identity beyond the last block's rows.  Four threads of one warp compute column c
// by substitution on e_c in float-float arithmetic, each on every fourth row (columns
// of L^-1 by forward, of U^-1 by back substitution with the diagonal reciprocals
// taken in FP64), the block and the columns in shared memory (columns row-major with
// a padded row, so that the final column-major write reads rows without bank
// conflicts).  With one thread per column, the first columns' chains (2016 updates
// for column 0) made it 220 us per CTA.
constexpr int kInvLd = kTrsvB + 1;
constexpr size_t kTriInvSmem = sizeof(Ffc) * ((size_t)kTrsvB * kTrsvB + (size_t)kTrsvB * kInvLd);
__global__ void __launch_bounds__(4 * kTrsvB) tri_inv_ff_kernel(const float4* __restrict__ A, long long lda, int n,
                                                                long long astride, float4* __restrict__ inv) {
  extern __shared__ __align__(16) unsigned char tri_inv_smem[];
  Ffc* T = reinterpret_cast<Ffc*>(tri_inv_smem);  // the block, column-major
  Ffc* Y = T + kTrsvB * kTrsvB;                     // Y[i * kInvLd + c]: row i of column c
  __shared__ Ffc dinv[kTrsvB];
  const int b = blockIdx.x, mat = blockIdx.y;
  const bool upper = blockIdx.z == 1;
  const int nblk = gridDim.x;
  const int r0 = b * kTrsvB;
  const int rows = min(kTrsvB, n - r0);
  const int tid = threadIdx.x;
  // column c of the inverse by the four threads (c, q) of one warp, rows q + 4 i each
  const int c = tid >> 2, q = tid & 3;
  A += (size_t)mat * astride;
  const Ffc zero{Ff{0.f, 0.f}, Ff{0.f, 0.f}}, one{Ff{1.f, 0.f}, Ff{0.f, 0.f}};
  for (int idx = tid; idx < kTrsvB * kTrsvB; idx += blockDim.x) {
    const int j = idx / kTrsvB, i = idx - j * kTrsvB;
    T[idx] = (i < rows && j < rows) ? ffc_ld(A, (size_t)(r0 + j) * lda + r0 + i) : zero;
    Y[(size_t)i * kInvLd + j] = i == j ? one : zero;
  }
  if (upper && tid < kTrsvB) {
    double2 d = make_double2(1.0, 0.0);
    if (tid < rows) d = ffc_dbl(ffc_ld(A, (size_t)(r0 + tid) * lda + r0 + tid));
    dinv[tid] = ffc_of(crecip(d));
  }
  __syncthreads();
  if (!upper) {
    // forward substitution on e_c: row k is final after step k - 1
    for (int k = 0; k + 1 < rows; ++k) {
      __syncwarp();
      if (c <= k && c < rows) {
        const Ffc yk = Y[(size_t)k * kInvLd + c];
        for (int i = q; i < rows; i += 4)
          if (i > k) Y[(size_t)i * kInvLd + c] = ffc_fms(Y[(size_t)i * kInvLd + c], T[(size_t)k * kTrsvB + i], yk);
      }
    }
  } else {
    // back substitution on e_c: row k is scaled by 1 / u_kk, then taken off the rows above
    for (int k = rows - 1; k >= 0; --k) {
      __syncwarp();
      Ffc yk = zero;
      if (c >= k && c < rows) yk = ffc_mul(Y[(size_t)k * kInvLd + c], dinv[k]);
      __syncwarp();  // every thread of the column has read row k before its owner writes it
      if (c >= k && c < rows) {
        if ((k & 3) == q) Y[(size_t)k * kInvLd + c] = yk;
        for (int i = q; i < k; i += 4)
          Y[(size_t)i * kInvLd + c] = ffc_fms(Y[(size_t)i * kInvLd + c], T[(size_t)k * kTrsvB + i], yk);
      }
    }
  }
  __syncthreads();
  float4* out = inv + (((size_t)mat * nblk + b) * 2 + (upper ? 1 : 0)) * kTrsvB * kTrsvB;
  for (int idx = tid; idx < kTrsvB * kTrsvB; idx += blockDim.x) {
    // entry (i, j) of the inverse at j * kTrsvB + i (consecutive threads, consecutive i)
    const int j = idx / kTrsvB, i = idx - j * kTrsvB;
    const Ffc v = Y[(size_t)i * kInvLd + j];
    out[idx] = make_float4(v.re.h, v.im.h, v.re.l, v.im.l);
  }
}

// The inverses of the factors' kTrsvB x kTrsvB diagonal blocks for trsv_kernel, in
// the factors' own arithmetic: tri_inv_ff_kernel's grid, layout and four-threads-per-
// column substitution on e_c (L^-1 by forward substitution, U^-1 by back
// substitution with the reciprocals of U's diagonal taken in FP64).
template <typename C>
__global__ void __launch_bounds__(4 * kTrsvB) tri_inv_kernel(const C* __restrict__ A, long long lda, int n,
                                                             long long astride, C* __restrict__ inv) {
  extern __shared__ __align__(16) unsigned char tri_inv_c_smem[];
  C* T = reinterpret_cast<C*>(tri_inv_c_smem);  // the block, column-major
  C* Y = T + kTrsvB * kTrsvB;                    // Y[i * kInvLd + c]: row i of column c
  __shared__ C dinv[kTrsvB];
  using R = decltype(C{}.x);
  const int b = blockIdx.x, mat = blockIdx.y;
  const bool upper = blockIdx.z == 1;
  const int nblk = gridDim.x;
  const int r0 = b * kTrsvB;
  const int rows = min(kTrsvB, n - r0);
  const int tid = threadIdx.x;
  const int c = tid >> 2, q = tid & 3;
  A += (size_t)mat * astride;
  const C zero = cmake<C>(0, 0), one = cmake<C>(1, 0);
  for (int idx = tid; idx < kTrsvB * kTrsvB; idx += blockDim.x) {
    const int j = idx / kTrsvB, i = idx - j * kTrsvB;
    T[idx] = (i < rows && j < rows) ? A[(size_t)(r0 + j) * lda + r0 + i] : zero;
    Y[(size_t)i * kInvLd + j] = i == j ? one : zero;
  }
  if (upper && tid < kTrsvB) {
    double2 d = make_double2(1.0, 0.0);
    if (tid < rows) {
      const C v = A[(size_t)(r0 + tid) * lda + r0 + tid];
      d = make_double2((double)v.x, (double)v.y);
    }
    const double2 rc = crecip(d);
    dinv[tid] = cmake<C>((R)rc.x, (R)rc.y);
  }
  __syncthreads();
  if (!upper) {
    for (int k = 0; k + 1 < rows; ++k) {
      __syncwarp();
      if (c <= k && c < rows) {
        const C yk = Y[(size_t)k * kInvLd + c];
        for (int i = q; i < rows; i += 4)
          if (i > k) Y[(size_t)i * kInvLd + c] = cfms(Y[(size_t)i * kInvLd + c], T[(size_t)k * kTrsvB + i], yk);
      }
    }
  } else {
    for (int k = rows - 1; k >= 0; --k) {
      __syncwarp();
      C yk = zero;
      if (c >= k && c < rows) yk = cmul(Y[(size_t)k * kInvLd + c], dinv[k]);
      __syncwarp();  // every thread of the column has read row k before its owner writes it
      if (c >= k && c < rows) {
        if ((k & 3) == q) Y[(size_t)k * kInvLd + c] = yk;
        for (int i = q; i < k; i += 4)
          Y[(size_t)i * kInvLd + c] = cfms(Y[(size_t)i * kInvLd + c], T[(size_t)k * kTrsvB + i], yk);
      }
    }
  }
  __syncthreads();
  C* out = inv + (((size_t)mat * nblk + b) * 2 + (upper ? 1 : 0)) * kTrsvB * kTrsvB;
  for (int idx = tid; idx < kTrsvB * kTrsvB; idx += blockDim.x) {
    const int j = idx / kTrsvB, i = idx - j * kTrsvB;
    out[idx] = Y[(size_t)i * kInvLd + j];
  }
}

// Complex128 entries to float-float in place, (re, im) -> (hi.re, hi.im, lo.re,
// lo.im) with hi = fp32(v), lo = fp32(v - hi); and back (hi + lo is exact in FP64).
__global__ void split_ff_kernel(double2* a, size_t count) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
    const double2 v = a[i];
    const Ff re = ff_of(v.x), im = ff_of(v.y);
    reinterpret_cast<float4*>(a)[i] = make_float4(re.h, im.h, re.l, im.l);
  }
}

__global__ void merge_ff_kernel(double2* a, size_t count) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
    const float4 v = reinterpret_cast<const float4*>(a)[i];
    a[i] = make_double2((double)v.x + (double)v.z, (double)v.y + (double)v.w);
  }
}

// ------------------------------------------- float-float cluster panel ----
// The second tier's panels (FP64-grade factors under the digit-plane tensor-core
// updates) in float-float arithmetic: panel_cluster_la_kernel's cluster, look-ahead,
// publication and bounded barriers, with the rows held as float-float values in
// shared memory (16 bytes each, as complex128), read from and written back to the
// complex128 matrix.  Its rank-1 updates, the bulk of the panel's work, run on the
// FP32 pipe instead of GB300's narrow FP64 pipe, at about 2^-48 per operation, below
// the second tier's factorisation error (about 2^-45).  The pivot of a column is the
// row with the largest |re| + |im| of the heads (within 2^-24 of the FP64 choice; on
// a near tie either row is a valid partial pivot); its reciprocal is computed once
// per CTA in FP64.  FFS: the matrix itself holds float-float values (float4 hi.re,
// hi.im, lo.re, lo.im per entry, LuWorkspace::ff_storage), read and written as they
// are; else complex128, converted on the way in and out.
struct ClusterPubFf {
  float val;
  int row;
  int pad[2];  // cand starts 16-byte aligned
  Ffc cand[64];
  Ffc diag[64];
};
static_assert(sizeof(ClusterPubFf) == sizeof(ClusterPub<double2>), "same layout as the FP64 panel's");

__device__ __forceinline__ Ffc ld_cluster_ffc(uint32_t a) {
  float4 v;
  asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(a)
               : "memory");
  return Ffc{Ff{v.x, v.y}, Ff{v.z, v.w}};
}

__device__ __forceinline__ float ffc_abs1(const Ffc& a) { return fabsf(a.re.h) + fabsf(a.im.h); }

template <bool FFS>
__global__ void __launch_bounds__(kClusterThreads, 1) panel_cluster_la_ff_kernel(double2* __restrict__ A,
                                                                                 long long lda, int n, int j0,
                                                                                 int w, int rpc,
                                                                                 int* __restrict__ ipiv,
                                                                                 GridBarrier* __restrict__ gb,
                                                                                 long long astride) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ClusterPubFf* pub = reinterpret_cast<ClusterPubFf*>(smem_raw);  // [2]
  Ffc* prw_buf = reinterpret_cast<Ffc*>(pub + 2);  // pivot rows of columns j - 1 and j, 2 x 64
  Ffc* dgr = prw_buf + 128;                        // diagonal row, 64
  Ffc* tile = dgr + 64;                            // column-major rpc x w
  __shared__ long long red_k[2][kClusterThreads / 32];
  __shared__ int red_r[2][kClusterThreads / 32];
  __shared__ Ffc s_inv;  // 1 / pivot of the current column, computed once per CTA
  __shared__ int s_prw;  // pivot row of the current column

  A += (size_t)blockIdx.y * astride;
  ipiv += (size_t)blockIdx.y * n;
  gb += blockIdx.y;
  const unsigned cs = gridDim.x;  // the cluster spans blockIdx.x
  const unsigned rank = cluster_rank();
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int base = j0 + (int)rank * rpc;
  const int cnt = max(0, min(rpc, n - base));
  const Ffc fzero{Ff{0.f, 0.f}, Ff{0.f, 0.f}};

  if (t < cnt) {
    const int gr = base + t;
    for (int c0 = 0; c0 < w; c0 += 16) {
      double2 v[16];
#pragma unroll
      for (int u = 0; u < 16; ++u)
        if (c0 + u < w) v[u] = A[(size_t)(j0 + c0 + u) * lda + gr];
#pragma unroll
      for (int u = 0; u < 16; ++u)
        if (c0 + u < w) {
          if constexpr (FFS) {
            const float4 f = *reinterpret_cast<const float4*>(&v[u]);
            tile[(size_t)(c0 + u) * rpc + t] = Ffc{Ff{f.x, f.z}, Ff{f.y, f.w}};
          } else {
            tile[(size_t)(c0 + u) * rpc + t] = ffc_of(v[u]);
          }
        }
    }
  }
  __syncthreads();

  // this CTA's candidate for column jc among its rows >= j0 + jc (first on ties),
  // published with the candidate row and, from its owner, row j0 + jc
  auto publish = [&](int jc) {
    const int gjc = j0 + jc;
    const int pc = jc & 1;
    long long best = order_key(-1.0f);
    int brow = INT_MAX;
    if (t < cnt && base + t >= gjc) {
      best = order_key(ffc_abs1(tile[(size_t)jc * rpc + t]));
      brow = base + t;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int orow = __shfl_xor_sync(0xffffffffu, brow, o);
      if (ov > best || (ov == best && orow < brow)) {
        best = ov;
        brow = orow;
      }
    }
    if (lane == 0) {
      red_k[pc][warp] = best;
      red_r[pc][warp] = brow;
    }
    __syncthreads();
    if (t < w) {  // only these threads publish
      best = order_key(-1.0f);
      brow = INT_MAX;
#pragma unroll
      for (int q = 0; q < kClusterThreads / 32; ++q) {
        const long long v = red_k[pc][q];
        const int r = red_r[pc][q];
        if (v > best || (v == best && r < brow)) {
          best = v;
          brow = r;
        }
      }
      ClusterPubFf& my = pub[pc];
      if (t == 0) {
        my.val = key_value<float>(best);
        my.row = brow;
      }
      if (best >= 0) my.cand[t] = tile[(size_t)t * rpc + (brow - base)];
      if (gjc >= base && gjc < base + cnt) my.diag[t] = tile[(size_t)t * rpc + (gjc - base)];
    }
    // every read of the tile for the publication is done before the rows change
    __syncthreads();
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
  };

  publish(0);
  Ffc lr_l = fzero;  // this row's multiplier of the current column
  for (int j = 0; j < w; ++j) {
    const int gj = j0 + j;
    const int par = j & 1;
    Ffc* prow = prw_buf + 64 * par;               // pivot row of column j
    const Ffc* pprev = prw_buf + 64 * (par ^ 1);  // pivot row of column j - 1
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    const unsigned owner_gj = (unsigned)((gj - j0) / rpc);  // the CTA holding row gj
    int r = INT_MAX, q = -1;
    if (warp * 32 < w) {
      long long v = order_key(-1.0f);
      if (lane < (int)cs) {
        v = order_key(ld_cluster_f32(map_rank(&pub[par].val, lane)));
        r = ld_cluster_s32(map_rank(&pub[par].row, lane));
        q = lane;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const long long ov = __shfl_xor_sync(0xffffffffu, v, o);
        const int orow = __shfl_xor_sync(0xffffffffu, r, o);
        const int oq = __shfl_xor_sync(0xffffffffu, q, o);
        if (ov > v || (ov == v && orow < r)) {
          v = ov;
          r = orow;
          q = oq;
        }
      }
      if (t == 0) s_prw = r;
    }
    if (t < w) {
      const int prw = r;
      // the published rows lag the update of column j - 1 in their columns > j
      Ffc pv = ld_cluster_ffc(map_rank(&pub[par].cand[t], (unsigned)q));
      if (j > 0 && t > j) pv = ffc_fms(pv, ld_cluster_ffc(map_rank(&pub[par].cand[j - 1], (unsigned)q)), pprev[t]);
      prow[t] = pv;
      // the pivot's reciprocal once for the CTA, in FP64
      if (t == j) {
        const double2 d = ffc_dbl(pv);
        s_inv = (d.x == 0.0 && d.y == 0.0) ? fzero : ffc_of(crecip(d));
      }
      if (prw != gj) {
        Ffc dv = ld_cluster_ffc(map_rank(&pub[par].diag[t], owner_gj));
        if (j > 0 && t > j) dv = ffc_fms(dv, ld_cluster_ffc(map_rank(&pub[par].diag[j - 1], owner_gj)), pprev[t]);
        dgr[t] = dv;
      }
    }
    __syncthreads();
    const int prw = s_prw;
    if (rank == 0 && t == 0) ipiv[gj] = prw + 1;
    const Ffc piv = prow[j];
    const bool zero = piv.re.h == 0.f && piv.im.h == 0.f;
    if (zero && rank == 0 && t == 0) atomicCAS(&gb->info, 0, gj + 1);
    // this thread's row: interchange, scale, then column j + 1 only
    lr_l = fzero;
    if (t < cnt) {
      const int gr = base + t;
      if (prw != gj) {
        if (gr == prw)
          for (int c = 0; c < w; ++c) tile[(size_t)c * rpc + t] = dgr[c];
        else if (gr == gj)
          for (int c = 0; c < w; ++c) tile[(size_t)c * rpc + t] = prow[c];
      }
      if (gr > gj) {
        Ffc l = tile[(size_t)j * rpc + t];
        if (!zero) {
          l = ffc_mul(l, s_inv);
          tile[(size_t)j * rpc + t] = l;
        }
        lr_l = l;
        if (j + 1 < w) tile[(size_t)(j + 1) * rpc + t] = ffc_fms(tile[(size_t)(j + 1) * rpc + t], l, prow[j + 1]);
      }
    }
    if (j + 1 < w) {
      __syncthreads();  // column j + 1 of every row is current
      publish(j + 1);
      // the rest of this thread's row while the cluster meets
      // (four columns per step, loaded before any is stored: their float-float chains
      // are independent, so the scheduler interleaves them)
      if (t < cnt && base + t > gj) {
        int c = j + 2;
        for (; c + 3 < w; c += 4) {
          Ffc a[4], p[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            a[u] = tile[(size_t)(c + u) * rpc + t];
            p[u] = prow[c + u];
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) tile[(size_t)(c + u) * rpc + t] = ffc_fms(a[u], lr_l, p[u]);
        }
        for (; c < w; ++c) tile[(size_t)c * rpc + t] = ffc_fms(tile[(size_t)c * rpc + t], lr_l, prow[c]);
      }
    }
  }
  // no CTA leaves while another may still read its shared memory
  cluster_sync_all();
  if (t < cnt)
    for (int c = 0; c < w; ++c) {
      const Ffc v = tile[(size_t)c * rpc + t];
      double2* dst = &A[(size_t)(j0 + c) * lda + base + t];
      if constexpr (FFS)
        *reinterpret_cast<float4*>(dst) = make_float4(v.re.h, v.im.h, v.re.l, v.im.l);
      else
        *dst = ffc_dbl(v);
    }
}

template __global__ void panel_cluster_la_ff_kernel<false>(double2*, long long, int, int, int, int, int*,
                                                           GridBarrier*, long long);
template __global__ void panel_cluster_la_ff_kernel<true>(double2*, long long, int, int, int, int, int*,
                                                          GridBarrier*, long long);

// Unit-lower block solve of the second tier in float-float arithmetic, B <- L^-1 B for
// an nb x nb unit lower L (nb <= 32): trsm_kernel's structure (L and 16 columns of B
// in shared memory, the block's elements updated in parallel, one barrier per row of
// the triangle, each element's updates in increasing k) on the FP32 pipe.
// FFS: the factors are held as float-float (float4 hi.re, hi.im, lo.re, lo.im); else
// as complex128, split into float-float on load and rounded back to FP64 on store.
// The result carries about 2^-48 relative error per operation, below the second
// tier's digit-plane updates' 2^-45.  A float-float update is a long dependent chain
// of FP32 operations, so the work of a row step is spread over the block's threads;
// one column per thread of one warp, tried first, left every chain's latency exposed
// (227 us per 24-column solve).
template <bool FFS>
__device__ __forceinline__ Ffc ffc_load(const void* p, size_t i) {
  if constexpr (FFS)
    return ffc_ld(reinterpret_cast<const float4*>(p), i);
  else
    return ffc_of(reinterpret_cast<const double2*>(p)[i]);
}

template <bool FFS>
__global__ void __launch_bounds__(256) trsm_lower_ff_kernel(const double2* __restrict__ T, long long ldt,
                                                            double2* __restrict__ B, long long ldb, int nb,
                                                            int ncols, long long tstride, long long bstride) {
  extern __shared__ __align__(16) unsigned char trsm_ff_smem[];
  T += (size_t)blockIdx.y * tstride;
  B += (size_t)blockIdx.y * bstride;
  Ffc* Ts = reinterpret_cast<Ffc*>(trsm_ff_smem);  // nb x nb, column-major
  Ffc* Bs = Ts + (size_t)nb * nb;                   // nb x kTrsmCols, column-major
  const int tid = threadIdx.x;
  const int c0 = blockIdx.x * kTrsmCols;
  const int nc = min(kTrsmCols, ncols - c0);
  for (int idx = tid; idx < nb * nb; idx += blockDim.x) {
    const int c = idx / nb, r = idx - c * nb;
    // the unit diagonal and the upper part are never read
    Ts[idx] = r > c ? ffc_load<FFS>(T, (size_t)c * ldt + r) : Ffc{Ff{0.f, 0.f}, Ff{0.f, 0.f}};
  }
  for (int idx = tid; idx < nb * nc; idx += blockDim.x) {
    const int c = idx / nb, r = idx - c * nb;
    Bs[idx] = ffc_load<FFS>(B, (size_t)(c0 + c) * ldb + r);
  }
  __syncthreads();
  const int total = nb * nc;
  for (int k = 0; k < nb - 1; ++k) {
    for (int idx = tid; idx < total; idx += blockDim.x) {
      const int c = idx / nb, r = idx - c * nb;
      if (r > k) Bs[c * nb + r] = ffc_fms(Bs[c * nb + r], Ts[(size_t)k * nb + r], Bs[c * nb + k]);
    }
    __syncthreads();
  }
  for (int idx = tid; idx < total; idx += blockDim.x) {
    const int c = idx / nb, r = idx - c * nb;
    const Ffc v = Bs[idx];
    if constexpr (FFS)
      reinterpret_cast<float4*>(B)[(size_t)(c0 + c) * ldb + r] = make_float4(v.re.h, v.im.h, v.re.l, v.im.l);
    else
      B[(size_t)(c0 + c) * ldb + r] = ffc_dbl(v);
  }
}

// ------------------------------------------- conjugate-transpose trsv ----
// Solves with the conjugate transposes of the factors, the second kind of solve of
// the condition estimator (A^H x = b with P A = L U): U^H y = b by forward
// substitution (U^H lower, diagonal conj(u_ii)), then L^H z = y by back substitution
// (unit diagonal); lu_solve_h_t applies x = P^T z.  Row i of U^H or L^H is column i
// of the factor storage, so a block's off-diagonal tiles are read along the factor's
// columns (coalesced): thread (column q of the tile, row group g) keeps the partial
// sums of its 16 rows g + 4i, reduced across the tile's columns once, after the last
// tile.  Ticket order, ready flags and bounded waits are trsv_kernel's.
constexpr int kTrsvLd = kTrsvB + 1;  // padded leading dimension of the diagonal tile

template <typename C, bool LH>  // LH = false: U^H (forward); true: L^H (backward)
__global__ void __launch_bounds__(256) trsv_h_kernel(const C* __restrict__ A, long long lda, int n, C* x,
                                                     int* flags, unsigned int* ticket, int epoch, int* err,
                                                     long long astride, int flag_stride,
                                                     const int* __restrict__ sel) {
  using R = decltype(C{}.x);
  __shared__ C xs[kTrsvB];
  __shared__ C part[2][kTrsvB];
  __shared__ int s_b, s_m, s_ok;
  __shared__ R dg_r[kTrsvB], dg_inv[kTrsvB];
  __shared__ int dg_sw[kTrsvB];
  const int tid = threadIdx.x;
  const int nblk = (n + kTrsvB - 1) / kTrsvB;
  const int batch = (int)gridDim.x / nblk;
  if (tid == 0) {
    const unsigned t = atomicAdd(ticket, 1u);
    const int bi = (int)(t / (unsigned)batch);
    s_m = (int)(t % (unsigned)batch);
    s_b = LH ? nblk - 1 - bi : bi;
    s_ok = 1;
  }
  __syncthreads();
  const int b = s_b;
  if (b < 0 || b >= nblk) return;
  const int mat = sel ? sel[s_m] : s_m;
  A += (size_t)mat * astride;
  x += (size_t)mat * n;
  flags += (size_t)s_m * flag_stride;
  const int r0 = b * kTrsvB;
  const int rows = min(kTrsvB, n - r0);
  // diagonal tile of T (T = U^H or L^H): Ds[c * kTrsvLd + q] = T[r0 + q][r0 + c]
  // = conj(A[(r0 + q) * lda + r0 + c]), read along A's columns
  extern __shared__ __align__(16) unsigned char trsv_smem[];
  C* Ds = reinterpret_cast<C*>(trsv_smem);
  for (int idx = tid; idx < kTrsvB * kTrsvB; idx += blockDim.x) {
    const int q = idx / kTrsvB, c = idx - q * kTrsvB;
    C v = cmake<C>(0, 0);
    if (q < rows && c < rows) {
      const C a = A[(size_t)(r0 + q) * lda + r0 + c];
      v = cmake<C>(a.x, -a.y);
    }
    Ds[c * kTrsvLd + q] = v;
  }
  if (!LH && tid < kTrsvB) {
    // forward substitution with U^H divides by conj(u_cc): Smith's ratio and
    // reciprocal of each diagonal entry, ahead of the waits
    const int c = tid;
    C d = cmake<C>(1, 0);
    if (c < rows) {
      const C a = A[(size_t)(r0 + c) * lda + r0 + c];
      d = cmake<C>(a.x, -a.y);
    }
    if (fabs(d.x) >= fabs(d.y)) {
      const R q = d.y / d.x;
      dg_r[c] = q;
      dg_inv[c] = R(1) / (d.x + d.y * q);
      dg_sw[c] = 0;
    } else {
      const R q = d.x / d.y;
      dg_r[c] = q;
      dg_inv[c] = R(1) / (d.y + d.x * q);
      dg_sw[c] = 1;
    }
  }
  constexpr int kPer = kTrsvB / 4;
  const int q = tid & (kTrsvB - 1), g = tid >> 6;
  // this thread's entries of an off-diagonal tile: T[r0 + g + 4i][c0 + q]
  // = conj(A[(r0 + g + 4i) * lda + c0 + q])
  auto load_tile = [&](int j, C* dst) {
    const int c0 = j * kTrsvB;
    const int cols = min(kTrsvB, n - c0);
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int rr = g + 4 * i;
      dst[i] = (rr < rows && q < cols) ? A[(size_t)(r0 + rr) * lda + c0 + q] : cmake<C>(0, 0);
    }
  };
  C acc[kPer];
#pragma unroll
  for (int i = 0; i < kPer; ++i) acc[i] = cmake<C>(0, 0);
  const int nsteps = LH ? nblk - 1 - b : b;
  C a_cur[kPer];
  if (nsteps > 0) load_tile(LH ? nblk - 1 : 0, a_cur);
  for (int step = 0; step < nsteps; ++step) {
    const int j = LH ? nblk - 1 - step : step;
    if (tid == 0) {
      const unsigned long long t0 = global_ns();
      while (ld_acquire_i32(&flags[j]) != epoch) {
        if (ld_volatile_i32(err) || global_ns() - t0 > kTrsvWaitNs) {
          atomicExch(err, 1);
          s_ok = 0;
          break;
        }
        __nanosleep(20);
      }
    }
    __syncthreads();
    if (!s_ok) return;
    const int c0 = j * kTrsvB;
    const int cols = min(kTrsvB, n - c0);
    if (tid < cols) xs[tid] = __ldcg(&x[c0 + tid]);
    __syncthreads();
    C a_next[kPer];
    if (step + 1 < nsteps) load_tile(LH ? j - 1 : j + 1, a_next);
    if (q < cols) {
      const C xq = xs[q];
#pragma unroll
      for (int i = 0; i < kPer; ++i) acc[i] = cfms(acc[i], cmake<C>(a_cur[i].x, -a_cur[i].y), xq);
    }
#pragma unroll
    for (int i = 0; i < kPer; ++i) a_cur[i] = a_next[i];
    __syncthreads();
  }
  // -sum over the tile columns of T x: each warp holds half of the columns for the
  // rows of its group g
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    R re = acc[i].x, im = acc[i].y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_xor_sync(0xffffffffu, re, o);
      im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if ((tid & 31) == 0) part[q >> 5][g + 4 * i] = cmake<C>(re, im);
  }
  __syncthreads();
  if (tid < 32) {
    C s0 = cmake<C>(0, 0), s1 = cmake<C>(0, 0);
    if (tid < rows) {
      const C b0 = x[r0 + tid];
      s0 = cmake<C>(b0.x + (part[0][tid].x + part[1][tid].x), b0.y + (part[0][tid].y + part[1][tid].y));
    }
    if (tid + 32 < rows) {
      const int qq = tid + 32;
      const C b1 = x[r0 + qq];
      s1 = cmake<C>(b1.x + (part[0][qq].x + part[1][qq].x), b1.y + (part[0][qq].y + part[1][qq].y));
    }
    if (!LH) {
      auto div_diag = [&](C a, int c) -> C {
        const R qq = dg_r[c], inv = dg_inv[c];
        return dg_sw[c] ? cmake<C>((a.x * qq + a.y) * inv, (a.y * qq - a.x) * inv)
                        : cmake<C>((a.x + a.y * qq) * inv, (a.y - a.x * qq) * inv);
      };
      for (int c = 0; c < rows; ++c) {
        if (c < 32) {
          if (tid == c) s0 = div_diag(s0, c);
        } else {
          if (tid + 32 == c) s1 = div_diag(s1, c);
        }
        const R xr = __shfl_sync(0xffffffffu, c < 32 ? s0.x : s1.x, c & 31);
        const R xi = __shfl_sync(0xffffffffu, c < 32 ? s0.y : s1.y, c & 31);
        const C xc = cmake<C>(xr, xi);
        if (tid > c && tid < rows) s0 = cfms(s0, Ds[c * kTrsvLd + tid], xc);
        if (tid + 32 > c && tid + 32 < rows) s1 = cfms(s1, Ds[c * kTrsvLd + tid + 32], xc);
      }
    } else {
      for (int c = rows - 1; c >= 0; --c) {
        const R xr = __shfl_sync(0xffffffffu, c < 32 ? s0.x : s1.x, c & 31);
        const R xi = __shfl_sync(0xffffffffu, c < 32 ? s0.y : s1.y, c & 31);
        const C xc = cmake<C>(xr, xi);
        if (tid < c && tid < rows) s0 = cfms(s0, Ds[c * kTrsvLd + tid], xc);
        if (tid + 32 < c && tid + 32 < rows) s1 = cfms(s1, Ds[c * kTrsvLd + tid + 32], xc);
      }
    }
    if (tid < rows) x[r0 + tid] = s0;
    if (tid + 32 < rows) x[r0 + tid + 32] = s1;
    __threadfence();
  }
  __syncthreads();
  if (tid == 0) st_release_i32(&flags[b], epoch);
}

// dst[c][perm[c][i]] = src[c][i]: x = P^T z for the vectors of a batch (column c of
// the compact src goes to vector sel[c] of dst, or c)
template <typename C>
__global__ void scatter_rows_kernel(const C* __restrict__ src, C* __restrict__ dst, const int* __restrict__ perm,
                                    int n, const int* __restrict__ sel) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i >= n) return;
  const int p = perm[(size_t)c * n + i];
  if (p >= 0 && p < n) dst[(size_t)(sel ? sel[c] : c) * n + p] = src[(size_t)c * n + i];
}

// ------------------------------------------------------- permutation ----
// perm[i] = original row that ends up in row i after the interchanges ipiv[0..n).
__global__ void pivots_to_perm_kernel(const int* __restrict__ ipiv, int n, int* __restrict__ perm,
                                      const int* __restrict__ sel) {
  extern __shared__ int sp[];
  // one block per matrix of a batch (sel: the batch's matrices, else all)
  ipiv += (size_t)(sel ? sel[blockIdx.x] : (int)blockIdx.x) * n;
  perm += (size_t)blockIdx.x * n;
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
                                   long long ldd, const int* __restrict__ perm, int n, int nrhs,
                                   int perm_stride, const int* __restrict__ sel, int perm_by_matrix = 0) {
  // column c: a right-hand side of one matrix (perm_stride 0) or the right-hand
  // side of matrix c of a batch (perm_stride n; with sel, of matrix sel[c], whose
  // vector is column sel[c] of dst).  The permutations are one per column, or with
  // perm_by_matrix one per matrix of the whole batch (precomputed, lu_pivots_to_perm)
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  const int cd = sel ? sel[c] : c;
  const int pc = perm_by_matrix ? cd : c;
  if (i < n && c < nrhs) dst[(size_t)cd * ldd + i] = src[(size_t)c * lds + perm[(size_t)pc * perm_stride + i]];
}

// dst[c] = src[sel[c]] for the n-vectors of the selected matrices of a batch
template <typename C>
__global__ void gather_vecs_kernel(const C* __restrict__ src, int n, C* __restrict__ dst,
                                   const int* __restrict__ sel) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i < n) dst[(size_t)c * n + i] = src[(size_t)sel[c] * n + i];
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
  // barrier + stage of one matrix, sized for the larger (FP64) configuration
  (void)elem_bytes;
  return sizeof(GridBarrier) + 256 + sizeof(PanelStage<double2, 64>) + 256;
}

// Dynamic shared memory of panel_kernel: the block's rows, the pivot row and, for
// FP32, the gathered candidates (rows, values, row numbers) and the diagonal row.
template <typename C, int NB>
size_t panel_smem(int rpc, int P) {
  using R = decltype(C{}.x);
  size_t bytes = (size_t)rpc * NB * sizeof(C) + NB * sizeof(C);
  if (sizeof(R) == 4) bytes += (size_t)P * NB * sizeof(C) + NB * sizeof(C) + (size_t)P * (sizeof(R) + sizeof(int));
  return bytes;
}

// Launch shape of one panel of m rows.  FP32: the row-owner kernel with one row per
// thread (rpc <= NT) while its shared memory fits.  Otherwise panel_kernel with at
// least kMinRows rows per block: FP64 rank-1 updates are costly, so many blocks share
// them; FP32 panels are latency-bound, so fewer blocks make each barrier cheaper.
// WMOM_NO_CLUSTER_PANEL=1 keeps the FP32 panels on the cooperative kernels.
// WMOM_PANEL_LOOKAHEAD=0 selects the cluster panel without the one-column look-ahead
// (same factors bit for bit).
bool panel_lookahead() {
  const char* e = std::getenv("WMOM_PANEL_LOOKAHEAD");
  return !(e && e[0] == '0');
}

// Widest FP64 cluster panel: WMOM_FP64_PANEL_W (16 .. 32, a multiple of 8) if set,
// else the workspace's choice (LuWorkspace::panel_w64), else 32 columns.  The panel's
// rank-1 updates run on GB300's narrow FP64 pipe, and their work grows with the width.
int fp64_panel_width(int ws_choice) {
  static const int env = [] {
    const char* e = std::getenv("WMOM_FP64_PANEL_W");
    const int v = e ? std::atoi(e) : 0;
    return v >= 16 && v <= 32 ? (v & ~7) : 0;
  }();
  if (env) return env;
  return ws_choice >= 16 && ws_choice <= 32 ? (ws_choice & ~7) : 32;
}

bool cluster_panels_disabled() {
  const char* e = std::getenv("WMOM_NO_CLUSTER_PANEL");
  return e && e[0] == '1';
}

struct PanelLaunch {
  bool rows = false;
  bool cluster = false;  // panel_cluster_kernel: P = cluster size
  int rpt = 1;           // rows per thread of panel_cluster_kernel
  int P = 1, rpc = 1;
  int w = 64;            // panel width
  size_t smem = 0;
};

template <bool FFS>
__global__ void panel_cluster_la_ff_kernel(double2* __restrict__ A, long long lda, int n, int j0, int w, int rpc,
                                           int* __restrict__ ipiv, GridBarrier* __restrict__ gb,
                                           long long astride);

// The second tier's panels in float-float arithmetic (panel_cluster_la_ff_kernel);
// WMOM_FF_PANEL=0 keeps them in FP64 (read at every panel, so that a test can
// compare both in one process).
bool ff_panels() {
  const char* e = std::getenv("WMOM_FF_PANEL");
  return !(e && e[0] == '0');
}

// With float-float panels, the second tier's block solves in float-float arithmetic as
// well (trsm_lower_ff_kernel<false>); WMOM_FF_TRSM=0 keeps them in FP64.
bool ff_trsm() {
  const char* e = std::getenv("WMOM_FF_TRSM");
  return ff_panels() && !(e && e[0] == '0');
}

// Largest cluster size this device schedules for panel_cluster_kernel (8 is the
// portable limit; 16 where the device allows it), probed once per device.
int max_cluster_size(const DeviceLimits& lim) {
  static std::mutex mu;
  static std::map<int, int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(dev);
  if (it != cache.end()) return it->second;
  int best = 0;
  const size_t smem = (size_t)lim.smem_optin - 4096;
  auto prepare = [&](const void* k) {
    return allow_dynamic_smem(k, smem) == cudaSuccess &&
           cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
  };
  if (prepare((const void*)panel_cluster_kernel<float2, 1>) && prepare((const void*)panel_cluster_kernel<float2, 2>) &&
      prepare((const void*)panel_cluster_kernel<double2, 1>) &&
      prepare((const void*)panel_cluster_la_kernel<float2, 1>) &&
      prepare((const void*)panel_cluster_la_kernel<float2, 2>) &&
      prepare((const void*)panel_cluster_la_kernel<double2, 1>) &&
      prepare((const void*)panel_cluster_la_ff_kernel<false>) && prepare((const void*)panel_cluster_la_ff_kernel<true>)) {
    for (int cs = kClusterMax; cs >= 1 && !best; cs /= 2) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(cs, 1, 1);
      cfg.blockDim = dim3(kClusterThreads, 1, 1);
      cfg.dynamicSmemBytes = smem;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = cs;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      int nclusters = 0;
      if (cudaOccupancyMaxActiveClusters(&nclusters, (const void*)panel_cluster_kernel<float2, 1>, &cfg) ==
              cudaSuccess &&
          nclusters >= 1)
        best = cs;
    }
  }
  cudaGetLastError();
  cache[dev] = best;
  return best;
}

// Clusters of cs CTAs of `kern` (kClusterThreads threads, smem bytes each) that can
// be resident at once (cudaOccupancyMaxActiveClusters; no launch), cached per
// device.  A cluster sits inside one GPC, so on a GB300 at one CTA per SM only 7
// clusters of 16 CTAs fit, 13 of 10 and 15 of 8, not 152 / cs.
int active_clusters(const void* kern, int cs, size_t smem) {
  static std::mutex mu;
  static std::map<std::tuple<int, const void*, int, size_t>, int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  const auto key = std::make_tuple(dev, kern, cs, (smem + 1023) / 1024);
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int n = 0;
  if (allow_dynamic_smem(kern, smem) == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs, 1, 1);
    cfg.blockDim = dim3(kClusterThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) n = 0;
  }
  cudaGetLastError();
  cache[key] = n;
  return n;
}

// batch: the matrices of the launch (0: not known).  Cluster panels with one row per
// thread then take, where their default cluster (the smallest power of two holding
// the rows, or for the FP64 / float-float panels the rows at the target height) cannot
// hold the whole batch at once, the smallest cluster of any size that can, at the
// same width: so that the batch runs in one wave instead of two.  The panel's results
// do not depend on the cluster size (each row's arithmetic is the same in whichever
// CTA holds it, and the pivot search breaks ties by row index), only on the width,
// which stays.
template <typename C>
PanelLaunch panel_launch(int m, const DeviceLimits& lim, bool fp64_cluster = false, int wmax = 0,
                         int wmax64 = 0, int batch = 0) {
  constexpr int NB = PanelCfg<C>::NB;
  constexpr int NT = PanelCfg<C>::NT;
  using R = decltype(C{}.x);
  PanelLaunch pl;
  const size_t cap = (size_t)lim.smem_optin - 4096;
  if (!cluster_panels_disabled() && (sizeof(R) == 4 || fp64_cluster)) {
    // FP32: one row per thread in the smallest cluster (the cluster barrier and the
    // remote reads cost more per column as the cluster grows); two rows per thread
    // only for panels taller than 16 x 512 rows, which would otherwise need the
    // cooperative kernel.  Two rows per thread in 8 CTAs instead of one in 16 for an
    // N = 8192 batch of 12 was measured: the panel became 40% faster, but its
    // 24-column width cost more in triangular solves, updates and launches.  The panel
    // is 64 columns wide where the rows leave room, else narrower.
    // FP64 (only with a tensor-core trailing update, fp64_cluster): the rank-1 row
    // updates run on the FP64 pipe (about 2 FMA per clock per SM), so the cluster
    // starts at about 256 rows per CTA (more SMs per matrix) and the panel is at most
    // 32 columns wide (its FP64 work grows with the width; the tensor-core updates
    // take K = span x width).  The plain FP64 form keeps the cooperative 64-column
    // panels: its SIMT FP64 update loses more at K = 24-32 than the narrow cluster
    // panels save (measured 0.64 vs 0.76 freq-solves/s at N = 8192, 24.0 vs 27.3 at
    // N = 2048).
    const int csmax = max_cluster_size(lim);
    // publication slots, two pivot rows and the diagonal row (the look-ahead kernel's
    // layout; the other kernel uses one pivot row less)
    const size_t head = 2 * sizeof(ClusterPub<C>) + 3 * 64 * sizeof(C);
    // FP32 panels: at most wmax columns when the tuner chose narrower ones
    const int wcap = sizeof(R) == 4 ? (wmax >= 16 && wmax < 64 ? wmax : 64) : fp64_panel_width(wmax64);
    auto try_shape = [&](int rpt, int cs_lo, int cs_hi, int wmin) -> bool {
      for (int cs = cs_lo; cs <= std::min(cs_hi, csmax); cs *= 2) {
        const int rpc = (m + cs - 1) / cs;
        if (rpc > rpt * kClusterThreads || (rpt > 1 && rpc <= kClusterThreads)) continue;
        int w = (int)std::min<size_t>(wcap, (cap - head) / ((size_t)rpc * sizeof(C)));
        if (w < wcap) w &= ~7;
        if (w < wmin) continue;
        pl.cluster = true;
        pl.rpt = rpt;
        pl.P = cs;
        pl.rpc = rpc;
        pl.w = w;
        pl.smem = head + (size_t)rpc * w * sizeof(C);
        return true;
      }
      return false;
    };
    // a batch that the chosen cluster size cannot hold at once: the smallest cluster of
    // any size that can, one row per thread, at the same width
    auto one_wave = [&](const void* kern) {
      if (batch <= 1 || pl.rpt != 1 || active_clusters(kern, pl.P, pl.smem) >= batch) return;
      const int rows_fit = (int)std::min<size_t>(kClusterThreads, (cap - head) / ((size_t)pl.w * sizeof(C)));
      for (int cs = std::max(1, (m + rows_fit - 1) / rows_fit); cs <= std::min(kClusterMax, csmax); ++cs) {
        const int rpc = (m + cs - 1) / cs;
        const size_t smem = head + (size_t)rpc * pl.w * sizeof(C);
        if (rpc > kClusterThreads || smem > cap) continue;
        if (active_clusters(kern, cs, smem) >= batch) {
          pl.P = cs;
          pl.rpc = rpc;
          pl.smem = smem;
          return;
        }
      }
    };
    if (sizeof(R) == 4) {
      if (try_shape(1, 1, kClusterMax, 32)) {
        one_wave((const void*)panel_cluster_la_kernel<float2, 1>);
        return pl;
      }
      if (try_shape(2, 1, kClusterMax, 24)) return pl;
    } else {
      // rows per CTA: 256 for the FP64 panel (its rank-1 updates want the SMs); the
      // float-float panel, whose updates run on the FP32 pipe, takes 512 where the
      // whole panel width fits at that height (fewer CTAs meet at each column's
      // cluster barrier; N = 8192 grid, 24-column panels: 835 -> 830 ms per step)
      static const int env_target = [] {
        const char* e = std::getenv("WMOM_FP64_PANEL_ROWS");
        const int v = e ? std::atoi(e) : 0;
        return v >= 16 && v <= 512 ? v : 0;
      }();
      const int target = env_target ? env_target
                         : (ff_panels() && (size_t)kClusterThreads * wcap * sizeof(C) + head <= cap) ? 512
                                                                                                   : 256;
      int cs0 = 1;
      while (cs0 < kClusterMax && (m + cs0 - 1) / cs0 > target) cs0 *= 2;
      if (try_shape(1, cs0, kClusterMax, 16)) {
        one_wave(ff_panels() ? (const void*)panel_cluster_la_ff_kernel<false>
                             : (const void*)panel_cluster_la_kernel<double2, 1>);
        return pl;
      }
    }
  }
  if (sizeof(R) == 4) {
    const int P = (m + NT - 1) / NT;
    const int rpc = (m + P - 1) / P;
    const size_t smem = ((size_t)rpc + (size_t)P + 1) * NB * sizeof(C) + (size_t)P * (sizeof(R) + sizeof(int));
    if (P <= std::min(lim.sms, kMaxPanelBlocks) && smem <= cap) {
      pl.rows = true;
      pl.P = P;
      pl.rpc = rpc;
      pl.smem = smem;
      return pl;
    }
  }
  constexpr int kMinRows = sizeof(R) == 8 ? 16 : 128;
  int P = std::max(1, std::min({lim.sms, kMaxPanelBlocks, (m + kMinRows - 1) / kMinRows}));
  int rpc = (m + P - 1) / P;
  size_t smem = (size_t)rpc * NB * sizeof(C) + NB * sizeof(C);
  while (smem > cap && P < std::min(lim.sms, kMaxPanelBlocks)) {
    ++P;
    rpc = (m + P - 1) / P;
    smem = (size_t)rpc * NB * sizeof(C) + NB * sizeof(C);
  }
  pl.P = (m + rpc - 1) / rpc;
  pl.rpc = rpc;
  pl.smem = panel_smem<C, NB>(rpc, pl.P);
  return pl;
}

size_t lu_stage_offset(int max_batch) {
  return ((size_t)max_batch * sizeof(GridBarrier) + 255) & ~(size_t)255;
}

size_t lu_stage_bytes(int max_batch) { return (size_t)max_batch * sizeof(PanelStage<double2, 64>); }

template <typename C>
cudaError_t lu_factor_t(C* A, long long lda, int n, int* ipiv, LuWorkspace* ws, cudaStream_t s,
                        GemmHook<C> gemm_hook, int batch, long long astride, int span) {
  constexpr int NB = PanelCfg<C>::NB;
  constexpr int NT = PanelCfg<C>::NT;
  using Stage = PanelStage<C, NB>;
  if (batch < 1 || batch > ws->max_batch || (batch > 1 && astride < lda * (long long)n))
    return cudaErrorInvalidValue;
  const DeviceLimits lim = device_limits();
  GridBarrier* gb = ws->barrier;
  Stage* st = reinterpret_cast<Stage*>(ws->stage);
  cudaError_t e;
  unsigned int bar_base = 0;  // arrivals of earlier panels on the counting barrier

  // panel of columns [jp, jp + w), rows jp..n-1 (cooperative launch)
  auto panel = [&](int jp, int w) -> cudaError_t {
    const int m = n - jp;
    const PanelLaunch pl = panel_launch<C>(m, lim, gemm_hook != nullptr, ws->panel_w, ws->panel_w64, batch);
    const int P = pl.P;
    if (ws->ff_storage && !pl.cluster) return cudaErrorInvalidValue;  // see ff_tier2_supported
    {
      if (pl.cluster) {
        if (w > pl.w) return cudaErrorInvalidValue;
        const bool la = panel_lookahead();
        const void* ck = la ? (pl.rpt == 2 ? (const void*)panel_cluster_la_kernel<C, 2>
                                           : (const void*)panel_cluster_la_kernel<C, 1>)
                            : (pl.rpt == 2 ? (const void*)panel_cluster_kernel<C, 2>
                                           : (const void*)panel_cluster_kernel<C, 1>);
        cudaError_t ce = allow_dynamic_smem(ck, pl.smem);
        if (ce != cudaSuccess) return ce;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(P, batch, 1);
        cfg.blockDim = dim3(kClusterThreads, 1, 1);
        cfg.dynamicSmemBytes = pl.smem;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = P;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        stats::Scope sc(stats::kPanel, s, 8.0 * m * (double)w * w / 2.0 * batch);
        if constexpr (std::is_same<C, double2>::value) {
          if (ws->ff_storage) {
            // float-float storage is only set up for these panels (ff_tier2_supported)
            if (!(la && pl.rpt == 1 && gemm_hook != nullptr)) return cudaErrorInvalidValue;
            ce = allow_dynamic_smem((const void*)panel_cluster_la_ff_kernel<true>, pl.smem);
            if (ce != cudaSuccess) return ce;
            return cudaLaunchKernelEx(&cfg, panel_cluster_la_ff_kernel<true>, A, lda, n, jp, w, pl.rpc, ipiv, gb,
                                      astride);
          }
          if (la && pl.rpt == 1 && gemm_hook != nullptr && ff_panels()) {
            ce = allow_dynamic_smem((const void*)panel_cluster_la_ff_kernel<false>, pl.smem);
            if (ce != cudaSuccess) return ce;
            return cudaLaunchKernelEx(&cfg, panel_cluster_la_ff_kernel<false>, A, lda, n, jp, w, pl.rpc, ipiv, gb,
                                      astride);
          }
        }
        if (la)
          return pl.rpt == 2 ? cudaLaunchKernelEx(&cfg, panel_cluster_la_kernel<C, 2>, A, lda, n, jp, w, pl.rpc, ipiv,
                                                  gb, astride)
                             : cudaLaunchKernelEx(&cfg, panel_cluster_la_kernel<C, 1>, A, lda, n, jp, w, pl.rpc, ipiv,
                                                  gb, astride);
        return pl.rpt == 2 ? cudaLaunchKernelEx(&cfg, panel_cluster_kernel<C, 2>, A, lda, n, jp, w, pl.rpc, ipiv, gb,
                                                astride)
                           : cudaLaunchKernelEx(&cfg, panel_cluster_kernel<C, 1>, A, lda, n, jp, w, pl.rpc, ipiv, gb,
                                                astride);
      }
    }
    const void* kern = pl.rows ? (const void*)panel_rows_kernel<C, NB, NT> : (const void*)panel_kernel<C, NB, NT>;
    cudaError_t pe = allow_dynamic_smem(kern, pl.smem);
    if (pe != cudaSuccess) return pe;
    int per_sm = 0;
    pe = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, pl.smem);
    if (pe != cudaSuccess) return pe;
    if (per_sm * lim.sms < P * batch) return cudaErrorCooperativeLaunchTooLarge;
    C* Ap = A;
    long long ldap = lda, astr = astride;
    int np = n, j0p = jp, nbp = w, rpcp = pl.rpc;
    int* ipivp = ipiv;
    // a test may make every barrier of this panel wait for arrivals that never come
    // (bounded: the wait gives up and the factorisation reports a timeout)
    unsigned int basep = bar_base + g_panel_missing_arrivals.load(std::memory_order_relaxed);
    void* args[] = {&Ap, &ldap, &np, &j0p, &nbp, &rpcp, &ipivp, &st, &gb, &basep, &astr};
    {
      stats::Scope sc(stats::kPanel, s, 8.0 * m * (double)w * w / 2.0 * batch);
      pe = cudaLaunchCooperativeKernel(kern, dim3(P, batch), dim3(NT), args, pl.smem, s);
    }
    bar_base += (unsigned int)P * (unsigned int)w;
    return pe;
  };
  // the interchanges of panel [jp, jp + w) on every other column
  auto laswp = [&](int jp, int w) -> cudaError_t {
    const int other = n - w;
    if (other <= 0) return cudaSuccess;
    stats::Scope sc(stats::kLaswp, s, 2.0 * w * other * sizeof(C) * batch);
    laswp_kernel<C><<<dim3((other + 127) / 128, batch), 128, 0, s>>>(A, lda, n, jp, jp + w, jp, w, ipiv, astride, n);
    return cudaGetLastError();
  };
  // rows [jp, jp + w) of columns [c0, c0 + nc) <- L(jp..jp+w)^-1 times themselves
  auto trsm = [&](int jp, int w, int c0, int nc) -> cudaError_t {
    if (nc <= 0) return cudaSuccess;
    const C* T = A + (size_t)jp * lda + jp;
    C* Bb = A + (size_t)c0 * lda + jp;
    cudaError_t te;
    if constexpr (std::is_same<C, float2>::value) {
      // one thread per column, L11 from shared memory, rows in register blocks of 16
      // (the same per-element order of updates as trsm_kernel, so the same results)
      const size_t tsmem = (64 * 64 + 64 * (kTrsmColThreads + 1)) * sizeof(C);
      te = allow_dynamic_smem((const void*)trsm_lower_cols_kernel<C>, tsmem);
      if (te != cudaSuccess) return te;
      stats::Scope sc(stats::kTrsm, s, 4.0 * w * (double)w * nc * batch);
      trsm_lower_cols_kernel<C><<<dim3((nc + kTrsmColThreads - 1) / kTrsmColThreads, batch), kTrsmColThreads,
                                  tsmem, s>>>(T, lda, Bb, lda, w, nc, astride, astride);
    } else {
      if (ws->ff_storage || (gemm_hook != nullptr && w <= 32 && ff_trsm())) {
        // the second tier: float-float arithmetic on the FP32 pipe, on float-float
        // storage or on complex128 (split on load, rounded back on store), for every
        // width up to 32.  Against the FP64 kernels below: N = 8192 grid, 9 second-tier
        // matrices, 51 ms per step in FP64; 256-frequency N = 2048 grid 145 ms.
        if (w > 32) return cudaErrorInvalidValue;
        const size_t fsmem = ((size_t)w * w + (size_t)w * kTrsmCols) * sizeof(Ffc);
        stats::Scope sc(stats::kTrsm, s, 4.0 * w * (double)w * nc * batch);
        if (ws->ff_storage)
          trsm_lower_ff_kernel<true><<<dim3((nc + kTrsmCols - 1) / kTrsmCols, batch), 256, fsmem, s>>>(
              T, lda, Bb, lda, w, nc, astride, astride);
        else
          trsm_lower_ff_kernel<false><<<dim3((nc + kTrsmCols - 1) / kTrsmCols, batch), 256, fsmem, s>>>(
              T, lda, Bb, lda, w, nc, astride, astride);
        return cudaGetLastError();
      }
      // FP64: the work is bound by the SMs' FP64 pipes.  Panels of 8 .. 32 columns
      // (the second tier's) take the one-warp, column-in-registers kernel when their
      // columns give every SM at least two warps; narrower right-hand sides (the
      // in-group solves of `span` panels, the late trailing columns) and wider
      // panels (the plain form's cooperative 64-column ones) spread their rows over
      // CTAs of 16 columns (the FP32 one-thread-per-column kernel, 128 columns per
      // CTA, pads to 64 rows and was 4x slower on the second tier's late panels).
      // Measured on the N = 8192 grid (9 second-tier matrices) and the 256-frequency
      // N = 2048 grid, trsm class: 71 / 172 ms with trsm_kernel alone, 66 / 196 with
      // the register kernel on every solve (a one-warp block is too little FP64 work
      // for the 24-column in-group solves), 51 / 143 with this choice.
      const long long warps = (long long)((nc + 31) / 32) * batch;
      if ((w == 8 || w == 16 || w == 24 || w == 32) && warps >= 2LL * lim.sms) {
        bool done = false;
        stats::Scope sc(stats::kTrsm, s, 4.0 * w * (double)w * nc * batch);
        te = trsm_lower_reg<C>(T, lda, Bb, lda, w, nc, astride, astride, batch, s, &done);
        if (done) return te;
      }
      const size_t tsmem = ((size_t)w * w + (size_t)w * kTrsmCols) * sizeof(C);
      te = allow_dynamic_smem((const void*)trsm_kernel<C, false>, tsmem);
      if (te != cudaSuccess) return te;
      stats::Scope sc(stats::kTrsm, s, 4.0 * w * (double)w * nc * batch);
      trsm_kernel<C, false><<<dim3((nc + kTrsmCols - 1) / kTrsmCols, batch), 256, tsmem, s>>>(T, lda, Bb, lda, w, nc,
                                                                                             astride, astride);
    }
    return cudaGetLastError();
  };
  // A[r0:r0+M, c0:c0+N] -= A[r0:r0+M, k0:k0+K] * A[k0:k0+K, c0:c0+N]
  auto update = [&](int r0, int c0, int M, int N, int k0, int K) -> cudaError_t {
    if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
    const C* Am = A + (size_t)k0 * lda + r0;
    const C* Bm = A + (size_t)c0 * lda + k0;
    C* Cm = A + (size_t)c0 * lda + r0;
    if (gemm_hook) return gemm_hook(ws, Am, lda, Bm, lda, Cm, lda, M, N, K, s, batch, astride);
    if constexpr (std::is_same<C, double2>::value)
      if (fp64_update_dmma()) return zgemm_sub_dmma(Am, lda, Bm, lda, Cm, lda, M, N, K, s, batch, astride);
    stats::Scope sc(stats::kGemm, s, 8.0 * M * (double)N * K * batch);
    dim3 grid((M + kGemmBM - 1) / kGemmBM, (N + kGemmBN - 1) / kGemmBN, batch);
    gemm_sub_kernel<C><<<grid, 256, 0, s>>>(Am, lda, Bm, lda, Cm, lda, M, N, K, astride);
    return cudaGetLastError();
  };
#define LU_TRY(x)                  \
  do {                             \
    e = (x);                       \
    if (e != cudaSuccess) return e; \
  } while (0)

  // With the tensor-core update, `span` panels share one trailing update (K = span
  // NB): inside the group each panel is brought up to date by thin updates from the
  // group's earlier panels, so the large update reads and writes the trailing matrix
  // 1/span as often.  Without the hook (FP64 SIMT GEMM,
  // bound by the FP64 pipe rather than by traffic) span is 1.
  const int S = gemm_hook ? std::max(1, std::min(span > 0 ? span : 2, kMaxSpan)) : 1;
  for (int j0 = 0; j0 < n;) {
    int c[kMaxSpan + 1], w[kMaxSpan];
    int np = 0;
    c[0] = j0;
    while (np < S && c[np] < n) {
      w[np] = std::min(panel_launch<C>(n - c[np], lim, gemm_hook != nullptr, ws->panel_w, ws->panel_w64).w,
                       n - c[np]);
      c[np + 1] = c[np] + w[np];
      ++np;
    }
    const int cr = c[np], rest = n - cr;
    for (int q = 0; q < np; ++q) {
      // panel q, then its U rows and its update for all the group's later panels at
      // once (one solve and one GEMM over columns c[q+1] .. cr instead of one per later
      // panel).  Every entry of those columns still receives the updates of panels
      // 0, 1, .. in that order, and both kernels compute each column (the GEMM each
      // entry) on its own, so the factors are those of one panel at a time, bit for
      // bit, with fewer and wider launches.
      LU_TRY(panel(c[q], w[q]));
      LU_TRY(laswp(c[q], w[q]));
      if (q + 1 < np) {
        LU_TRY(trsm(c[q], w[q], c[q + 1], cr - c[q + 1]));
        LU_TRY(update(c[q + 1], c[q + 1], n - c[q + 1], cr - c[q + 1], c[q], w[q]));
      }
    }
    if (rest > 0) {
      // U rows of the group for the trailing columns, then one update with K = c[np] - j0
      for (int p = 0; p < np; ++p) {
        LU_TRY(trsm(c[p], w[p], cr, rest));
        if (p + 1 < np) LU_TRY(update(c[p + 1], cr, cr - c[p + 1], rest, c[p], w[p]));
      }
      LU_TRY(update(cr, cr, rest, rest, j0, cr - j0));
    }
    j0 = cr;
  }
#undef LU_TRY
  return cudaSuccess;
}

template <typename C>
cudaError_t lu_solve_t(const C* A, long long lda, int n, const int* ipiv, C* B, long long ldb, int nrhs,
                       LuWorkspace* ws, cudaStream_t s, int batch, long long astride, const int* sel,
                       const C* inv, const int* perm_pre) {
  constexpr int NB = PanelCfg<C>::NB;
  cudaError_t e;
  if (batch < 1 || batch > ws->max_batch || ((batch > 1 || sel) && (nrhs != 1 || ldb != n)))
    return cudaErrorInvalidValue;
  if (n > ws->perm_cap) return cudaErrorInvalidValue;
  if (sel && !(nrhs == 1 && ws->flags)) return cudaErrorInvalidValue;
  // row interchanges: B <- P B through a permutation gather into the scratch copy
  if ((size_t)n * sizeof(int) > 200 * 1024) return cudaErrorInvalidValue;
  e = allow_dynamic_smem((const void*)pivots_to_perm_kernel, (n * sizeof(int)));
  if (e != cudaSuccess) return e;
  const bool pre = perm_pre != nullptr;
  stats::count(stats::kMisc, pre ? 1 : 2);
  if (!pre) pivots_to_perm_kernel<<<batch, 256, n * sizeof(int), s>>>(ipiv, n, ws->perm, sel);
  C* tmp = reinterpret_cast<C*>(ws->rhs);
  const int ncol = (batch > 1 || sel) ? batch : nrhs;  // columns of the gathered block
  if ((size_t)n * ncol * sizeof(C) > ws->rhs_bytes) return cudaErrorInvalidValue;
  if (sel) {
    stats::count(stats::kMisc);
    gather_vecs_kernel<C><<<dim3((n + 255) / 256, ncol), 256, 0, s>>>(B, n, tmp, sel);
  } else {
    e = cudaMemcpy2DAsync(tmp, (size_t)n * sizeof(C), B, (size_t)ldb * sizeof(C), (size_t)n * sizeof(C), ncol,
                          cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  }
  if (pre)
    gather_rows_kernel<C><<<dim3((n + 255) / 256, ncol), 256, 0, s>>>(tmp, n, B, ldb, perm_pre, n, ncol,
                                                                       (batch > 1 || sel) ? n : 0, sel, 1);
  else
    gather_rows_kernel<C><<<dim3((n + 255) / 256, ncol), 256, 0, s>>>(tmp, n, B, ldb, ws->perm, n, ncol,
                                                                       (batch > 1 || sel) ? n : 0, sel);
  if (nrhs == 1 && ws->flags) {
    const int nblk = (n + kTrsvB - 1) / kTrsvB;
    if (nblk > ws->flag_cap) return cudaErrorInvalidValue;
    const size_t dsmem = sizeof(C) * kTrsvB * kTrsvB;
    e = allow_dynamic_smem((const void*)trsv_kernel<C, false>, dsmem);
    if (e != cudaSuccess) return e;
    e = allow_dynamic_smem((const void*)trsv_kernel<C, true>, dsmem);
    if (e != cudaSuccess) return e;
    stats::Scope sc(stats::kTrsv, s, 8.0 * n * (double)n * batch, 2);
    for (int pass = 0; pass < 2; ++pass) {
      const int ep = ++ws->epoch;
      e = cudaMemsetAsync(ws->ticket, 0, sizeof(unsigned int) * batch, s);
      if (e != cudaSuccess) return e;
      if (pass == 0)
        trsv_kernel<C, false><<<nblk * batch, 256, dsmem, s>>>(A, lda, n, B, ws->flags, ws->ticket, ep,
                                                               &ws->barrier->err, astride, ws->flag_cap, sel, inv);
      else
        trsv_kernel<C, true><<<nblk * batch, 256, dsmem, s>>>(A, lda, n, B, ws->flags, ws->ticket, ep,
                                                              &ws->barrier->err, astride, ws->flag_cap, sel, inv);
    }
    return cudaGetLastError();
  }
  const size_t tsmem = ((size_t)NB * NB + (size_t)NB * kTrsmCols) * sizeof(C);
  e = allow_dynamic_smem((const void*)trsm_kernel<C, false>, tsmem);
  if (e != cudaSuccess) return e;
  e = allow_dynamic_smem((const void*)trsm_kernel<C, true>, tsmem);
  if (e != cudaSuccess) return e;
  // forward: L unit lower
  const int nblocks = (n + NB - 1) / NB;
  stats::Scope sc(stats::kTrsm, s, 8.0 * n * (double)n * nrhs, 4 * nblocks - 2);
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int kb = std::min(NB, n - k0);
    const size_t sm = ((size_t)kb * kb + (size_t)kb * kTrsmCols) * sizeof(C);
    trsm_kernel<C, false><<<(nrhs + kTrsmCols - 1) / kTrsmCols, 256, sm, s>>>(
        A + (size_t)k0 * lda + k0, lda, B + k0, ldb, kb, nrhs, 0, 0);
    const int below = n - k0 - kb;
    if (below > 0) {
      dim3 grid((below + kGemmBM - 1) / kGemmBM, (nrhs + kGemmBN - 1) / kGemmBN);
      gemm_sub_kernel<C><<<grid, 256, 0, s>>>(A + (size_t)k0 * lda + k0 + kb, lda, B + k0, ldb, B + k0 + kb,
                                              ldb, below, nrhs, kb, 0);
    }
  }
  // backward: U non-unit upper
  const int nblk = (n + NB - 1) / NB;
  for (int bi = nblk - 1; bi >= 0; --bi) {
    const int k0 = bi * NB;
    const int kb = std::min(NB, n - k0);
    const size_t sm = ((size_t)kb * kb + (size_t)kb * kTrsmCols) * sizeof(C);
    trsm_kernel<C, true><<<(nrhs + kTrsmCols - 1) / kTrsmCols, 256, sm, s>>>(
        A + (size_t)k0 * lda + k0, lda, B + k0, ldb, kb, nrhs, 0, 0);
    if (k0 > 0) {
      dim3 grid((k0 + kGemmBM - 1) / kGemmBM, (nrhs + kGemmBN - 1) / kGemmBN);
      gemm_sub_kernel<C><<<grid, 256, 0, s>>>(A + (size_t)k0 * lda, lda, B + k0, ldb, B, ldb, k0, nrhs, kb, 0);
    }
  }
  return cudaGetLastError();
}

cudaError_t ff_block_inverses(const float4* A, long long lda, int n, int batch, long long astride, float4* inv,
                              cudaStream_t s) {
  if (n <= 0 || batch < 1 || batch > 65535 || !inv) return cudaErrorInvalidValue;
  const int nblk = (n + kTrsvB - 1) / kTrsvB;
  cudaError_t e = allow_dynamic_smem((const void*)tri_inv_ff_kernel, kTriInvSmem);
  if (e != cudaSuccess) return e;
  stats::count(stats::kMisc);
  tri_inv_ff_kernel<<<dim3(nblk, batch, 2), 4 * kTrsvB, kTriInvSmem, s>>>(A, lda, n, astride, inv);
  return cudaGetLastError();
}

size_t ff_block_inverse_bytes(int n, int batch) {
  return (size_t)batch * ((n + kTrsvB - 1) / kTrsvB) * 2 * kTrsvB * kTrsvB * sizeof(float4);
}

template <typename C>
cudaError_t lu_block_inverses(const C* A, long long lda, int n, int batch, long long astride, C* inv,
                              cudaStream_t s) {
  if (n <= 0 || batch < 1 || batch > 65535 || !inv) return cudaErrorInvalidValue;
  const int nblk = (n + kTrsvB - 1) / kTrsvB;
  const size_t smem = sizeof(C) * ((size_t)kTrsvB * kTrsvB + (size_t)kTrsvB * kInvLd);
  cudaError_t e = allow_dynamic_smem((const void*)tri_inv_kernel<C>, smem);
  if (e != cudaSuccess) return e;
  stats::count(stats::kMisc);
  tri_inv_kernel<C><<<dim3(nblk, batch, 2), 4 * kTrsvB, smem, s>>>(A, lda, n, astride, inv);
  return cudaGetLastError();
}

template <typename C>
size_t lu_block_inverse_bytes(int n, int batch) {
  return (size_t)batch * ((n + kTrsvB - 1) / kTrsvB) * 2 * kTrsvB * kTrsvB * sizeof(C);
}

template cudaError_t lu_block_inverses<float2>(const float2*, long long, int, int, long long, float2*, cudaStream_t);
template size_t lu_block_inverse_bytes<float2>(int, int);

cudaError_t lu_pivots_to_perm(const int* ipiv, int n, int batch, int* perm, cudaStream_t s) {
  if (n <= 0 || batch < 1 || batch > 65535 || !perm || (size_t)n * sizeof(int) > 200 * 1024)
    return cudaErrorInvalidValue;
  cudaError_t e = allow_dynamic_smem((const void*)pivots_to_perm_kernel, (n * sizeof(int)));
  if (e != cudaSuccess) return e;
  stats::count(stats::kMisc);
  pivots_to_perm_kernel<<<batch, 256, n * sizeof(int), s>>>(ipiv, n, perm, nullptr);
  return cudaGetLastError();
}

cudaError_t lu_solve_ff(const float4* A, long long lda, int n, const int* ipiv, double2* B, LuWorkspace* ws,
                        cudaStream_t s, int batch, long long astride, const int* sel, const float4* inv,
                        const int* perm_pre) {
  if (batch < 1 || batch > ws->max_batch || !ws->flags || n > ws->perm_cap) return cudaErrorInvalidValue;
  if ((size_t)n * sizeof(int) > 200 * 1024) return cudaErrorInvalidValue;
  if ((size_t)n * batch * sizeof(double2) > ws->rhs_bytes) return cudaErrorInvalidValue;
  const int nblk = (n + kTrsvB - 1) / kTrsvB;
  if (nblk > ws->flag_cap) return cudaErrorInvalidValue;
  cudaError_t e = allow_dynamic_smem((const void*)pivots_to_perm_kernel, (n * sizeof(int)));
  if (e != cudaSuccess) return e;
  // B <- P B, as lu_solve_t's single-right-hand-side path
  stats::count(stats::kMisc, perm_pre ? 1 : 2);
  if (!perm_pre) pivots_to_perm_kernel<<<batch, 256, n * sizeof(int), s>>>(ipiv, n, ws->perm, sel);
  double2* tmp = reinterpret_cast<double2*>(ws->rhs);
  if (sel) {
    stats::count(stats::kMisc);
    gather_vecs_kernel<double2><<<dim3((n + 255) / 256, batch), 256, 0, s>>>(B, n, tmp, sel);
  } else {
    e = cudaMemcpyAsync(tmp, B, sizeof(double2) * (size_t)n * batch, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  }
  gather_rows_kernel<double2><<<dim3((n + 255) / 256, batch), 256, 0, s>>>(
      tmp, n, B, n, perm_pre ? perm_pre : ws->perm, n, batch, n, sel, perm_pre ? 1 : 0);
  const size_t dsmem = sizeof(Ffc) * kTrsvB * kTrsvB;
  e = allow_dynamic_smem((const void*)trsv_ff_kernel<false>, dsmem);
  if (e != cudaSuccess) return e;
  e = allow_dynamic_smem((const void*)trsv_ff_kernel<true>, dsmem);
  if (e != cudaSuccess) return e;
  stats::Scope sc(stats::kTrsv, s, 8.0 * n * (double)n * batch, 2);
  for (int pass = 0; pass < 2; ++pass) {
    const int ep = ++ws->epoch;
    e = cudaMemsetAsync(ws->ticket, 0, sizeof(unsigned int) * batch, s);
    if (e != cudaSuccess) return e;
    if (pass == 0)
      trsv_ff_kernel<false><<<nblk * batch, 256, dsmem, s>>>(A, lda, n, B, ws->flags, ws->ticket, ep,
                                                             &ws->barrier->err, astride, ws->flag_cap, sel, inv);
    else
      trsv_ff_kernel<true><<<nblk * batch, 256, dsmem, s>>>(A, lda, n, B, ws->flags, ws->ticket, ep,
                                                            &ws->barrier->err, astride, ws->flag_cap, sel, inv);
  }
  return cudaGetLastError();
}

cudaError_t split_ff_inplace(double2* a, size_t count, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  stats::count(stats::kMisc);
  const unsigned blocks = (unsigned)std::min<size_t>((count + 255) / 256, 152 * 16);
  split_ff_kernel<<<blocks, 256, 0, s>>>(a, count);
  return cudaGetLastError();
}

cudaError_t merge_ff_inplace(double2* a, size_t count, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  stats::count(stats::kMisc);
  const unsigned blocks = (unsigned)std::min<size_t>((count + 255) / 256, 152 * 16);
  merge_ff_kernel<<<blocks, 256, 0, s>>>(a, count);
  return cudaGetLastError();
}

template <typename C>
cudaError_t lu_solve_h_t(const C* A, long long lda, int n, const int* ipiv, C* B, LuWorkspace* ws, cudaStream_t s,
                         int batch, long long astride, const int* sel) {
  if (batch < 1 || batch > ws->max_batch || !ws->flags || n > ws->perm_cap) return cudaErrorInvalidValue;
  if ((size_t)n * sizeof(int) > 200 * 1024) return cudaErrorInvalidValue;
  if ((size_t)n * batch * sizeof(C) > ws->rhs_bytes) return cudaErrorInvalidValue;
  const int nblk = (n + kTrsvB - 1) / kTrsvB;
  if (nblk > ws->flag_cap) return cudaErrorInvalidValue;
  const size_t dsmem = sizeof(C) * kTrsvB * kTrsvLd;
  cudaError_t e = allow_dynamic_smem((const void*)trsv_h_kernel<C, false>, dsmem);
  if (e != cudaSuccess) return e;
  e = allow_dynamic_smem((const void*)trsv_h_kernel<C, true>, dsmem);
  if (e != cudaSuccess) return e;
  e = allow_dynamic_smem((const void*)pivots_to_perm_kernel, (n * sizeof(int)));
  if (e != cudaSuccess) return e;
  {
    stats::Scope sc(stats::kTrsv, s, 8.0 * n * (double)n * batch, 2);
    for (int pass = 0; pass < 2; ++pass) {
      const int ep = ++ws->epoch;
      e = cudaMemsetAsync(ws->ticket, 0, sizeof(unsigned int) * batch, s);
      if (e != cudaSuccess) return e;
      if (pass == 0)
        trsv_h_kernel<C, false><<<nblk * batch, 256, dsmem, s>>>(A, lda, n, B, ws->flags, ws->ticket, ep,
                                                                 &ws->barrier->err, astride, ws->flag_cap, sel);
      else
        trsv_h_kernel<C, true><<<nblk * batch, 256, dsmem, s>>>(A, lda, n, B, ws->flags, ws->ticket, ep,
                                                                &ws->barrier->err, astride, ws->flag_cap, sel);
    }
  }
  // x = P^T z: the row each entry of z came from
  stats::count(stats::kMisc, 3);
  pivots_to_perm_kernel<<<batch, 256, n * sizeof(int), s>>>(ipiv, n, ws->perm, sel);
  C* tmp = reinterpret_cast<C*>(ws->rhs);
  if (sel) {
    gather_vecs_kernel<C><<<dim3((n + 255) / 256, batch), 256, 0, s>>>(B, n, tmp, sel);
  } else {
    e = cudaMemcpyAsync(tmp, B, (size_t)n * batch * sizeof(C), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  }
  scatter_rows_kernel<C><<<dim3((n + 255) / 256, batch), 256, 0, s>>>(tmp, B, ws->perm, n, sel);
  return cudaGetLastError();
}

template <typename C>
int lu_max_batch(int n, bool fp64_cluster) {
  constexpr int NB = PanelCfg<C>::NB;
  constexpr int NT = PanelCfg<C>::NT;
  const DeviceLimits lim = device_limits();
  if (lim.sms <= 0 || n <= 0) return 1;
  static std::mutex mu;
  static std::map<std::pair<int, int>, int> cache;  // (device, n, fp64_cluster) -> batch
  int dev = 0;
  cudaGetDevice(&dev);
  const std::pair<int, int> key{2 * dev + (fp64_cluster ? 1 : 0), n};
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  // every panel's cooperative launch must fit co-resident; shapes change as the
  // panels shrink, so the smallest batch over all of them is the limit
  int best = kMaxLuBatch;
  for (int j0 = 0; j0 < n && best > 1; j0 += NB) {
    const PanelLaunch pl = panel_launch<C>(n - j0, lim, fp64_cluster);
    if (pl.cluster) continue;  // clusters are independent of one another
    const void* kern = pl.rows ? (const void*)panel_rows_kernel<C, NB, NT> : (const void*)panel_kernel<C, NB, NT>;
    if (allow_dynamic_smem(kern, pl.smem) != cudaSuccess) return 1;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, pl.smem) != cudaSuccess) return 1;
    best = std::min(best, per_sm * lim.sms / pl.P);
  }
  best = std::max(1, best);
  std::lock_guard<std::mutex> lk(mu);
  cache[key] = best;
  return best;
}

// Whether the second tier's LU of order n can hold its matrix in float-float form:
// every panel must be a one-row-per-thread look-ahead cluster panel (the panels that
// read and write that form), i.e. cluster panels on, look-ahead on, and the tallest
// panel (n rows) within one cluster.
bool ff_tier2_supported(int n, int panel_w64) {
  if (cluster_panels_disabled() || !panel_lookahead()) return false;
  const DeviceLimits lim = device_limits();
  const PanelLaunch pl = panel_launch<double2>(n, lim, true, 0, panel_w64);
  return pl.cluster && pl.rpt == 1;
}

template int lu_max_batch<double2>(int, bool);
template int lu_max_batch<float2>(int, bool);

template cudaError_t lu_factor_t<double2>(double2*, long long, int, int*, LuWorkspace*, cudaStream_t,
                                          GemmHook<double2>, int, long long, int);
template cudaError_t lu_factor_t<float2>(float2*, long long, int, int*, LuWorkspace*, cudaStream_t,
                                         GemmHook<float2>, int, long long, int);
template cudaError_t lu_solve_t<double2>(const double2*, long long, int, const int*, double2*, long long, int,
                                         LuWorkspace*, cudaStream_t, int, long long, const int*, const double2*,
                                         const int*);
template cudaError_t lu_solve_t<float2>(const float2*, long long, int, const int*, float2*, long long, int,
                                         LuWorkspace*, cudaStream_t, int, long long, const int*, const float2*,
                                         const int*);
template cudaError_t lu_solve_h_t<double2>(const double2*, long long, int, const int*, double2*, LuWorkspace*,
                                           cudaStream_t, int, long long, const int*);
template cudaError_t lu_solve_h_t<float2>(const float2*, long long, int, const int*, float2*, LuWorkspace*,
                                          cudaStream_t, int, long long, const int*);


}  // namespace wmom
