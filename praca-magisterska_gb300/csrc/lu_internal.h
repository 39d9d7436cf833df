// lu_internal.h -- LU / solve entry points shared by the C ABI layer.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace wmom {

constexpr int kMaxPanelBlocks = 256;

struct GridBarrier;

// Device scratch of one factorisation stream: the panel kernel's grid barrier and
// candidate staging, the row permutation of a solve and a right-hand-side copy.
struct LuWorkspace {
  GridBarrier* barrier = nullptr;
  void* stage = nullptr;
  int* perm = nullptr;
  void* rhs = nullptr;
  size_t rhs_bytes = 0;
  int perm_cap = 0;
};

size_t lu_workspace_bytes(int elem_bytes);

// Optional replacement of the trailing-update GEMM (Cm -= Am * Bm).
template <typename C>
using GemmHook = cudaError_t (*)(const C* Am, long long lda, const C* Bm, long long ldb, C* Cm,
                                 long long ldc, int M, int N, int K, cudaStream_t s);

template <typename C>
cudaError_t lu_factor_t(C* A, long long lda, int n, int* ipiv, LuWorkspace* ws, cudaStream_t s,
                        GemmHook<C> gemm_hook);

template <typename C>
cudaError_t lu_solve_t(const C* A, long long lda, int n, const int* ipiv, C* B, long long ldb, int nrhs,
                       LuWorkspace* ws, cudaStream_t s);

// Workspace management (api.cu).
cudaError_t lu_workspace_create(LuWorkspace* ws, int nmax, int nrhs_max);
void lu_workspace_destroy(LuWorkspace* ws);
cudaError_t lu_workspace_reset_barrier(LuWorkspace* ws, cudaStream_t s);
int lu_workspace_read_status(LuWorkspace* ws, int* info, cudaStream_t s);

}  // namespace wmom
