// lu_internal.h -- LU / solve entry points shared by the C ABI layer.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstddef>

namespace wmom {

constexpr int kMaxPanelBlocks = 256;
constexpr int kMaxLuBatch = 32;  // matrices per batched factorisation

// Largest batch whose cooperative panel launches all fit co-resident on this device
// (cluster panels impose no limit).  fp64_cluster: the FP64 factorisation runs with
// a tensor-core trailing update, whose panels are cluster panels where they fit.
template <typename C>
int lu_max_batch(int n, bool fp64_cluster = false);

struct GridBarrier;

// Device scratch of one factorisation stream, for up to max_batch matrices of one
// batched factorisation: per matrix the panel kernel's grid barrier and candidate
// staging, the row permutation of a solve, and a right-hand-side copy.
struct LuWorkspace {
  GridBarrier* barrier = nullptr;  // [max_batch]
  void* stage = nullptr;           // [max_batch] panel staging (FP64-sized)
  int* perm = nullptr;             // [max_batch * perm_cap]
  void* rhs = nullptr;
  size_t rhs_bytes = 0;
  int perm_cap = 0;
  int max_batch = 1;
  // single-launch triangular solves: per-block ready flags (epoch-tagged), ticket
  int* flags = nullptr;            // [max_batch * flag_cap]
  unsigned int* ticket = nullptr;  // [max_batch]
  int flag_cap = 0;
  int epoch = 0;
  // tensor-core trailing update: packed TF32 operand planes, grown on first use
  // (never inside a stream capture; tc_gen counts reallocations, so that a captured
  // factorisation is replayed only over the buffer it was captured with) and the
  // flag its bounded waits set on timeout
  float* tc_buf = nullptr;
  size_t tc_cap = 0;  // floats
  unsigned tc_gen = 0;
  int* tc_err = nullptr;
  // allocated from the device's stream-ordered pool (lu_workspace_create_async):
  // growing and freeing it never waits for work on other streams
  bool pooled = false;
  // shape of the precision form's factorisation, set from the autotuner's choice
  // for the order: FP32 columns of a tensor-core update tile (256 or 128; 0 = 256)
  // and the widest FP32 panel (0 = as wide as the panel's shared memory allows)
  int tile_n = 0;
  int panel_w = 0;
  // widest FP64 cluster panel of the precision form's second tier (0 = 32)
  int panel_w64 = 0;
  // the matrix being factored holds float-float values (float4: hi.re, hi.im,
  // lo.re, lo.im in place of each complex128; the second tier's storage): panels,
  // block solves and the digit-plane updates read and write that form
  bool ff_storage = false;
};

size_t lu_workspace_bytes(int elem_bytes);  // one matrix: barrier + staging
size_t lu_stage_offset(int max_batch);      // byte offset of the staging array
size_t lu_stage_bytes(int max_batch);

// Optional replacement of the trailing-update GEMM (Cm -= Am * Bm) for `batch`
// matrices whose operands are `bstride` elements apart; its scratch lives in `ws`.
template <typename C>
using GemmHook = cudaError_t (*)(LuWorkspace* ws, const C* Am, long long lda, const C* Bm, long long ldb, C* Cm,
                                 long long ldc, int M, int N, int K, cudaStream_t s, int batch,
                                 long long bstride);

// In-place LU of `batch` n x n matrices astride elements apart (pivots n apart).
// With a GEMM hook, `span` panels (1..kMaxSpan, 0 = default 2) share one trailing
// update.
constexpr int kMaxSpan = 8;
template <typename C>
cudaError_t lu_factor_t(C* A, long long lda, int n, int* ipiv, LuWorkspace* ws, cudaStream_t s,
                        GemmHook<C> gemm_hook, int batch = 1, long long astride = 0, int span = 0);

// Solves with the factors; batch > 1 needs nrhs == 1 and right-hand sides n apart.
// sel (device, `batch` entries): solve only these matrices of a larger batch (matrix
// sel[i] at A + sel[i] * astride, its right-hand side at B + sel[i] * n).
// inv (optional, one right-hand side): the inverses of the factors' 64 x 64 diagonal
// blocks (lu_block_inverses), which turn each block's substitution into one parallel
// product.
// perm_pre (optional, device, n ints per matrix of the whole batch, matrix i at
// perm_pre + i * n): the factors' row permutations from lu_pivots_to_perm, computed
// once per factorisation instead of on every solve.
template <typename C>
cudaError_t lu_solve_t(const C* A, long long lda, int n, const int* ipiv, C* B, long long ldb, int nrhs,
                       LuWorkspace* ws, cudaStream_t s, int batch = 1, long long astride = 0,
                       const int* sel = nullptr, const C* inv = nullptr, const int* perm_pre = nullptr);
// The row permutation of each of `batch` pivot vectors (ipiv, n apart, LAPACK 1-based)
// into perm (n apart): row i of P B is row perm[i] of B.
cudaError_t lu_pivots_to_perm(const int* ipiv, int n, int batch, int* perm, cudaStream_t s);
// The inverses of the 64 x 64 diagonal blocks of the factors (unit lower L and upper
// U) of `batch` matrices astride apart, into inv (lu_block_inverse_bytes): per matrix
// and block L^-1 then U^-1, column-major.  Instantiated for complex FP32.
template <typename C>
cudaError_t lu_block_inverses(const C* A, long long lda, int n, int batch, long long astride, C* inv,
                              cudaStream_t s);
template <typename C>
size_t lu_block_inverse_bytes(int n, int batch);

// Solves A^H x = b with the factors of lu_factor_t (the condition estimator's second
// kind of solve), one right-hand side per matrix, vectors n apart; batch and sel as
// lu_solve_t's.
template <typename C>
cudaError_t lu_solve_h_t(const C* A, long long lda, int n, const int* ipiv, C* B, LuWorkspace* ws, cudaStream_t s,
                         int batch = 1, long long astride = 0, const int* sel = nullptr);

// lu_solve_t with one right-hand side per matrix, for FP64-grade factors held as
// float-float entries (split_ff_inplace: float4 (hi.re, hi.im, lo.re, lo.im) in
// place of each complex128 entry, same layout), in compensated FP32 arithmetic
// (about 2^-48 relative per operation): the second tier's solves inside its FP64
// refinement.
// inv (optional): the inverses of the factors' 64 x 64 diagonal blocks
// (ff_block_inverses), which turn each block's substitution into one parallel product.
cudaError_t lu_solve_ff(const float4* A, long long lda, int n, const int* ipiv, double2* B, LuWorkspace* ws,
                        cudaStream_t s, int batch = 1, long long astride = 0, const int* sel = nullptr,
                        const float4* inv = nullptr, const int* perm_pre = nullptr);
// The inverses of the 64 x 64 diagonal blocks of the float-float factors (unit lower L
// and upper U) of `batch` matrices astride apart, into inv (ff_block_inverse_bytes),
// in float-float arithmetic: for lu_solve_ff.
cudaError_t ff_block_inverses(const float4* A, long long lda, int n, int batch, long long astride, float4* inv,
                              cudaStream_t s);
size_t ff_block_inverse_bytes(int n, int batch);
// Whether the second tier's LU of order n (FP64 cluster panels of at most panel_w64
// columns) can keep its matrix in float-float form (LuWorkspace::ff_storage).
bool ff_tier2_supported(int n, int panel_w64);
// `count` complex128 values to float-float in place (hi = fp32(v), lo = fp32(v - hi)),
// and back (exact).
cudaError_t split_ff_inplace(double2* a, size_t count, cudaStream_t s);
cudaError_t merge_ff_inplace(double2* a, size_t count, cudaStream_t s);

// The plain FP64 form's trailing update, C -= A B for complex FP64 column-major
// operands (`batch` matrices bstride apart): SIMT DFMA (gemm_sub_kernel, lu.cu) or
// DMMA on the FP64 tensor pipe (lu_dmma.cu).  WMOM_FP64_UPDATE=dmma selects the
// latter inside the plain form's LU.
cudaError_t zgemm_sub_simt(const double2* Am, long long lda, const double2* Bm, long long ldb, double2* Cm,
                           long long ldc, int M, int N, int K, cudaStream_t s, int batch, long long bstride);
cudaError_t zgemm_sub_dmma(const double2* Am, long long lda, const double2* Bm, long long ldb, double2* Cm,
                           long long ldc, int M, int N, int K, cudaStream_t s, int batch, long long bstride);
bool fp64_update_dmma();

// Test hook: arrivals every cooperative panel barrier waits for in addition to its
// blocks' own (0 in normal use).
extern std::atomic<unsigned int> g_panel_missing_arrivals;

// Workspace management (api.cu).
cudaError_t lu_workspace_create(LuWorkspace* ws, int nmax, int nrhs_max, int max_batch = 1);
// The same workspace from the device's stream-ordered pool, allocated and cleared in
// the order of `s`.  Factor sets that a serving loop creates and evicts while other
// streams run use it: cudaMalloc / cudaFree may wait for the whole device.
cudaError_t lu_workspace_create_async(LuWorkspace* ws, int nmax, int nrhs_max, int max_batch, cudaStream_t s);
// Frees a workspace.  A pooled one is returned to the pool on the calling thread's
// default stream: every call that used it must have finished (the library's entry
// points synchronise their stream before returning).
void lu_workspace_destroy(LuWorkspace* ws);
cudaError_t lu_workspace_reset_barrier(LuWorkspace* ws, cudaStream_t s);
// Returns nonzero when a wait of the last factorisation timed out; info[b] = the
// first zero-pivot column of matrix b (info may be null; batch entries read).
int lu_workspace_read_status(LuWorkspace* ws, int* info, cudaStream_t s, int batch = 1);

}  // namespace wmom
