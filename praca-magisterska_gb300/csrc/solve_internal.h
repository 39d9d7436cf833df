// solve_internal.h -- the frequency-sweep driver shared by the C ABI and the
// serving loop.
#pragma once

#include <cuda_runtime.h>

#include "lu_internal.h"
#include "wmom_internal.h"

namespace wmom {

struct SweepArgs {
  const Plan* plan = nullptr;
  const float* freq_mhz = nullptr;
  int nfreq = 0;
  int ngap = 1;
  float ampl = 1.f, phas_deg = 0.f;
  int mode = WMOM_MODE_FP64;
  double tol = 1e-12;
  double* currents = nullptr;  // host, nfreq*npls complex (optional)
  double* zin = nullptr;       // host, nfreq complex (optional)
  wmom_report* reports = nullptr;
  cudaStream_t stream = nullptr;
  LuWorkspace* ws = nullptr;
  size_t mem_budget = 0;  // bytes of device memory the sweep may use; 0 = automatic
  bool condest = false;   // estimate kappa_1 of every matrix (wmom_report.cond1)
};

wmom_status run_sweep(const SweepArgs& a);

// Z and its factors kept resident for a list of frequencies of one plan, so that new
// excitations only run the solves (and refinement).
// Factorisation shape chosen by the autotuner: matrices per batched launch and
// panels per tensor-core trailing update.
struct LuConfig {
  int batch = 1;
  int span = 0;
  int tile_n = 0;   // tensor-core update tile: FP32 columns (256 or 128; 0 = 256)
  int panel_w = 0;  // widest FP32 panel (0 = as wide as shared memory allows)
};

// The factorisation shape of cfg on the workspace that the factorisation uses.
inline void use_shape(LuWorkspace* ws, const LuConfig& cfg) {
  ws->tile_n = cfg.tile_n;
  ws->panel_w = cfg.panel_w;
}

struct FactorSet {
  const Plan* plan = nullptr;
  int mode = WMOM_MODE_MIXED;
  std::vector<float> freq;
  LuWorkspace* ws = nullptr;  // owned by the set
  int batch = 1;
  int span = 0;               // panels per tensor-core trailing update (tuned)
  double2* z64 = nullptr;     // nf matrices, FP64 (kept for the residual)
  void* lu = nullptr;         // nf factors: float2 (mixed) or double2 (FP64)
  int* ipiv = nullptr;        // nf * n
  std::vector<int> info;
  bool condest = false;       // estimate kappa_1 with every solve
  // order of the stored matrices: the plan's npls, or the padded order of the
  // geometry's size class when the set was factored in a batch of uneven geometries
  // (identity block beyond npls; factors_solve pads the excitation and returns npls
  // entries)
  int order = 0;
  // z64, lu and ipiv come from the stream-ordered pool (freed without waiting for
  // other streams)
  bool pooled = false;
};

wmom_status factors_build(FactorSet* fs, cudaStream_t s);

// Keeps up to an eighth of the device's memory (WMOM_POOL_RETAIN_GB) in the default
// stream-ordered pool between synchronisations; once per device.
void retain_pool_memory();

// Geometries of uneven order (solve.cu): the padded order of n's size class (four
// classes per octave, P <= 1.25 n); the factorisation shape of order n (the tuned
// span, tile and panels, else span 2 with the default tile and panels); and the
// batched fill + factorisation of `count` geometries of
// one class, one frequency each, into z64 (count matrices of order P) and lu / ipiv
// (complex64 or complex128 factors by mode), with an identity block beyond each
// geometry's order.
int padded_order(int n);
LuConfig tuned_shape(int n, int mode);
wmom_status factor_class(int mode, int P, const Plan* const* plans, const float* freq, int count, double2* z64,
                         void* lu, int* ipiv, int* info, LuWorkspace* ws, int span, cudaStream_t s);
wmom_status factors_solve(FactorSet* fs, int first, int count, int ngap, float ampl, float phas, double tol,
                          double* currents, double* zin, wmom_report* reports, cudaStream_t s);

// Condition estimates (condest.cu).  condest_t: est[k] = an estimate of
// ||A^-1||_1 for the factored matrices slots[0..m) (host list; matrix slot at
// lu + slot * astride, pivots at ipiv + slot * n), by LAPACK zlacn2's algorithm with
// batched solves; X holds one n-vector per slot (at X + slot * n) as scratch.  nreal
// <= n: the matrices' own order when they are stored at the padded order n with an
// identity block beyond nreal (the estimate is then that of the leading block).
template <typename C>
wmom_status condest_t(int n, int nreal, const C* lu, long long lda, long long astride, const int* ipiv,
                      const int* slots, int m, C* X, LuWorkspace* ws, cudaStream_t s, double* est);
// out_dev[b] = ||Z_b||_1 (maximum column sum of moduli) for nmat matrices zstride apart.
cudaError_t norm1_batch(const double2* Z, int n, long long lda, long long zstride, int nmat, double* out_dev,
                        cudaStream_t s);

// Device helpers (solve.cu).
// r[b] = v - Z[b] x[b] for nvec matrices zstride apart (vectors n apart), FP64;
// sel (device, nvec entries): only these matrices b of a larger batch; vsel (device,
// nvec entries): the vector slots of x and r that go with them, when they differ.
cudaError_t residual_fp64(const double2* Z, long long ldz, long long zstride, const double2* x, const double2* v,
                          int n, double2* r, double2* partial, int nvec, cudaStream_t s, const int* sel = nullptr,
                          const int* vsel = nullptr);
// out[b] = sum |x[b]_i|^2 for nvec vectors n apart (deterministic order).
cudaError_t sumsq_fp64(const double2* x, int n, double* out, int nvec, cudaStream_t s);
cudaError_t convert_flat_64_to_32(const double2* src, float2* dst, size_t count, cudaStream_t s);

// FP32 trailing-update GEMM on the tensor cores (lu_tc.cu); nullptr when the
// device has no tcgen05 path, in which case the SIMT GEMM is used.
GemmHook<float2> tc_gemm_hook();
// FP64-grade trailing-update GEMM on the bf16 tensor cores (lu_emul.cu), the second
// tier of the precision form; nullptr without a tcgen05 device or with WMOM_NO_EMUL.
GemmHook<double2> emul_gemm_hook();
namespace tc {
// 1 if a tensor-core GEMM wait on `ws` timed out since the last call (synchronises s)
int read_and_clear_error(LuWorkspace* ws, cudaStream_t s);
}

}  // namespace wmom
