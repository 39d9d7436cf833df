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
};

wmom_status run_sweep(const SweepArgs& a);

// Device helpers (solve.cu).
cudaError_t residual_fp64(const double2* Z, long long ldz, const double2* x, const double2* v, int n,
                          double2* r, double2* partial, cudaStream_t s);
cudaError_t sumsq_fp64(const double2* x, int n, double* out, cudaStream_t s);
cudaError_t convert_matrix_64_to_32(const double2* src, long long lds, float2* dst, long long ldd, int rows,
                                    int cols, cudaStream_t s);
cudaError_t convert_vec_64_to_32(const double2* src, float2* dst, int n, double scale, cudaStream_t s);
cudaError_t accumulate_vec_32_to_64(double2* x, const float2* d, int n, double scale, cudaStream_t s);

// FP32 trailing-update GEMM on the tensor cores (lu_tc.cu); nullptr when the
// device has no tcgen05 path, in which case the SIMT GEMM is used.
GemmHook<float2> tc_gemm_hook();
namespace tc {
int read_and_clear_error();  // 1 if a tensor-core GEMM wait timed out since the last call
}

}  // namespace wmom
