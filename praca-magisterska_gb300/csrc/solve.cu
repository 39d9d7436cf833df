// solve.cu -- the per-frequency solve of the reference's driver loop
// ("wersja referencyjna/Wire_MoM.cu":335-400: zmatrix -> zgetrf -> zgetrs ->
// Z_in = V[ngap-1]/I[ngap-1]), batched over frequencies on one device.
//
// FP64 form: fill (FP64) -> LU (FP64) -> solve (FP64).
// Mixed form: fill (FP64, kept) -> FP32 copy -> LU (FP32, tensor-core trailing
// updates) -> solve (FP32) -> iterative refinement: r = V - Z I in FP64 with the
// FP64 Z, correction solved with the FP32 factors, I += d in FP64; when the
// residual stops shrinking (or the FP32 factorisation hits a zero pivot) the FP64
// LU is used instead, and the report says so.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "lu_common.cuh"
#include "solve_internal.h"
#include "stats.h"

namespace wmom {

// ------------------------------------------------------------ kernels ----
constexpr int kGemvRows = 128;
constexpr int kGemvChunk = 512;

// partial[chunk*n + i] = sum over columns of chunk of Z[i, j] x[j]
__global__ void __launch_bounds__(kGemvRows) gemv_partial_kernel(const double2* __restrict__ Z, long long ldz,
                                                                 const double2* __restrict__ x, int n,
                                                                 double2* __restrict__ partial) {
  __shared__ double2 xs[kGemvChunk];
  const int i = blockIdx.x * kGemvRows + threadIdx.x;
  const int c0 = blockIdx.y * kGemvChunk;
  const int c1 = min(n, c0 + kGemvChunk);
  for (int j = c0 + threadIdx.x; j < c1; j += kGemvRows) xs[j - c0] = x[j];
  __syncthreads();
  if (i >= n) return;
  double re = 0.0, im = 0.0;
  const double2* zp = Z + (size_t)c0 * ldz + i;
  for (int j = c0; j < c1; ++j, zp += ldz) {
    const double2 a = *zp;
    const double2 b = xs[j - c0];
    re = fma(a.x, b.x, fma(-a.y, b.y, re));
    im = fma(a.x, b.y, fma(a.y, b.x, im));
  }
  partial[(size_t)blockIdx.y * n + i] = make_double2(re, im);
}

__global__ void residual_finish_kernel(const double2* __restrict__ v, const double2* __restrict__ partial,
                                       int nchunks, int n, double2* __restrict__ r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double re = 0.0, im = 0.0;
  for (int c = 0; c < nchunks; ++c) {
    const double2 p = partial[(size_t)c * n + i];
    re += p.x;
    im += p.y;
  }
  r[i] = make_double2(v[i].x - re, v[i].y - im);
}

// Deterministic sum of |x_i|^2 in one block (fixed order: strided partials, then a
// fixed tree).
__global__ void __launch_bounds__(1024) sumsq_kernel(const double2* __restrict__ x, int n, double* out) {
  __shared__ double sh[1024];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += 1024) acc = fma(x[i].x, x[i].x, fma(x[i].y, x[i].y, acc));
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 512; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

__global__ void __launch_bounds__(1024) sumsq_f32_kernel(const float2* __restrict__ x, int n, double scale,
                                                         double* out) {
  __shared__ double sh[1024];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += 1024) {
    const double a = (double)x[i].x * scale, b = (double)x[i].y * scale;
    acc = fma(a, a, fma(b, b, acc));
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 512; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

__global__ void convert_matrix_kernel(const double2* __restrict__ src, long long lds, float2* __restrict__ dst,
                                      long long ldd, int rows, int cols) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i < rows && j < cols) {
    const double2 a = src[(size_t)j * lds + i];
    dst[(size_t)j * ldd + i] = make_float2((float)a.x, (float)a.y);
  }
}

__global__ void convert_vec_kernel(const double2* __restrict__ src, float2* __restrict__ dst, int n,
                                   double scale) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = make_float2((float)(src[i].x * scale), (float)(src[i].y * scale));
}

__global__ void accumulate_vec_kernel(double2* __restrict__ x, const float2* __restrict__ d, int n,
                                      double scale) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    x[i].x += (double)d[i].x * scale;
    x[i].y += (double)d[i].y * scale;
  }
}

__global__ void widen_vec_kernel(const float2* __restrict__ d, double2* __restrict__ x, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = make_double2((double)d[i].x, (double)d[i].y);
}

cudaError_t residual_fp64(const double2* Z, long long ldz, const double2* x, const double2* v, int n,
                          double2* r, double2* partial, cudaStream_t s) {
  const int nchunks = (n + kGemvChunk - 1) / kGemvChunk;
  stats::Scope sc(stats::kResidual, s, 16.0 * n * (double)n, 2);
  gemv_partial_kernel<<<dim3((n + kGemvRows - 1) / kGemvRows, nchunks), kGemvRows, 0, s>>>(Z, ldz, x, n,
                                                                                           partial);
  residual_finish_kernel<<<(n + 255) / 256, 256, 0, s>>>(v, partial, nchunks, n, r);
  return cudaGetLastError();
}

cudaError_t sumsq_fp64(const double2* x, int n, double* out, cudaStream_t s) {
  stats::count(stats::kMisc);
  sumsq_kernel<<<1, 1024, 0, s>>>(x, n, out);
  return cudaGetLastError();
}

cudaError_t convert_matrix_64_to_32(const double2* src, long long lds, float2* dst, long long ldd, int rows,
                                    int cols, cudaStream_t s) {
  stats::Scope sc(stats::kMisc, s, 24.0 * rows * (double)cols);
  convert_matrix_kernel<<<dim3((rows + 255) / 256, cols), 256, 0, s>>>(src, lds, dst, ldd, rows, cols);
  return cudaGetLastError();
}

cudaError_t convert_vec_64_to_32(const double2* src, float2* dst, int n, double scale, cudaStream_t s) {
  stats::count(stats::kMisc);
  convert_vec_kernel<<<(n + 255) / 256, 256, 0, s>>>(src, dst, n, scale);
  return cudaGetLastError();
}

cudaError_t accumulate_vec_32_to_64(double2* x, const float2* d, int n, double scale, cudaStream_t s) {
  stats::count(stats::kMisc);
  accumulate_vec_kernel<<<(n + 255) / 256, 256, 0, s>>>(x, d, n, scale);
  return cudaGetLastError();
}

// ------------------------------------------------------------- driver ----
namespace {

struct DevBuf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  cudaError_t alloc(size_t bytes, cudaStream_t st) {
    s = st;
    return cudaMallocAsync(&p, std::max<size_t>(bytes, 16), st);
  }
  ~DevBuf() {
    if (p) cudaFreeAsync(p, s);
  }
  template <typename T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

#define SWEEP_TRY(call)                                 \
  do {                                                  \
    cudaError_t _e = (call);                            \
    if (_e != cudaSuccess) return wmom_fail_cuda(_e, #call); \
  } while (0)

struct Scalars {
  double vnorm2;
  double rnorm2;
  double dnorm2;  // last refinement correction
  double xnorm2;  // solution before that correction
};

}  // namespace

wmom_status run_sweep(const SweepArgs& a) {
  const Plan& p = *a.plan;
  const int n = p.npls;
  cudaStream_t s = a.stream;
  const size_t mat64 = sizeof(double2) * (size_t)n * n;
  const size_t mat32 = sizeof(float2) * (size_t)n * n;
  size_t budget = a.mem_budget;
  if (budget == 0) {
    size_t fr = 0, tot = 0;
    SWEEP_TRY(cudaMemGetInfo(&fr, &tot));
    budget = fr / 2;
  }
  const size_t fixed = mat64 + (a.mode == WMOM_MODE_MIXED ? mat32 : 0);
  if (budget < fixed + mat64) return WMOM_ERR_NOMEM;
  const int batch = (int)std::max<size_t>(1, std::min<size_t>((size_t)a.nfreq, (budget - fixed) / mat64));

  // excitation
  std::vector<double> vh(2 * (size_t)n);
  wmom_status st = wmom_excitation(n, a.ngap, a.ampl, a.phas_deg, vh.data());
  if (st != WMOM_OK) return st;

  DevBuf zall, zf, z32, ipiv, v64, x64, r64, d32, part, fpb, sc;
  SWEEP_TRY(zall.alloc(mat64 * batch, s));
  SWEEP_TRY(zf.alloc(mat64, s));
  if (a.mode == WMOM_MODE_MIXED) SWEEP_TRY(z32.alloc(mat32, s));
  SWEEP_TRY(ipiv.alloc(sizeof(int) * n, s));
  SWEEP_TRY(v64.alloc(sizeof(double2) * n, s));
  SWEEP_TRY(x64.alloc(sizeof(double2) * n, s));
  SWEEP_TRY(r64.alloc(sizeof(double2) * n, s));
  SWEEP_TRY(d32.alloc(sizeof(float2) * n, s));
  const int nchunks = (n + kGemvChunk - 1) / kGemvChunk;
  SWEEP_TRY(part.alloc(sizeof(double2) * (size_t)n * nchunks, s));
  SWEEP_TRY(fpb.alloc(sizeof(double) * 3 * batch, s));
  SWEEP_TRY(sc.alloc(sizeof(Scalars), s));
  SWEEP_TRY(cudaMemcpyAsync(v64.p, vh.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, s));
  SWEEP_TRY(sumsq_fp64(v64.as<double2>(), n, &sc.as<Scalars>()->vnorm2, s));
  Scalars hs{};
  SWEEP_TRY(cudaMemcpyAsync(&hs, sc.p, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  SWEEP_TRY(cudaStreamSynchronize(s));
  const double vnorm = std::sqrt(hs.vnorm2);

  const GemmHook<float2> hook32 = tc_gemm_hook();
  std::vector<double> fph(3 * (size_t)batch);
  std::vector<double2> xh(n);
  const double pi = std::acos(-1.0);
  wmom_status overall = WMOM_OK;

  auto factor64 = [&](const double2* Zk, int* info) -> wmom_status {
    SWEEP_TRY(cudaMemcpyAsync(zf.p, Zk, mat64, cudaMemcpyDeviceToDevice, s));
    SWEEP_TRY(lu_workspace_reset_barrier(a.ws, s));
    SWEEP_TRY(lu_factor_t<double2>(zf.as<double2>(), n, n, ipiv.as<int>(), a.ws, s, nullptr));
    const int err = lu_workspace_read_status(a.ws, info, s);
    SWEEP_TRY(cudaGetLastError());
    if (err) return WMOM_ERR_TIMEOUT;
    SWEEP_TRY(cudaMemcpyAsync(x64.p, v64.p, sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
    SWEEP_TRY(lu_solve_t<double2>(zf.as<double2>(), n, n, ipiv.as<int>(), x64.as<double2>(), n, 1, a.ws, s));
    return *info ? WMOM_ERR_SINGULAR : WMOM_OK;
  };
  auto residual_norm = [&](const double2* Zk, double* rel) -> wmom_status {
    SWEEP_TRY(residual_fp64(Zk, n, x64.as<double2>(), v64.as<double2>(), n, r64.as<double2>(),
                            part.as<double2>(), s));
    SWEEP_TRY(sumsq_fp64(r64.as<double2>(), n, &sc.as<Scalars>()->rnorm2, s));
    SWEEP_TRY(cudaMemcpyAsync(&hs, sc.p, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
    SWEEP_TRY(cudaStreamSynchronize(s));
    *rel = std::sqrt(hs.rnorm2) / vnorm;
    return WMOM_OK;
  };

  for (int f0 = 0; f0 < a.nfreq; f0 += batch) {
    const int nb = std::min(batch, a.nfreq - f0);
    for (int i = 0; i < nb; ++i) {
      const double ka = ka_from_mhz(a.freq_mhz[f0 + i]);
      const double eta0 = 120. * pi;
      fph[3 * i] = ka;
      fph[3 * i + 1] = ka * ka;
      fph[3 * i + 2] = eta0 / (4.0 * pi * ka);
    }
    SWEEP_TRY(cudaMemcpyAsync(fpb.p, fph.data(), sizeof(double) * 3 * nb, cudaMemcpyHostToDevice, s));
    SWEEP_TRY(launch_fill(p, fpb.as<double>(), nb, zall.as<double2>(), n, (long long)n * n, s));
    for (int i = 0; i < nb; ++i) {
      const int f = f0 + i;
      const double2* Zk = zall.as<double2>() + (size_t)i * n * n;
      wmom_report rep{};
      rep.rel_residual = -1.0;
      int info = 0;
      wmom_status fst = WMOM_OK;
      if (a.mode == WMOM_MODE_FP64) {
        fst = factor64(Zk, &info);
        rep.info = info;
        if (fst == WMOM_OK || fst == WMOM_ERR_SINGULAR) {
          const wmom_status rs = residual_norm(Zk, &rep.rel_residual);
          if (rs != WMOM_OK) return rs;
        }
      } else {
        // FP32 factorisation of the FP64 matrix
        SWEEP_TRY(convert_matrix_64_to_32(Zk, n, z32.as<float2>(), n, n, n, s));
        SWEEP_TRY(lu_workspace_reset_barrier(a.ws, s));
        SWEEP_TRY(lu_factor_t<float2>(z32.as<float2>(), n, n, ipiv.as<int>(), a.ws, s, hook32));
        const int err = lu_workspace_read_status(a.ws, &info, s) | (hook32 ? tc::read_and_clear_error() : 0);
        SWEEP_TRY(cudaGetLastError());
        if (err) return WMOM_ERR_TIMEOUT;
        bool fallback = info != 0;
        if (!fallback) {
          // initial solve in FP32
          SWEEP_TRY(convert_vec_64_to_32(v64.as<double2>(), d32.as<float2>(), n, 1.0, s));
          SWEEP_TRY(lu_solve_t<float2>(z32.as<float2>(), n, n, ipiv.as<int>(), d32.as<float2>(), n, 1, a.ws, s));
          stats::count(stats::kMisc);
          widen_vec_kernel<<<(n + 255) / 256, 256, 0, s>>>(d32.as<float2>(), x64.as<double2>(), n);
          SWEEP_TRY(cudaGetLastError());
          double prev = HUGE_VAL;
          int stall = 0;
          const int max_it = 40;
          for (int it = 0;; ++it) {
            double rel = 0.0;
            const wmom_status rs = residual_norm(Zk, &rel);
            if (rs != WMOM_OK) return rs;
            rep.rel_residual = rel;
            rep.iterations = it;
            if (!(rel == rel)) {  // NaN: refinement diverged
              fallback = true;
              break;
            }
            // converged: the residual target is met, or the last correction no longer
            // changes the solution at FP64 resolution (ill-conditioned systems whose
            // FP64 residual floor lies above the target)
            const double corr = it > 0 ? std::sqrt(hs.dnorm2 / hs.xnorm2) : HUGE_VAL;
            if (rel <= a.tol || corr <= 0x1p-48) break;
            if (rel > 0.5 * prev) {
              if (++stall >= 2) {
                fallback = true;
                break;
              }
            } else {
              stall = 0;
            }
            if (it >= max_it) {
              fallback = true;
              break;
            }
            prev = std::min(prev, rel);
            // correction: d = (LU32)^-1 r, scaled by a power of two to keep FP32 in range
            const double rn = rel * vnorm;
            const double scale = rn > 0 ? std::ldexp(1.0, -std::ilogb(rn)) : 1.0;
            SWEEP_TRY(convert_vec_64_to_32(r64.as<double2>(), d32.as<float2>(), n, scale, s));
            SWEEP_TRY(lu_solve_t<float2>(z32.as<float2>(), n, n, ipiv.as<int>(), d32.as<float2>(), n, 1, a.ws, s));
            stats::count(stats::kMisc);
            sumsq_f32_kernel<<<1, 1024, 0, s>>>(d32.as<float2>(), n, 1.0 / scale, &sc.as<Scalars>()->dnorm2);
            SWEEP_TRY(sumsq_fp64(x64.as<double2>(), n, &sc.as<Scalars>()->xnorm2, s));
            SWEEP_TRY(accumulate_vec_32_to_64(x64.as<double2>(), d32.as<float2>(), n, 1.0 / scale, s));
          }
        }
        if (fallback) {
          rep.fell_back = 1;
          fst = factor64(Zk, &info);
          if (fst == WMOM_OK || fst == WMOM_ERR_SINGULAR) {
            const wmom_status rs = residual_norm(Zk, &rep.rel_residual);
            if (rs != WMOM_OK) return rs;
          }
        }
        rep.info = info;
      }
      if (fst == WMOM_ERR_TIMEOUT) return fst;
      rep.status = fst;
      if (fst != WMOM_OK && overall == WMOM_OK) overall = fst;
      // results
      if (a.currents) {
        SWEEP_TRY(cudaMemcpyAsync(a.currents + 2 * (size_t)f * n, x64.p, sizeof(double2) * n,
                                  cudaMemcpyDeviceToHost, s));
        SWEEP_TRY(cudaStreamSynchronize(s));
        std::memcpy(xh.data(), a.currents + 2 * (size_t)f * n, sizeof(double2) * n);
      } else {
        SWEEP_TRY(cudaMemcpyAsync(xh.data() + (a.ngap - 1), x64.as<double2>() + (a.ngap - 1), sizeof(double2),
                                  cudaMemcpyDeviceToHost, s));
        SWEEP_TRY(cudaStreamSynchronize(s));
      }
      if (a.zin) {
        // Z_in = V[ngap-1] / I[ngap-1], Smith's formula
        const double vr = vh[2 * (a.ngap - 1)], vi = vh[2 * (a.ngap - 1) + 1];
        const double br = xh[a.ngap - 1].x, bi = xh[a.ngap - 1].y;
        double zr, zi;
        if (std::fabs(br) >= std::fabs(bi)) {
          const double r = bi / br, d = br + bi * r;
          zr = (vr + vi * r) / d;
          zi = (vi - vr * r) / d;
        } else {
          const double r = br / bi, d = bi + br * r;
          zr = (vr * r + vi) / d;
          zi = (vi * r - vr) / d;
        }
        a.zin[2 * (size_t)f] = zr;
        a.zin[2 * (size_t)f + 1] = zi;
      }
      if (a.reports) a.reports[f] = rep;
    }
  }
  SWEEP_TRY(cudaStreamSynchronize(s));
  return overall;
}

}  // namespace wmom
