// solve.cu -- the per-frequency solve of the reference's driver loop
// ("wersja referencyjna/Wire_MoM.cu":335-400: zmatrix -> zgetrf -> zgetrs ->
// Z_in = V[ngap-1]/I[ngap-1]), batched over frequencies on one device.
//
// FP64 form: fill (FP64) -> LU (FP64) -> solve (FP64).
// Mixed form: fill (FP64, kept) -> FP32 copy -> LU (FP32, tensor-core trailing
// updates) -> solve (FP32) -> iterative refinement: r = V - Z I in FP64 with the
// FP64 Z, correction solved with the FP32 factors, I += d in FP64; a matrix whose
// residual stops shrinking (or whose FP32 factorisation hits a zero pivot) is
// solved with the FP64 LU instead, and its report says so.
//
// Frequencies are processed in groups of B matrices that go through ONE batched
// launch sequence (fill, factor, solves, refinement with a per-matrix activity
// mask).  B is picked per (order, form) by timing the candidate batch widths on
// the first group (autotuner; WMOM_LU_BATCH overrides).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <vector>

#include "lu_common.cuh"
#include "solve_internal.h"
#include "stats.h"

namespace wmom {

// ------------------------------------------------------------ kernels ----
constexpr int kGemvRows = 128;
constexpr int kGemvChunk = 512;

// partial[chunk*n + i] = sum over the columns of a chunk of Z[i, j] x[j]; blockIdx.z = matrix
// (sel: the z-th selected matrix is Z's sel[z]; its vector is x's vsel[z], or sel[z])
__global__ void __launch_bounds__(kGemvRows) gemv_partial_kernel(const double2* __restrict__ Z, long long ldz,
                                                                 long long zstride, const double2* __restrict__ x,
                                                                 int n, double2* __restrict__ partial,
                                                                 const int* __restrict__ sel,
                                                                 const int* __restrict__ vsel) {
  __shared__ double2 xs[kGemvChunk];
  const int mat = sel ? sel[blockIdx.z] : (int)blockIdx.z;
  Z += (size_t)mat * zstride;
  x += (size_t)(vsel ? vsel[blockIdx.z] : mat) * n;
  partial += (size_t)blockIdx.z * gridDim.y * n;
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

// r = v - sum of the partials in chunk order (deterministic); blockIdx.y = matrix
// (sel: the y-th selected matrix, sel[y])
__global__ void residual_finish_kernel(const double2* __restrict__ v, const double2* __restrict__ partial,
                                       int nchunks, int n, double2* __restrict__ r, const int* __restrict__ sel,
                                       const int* __restrict__ vsel) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  partial += (size_t)blockIdx.y * nchunks * n;
  r += (size_t)(vsel ? vsel[blockIdx.y] : (sel ? sel[blockIdx.y] : (int)blockIdx.y)) * n;
  if (i >= n) return;
  double re = 0.0, im = 0.0;
  for (int c = 0; c < nchunks; ++c) {
    const double2 p = partial[(size_t)c * n + i];
    re += p.x;
    im += p.y;
  }
  r[i] = make_double2(v[i].x - re, v[i].y - im);
}

// Deterministic sum of |x_i|^2 per vector (one block per vector of a batch: fixed
// strided partials, then a fixed tree).
__global__ void __launch_bounds__(1024) sumsq_kernel(const double2* __restrict__ x, int n, double* out) {
  __shared__ double sh[1024];
  x += (size_t)blockIdx.x * n;
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += 1024) acc = fma(x[i].x, x[i].x, fma(x[i].y, x[i].y, acc));
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 512; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(1024) sumsq_f32_kernel(const float2* __restrict__ x, int n,
                                                         const double* __restrict__ scale, double* out) {
  __shared__ double sh[1024];
  x += (size_t)blockIdx.x * n;
  const double sc = scale[blockIdx.x];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += 1024) {
    const double a = (double)x[i].x * sc, b = (double)x[i].y * sc;
    acc = fma(a, a, fma(b, b, acc));
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 512; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

__global__ void convert_flat_kernel(const double2* __restrict__ src, float2* __restrict__ dst, size_t count) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
    const double2 a = src[i];
    dst[i] = make_float2((float)a.x, (float)a.y);
  }
}

// dst[b] = (float)(src[b] * scale[b]) for the vectors of a batch
__global__ void convert_vec_kernel(const double2* __restrict__ src, float2* __restrict__ dst, int n, int nvec,
                                   const double* __restrict__ scale) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)n * nvec) return;
  const double sc = scale ? scale[i / n] : 1.0;
  dst[i] = make_float2((float)(src[i].x * sc), (float)(src[i].y * sc));
}

// x[b] += d[b] * inv[b] where active[b]
__global__ void accumulate_vec_kernel(double2* __restrict__ x, const float2* __restrict__ d, int n, int nvec,
                                      const double* __restrict__ inv, const int* __restrict__ active) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)n * nvec) return;
  const size_t b = i / n;
  if (!active[b]) return;
  x[i].x += (double)d[i].x * inv[b];
  x[i].y += (double)d[i].y * inv[b];
}

// v[b] *= scale[b] (powers of two: exact), every vector of the batch
__global__ void scale_vec64_kernel(double2* __restrict__ v, int n, int nvec, const double* __restrict__ scale) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)n * nvec) return;
  const double sc = scale[i / n];
  v[i].x *= sc;
  v[i].y *= sc;
}

// x[b] += d[b] where active[b] (FP64 corrections of the second tier)
__global__ void accumulate64_kernel(double2* __restrict__ x, const double2* __restrict__ d, int n, int nvec,
                                    const int* __restrict__ active) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)n * nvec) return;
  if (!active[i / n]) return;
  x[i].x += d[i].x;
  x[i].y += d[i].y;
}

// partial[chunk*n + i] = sum over the chunk's columns of cabs1(Z[i, j]) cabs1(x[j]),
// cabs1(z) = |re z| + |im z|: the |Z| |x| of the componentwise backward error
__global__ void __launch_bounds__(kGemvRows) absgemv_partial_kernel(const double2* __restrict__ Z, long long ldz,
                                                                    const double2* __restrict__ x, int n,
                                                                    double* __restrict__ partial) {
  __shared__ double xs[kGemvChunk];
  const int i = blockIdx.x * kGemvRows + threadIdx.x;
  const int c0 = blockIdx.y * kGemvChunk;
  const int c1 = min(n, c0 + kGemvChunk);
  for (int j = c0 + threadIdx.x; j < c1; j += kGemvRows) xs[j - c0] = fabs(x[j].x) + fabs(x[j].y);
  __syncthreads();
  if (i >= n) return;
  double acc = 0.0;
  const double2* zp = Z + (size_t)c0 * ldz + i;
  for (int j = c0; j < c1; ++j, zp += ldz) {
    const double2 a = *zp;
    acc = fma(fabs(a.x) + fabs(a.y), xs[j - c0], acc);
  }
  partial[(size_t)blockIdx.y * n + i] = acc;
}

// *out = max_i cabs1(r_i) / ((|Z| |x|)_i + cabs1(v_i)) (one block; the Oettli-Prager
// componentwise backward error of x, as LAPACK's zgerfs measures it)
__global__ void __launch_bounds__(1024) berr_finish_kernel(const double2* __restrict__ r,
                                                           const double2* __restrict__ v,
                                                           const double* __restrict__ partial, int nchunks, int n,
                                                           double* out) {
  __shared__ double sh[1024];
  double w = 0.0;
  for (int i = threadIdx.x; i < n; i += 1024) {
    double den = fabs(v[i].x) + fabs(v[i].y);
    for (int c = 0; c < nchunks; ++c) den += partial[(size_t)c * n + i];
    const double num = fabs(r[i].x) + fabs(r[i].y);
    if (num > 0.0) w = fmax(w, den > 0.0 ? num / den : HUGE_VAL);
  }
  sh[threadIdx.x] = w;
  __syncthreads();
  for (int s = 512; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

__global__ void widen_vec_kernel(const float2* __restrict__ d, double2* __restrict__ x, size_t count) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < count) x[i] = make_double2((double)d[i].x, (double)d[i].y);
}

// Lumped loads: one thread per matrix adds its loads in list order.
__global__ void add_loads_kernel(double2* __restrict__ Z, long long ldz, long long zstride, const int* __restrict__ idx,
                                 const double2* __restrict__ val, int nloads, int nk) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nk) return;
  for (int l = 0; l < nloads; ++l) {
    const int d = idx[l] - 1;
    double2* p = Z + (size_t)k * zstride + (size_t)d * ldz + d;
    const double2 a = val[(size_t)k * nloads + l];
    p->x += a.x;
    p->y += a.y;
  }
}

cudaError_t residual_fp64(const double2* Z, long long ldz, long long zstride, const double2* x, const double2* v,
                          int n, double2* r, double2* partial, int nvec, cudaStream_t s, const int* sel,
                          const int* vsel) {
  const int nchunks = (n + kGemvChunk - 1) / kGemvChunk;
  stats::Scope sc(stats::kResidual, s, 16.0 * n * (double)n * nvec, 2);
  gemv_partial_kernel<<<dim3((n + kGemvRows - 1) / kGemvRows, nchunks, nvec), kGemvRows, 0, s>>>(
      Z, ldz, zstride, x, n, partial, sel, vsel);
  residual_finish_kernel<<<dim3((n + 255) / 256, nvec), 256, 0, s>>>(v, partial, nchunks, n, r, sel, vsel);
  return cudaGetLastError();
}

cudaError_t sumsq_fp64(const double2* x, int n, double* out, int nvec, cudaStream_t s) {
  stats::count(stats::kMisc);
  sumsq_kernel<<<nvec, 1024, 0, s>>>(x, n, out);
  return cudaGetLastError();
}

cudaError_t convert_flat_64_to_32(const double2* src, float2* dst, size_t count, cudaStream_t s) {
  stats::Scope sc(stats::kMisc, s, 24.0 * (double)count);
  convert_flat_kernel<<<4 * 152, 256, 0, s>>>(src, dst, count);
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

#define SWEEP_TRY(call)                                      \
  do {                                                       \
    cudaError_t _e = (call);                                 \
    if (_e != cudaSuccess) return wmom_fail_cuda(_e, #call); \
  } while (0)

// Per-matrix scalars of a group, one D2H per refinement step.
struct GroupScalars {
  double rnorm2[kMaxLuBatch];
  double dnorm2[kMaxLuBatch];
  double xnorm2[kMaxLuBatch];
  double berr[kMaxLuBatch];    // componentwise backward errors of the second tier
  double anorm[kMaxLuBatch];   // ||Z||_1 of the group's matrices (condition estimates)
  double vnorm2;
};

// Autotuned factorisation shape per (order bucket, form).
std::mutex g_tune_mu;
std::map<std::pair<int, int>, LuConfig> g_tuned;

int env_int(const char* name, int lo, int hi) {
  const char* e = std::getenv(name);
  if (!e) return 0;
  const int b = std::atoi(e);
  return (b >= lo && b <= hi) ? b : 0;
}

// Krylov space per GMRES cycle and cycles per correction of the Krylov refinement
// (WMOM_GMRES_RESTART, WMOM_GMRES_CYCLES override).
int gmres_restart() {
  const int v = env_int("WMOM_GMRES_RESTART", 4, 400);
  return v ? v : 30;
}
// GMRES refinement with the FP32 factors before the FP64-grade tiers: on by default
// only without the tensor-core second tier, which serves a stalled matrix in less
// time than GMRES (measured on the grid workloads: 6.12 vs 5.83 freq-solves/s at
// N = 8192, 67.9 vs 57.8 at N = 2048).  WMOM_KRYLOV=1 / 0 forces it on / off.
bool krylov_enabled() {
  const char* e = std::getenv("WMOM_KRYLOV");
  if (e && e[0] == '1') return true;
  if (e && e[0] == '0') return false;
  return emul_gemm_hook() == nullptr;
}
int gmres_cycles() {
  const int v = env_int("WMOM_GMRES_CYCLES", 1, 20);
  return v ? v : 2;
}

}  // namespace

// Vectors, scalars and the FP64-fallback factor of one group of up to B matrices.
struct GroupScratch {
  int n = 0, B = 0;
  cudaStream_t s = nullptr;
  DevBuf vrep, x64, r64, d32, part, sc, scal, actv, sel, fb_lu, fb_ipiv, fb_x, fb_r;
  int fb_cap = 0;          // matrices per batched FP64-grade factorisation (tiers 2, 3)
  std::vector<double> vh;  // excitation on the host
  double vnorm = 0.0;
  GroupScalars hs{};
};

namespace {

wmom_status scratch_init(GroupScratch* g, int n, int B, int ngap, float ampl, float phas, cudaStream_t s) {
  g->n = n;
  g->B = B;
  g->s = s;
  const int nchunks = (n + kGemvChunk - 1) / kGemvChunk;
  g->vh.assign(2 * (size_t)n, 0.0);
  wmom_status st = wmom_excitation(n, ngap, ampl, phas, g->vh.data());
  if (st != WMOM_OK) return st;
  SWEEP_TRY(g->vrep.alloc(sizeof(double2) * (size_t)n * B, s));
  SWEEP_TRY(g->x64.alloc(sizeof(double2) * (size_t)n * B, s));
  SWEEP_TRY(g->r64.alloc(sizeof(double2) * (size_t)n * B, s));
  SWEEP_TRY(g->d32.alloc(sizeof(float2) * (size_t)n * B, s));
  SWEEP_TRY(g->part.alloc(sizeof(double2) * (size_t)n * nchunks * B, s));
  SWEEP_TRY(g->sc.alloc(sizeof(GroupScalars), s));
  SWEEP_TRY(g->scal.alloc(sizeof(double) * 2 * kMaxLuBatch, s));
  SWEEP_TRY(g->actv.alloc(sizeof(int) * kMaxLuBatch, s));
  SWEEP_TRY(g->sel.alloc(sizeof(int) * 2 * kMaxLuBatch, s));
  for (int b = 0; b < B; ++b)
    SWEEP_TRY(cudaMemcpyAsync(g->vrep.as<double2>() + (size_t)b * n, g->vh.data(), sizeof(double2) * n,
                              cudaMemcpyHostToDevice, s));
  GroupScalars* dsc = g->sc.as<GroupScalars>();
  SWEEP_TRY(sumsq_fp64(g->vrep.as<double2>(), n, &dsc->vnorm2, 1, s));
  SWEEP_TRY(cudaMemcpyAsync(&g->hs, dsc, sizeof(GroupScalars), cudaMemcpyDeviceToHost, s));
  SWEEP_TRY(cudaStreamSynchronize(s));
  g->vnorm = std::sqrt(g->hs.vnorm2);
  return WMOM_OK;
}

// relative residuals of x64[0..nb) against Z (nb matrices, contiguous)
wmom_status group_residuals(GroupScratch& g, const double2* Z, int nb) {
  const int n = g.n;
  GroupScalars* dsc = g.sc.as<GroupScalars>();
  SWEEP_TRY(residual_fp64(Z, n, (long long)n * n, g.x64.as<double2>(), g.vrep.as<double2>(), n,
                          g.r64.as<double2>(), g.part.as<double2>(), nb, g.s));
  SWEEP_TRY(sumsq_fp64(g.r64.as<double2>(), n, dsc->rnorm2, nb, g.s));
  SWEEP_TRY(cudaMemcpyAsync(&g.hs, dsc, sizeof(GroupScalars), cudaMemcpyDeviceToHost, g.s));
  SWEEP_TRY(cudaStreamSynchronize(g.s));
  return WMOM_OK;
}

}  // namespace

// ------------------------------------------------------------- GMRES-IR ----
// Left-preconditioned restarted GMRES in FP64 on M^-1 Z d = M^-1 r with M = the FP32
// LU factors: the refinement for systems too ill-conditioned for the plain FP32
// correction (kappa * u_fp32 >~ 1), before resorting to the FP64 LU.

// y = sum of the partial products (chunk order)
__global__ void matvec_finish_kernel(const double2* __restrict__ partial, int nchunks, int n,
                                     double2* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double re = 0.0, im = 0.0;
  for (int c = 0; c < nchunks; ++c) {
    const double2 p = partial[(size_t)c * n + i];
    re += p.x;
    im += p.y;
  }
  y[i] = make_double2(re, im);
}

// h[i] = conj(V_i) . w, one block per vector, fixed reduction order
__global__ void __launch_bounds__(1024) cdot_many_kernel(const double2* __restrict__ V, int n,
                                                         const double2* __restrict__ w, double2* __restrict__ h) {
  __shared__ double sr[1024], si[1024];
  const double2* v = V + (size_t)blockIdx.x * n;
  double re = 0.0, im = 0.0;
  for (int i = threadIdx.x; i < n; i += 1024) {
    const double2 a = v[i], b = w[i];
    re = fma(a.x, b.x, fma(a.y, b.y, re));
    im = fma(a.x, b.y, fma(-a.y, b.x, im));
  }
  sr[threadIdx.x] = re;
  si[threadIdx.x] = im;
  __syncthreads();
  for (int s = 512; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sr[threadIdx.x] += sr[threadIdx.x + s];
      si[threadIdx.x] += si[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) h[blockIdx.x] = make_double2(sr[0], si[0]);
}

// w -= sum_i h[i] V_i   (sign = -1)   or   w += sum_i h[i] V_i   (sign = +1)
__global__ void caxpy_many_kernel(double2* __restrict__ w, const double2* __restrict__ V, int k, int n,
                                  const double2* __restrict__ h, double sign) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double re = w[i].x, im = w[i].y;
  for (int q = 0; q < k; ++q) {
    const double2 c = h[q], v = V[(size_t)q * n + i];
    re = fma(sign * c.x, v.x, fma(-sign * c.y, v.y, re));
    im = fma(sign * c.x, v.y, fma(sign * c.y, v.x, im));
  }
  w[i] = make_double2(re, im);
}

__global__ void rscale_kernel(const double2* __restrict__ w, double2* __restrict__ v, int n, double s) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = make_double2(w[i].x * s, w[i].y * s);
}

namespace {

struct Cplx {
  double re, im;
};
inline Cplx cm(Cplx a, Cplx b) { return Cplx{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline Cplx cconj(Cplx a) { return Cplx{a.re, -a.im}; }
inline double cabsd(Cplx a) { return std::hypot(a.re, a.im); }

}  // namespace

// d = GMRES(m) solution of M^-1 Z d = M^-1 r for ONE matrix.  z/lu/ipiv address that
// matrix; r (device, n) is the right-hand side; d (device, n) receives the
// correction.  Returns the inner steps taken in *steps.
wmom_status gmres_correction(int n, const double2* Z, const float2* lu, const int* ipiv, const double2* r,
                             double2* d, LuWorkspace* ws, cudaStream_t s, int m, int max_cycles, double inner_tol,
                             int* steps) {
  const int nchunks = (n + kGemvChunk - 1) / kGemvChunk;
  DevBuf V, w, part, h, f32, nrm;
  SWEEP_TRY(V.alloc(sizeof(double2) * (size_t)n * (m + 1), s));
  SWEEP_TRY(w.alloc(sizeof(double2) * n, s));
  SWEEP_TRY(part.alloc(sizeof(double2) * (size_t)n * nchunks, s));
  SWEEP_TRY(h.alloc(sizeof(double2) * (m + 2) * 2, s));
  SWEEP_TRY(f32.alloc(sizeof(float2) * n, s));
  SWEEP_TRY(nrm.alloc(sizeof(double) * 2, s));
  const unsigned vb = (unsigned)((n + 255) / 256);
  double2* Vp = V.as<double2>();
  double2* wp = w.as<double2>();
  double2* hp = h.as<double2>();
  double* np_ = nrm.as<double>();
  // preconditioner: dst = M^-1 src (FP32 solve of the src scaled into range)
  auto precond = [&](const double2* src, double2* dst) -> wmom_status {
    double ss = 0.0;
    SWEEP_TRY(sumsq_fp64(src, n, np_, 1, s));
    SWEEP_TRY(cudaMemcpyAsync(&ss, np_, sizeof(double), cudaMemcpyDeviceToHost, s));
    SWEEP_TRY(cudaStreamSynchronize(s));
    const double rn = std::sqrt(ss);
    const double scl = (rn > 0 && std::isfinite(rn)) ? std::ldexp(1.0, -std::ilogb(rn)) : 1.0;
    DevBuf sc2;
    SWEEP_TRY(sc2.alloc(sizeof(double) * 2, s));
    const double hsc[2] = {scl, 1.0 / scl};
    SWEEP_TRY(cudaMemcpyAsync(sc2.p, hsc, sizeof(hsc), cudaMemcpyHostToDevice, s));
    stats::count(stats::kMisc, 2);
    convert_vec_kernel<<<vb, 256, 0, s>>>(src, f32.as<float2>(), n, 1, sc2.as<double>());
    SWEEP_TRY(lu_solve_t<float2>(lu, n, n, ipiv, f32.as<float2>(), n, 1, ws, s, 1, 0));
    widen_vec_kernel<<<vb, 256, 0, s>>>(f32.as<float2>(), dst, (size_t)n);
    rscale_kernel<<<vb, 256, 0, s>>>(dst, dst, n, 1.0 / scl);
    SWEEP_TRY(cudaStreamSynchronize(s));  // hsc lives on this frame
    return cudaGetLastError() == cudaSuccess ? WMOM_OK : WMOM_ERR_CUDA;
  };
  auto norm = [&](const double2* x, double* out) -> wmom_status {
    SWEEP_TRY(sumsq_fp64(x, n, np_, 1, s));
    double ss = 0.0;
    SWEEP_TRY(cudaMemcpyAsync(&ss, np_, sizeof(double), cudaMemcpyDeviceToHost, s));
    SWEEP_TRY(cudaStreamSynchronize(s));
    *out = std::sqrt(ss);
    return WMOM_OK;
  };
  SWEEP_TRY(cudaMemsetAsync(d, 0, sizeof(double2) * n, s));
  *steps = 0;
  // initial residual of the preconditioned system for d = 0: M^-1 r
  DevBuf r0;
  SWEEP_TRY(r0.alloc(sizeof(double2) * n, s));
  SWEEP_TRY(cudaMemcpyAsync(r0.p, r, sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
  double beta0 = -1.0;
  for (int cycle = 0; cycle < max_cycles; ++cycle) {
    wmom_status st = precond(r0.as<double2>(), wp);
    if (st != WMOM_OK) return st;
    double beta = 0.0;
    st = norm(wp, &beta);
    if (st != WMOM_OK) return st;
    if (beta0 < 0) beta0 = beta;
    if (!(beta > 0) || beta <= inner_tol * beta0) break;
    stats::count(stats::kMisc);
    rscale_kernel<<<vb, 256, 0, s>>>(wp, Vp, n, 1.0 / beta);
    std::vector<Cplx> H((size_t)(m + 1) * m, Cplx{0, 0}), g(m + 1, Cplx{0, 0});
    std::vector<double> cs(m);
    std::vector<Cplx> sn(m);
    g[0] = Cplx{beta, 0.0};
    int jlast = -1;
    for (int j = 0; j < m; ++j) {
      // w = M^-1 Z v_j
      stats::count(stats::kMisc, 1);
      {
        stats::Scope sc(stats::kResidual, s, 16.0 * n * (double)n, 1);
        gemv_partial_kernel<<<dim3((n + kGemvRows - 1) / kGemvRows, nchunks, 1), kGemvRows, 0, s>>>(
            Z, n, 0, Vp + (size_t)j * n, n, part.as<double2>(), nullptr, nullptr);
      }
      matvec_finish_kernel<<<vb, 256, 0, s>>>(part.as<double2>(), nchunks, n, wp);
      st = precond(wp, wp);
      if (st != WMOM_OK) return st;
      // classical Gram-Schmidt, twice
      std::vector<double2> hh(2 * (j + 1));
      stats::count(stats::kMisc, 4);
      cdot_many_kernel<<<j + 1, 1024, 0, s>>>(Vp, n, wp, hp);
      caxpy_many_kernel<<<vb, 256, 0, s>>>(wp, Vp, j + 1, n, hp, -1.0);
      cdot_many_kernel<<<j + 1, 1024, 0, s>>>(Vp, n, wp, hp + (m + 2));
      caxpy_many_kernel<<<vb, 256, 0, s>>>(wp, Vp, j + 1, n, hp + (m + 2), -1.0);
      SWEEP_TRY(cudaMemcpyAsync(hh.data(), hp, sizeof(double2) * (j + 1), cudaMemcpyDeviceToHost, s));
      SWEEP_TRY(cudaMemcpyAsync(hh.data() + (j + 1), hp + (m + 2), sizeof(double2) * (j + 1), cudaMemcpyDeviceToHost,
                                s));
      double hn = 0.0;
      st = norm(wp, &hn);
      if (st != WMOM_OK) return st;
      for (int i = 0; i <= j; ++i)
        H[(size_t)i * m + j] = Cplx{hh[i].x + hh[j + 1 + i].x, hh[i].y + hh[j + 1 + i].y};
      H[(size_t)(j + 1) * m + j] = Cplx{hn, 0.0};
      // previous rotations, then a new one zeroing H[j+1][j]
      for (int i = 0; i < j; ++i) {
        const Cplx a = H[(size_t)i * m + j], b = H[(size_t)(i + 1) * m + j];
        const Cplx t1 = Cplx{cs[i] * a.re + (sn[i].re * b.re - sn[i].im * b.im), cs[i] * a.im + (sn[i].re * b.im + sn[i].im * b.re)};
        const Cplx cb = cm(cconj(sn[i]), a);
        H[(size_t)(i + 1) * m + j] = Cplx{-cb.re + cs[i] * b.re, -cb.im + cs[i] * b.im};
        H[(size_t)i * m + j] = t1;
      }
      const Cplx a = H[(size_t)j * m + j];
      const double bb = hn, aa = cabsd(a);
      const double rr = std::hypot(aa, bb);
      if (rr == 0.0) {
        jlast = j - 1;
        break;
      }
      cs[j] = aa / rr;
      sn[j] = aa > 0 ? Cplx{(a.re / aa) * bb / rr, (a.im / aa) * bb / rr} : Cplx{1.0, 0.0};
      // with this phase choice the rotated entry is (a/|a|) * rr
      H[(size_t)j * m + j] = aa > 0 ? Cplx{a.re / aa * rr, a.im / aa * rr} : Cplx{rr, 0.0};
      H[(size_t)(j + 1) * m + j] = Cplx{0.0, 0.0};
      const Cplx gj = g[j];
      g[j + 1] = Cplx{-(sn[j].re * gj.re + sn[j].im * gj.im) / 1.0, -(sn[j].re * gj.im - sn[j].im * gj.re)};
      g[j] = Cplx{cs[j] * gj.re, cs[j] * gj.im};
      // keep the rotation consistent: g_{j+1} = -conj(s) g_j, g_j = c g_j
      ++*steps;
      jlast = j;
      const double resid = cabsd(g[j + 1]);
      if (resid <= inner_tol * beta0 || hn == 0.0) break;
      if (j + 1 < m) {
        stats::count(stats::kMisc);
        rscale_kernel<<<vb, 256, 0, s>>>(wp, Vp + (size_t)(j + 1) * n, n, 1.0 / hn);
      }
    }
    if (jlast < 0) break;
    // y = H^-1 g (upper triangular), d += V y
    const int k = jlast + 1;
    std::vector<Cplx> y(k);
    for (int i = k - 1; i >= 0; --i) {
      Cplx acc = g[i];
      for (int q = i + 1; q < k; ++q) {
        const Cplx t = cm(H[(size_t)i * m + q], y[q]);
        acc = Cplx{acc.re - t.re, acc.im - t.im};
      }
      const Cplx hd = H[(size_t)i * m + i];
      const double den = hd.re * hd.re + hd.im * hd.im;
      y[i] = Cplx{(acc.re * hd.re + acc.im * hd.im) / den, (acc.im * hd.re - acc.re * hd.im) / den};
    }
    std::vector<double2> yd(k);
    for (int i = 0; i < k; ++i) yd[i] = make_double2(y[i].re, y[i].im);
    SWEEP_TRY(cudaMemcpyAsync(hp, yd.data(), sizeof(double2) * k, cudaMemcpyHostToDevice, s));
    stats::count(stats::kMisc);
    caxpy_many_kernel<<<vb, 256, 0, s>>>(d, Vp, k, n, hp, +1.0);
    SWEEP_TRY(cudaStreamSynchronize(s));  // yd lives on this frame
    // next cycle: r0 = r - Z d (FP64)
    SWEEP_TRY(residual_fp64(Z, n, 0, d, r, n, r0.as<double2>(), part.as<double2>(), 1, s));
    double cur = 0.0;
    st = precond(r0.as<double2>(), wp);
    if (st != WMOM_OK) return st;
    st = norm(wp, &cur);
    if (st != WMOM_OK) return st;
    if (cur <= inner_tol * beta0) break;
  }
  return WMOM_OK;
}

// Factorises bg matrices Z64 (contiguous).  Mixed: FP32 copy into lu32, tensor-core
// LU; FP64: copy into lu64, FP64 LU.  info[b] = LAPACK info of matrix b.  When ms
// is given the factorisation is timed with events on the stream.
// A captured factorisation (CUDA graph) of one (order, batch, buffers) combination:
// every group of a sweep factors into the same buffers, so the whole launch sequence
// of the blocked LU (a cooperative panel launch, interchanges, triangular solve and
// tensor-core update per panel) is captured once and replayed per group.
struct FactorGraph {
  cudaGraphExec_t exec = nullptr;
  int mode = -1, n = 0, bg = 0;
  const void* lu = nullptr;
  const int* ipiv = nullptr;
  int span = 0;
  int tile_n = 0, panel_w = 0;    // shape of the captured factorisation
  const float* tc_buf = nullptr;  // tensor-core scratch the capture used
  unsigned tc_gen = 0;
  bool failed = false;  // capture unsupported here: launch directly
  long long launches[stats::kNumCls] = {};  // kernel launches of one replay
  ~FactorGraph() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

namespace {
bool graphs_enabled() {
  const char* e = std::getenv("WMOM_NO_GRAPHS");
  return !(e && e[0] == '1');
}
}  // namespace

wmom_status factor_group(int mode, int n, const double2* Z64, int bg, float2* lu32, double2* lu64, int* ipiv,
                         LuWorkspace* ws, cudaStream_t s, int* info, float* ms, FactorGraph* graph, int span) {
  const size_t nn = (size_t)n * n;
  SWEEP_TRY(lu_workspace_reset_barrier(ws, s));
  if (mode == WMOM_MODE_MIXED)
    SWEEP_TRY(convert_flat_64_to_32(Z64, lu32, nn * bg, s));
  else if (Z64 != lu64)  // Z64 == lu64: the matrices were copied in already
    SWEEP_TRY(cudaMemcpyAsync(lu64, Z64, sizeof(double2) * nn * bg, cudaMemcpyDeviceToDevice, s));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (ms) {
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
  }
  const GemmHook<float2> hook32 = tc_gemm_hook();
  const void* lu = mode == WMOM_MODE_MIXED ? (const void*)lu32 : (const void*)lu64;
  auto direct = [&]() -> cudaError_t {
    return mode == WMOM_MODE_MIXED ? lu_factor_t<float2>(lu32, n, n, ipiv, ws, s, hook32, bg, (long long)nn, span)
                                   : lu_factor_t<double2>(lu64, n, n, ipiv, ws, s, nullptr, bg, (long long)nn);
  };
  cudaError_t fe = cudaSuccess;
  if (graph && graph->exec && (graph->tc_buf != ws->tc_buf || graph->tc_gen != ws->tc_gen)) {
    // the scratch was reallocated since the capture: capture again on the next use
    cudaGraphExecDestroy(graph->exec);
    graph->exec = nullptr;
  }
  const bool same_shape = graph && graph->tile_n == ws->tile_n && graph->panel_w == ws->panel_w;
  if (graph && graph->exec && !same_shape) {
    // the workspace's factorisation shape changed since the capture
    cudaGraphExecDestroy(graph->exec);
    graph->exec = nullptr;
  }
  if (graph && graph->exec && graph->mode == mode && graph->n == n && graph->bg == bg && graph->lu == lu &&
      graph->ipiv == ipiv && graph->span == span) {
    stats::add_counts(graph->launches);
    fe = cudaGraphLaunch(graph->exec, s);
  } else if (graph && !graph->failed && graphs_enabled() && same_shape && graph->mode == mode &&
             graph->n == n && graph->bg == bg && graph->lu == lu && graph->ipiv == ipiv && graph->span == span) {
    // second use of these buffers: capture the sequence, then replay it from now on
    cudaGraph_t g = nullptr;
    long long before[stats::kNumCls], after[stats::kNumCls];
    stats::snapshot(before);
    fe = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (fe == cudaSuccess) {
      const cudaError_t ce = direct();
      fe = cudaStreamEndCapture(s, &g);
      if (ce != cudaSuccess) fe = ce;
    }
    stats::snapshot(after);
    for (int i = 0; i < stats::kNumCls; ++i) graph->launches[i] = after[i] - before[i];
    if (fe == cudaSuccess) fe = cudaGraphInstantiate(&graph->exec, g, 0);
    if (g) cudaGraphDestroy(g);
    graph->tc_buf = ws->tc_buf;
    graph->tc_gen = ws->tc_gen;
    if (fe == cudaSuccess) {
      fe = cudaGraphLaunch(graph->exec, s);
    } else {
      // the capture counted launches that never ran
      for (int i = 0; i < stats::kNumCls; ++i) graph->launches[i] = -graph->launches[i];
      stats::add_counts(graph->launches);
      cudaGetLastError();  // clear the capture error, launch directly from now on
      graph->failed = true;
      if (graph->exec) {
        cudaGraphExecDestroy(graph->exec);
        graph->exec = nullptr;
      }
      fe = direct();
    }
  } else {
    if (graph && !graph->exec) {
      // remember the shape; the next group with the same shape is captured
      graph->mode = mode;
      graph->n = n;
      graph->bg = bg;
      graph->lu = lu;
      graph->ipiv = ipiv;
      graph->span = span;
      graph->tile_n = ws->tile_n;
      graph->panel_w = ws->panel_w;
    }
    fe = direct();
  }
  if (ms) {
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  if (fe != cudaSuccess) return wmom_fail_cuda(fe, "lu_factor_t");
  int err = lu_workspace_read_status(ws, info, s, bg);
  if (mode == WMOM_MODE_MIXED && hook32) err |= tc::read_and_clear_error(ws, s);
  SWEEP_TRY(cudaGetLastError());
  return err ? WMOM_ERR_TIMEOUT : WMOM_OK;
}

wmom_status choose_lu_config(int mode, int n, int limit, const double2* Z64, LuWorkspace* ws, cudaStream_t s,
                             size_t budget, LuConfig* out, bool timing);

namespace {

// In-place FP64 LU of the bg matrices in lu64 (n*n apart) whose trailing updates
// run through `hook` (the digit-plane tensor-core GEMM): the second tier's factors.
wmom_status factor_emul(int n, double2* lu64, int bg, int* ipiv, LuWorkspace* ws, cudaStream_t s, int* info,
                        GemmHook<double2> hook, bool ff) {
  SWEEP_TRY(lu_workspace_reset_barrier(ws, s));
  // Shape: span panels per tensor-core update, of at most w columns, K = span w <= 96
  // (the most one launch of the digit-plane GEMM takes).  Measured per 12-frequency
  // step (instrumented):
  //   N = 8192 grid: spans 1 / 2 / 3 of 32 columns 6.70 / 8.66 / 9.67 freq-solves/s;
  //     then w / span 32/3, 24/4, 16/6, 16/4: 946, 918, 932, 1032 ms;
  //   N = 2048 grid, 256 frequencies: 32/3, 24/4, 16/6, 16/4: 1192, 1201, 1239, 1213 ms.
  // Narrower panels cut the panels' and the triangular solves' FP64 work, at the
  // price of more, thinner launches, which only pays at large orders.
  // WMOM_EMUL_SPAN and WMOM_FP64_PANEL_W override.
  const bool large = n > 4096;
  const int es = env_int("WMOM_EMUL_SPAN", 1, kMaxSpan);
  const int saved_w64 = ws->panel_w64;
  ws->panel_w64 = large ? 24 : 32;
  ws->ff_storage = ff;  // lu64 holds float-float values (split_ff_inplace) when set
  const cudaError_t fe =
      lu_factor_t<double2>(lu64, n, n, ipiv, ws, s, hook, bg, (long long)n * n, es ? es : (large ? 4 : 3));
  ws->panel_w64 = saved_w64;
  ws->ff_storage = false;
  if (fe != cudaSuccess) return wmom_fail_cuda(fe, "lu_factor_t (tier 2)");
  int err = lu_workspace_read_status(ws, info, s, bg);
  err |= tc::read_and_clear_error(ws, s);
  SWEEP_TRY(cudaGetLastError());
  return err ? WMOM_ERR_TIMEOUT : WMOM_OK;
}

}  // namespace

// Solves bg systems Z64[b] x = V with the factors of factor_group; the solutions end
// in g.x64[0..bg).  Mixed: FP32 solve, FP64 refinement with a per-matrix activity
// mask, FP64 LU for the matrices that stall.
//
// Probe (mixed form, 0 < probe < bg, factor_rest given): the caller has FP32 factors
// for matrices [0, probe) only, the group's highest frequencies.  Those refine in
// tier 1 first.  If the lowest of them (matrix probe - 1) needs FP64-grade factors,
// matrices [probe, bg) -- lower frequencies, worse conditioned -- go straight to the
// second tier with it; otherwise factor_rest(probe, bg - probe, info + probe) gives
// them FP32 factors and they refine in tier 1 as well.
wmom_status solve_group(int mode, int n, const double2* Z64, int bg, const float2* lu32, const double2* lu64,
                        const int* ipiv, const int* info_in, double tol, LuWorkspace* ws, GroupScratch& g,
                        wmom_report* rep, bool condest, int nreal, bool direct_t2, int probe = 0,
                        const std::function<wmom_status(int, int, int*)>* factor_rest = nullptr) {
  int info[kMaxLuBatch] = {};
  std::copy(info_in, info_in + bg, info);
  if (nreal <= 0) nreal = n;
  const size_t nn = (size_t)n * n;
  cudaStream_t s = g.s;
  GroupScalars& hs = g.hs;
  GroupScalars* dsc = g.sc.as<GroupScalars>();
  for (int b = 0; b < bg; ++b) {
    rep[b] = wmom_report{};
    rep[b].rel_residual = -1.0;
    rep[b].info = info[b];
  }
  // condition estimates: ||Z||_1 now (read back with the next scalars), ||Z^-1||_1
  // from the factors behind each matrix's solution once it is final
  if (condest) SWEEP_TRY(norm1_batch(Z64, nreal, n, (long long)nn, bg, dsc->anorm, s));
  auto estimate = [&](auto* lu, const int* piv, auto* X, const std::vector<int>& slots,
                      const std::vector<int>& mats) -> wmom_status {
    if (!condest || slots.empty()) return WMOM_OK;
    std::vector<double> est(slots.size(), 0.0);
    const wmom_status cs = condest_t(n, nreal, lu, (long long)n, (long long)nn, piv, slots.data(),
                                     (int)slots.size(), X, ws, s, est.data());
    if (cs != WMOM_OK) return cs;
    for (size_t q = 0; q < slots.size(); ++q) rep[mats[q]].cond1 = hs.anorm[mats[q]] * est[q];
    return WMOM_OK;
  };
  // Componentwise backward errors max_i |r_i| / (|Z||x| + |V|)_i (LAPACK zgerfs'
  // measure, |z| = |re| + |im|) of the solutions in vector slots slot[q] of x and r,
  // matrix mat[q] of Zb, read back into hs.berr[slot[q]].  A refined solution whose
  // backward error is at most 4 sqrt(n) eps (eps = 2^-53) is as good as an FP64 LU's:
  // it solves a system within that relative distance of Z, entry by entry.
  const double eps64 = 0x1p-53;
  const double berr_ok = 4.0 * std::sqrt((double)n) * eps64;
  auto backward_errors = [&](const double2* Zb, const double2* x, const double2* r, const int* slot, const int* mat,
                             int cnt) -> wmom_status {
    if (cnt == 0) return WMOM_OK;
    const int nch = (n + kGemvChunk - 1) / kGemvChunk;
    double* part = reinterpret_cast<double*>(g.part.p);
    for (int q = 0; q < cnt; ++q) {
      stats::count(stats::kMisc, 2);
      absgemv_partial_kernel<<<dim3((n + kGemvRows - 1) / kGemvRows, nch), kGemvRows, 0, s>>>(
          Zb + (size_t)mat[q] * nn, n, x + (size_t)slot[q] * n, n, part);
      berr_finish_kernel<<<1, 1024, 0, s>>>(r + (size_t)slot[q] * n, g.vrep.as<double2>(), part, nch, n,
                                            &dsc->berr[slot[q]]);
      SWEEP_TRY(cudaGetLastError());
    }
    SWEEP_TRY(cudaMemcpyAsync(&hs, dsc, sizeof(GroupScalars), cudaMemcpyDeviceToHost, s));
    SWEEP_TRY(cudaStreamSynchronize(s));
    return WMOM_OK;
  };
  // WMOM_TRACE_REFINE=1: one line per refinement step and matrix on stderr
  const char* trace_env = std::getenv("WMOM_TRACE_REFINE");
  const bool trace = trace_env && trace_env[0] == '1';
  const char* t1_env = std::getenv("WMOM_T1_BERR");
  const bool t1_berr = !(t1_env && t1_env[0] == '0');
  if (mode == WMOM_MODE_FP64) {
    SWEEP_TRY(cudaMemcpyAsync(g.x64.p, g.vrep.p, sizeof(double2) * n * bg, cudaMemcpyDeviceToDevice, s));
    SWEEP_TRY(lu_solve_t<double2>(lu64, n, n, ipiv, g.x64.as<double2>(), n, 1, ws, s, bg, (long long)nn));
    const wmom_status rs = group_residuals(g, Z64, bg);
    if (rs != WMOM_OK) return rs;
    for (int b = 0; b < bg; ++b) {
      rep[b].status = info[b] ? WMOM_ERR_SINGULAR : WMOM_OK;
      rep[b].rel_residual = std::sqrt(hs.rnorm2[b]) / g.vnorm;
    }
    std::vector<int> all;
    for (int b = 0; b < bg; ++b)
      if (info[b] == 0) all.push_back(b);
    return estimate(lu64, ipiv, g.r64.as<double2>(), all, all);
  }
  bool fallback[kMaxLuBatch] = {}, active[kMaxLuBatch] = {};
  int stall[kMaxLuBatch] = {};
  double prev[kMaxLuBatch], last[kMaxLuBatch], rel_first[kMaxLuBatch], rel_best[kMaxLuBatch];
  const bool probing = mode == WMOM_MODE_MIXED && !direct_t2 && probe > 0 && probe < bg && factor_rest;
  const int t1_end = probing ? probe : bg;
  for (int b = 0; b < bg; ++b) {
    fallback[b] = direct_t2 || info[b] != 0;
    active[b] = !fallback[b] && b < t1_end;
    prev[b] = last[b] = rel_first[b] = rel_best[b] = HUGE_VAL;
  }
  // With the tensor-core second tier, a matrix whose refinement contracts slowly
  // leaves tier 1 once the steps it still needs (extrapolated from its last step)
  // would cost more than a second-tier factorisation: a step costs O(N^2) (residual
  // and two triangular solves), the factorisation O(N^3), so the limit grows with N
  // (8 steps at N = 2048, 32 at N = 8192).
  const bool tier2 = emul_gemm_hook() != nullptr;
  const double step_budget = std::max(8.0, n / 256.0);
  const unsigned vgrid = (unsigned)(((size_t)n * bg + 255) / 256);
  std::vector<int> hact(kMaxLuBatch, 0);
  std::vector<double> hscale(2 * kMaxLuBatch, 1.0);
  const int max_it = 40;
  // direct_t2: the caller predicts that no matrix of the group is served by its FP32
  // factors (none were computed); the group goes straight to the second tier
  // The FP32 solves of tier 1 multiply by the inverses of the factors' 64 x 64
  // diagonal blocks (lu_block_inverses, once per factorisation) instead of
  // substituting through each block with one warp: most of tier 1's later steps solve
  // one or two slowly converging matrices, whose solves are that chain of blocks.
  // WMOM_TRSV_INV=0 keeps the substitution.
  DevBuf t1inv;
  const size_t inv_per = lu_block_inverse_bytes<float2>(n, 1) / sizeof(float2);
  {
    const char* ie = std::getenv("WMOM_TRSV_INV");
    if (mode == WMOM_MODE_MIXED && !direct_t2 && !(ie && ie[0] == '0'))
      SWEEP_TRY(t1inv.alloc(lu_block_inverse_bytes<float2>(n, bg), s));
  }
  float2* t1invp = t1inv.p ? t1inv.as<float2>() : nullptr;
  // the factors' row permutations, once per factorisation (every solve of a matrix
  // applies the same one)
  DevBuf t1perm;
  if (mode == WMOM_MODE_MIXED && !direct_t2) SWEEP_TRY(t1perm.alloc(sizeof(int) * (size_t)n * bg, s));
  // Tier 1 for matrices [b0, b1): FP32 solve, then FP64 refinement of the active ones.
  auto tier1 = [&](int b0, int b1) -> wmom_status {
    if (t1invp)
      SWEEP_TRY(lu_block_inverses<float2>(lu32 + (size_t)b0 * nn, n, n, b1 - b0, (long long)nn,
                                          t1invp + (size_t)b0 * inv_per, s));
    SWEEP_TRY(lu_pivots_to_perm(ipiv + (size_t)b0 * n, n, b1 - b0, t1perm.as<int>() + (size_t)b0 * n, s));
    // the matrices still refining: residuals and corrections are computed for these
    // only (one slowly converging matrix no longer keeps its whole batch busy)
    std::vector<int> hsel(kMaxLuBatch, 0);
    int nsel = 0;
    for (int b = b0; b < b1; ++b)
      if (active[b]) hsel[nsel++] = b;
    SWEEP_TRY(cudaMemcpyAsync(g.sel.p, hsel.data(), sizeof(int) * kMaxLuBatch, cudaMemcpyHostToDevice, s));
    // initial solve in FP32
    stats::count(stats::kMisc, 2);
    convert_vec_kernel<<<vgrid, 256, 0, s>>>(g.vrep.as<double2>(), g.d32.as<float2>(), n, bg, nullptr);
    if (b0 == 0 && b1 == bg) {
      SWEEP_TRY(lu_solve_t<float2>(lu32, n, n, ipiv, g.d32.as<float2>(), n, 1, ws, s, bg, (long long)nn, nullptr,
                                   t1invp, t1perm.as<int>()));
    } else if (nsel > 0) {
      SWEEP_TRY(lu_solve_t<float2>(lu32, n, n, ipiv, g.d32.as<float2>(), n, 1, ws, s, nsel, (long long)nn,
                                   g.sel.as<int>(), t1invp, t1perm.as<int>()));
    }
    const size_t wcount = (size_t)n * (b1 - b0);
    widen_vec_kernel<<<(unsigned)((wcount + 255) / 256), 256, 0, s>>>(g.d32.as<float2>() + (size_t)b0 * n,
                                                                     g.x64.as<double2>() + (size_t)b0 * n, wcount);
    SWEEP_TRY(cudaGetLastError());
    for (int it = 0;; ++it) {
      if (nsel == 0) break;
      {
        GroupScalars* dscr = g.sc.as<GroupScalars>();
        SWEEP_TRY(residual_fp64(Z64, n, (long long)nn, g.x64.as<double2>(), g.vrep.as<double2>(), n,
                                g.r64.as<double2>(), g.part.as<double2>(), nsel, s, g.sel.as<int>()));
        SWEEP_TRY(sumsq_fp64(g.r64.as<double2>(), n, dscr->rnorm2, bg, s));
        SWEEP_TRY(cudaMemcpyAsync(&hs, dscr, sizeof(GroupScalars), cudaMemcpyDeviceToHost, s));
        SWEEP_TRY(cudaStreamSynchronize(s));
      }
      int nact = 0, nleave = 0, leave[kMaxLuBatch];
      for (int b = 0; b < bg; ++b) {
        if (!active[b]) continue;
        const double rel = std::sqrt(hs.rnorm2[b]) / g.vnorm;
        rep[b].rel_residual = rel;
        rep[b].iterations = it;
        if (it == 0) rel_first[b] = rel;
        if (rel < rel_best[b]) rel_best[b] = rel;
        // converged: the target is met, or the last correction no longer changes the
        // solution at FP64 resolution (systems whose FP64 residual floor lies above
        // the target); diverged: FP64 fallback; stalled, out of steps or converging
        // too slowly: FP64 fallback unless the solution is already backward stable
        const double corr = it > 0 ? std::sqrt(hs.dnorm2[b] / hs.xnorm2[b]) : HUGE_VAL;
        if (trace)
          std::fprintf(stderr, "wmom refine: tier 1 matrix %d step %d rel %.3e corr %.3e\n", b, it, rel, corr);
        if (!(rel == rel)) {
          fallback[b] = true;
          active[b] = false;
        } else if (rel <= tol || corr <= 0x1p-48) {
          active[b] = false;
        } else if ((rel > 0.5 * prev[b] && ++stall[b] >= 2) || it >= max_it ||
                   (tier2 && it >= 3 && rel < last[b] &&
                    std::log(tol / rel) / std::log(rel / last[b]) > step_budget)) {
          active[b] = false;
          leave[nleave++] = b;
        } else {
          if (rel <= 0.5 * prev[b]) stall[b] = 0;
          prev[b] = std::min(prev[b], rel);
          last[b] = rel;
          ++nact;
        }
      }
      // A matrix whose refinement stopped at the FP64 residual floor of its system
      // (above tol when kappa is large) keeps its tier-1 solution if that solution is
      // backward stable at FP64 level, the test the second tier accepts by; the FP64-
      // grade factorisation would only reach the same floor.
      // (WMOM_T1_BERR=0 turns this off: every such matrix then falls back.)
      if (!t1_berr)
        for (int q = 0; q < nleave; ++q) fallback[leave[q]] = true;
      if (nleave > 0 && t1_berr) {
        const wmom_status bs =
            backward_errors(Z64, g.x64.as<double2>(), g.r64.as<double2>(), leave, leave, nleave);
        if (bs != WMOM_OK) return bs;
        for (int q = 0; q < nleave; ++q) {
          const int b = leave[q];
          fallback[b] = !(hs.berr[b] <= berr_ok);
          if (trace)
            std::fprintf(stderr, "wmom refine: tier 1 matrix %d leaves at step %d, backward error %.3e -> %s\n", b,
                         it, hs.berr[b], fallback[b] ? "fallback" : "accepted");
        }
      }
      if (nact == 0) break;
      // correction d = (LU32)^-1 r per active matrix, scaled by a power of two
      for (int b = 0; b < bg; ++b) {
        const double rn = std::sqrt(hs.rnorm2[b]);
        const double scl = (active[b] && rn > 0 && std::isfinite(rn)) ? std::ldexp(1.0, -std::ilogb(rn)) : 1.0;
        hscale[b] = scl;
        hscale[kMaxLuBatch + b] = 1.0 / scl;
        hact[b] = active[b] ? 1 : 0;
      }
      nsel = 0;
      for (int b = 0; b < bg; ++b)
        if (active[b]) hsel[nsel++] = b;
      SWEEP_TRY(cudaMemcpyAsync(g.scal.p, hscale.data(), sizeof(double) * 2 * kMaxLuBatch, cudaMemcpyHostToDevice, s));
      SWEEP_TRY(cudaMemcpyAsync(g.actv.p, hact.data(), sizeof(int) * kMaxLuBatch, cudaMemcpyHostToDevice, s));
      SWEEP_TRY(cudaMemcpyAsync(g.sel.p, hsel.data(), sizeof(int) * kMaxLuBatch, cudaMemcpyHostToDevice, s));
      const double* dscale = g.scal.as<double>();
      const double* dinv = dscale + kMaxLuBatch;
      stats::count(stats::kMisc, 4);
      convert_vec_kernel<<<vgrid, 256, 0, s>>>(g.r64.as<double2>(), g.d32.as<float2>(), n, bg, dscale);
      SWEEP_TRY(lu_solve_t<float2>(lu32, n, n, ipiv, g.d32.as<float2>(), n, 1, ws, s, nsel, (long long)nn,
                                   nsel == bg ? nullptr : g.sel.as<int>(), t1invp, t1perm.as<int>()));

      sumsq_f32_kernel<<<bg, 1024, 0, s>>>(g.d32.as<float2>(), n, dinv, dsc->dnorm2);
      sumsq_kernel<<<bg, 1024, 0, s>>>(g.x64.as<double2>(), n, dsc->xnorm2);
      accumulate_vec_kernel<<<vgrid, 256, 0, s>>>(g.x64.as<double2>(), g.d32.as<float2>(), n, bg, dinv,
                                                  g.actv.as<int>());
      SWEEP_TRY(cudaGetLastError());
    }
    int tmp_info[kMaxLuBatch];
    if (lu_workspace_read_status(ws, tmp_info, s, 1)) return WMOM_ERR_TIMEOUT;
    // GMRES-IR for the matrices whose plain refinement made progress (at least a
    // factor kKrylovEntry below the first residual) before it stalled: their FP32
    // factors are still a usable preconditioner.  The others -- refinement diverged or
    // barely moved, i.e. kappa * u_fp32 >> 1 -- go straight to the FP64 LU.
    constexpr double kKrylovEntry = 1e-3;
    for (int b = b0; b < b1; ++b) {
      if (!krylov_enabled()) break;
      if (!fallback[b] || info[b] != 0) continue;
      if (!(rel_best[b] <= kKrylovEntry * rel_first[b])) continue;
      double2* xb = g.x64.as<double2>() + (size_t)b * n;
      const double2* Zb = Z64 + (size_t)b * nn;
      const float2* lub = lu32 + (size_t)b * nn;
      const int* ipb = ipiv + (size_t)b * n;
      DevBuf dv;
      SWEEP_TRY(dv.alloc(sizeof(double2) * n, s));
      // budget: a correction must cut the residual by kKrylovGain, else the FP32
      // factors are too poor a preconditioner here and the FP64 LU takes over
      constexpr double kKrylovGain = 1e-2;
      double prevr = HUGE_VAL, corr = HUGE_VAL;
      bool ok = false;
      for (int outer = 0; outer < 6; ++outer) {
        SWEEP_TRY(residual_fp64(Zb, n, 0, xb, g.vrep.as<double2>(), n, g.r64.as<double2>(), g.part.as<double2>(), 1,
                                s));
        SWEEP_TRY(sumsq_fp64(g.r64.as<double2>(), n, dsc->rnorm2, 1, s));
        SWEEP_TRY(sumsq_fp64(xb, n, dsc->xnorm2, 1, s));
        SWEEP_TRY(cudaMemcpyAsync(&hs, dsc, sizeof(GroupScalars), cudaMemcpyDeviceToHost, s));
        SWEEP_TRY(cudaStreamSynchronize(s));
        const double rel = std::sqrt(hs.rnorm2[0]) / g.vnorm;
        if (!(rel == rel)) {
          // diverged plain refinement: start the Krylov refinement from zero
          SWEEP_TRY(cudaMemsetAsync(xb, 0, sizeof(double2) * n, s));
          prevr = HUGE_VAL;
          continue;
        }
        rep[b].rel_residual = rel;
        if (rel <= tol || corr <= 0x1p-48) {
          ok = true;
          break;
        }
        if (rel > kKrylovGain * prevr) break;
        prevr = rel;
        int steps = 0;
        const wmom_status gs = gmres_correction(n, Zb, lub, ipb, g.r64.as<double2>(), dv.as<double2>(), ws, s,
                                                gmres_restart(), gmres_cycles(), 1e-10, &steps);
        if (gs != WMOM_OK) return gs;
        rep[b].krylov_steps += steps;
        rep[b].iterations += 1;
        const double xn = std::sqrt(hs.xnorm2[0]);
        SWEEP_TRY(sumsq_fp64(dv.as<double2>(), n, dsc->dnorm2, 1, s));
        SWEEP_TRY(cudaMemcpyAsync(&hs, dsc, sizeof(GroupScalars), cudaMemcpyDeviceToHost, s));
        SWEEP_TRY(cudaStreamSynchronize(s));
        corr = xn > 0 ? std::sqrt(hs.dnorm2[0]) / xn : HUGE_VAL;
        // x += d
        stats::count(stats::kMisc);
        std::vector<double2> onec(1, make_double2(1.0, 0.0));
        DevBuf cbuf;
        SWEEP_TRY(cbuf.alloc(sizeof(double2), s));
        SWEEP_TRY(cudaMemcpyAsync(cbuf.p, onec.data(), sizeof(double2), cudaMemcpyHostToDevice, s));
        caxpy_many_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(xb, dv.as<double2>(), 1, n, cbuf.as<double2>(),
                                                                      +1.0);
        SWEEP_TRY(cudaStreamSynchronize(s));
      }
      if (ok) fallback[b] = false;
    }
    return WMOM_OK;
  };
  if (!direct_t2) {
    wmom_status ts = tier1(0, t1_end);
    if (ts != WMOM_OK) return ts;
    if (probing) {
      const bool predict_rest = fallback[probe - 1];
      if (trace)
        std::fprintf(stderr, "wmom refine: probe of %d of %d matrices: matrices %d..%d %s\n", probe, bg, probe,
                     bg - 1, predict_rest ? "go to the second tier" : "get FP32 factors");
      if (predict_rest) {
        for (int b = probe; b < bg; ++b) fallback[b] = true;
      } else {
        ts = (*factor_rest)(probe, bg - probe, info + probe);
        if (ts != WMOM_OK) return ts;
        for (int b = probe; b < bg; ++b) {
          rep[b].info = info[b];
          fallback[b] = info[b] != 0;
          active[b] = !fallback[b];
        }
        ts = tier1(probe, bg);
        if (ts != WMOM_OK) return ts;
      }
    }
    for (int b = 0; b < bg; ++b)
      if (!fallback[b]) {
        rep[b].status = WMOM_OK;
        rep[b].tier = 1;
      }
    {
      // tier 1: the FP32 factors (their estimate is kappa of the FP32-rounded Z, which
      // refinement only reaches when kappa * u_fp32 < 1)
      std::vector<int> t1;
      for (int b = 0; b < bg; ++b)
        if (!fallback[b]) t1.push_back(b);
      const wmom_status cs = estimate(lu32, ipiv, g.d32.as<float2>(), t1, t1);
      if (cs != WMOM_OK) return cs;
    }
  }
  // The matrices the FP32 factors could not serve get FP64-grade factors, batched
  // as wide as the plain FP64 form batches at this order (copies in the scratch
  // factor buffer, so that their panels run side by side).
  //   Tier 2: FP64 LU whose trailing updates run on the bf16 tensor cores from
  //   digit planes (lu_emul.cu), then FP64 refinement as above.  A matrix is accepted
  //   when its residual meets tol or the correction no longer changes x at FP64
  //   resolution; when its refinement stalls instead (the FP64 residual floor of an
  //   ill-conditioned system), it is accepted if its componentwise backward error
  //   max_i |r_i| / (|Z||x| + |V|)_i (LAPACK zgerfs' measure, with |z| = |re| + |im|)
  //   is at most 4 sqrt(n) eps, eps = 2^-53: such a solution is as good as an FP64
  //   LU's, from which it differs by about kappa * eps.
  //   Tier 3: plain FP64 LU for the matrices whose tier-2 refinement stalled, and for
  //   every matrix when the device has no tensor-core path (or WMOM_NO_EMUL is set).
  int nfb = 0, fb[kMaxLuBatch];
  for (int b = 0; b < bg; ++b)
    if (fallback[b]) fb[nfb++] = b;
  if (nfb == 0) return WMOM_OK;
  const GemmHook<double2> emul = emul_gemm_hook();
  if (g.fb_cap == 0) {
    size_t fr = 0, tot = 0;
    SWEEP_TRY(cudaMemGetInfo(&fr, &tot));
    int cap = 1;
    if (emul) {
      // with its updates on the tensor cores the second tier's time goes to the FP64
      // panels, which run side by side across a batch: as wide as co-residency of
      // the panel, the workspace and a quarter of the free memory allow
      cap = std::min({g.B, ws->max_batch, kMaxLuBatch, lu_max_batch<double2>(n, true)});
      const int eb = env_int("WMOM_LU_BATCH", 1, kMaxLuBatch);
      if (eb) cap = std::min(cap, eb);
      while (cap > 1 && (size_t)cap * nn * sizeof(double2) > fr / 4) --cap;
    } else {
      LuConfig c64;
      const wmom_status cs = choose_lu_config(WMOM_MODE_FP64, n, g.B, nullptr, ws, s, fr / 2, &c64, false);
      if (cs != WMOM_OK) return cs;
      cap = c64.batch;
    }
    cap = std::max(1, std::min(cap, g.B));
    SWEEP_TRY(g.fb_lu.alloc(sizeof(double2) * nn * cap, s));
    SWEEP_TRY(g.fb_ipiv.alloc(sizeof(int) * (size_t)n * cap, s));
    SWEEP_TRY(g.fb_x.alloc(sizeof(double2) * (size_t)n * cap, s));
    SWEEP_TRY(g.fb_r.alloc(sizeof(double2) * (size_t)n * cap, s));
    g.fb_cap = cap;
  }
  double2* flu = g.fb_lu.as<double2>();
  double2* fx = g.fb_x.as<double2>();
  double2* frr = g.fb_r.as<double2>();
  int* fpiv = g.fb_ipiv.as<int>();
  for (int c0 = 0; c0 < nfb; c0 += g.fb_cap) {
    const int cn = std::min(g.fb_cap, nfb - c0);
    bool plain[kMaxLuBatch];
    for (int j = 0; j < cn; ++j) {
      plain[j] = true;
      rep[fb[c0 + j]].fell_back = 1;
    }
    if (emul) {
      for (int j = 0; j < cn; ++j)
        SWEEP_TRY(cudaMemcpyAsync(flu + (size_t)j * nn, Z64 + (size_t)fb[c0 + j] * nn, sizeof(double2) * nn,
                                  cudaMemcpyDeviceToDevice, s));
      int inf[kMaxLuBatch] = {};
      // With WMOM_FF_TIER2=1 the second tier factors in float-float form where its
      // panels allow (ff_tier2_supported): the matrices are split in place first, and
      // panels, block solves and the digit-plane updates' C work on that form on the
      // FP32 pipe.  Measured per step (N = 8192 grid / 256-frequency N = 2048 grid):
      // 888 / 896 ms against 869 / 904 ms with complex128 storage and float-float
      // panels, the default.  The panels and block solves gain 21 ms, but the
      // digit-plane packs then convert every entry back to FP64 (+43 ms), and the
      // update's epilogue does not speed up (its bound is the tcgen05 instruction
      // path).  By default the factors are split after the factorisation.  Either way
      // the solves below run in compensated FP32 (lu_solve_ff: about 2^-48 per
      // operation, below the factors' own error), with every right-hand side scaled
      // by a power of two to a norm near 1, inside FP32's range.  The condition
      // estimate merges them back to FP64 first.
      const char* ffe = std::getenv("WMOM_FF_TIER2");
      const bool ff = ffe && ffe[0] == '1' && ff_tier2_supported(n, n > 4096 ? 24 : 32);
      if (ff) SWEEP_TRY(split_ff_inplace(flu, nn * cn, s));
      const wmom_status fst = factor_emul(n, flu, cn, fpiv, ws, s, inf, emul, ff);
      if (fst != WMOM_OK) return fst;
      if (!ff) SWEEP_TRY(split_ff_inplace(flu, nn * cn, s));
      const float4* fff = reinterpret_cast<const float4*>(flu);
      // the inverses of the factors' 64 x 64 diagonal blocks, once per factorisation:
      // every solve below then takes each block in one parallel product instead of a
      // 64-step substitution by one warp (WMOM_FF_TRSV_INV=0 keeps the substitution)
      DevBuf finv;
      const float4* finvp = nullptr;
      {
        const char* ie = std::getenv("WMOM_FF_TRSV_INV");
        if (!(ie && ie[0] == '0')) {
          SWEEP_TRY(finv.alloc(ff_block_inverse_bytes(n, cn), s));
          SWEEP_TRY(ff_block_inverses(fff, n, n, cn, (long long)nn, finv.as<float4>(), s));
          finvp = finv.as<float4>();
        }
      }
      // the chunk's row permutations, once for all its solves
      DevBuf fperm;
      SWEEP_TRY(fperm.alloc(sizeof(int) * (size_t)n * cn, s));
      SWEEP_TRY(lu_pivots_to_perm(fpiv, n, cn, fperm.as<int>(), s));
      double* dscale = g.scal.as<double>();
      auto scale_slots = [&](double2* v, const double* norm, int cnt) -> wmom_status {
        for (int j = 0; j < kMaxLuBatch; ++j) {
          const double rn = j < cnt ? norm[j] : 0.0;
          const double sc = (rn > 0 && std::isfinite(rn)) ? std::ldexp(1.0, -std::ilogb(rn)) : 1.0;
          hscale[j] = sc;
          hscale[kMaxLuBatch + j] = 1.0 / sc;
        }
        SWEEP_TRY(cudaMemcpyAsync(g.scal.p, hscale.data(), sizeof(double) * 2 * kMaxLuBatch, cudaMemcpyHostToDevice,
                                  s));
        stats::count(stats::kMisc);
        scale_vec64_kernel<<<(unsigned)(((size_t)n * cnt + 255) / 256), 256, 0, s>>>(v, n, cnt, dscale);
        SWEEP_TRY(cudaGetLastError());
        return WMOM_OK;
      };
      auto unscale_slots = [&](double2* v, int cnt) -> wmom_status {
        stats::count(stats::kMisc);
        scale_vec64_kernel<<<(unsigned)(((size_t)n * cnt + 255) / 256), 256, 0, s>>>(v, n, cnt,
                                                                                    dscale + kMaxLuBatch);
        SWEEP_TRY(cudaGetLastError());
        return WMOM_OK;
      };
      // x = LU^-1 V (every slot of vrep holds the excitation)
      SWEEP_TRY(cudaMemcpyAsync(fx, g.vrep.p, sizeof(double2) * (size_t)n * cn, cudaMemcpyDeviceToDevice, s));
      {
        std::vector<double> vn(kMaxLuBatch, g.vnorm);
        wmom_status ss = scale_slots(fx, vn.data(), cn);
        if (ss != WMOM_OK) return ss;
        SWEEP_TRY(lu_solve_ff(fff, n, n, fpiv, fx, ws, s, cn, (long long)nn, nullptr, finvp, fperm.as<int>()));
        ss = unscale_slots(fx, cn);
        if (ss != WMOM_OK) return ss;
      }
      bool act[kMaxLuBatch];
      int stall2[kMaxLuBatch] = {};
      double prev2[kMaxLuBatch];
      for (int j = 0; j < cn; ++j) {
        act[j] = inf[j] == 0;
        prev2[j] = HUGE_VAL;
      }
      // the chunk's active matrices in one residual launch: matrix fb[c0 + j] of Z64,
      // vector slot j of fx / frr
      std::vector<int> zsel2(2 * kMaxLuBatch, 0);
      for (int it = 0;; ++it) {
        int na = 0;
        for (int j = 0; j < cn; ++j)
          if (act[j]) {
            zsel2[na] = fb[c0 + j];
            zsel2[kMaxLuBatch + na] = j;
            ++na;
          }
        if (na > 0) {
          SWEEP_TRY(cudaMemcpyAsync(g.sel.p, zsel2.data(), sizeof(int) * 2 * kMaxLuBatch, cudaMemcpyHostToDevice, s));
          SWEEP_TRY(residual_fp64(Z64, n, (long long)nn, fx, g.vrep.as<double2>(), n, frr, g.part.as<double2>(), na,
                                  s, g.sel.as<int>(), g.sel.as<int>() + kMaxLuBatch));
        }
        SWEEP_TRY(sumsq_fp64(frr, n, dsc->rnorm2, cn, s));
        SWEEP_TRY(sumsq_fp64(fx, n, dsc->xnorm2, cn, s));
        SWEEP_TRY(cudaMemcpyAsync(&hs, dsc, sizeof(GroupScalars), cudaMemcpyDeviceToHost, s));
        SWEEP_TRY(cudaStreamSynchronize(s));
        int nact = 0, ncheck = 0, cslot[kMaxLuBatch], cmat[kMaxLuBatch];
        bool stalled[kMaxLuBatch] = {}, check[kMaxLuBatch] = {};
        for (int j = 0; j < cn; ++j) {
          if (!act[j]) continue;
          const int b = fb[c0 + j];
          const double xn = std::sqrt(hs.xnorm2[j]);
          const double rel = std::sqrt(hs.rnorm2[j]) / g.vnorm;
          const double corr = it > 0 && xn > 0 ? std::sqrt(hs.dnorm2[j]) / xn : HUGE_VAL;
          rep[b].iterations += it > 0 ? 1 : 0;
          if (trace)
            std::fprintf(stderr, "wmom refine: tier 2 matrix %d step %d rel %.3e corr %.3e\n", b, it, rel, corr);
          if (!(rel == rel)) {
            act[j] = false;
          } else if (rel <= tol || corr <= 0x1p-48) {
            act[j] = false;
            plain[j] = false;
          } else if ((rel > 0.5 * prev2[j] && ++stall2[j] >= 2) || it >= max_it) {
            act[j] = false;
            stalled[j] = true;
          } else {
            // a step that did not halve the residual: the solution may already sit at
            // the FP64 residual floor, where further steps only move it by rounding
            check[j] = rel > 0.5 * prev2[j];
            if (rel <= 0.5 * prev2[j]) stall2[j] = 0;
            prev2[j] = std::min(prev2[j], rel);
            ++nact;
          }
          if (stalled[j] || check[j]) {
            cslot[ncheck] = j;
            cmat[ncheck++] = b;
          }
        }
        // stalled or at the floor: accepted at FP64 level of the componentwise
        // backward error (a stalled matrix that fails it goes to tier 3; one at a
        // non-halving step that fails it keeps refining)
        if (ncheck > 0) {
          const wmom_status bs = backward_errors(Z64, fx, frr, cslot, cmat, ncheck);
          if (bs != WMOM_OK) return bs;
          for (int q = 0; q < ncheck; ++q) {
            const int j = cslot[q];
            const bool ok = hs.berr[j] <= berr_ok;
            if (trace)
              std::fprintf(stderr, "wmom refine: tier 2 matrix %d %s at step %d, backward error %.3e -> %s\n",
                           cmat[q], stalled[j] ? "stalls" : "did not halve", it, hs.berr[j],
                           ok ? "accepted" : (stalled[j] ? "tier 3" : "continues"));
            if (!ok) continue;
            plain[j] = false;
            if (check[j]) {
              act[j] = false;
              --nact;
            }
          }
        }
        if (nact == 0) break;
        // d = LU^-1 r for the chunk's active matrices; x += d where active
        int nsa = 0;
        for (int j = 0; j < cn; ++j) {
          hact[j] = act[j] ? 1 : 0;
          if (act[j]) zsel2[nsa++] = j;
        }
        SWEEP_TRY(cudaMemcpyAsync(g.actv.p, hact.data(), sizeof(int) * kMaxLuBatch, cudaMemcpyHostToDevice, s));
        SWEEP_TRY(cudaMemcpyAsync(g.sel.p, zsel2.data(), sizeof(int) * kMaxLuBatch, cudaMemcpyHostToDevice, s));
        {
          std::vector<double> rn(kMaxLuBatch, 0.0);
          for (int j = 0; j < cn; ++j) rn[j] = act[j] ? std::sqrt(hs.rnorm2[j]) : 0.0;
          wmom_status ss = scale_slots(frr, rn.data(), cn);
          if (ss != WMOM_OK) return ss;
          SWEEP_TRY(lu_solve_ff(fff, n, n, fpiv, frr, ws, s, nsa, (long long)nn,
                                nsa == cn ? nullptr : g.sel.as<int>(), finvp, fperm.as<int>()));
          ss = unscale_slots(frr, cn);
          if (ss != WMOM_OK) return ss;
        }
        SWEEP_TRY(sumsq_fp64(frr, n, dsc->dnorm2, cn, s));
        stats::count(stats::kMisc);
        accumulate64_kernel<<<(unsigned)(((size_t)n * cn + 255) / 256), 256, 0, s>>>(fx, frr, n, cn,
                                                                                   g.actv.as<int>());
        SWEEP_TRY(cudaGetLastError());
      }
      std::vector<int> s2, m2;
      for (int j = 0; j < cn; ++j)
        if (!plain[j]) {
          const int b = fb[c0 + j];
          rep[b].tier = 2;
          rep[b].info = 0;
          rep[b].status = WMOM_OK;
          s2.push_back(j);
          m2.push_back(b);
        }
      // before tier 3 reuses the scratch factors, with the factors back in FP64
      if (condest && !s2.empty()) SWEEP_TRY(merge_ff_inplace(flu, nn * cn, s));
      const wmom_status cs = estimate(flu, fpiv, frr, s2, m2);
      if (cs != WMOM_OK) return cs;
    }
    // tier 3: the chunk's remaining matrices, compacted into the scratch buffer
    int n3 = 0, idx3[kMaxLuBatch];
    for (int j = 0; j < cn; ++j)
      if (plain[j]) idx3[n3++] = j;
    if (n3 > 0) {
      for (int i = 0; i < n3; ++i)
        SWEEP_TRY(cudaMemcpyAsync(flu + (size_t)i * nn, Z64 + (size_t)fb[c0 + idx3[i]] * nn, sizeof(double2) * nn,
                                  cudaMemcpyDeviceToDevice, s));
      int inf[kMaxLuBatch] = {};
      const wmom_status fst = factor_group(WMOM_MODE_FP64, n, flu, n3, nullptr, flu, fpiv, ws, s, inf, nullptr,
                                           nullptr, 1);
      if (fst != WMOM_OK) return fst;
      SWEEP_TRY(cudaMemcpyAsync(frr, g.vrep.p, sizeof(double2) * (size_t)n * n3, cudaMemcpyDeviceToDevice, s));
      SWEEP_TRY(lu_solve_t<double2>(flu, n, n, fpiv, frr, n, 1, ws, s, n3, (long long)nn));
      std::vector<int> s3, m3;
      for (int i = 0; i < n3; ++i) {
        const int j = idx3[i], b = fb[c0 + j];
        SWEEP_TRY(cudaMemcpyAsync(fx + (size_t)j * n, frr + (size_t)i * n, sizeof(double2) * n,
                                  cudaMemcpyDeviceToDevice, s));
        rep[b].tier = 3;
        rep[b].info = inf[i];
        rep[b].status = inf[i] ? WMOM_ERR_SINGULAR : WMOM_OK;
        if (inf[i] == 0) {
          s3.push_back(i);
          m3.push_back(b);
        }
      }
      const wmom_status cs = estimate(flu, fpiv, frr, s3, m3);
      if (cs != WMOM_OK) return cs;
    }
    for (int j = 0; j < cn; ++j)
      SWEEP_TRY(cudaMemcpyAsync(g.x64.as<double2>() + (size_t)fb[c0 + j] * n, fx + (size_t)j * n,
                                sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
  }
  const wmom_status rs = group_residuals(g, Z64, bg);
  if (rs != WMOM_OK) return rs;
  for (int j = 0; j < nfb; ++j) rep[fb[j]].rel_residual = std::sqrt(hs.rnorm2[fb[j]]) / g.vnorm;
  return WMOM_OK;
}

namespace {

// Currents / Z_in / reports of a solved group to the caller's host arrays.
// nout (<= g.n, 0 = g.n): the entries of each solution the caller receives -- the
// geometry's own order when its matrices are stored at a larger padded order.
wmom_status group_results(GroupScratch& g, int bg, int ngap, const wmom_report* rep, int f, double* currents,
                          double* zin, wmom_report* reports, wmom_status* overall, int nout = 0) {
  const int n = g.n;
  if (nout <= 0) nout = n;
  std::vector<double2> xh((size_t)n * bg);
  if (currents && nout == n) {
    SWEEP_TRY(cudaMemcpyAsync(currents + 2 * (size_t)f * n, g.x64.p, sizeof(double2) * (size_t)n * bg,
                              cudaMemcpyDeviceToHost, g.s));
    SWEEP_TRY(cudaStreamSynchronize(g.s));
    std::memcpy(xh.data(), currents + 2 * (size_t)f * n, sizeof(double2) * (size_t)n * bg);
  } else {
    if (currents)
      SWEEP_TRY(cudaMemcpy2DAsync(currents + 2 * (size_t)f * nout, sizeof(double2) * nout, g.x64.p,
                                  sizeof(double2) * n, sizeof(double2) * nout, bg, cudaMemcpyDeviceToHost, g.s));
    for (int b = 0; b < bg; ++b)
      SWEEP_TRY(cudaMemcpyAsync(xh.data() + (size_t)b * n + (ngap - 1), g.x64.as<double2>() + (size_t)b * n + (ngap - 1),
                                sizeof(double2), cudaMemcpyDeviceToHost, g.s));
    SWEEP_TRY(cudaStreamSynchronize(g.s));
  }
  for (int b = 0; b < bg; ++b) {
    if (zin) {
      // Z_in = V[ngap-1] / I[ngap-1], Smith's formula
      const double vr = g.vh[2 * (ngap - 1)], vi = g.vh[2 * (ngap - 1) + 1];
      const double br = xh[(size_t)b * n + ngap - 1].x, bi = xh[(size_t)b * n + ngap - 1].y;
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
      zin[2 * (size_t)(f + b)] = zr;
      zin[2 * (size_t)(f + b) + 1] = zi;
    }
    if (rep[b].status != WMOM_OK && *overall == WMOM_OK) *overall = (wmom_status)rep[b].status;
    if (reports) reports[f + b] = rep[b];
  }
  return WMOM_OK;
}

// Fills nk matrices (frequencies freq[0..nk)) into Z and adds the plan's loads.  The
// host staging vectors are copied from pageable memory (staged before each copy call
// returns) and the device ones are freed in stream order, so `sync` = false leaves
// the work in flight.
wmom_status fill_batch(const Plan& p, const float* freq, int nk, double2* Z, cudaStream_t s, bool sync = true) {
  const int n = p.npls;
  const size_t nn = (size_t)n * n;
  std::vector<FreqParams> fph(nk);
  for (int i = 0; i < nk; ++i) fph[i] = freq_params(ka_from_mhz(freq[i]));
  DevBuf fpb;
  SWEEP_TRY(fpb.alloc(sizeof(FreqParams) * nk, s));
  SWEEP_TRY(cudaMemcpyAsync(fpb.p, fph.data(), sizeof(FreqParams) * nk, cudaMemcpyHostToDevice, s));
  SWEEP_TRY(launch_fill(p, fpb.as<double>(), nk, Z, n, (long long)nn, s));
  if (!p.load_idx.empty()) {
    // R + j*2*pi*f[MHz]*L[uH] on the loaded diagonal entries (REF/Wire_MoM.cu:346-363)
    const int nl = (int)p.load_idx.size();
    const double pi = std::acos(-1.0);
    std::vector<double2> lv((size_t)nk * nl);
    for (int i = 0; i < nk; ++i)
      for (int l = 0; l < nl; ++l)
        lv[(size_t)i * nl + l] = make_double2(p.load_r[l], 2. * pi * freq[i] * p.load_l_uh[l]);
    DevBuf li, lvd;
    SWEEP_TRY(li.alloc(sizeof(int) * nl, s));
    SWEEP_TRY(lvd.alloc(sizeof(double2) * lv.size(), s));
    SWEEP_TRY(cudaMemcpyAsync(li.p, p.load_idx.data(), sizeof(int) * nl, cudaMemcpyHostToDevice, s));
    SWEEP_TRY(cudaMemcpyAsync(lvd.p, lv.data(), sizeof(double2) * lv.size(), cudaMemcpyHostToDevice, s));
    stats::count(stats::kMisc);
    add_loads_kernel<<<(nk + 127) / 128, 128, 0, s>>>(Z, n, (long long)nn, li.as<int>(), lvd.as<double2>(), nl, nk);
    SWEEP_TRY(cudaGetLastError());
  }
  if (sync) SWEEP_TRY(cudaStreamSynchronize(s));
  return WMOM_OK;
}

}  // namespace

// Picks the factorisation shape for order n: the batch width (matrices per launch,
// up to what the cooperative panel keeps co-resident and a quarter of `budget`) and,
// for the precision form, the span (panels per tensor-core trailing update), the
// tensor-core tile (128 x 256 or 128 x 128 real outputs) and the widest FP32 panel
// (64 columns or as many as shared memory allows, 48 or 32).  It times factorisations
// of copies of the first matrix: widths 1, 2, 4, ... and the widest at span 2, then
// spans 1, 2, 4 at the chosen width, then the narrow tile, then the narrower panels;
// a change is kept only when it is clearly faster (3%).  Results are cached per
// (n / 256, form); WMOM_LU_BATCH, WMOM_LU_SPAN, WMOM_TC_TILE (128 or 256) and
// WMOM_PANEL_W (16-64) override.  Without `timing` (requests on a serving path, where
// trial factorisations would add to a request's latency) a cached result is used if
// there is one, else the widest batch up to `limit` at span 2 with the default tile
// and panels, and nothing is cached.
wmom_status choose_lu_config(int mode, int n, int limit, const double2* Z64, LuWorkspace* ws, cudaStream_t s,
                             size_t budget, LuConfig* out, bool timing) {
  const size_t nn = (size_t)n * n;
  const size_t mat = mode == WMOM_MODE_MIXED ? sizeof(float2) * nn : sizeof(double2) * nn;
  int bmax = std::min({ws->max_batch, kMaxLuBatch, limit,
                       mode == WMOM_MODE_MIXED ? lu_max_batch<float2>(n) : lu_max_batch<double2>(n)});
  while (bmax > 1 && (size_t)bmax * mat > budget / 4) bmax /= 2;
  bmax = std::max(bmax, 1);
  const int eb = env_int("WMOM_LU_BATCH", 1, kMaxLuBatch), es = env_int("WMOM_LU_SPAN", 1, kMaxSpan);
  const int et = env_int("WMOM_TC_TILE", 128, 256), ep = env_int("WMOM_PANEL_W", 16, 64);
  const int etile = et == 128 || et == 256 ? et : 0;
  if (mode != WMOM_MODE_MIXED) {
    // the FP64 form is bound by the FP64 pipe at every width worth batching
    *out = LuConfig{eb ? std::min(eb, bmax) : (n <= 2048 ? bmax : 1), 1};
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[{(n + 255) / 256, mode}] = *out;
    return WMOM_OK;
  }
  if (eb && es) {
    *out = LuConfig{std::min(eb, bmax), es, etile, ep};
    return WMOM_OK;
  }
  const std::pair<int, int> key{(n + 255) / 256, mode};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      *out = LuConfig{eb ? std::min(eb, bmax) : std::min(it->second.batch, bmax), es ? es : it->second.span,
                      etile ? etile : it->second.tile_n, ep ? ep : it->second.panel_w};
      return WMOM_OK;
    }
  }
  const int bcap = eb ? std::min(eb, bmax) : bmax;
  if (!timing) {
    *out = LuConfig{bcap, es ? es : 2, etile, ep};
    return WMOM_OK;
  }
  DevBuf rep64, lu, piv;
  SWEEP_TRY(rep64.alloc(sizeof(double2) * nn * bcap, s));
  SWEEP_TRY(lu.alloc(sizeof(float2) * nn * bcap, s));
  SWEEP_TRY(piv.alloc(sizeof(int) * (size_t)n * bcap, s));
  for (int b = 0; b < bcap; ++b)
    SWEEP_TRY(cudaMemcpyAsync(rep64.as<double2>() + (size_t)b * nn, Z64, sizeof(double2) * nn,
                              cudaMemcpyDeviceToDevice, s));
  const LuConfig saved{0, 0, ws->tile_n, ws->panel_w};
  auto time_one = [&](const LuConfig& c, float* per) -> wmom_status {
    float ms = 0.f;
    int info[kMaxLuBatch];
    use_shape(ws, c);
    const wmom_status st = factor_group(mode, n, rep64.as<double2>(), c.batch, lu.as<float2>(), nullptr,
                                        piv.as<int>(), ws, s, info, &ms, nullptr, c.span);
    use_shape(ws, saved);
    *per = ms / c.batch;
    return st;
  };
  // widths first (at the default span), then spans at the chosen width: the span's
  // saving is trailing-matrix traffic, which only shows at the width that will run
  LuConfig best{eb ? bcap : 1, es ? es : 2, etile, ep};
  float best_t = 1e30f;
  if (!eb) {
    // widths 1, 2, 4, ... and the widest one allowed (e.g. a whole 12-frequency sweep in
    // one group: its panels then run once for all of them)
    std::vector<int> cands;
    for (int c = 1; c <= bcap; c *= 2) cands.push_back(c);
    if (cands.back() != bcap) cands.push_back(bcap);
    for (int cand : cands) {
      float per = 0.f;
      LuConfig c = best;
      c.batch = cand;
      const wmom_status st = time_one(c, &per);
      if (st != WMOM_OK) return st;
      if (per < best_t * 0.95f) {
        best_t = per;
        best.batch = cand;
      }
    }
  }
  if (!es) {
    best_t = 1e30f;
    int cur = best.span;
    for (int span = 1; span <= 4; span *= 2) {
      // the better of two trials: the spans' differences (a few percent of a
      // factorisation) are near one trial's noise
      float per = 0.f, per2 = 0.f;
      LuConfig c = best;
      c.span = span;
      wmom_status st = time_one(c, &per);
      if (st != WMOM_OK) return st;
      st = time_one(c, &per2);
      if (st != WMOM_OK) return st;
      per = std::min(per, per2);
      // keep the default unless another span is clearly faster
      const float margin = span == cur ? 1.0f : 0.97f;
      if (per < best_t * margin) {
        best_t = per;
        best.span = span;
      }
    }
  } else {
    const wmom_status st = time_one(best, &best_t);
    if (st != WMOM_OK) return st;
  }
  // best_t is now the time of `best`; the narrow tile, then narrower panels
  if (!etile) {
    float per = 0.f;
    LuConfig c = best;
    c.tile_n = 128;
    const wmom_status st = time_one(c, &per);
    if (st != WMOM_OK) return st;
    if (per < best_t * 0.97f) {
      best_t = per;
      best.tile_n = 128;
    }
  }
  if (!ep) {
    for (int pw : {48, 32}) {
      float per = 0.f;
      LuConfig c = best;
      c.panel_w = pw;
      const wmom_status st = time_one(c, &per);
      if (st != WMOM_OK) return st;
      if (per < best_t * 0.97f) {
        best_t = per;
        best.panel_w = pw;
      }
    }
  }
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[key] = best;
  }
  *out = best;
  return WMOM_OK;
}

// The sweep's buffers (Z of a frequency batch and its factors: about 19 GB at
// N = 8192 and 12 frequencies) and resident factor sets come from the stream-ordered
// allocator.  With the default pool's release threshold of 0 that memory is handed
// back at every synchronisation and mapped again by the next sweep; the pool of this
// process keeps up to an eighth of the device's memory instead (WMOM_POOL_RETAIN_GB
// overrides, 0 keeps the default).
void retain_pool_memory() {
  static std::mutex mu;
  static std::vector<char> done;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  std::lock_guard<std::mutex> lk(mu);
  if ((int)done.size() <= dev) done.resize(dev + 1, 0);
  if (done[dev]) return;
  done[dev] = 1;
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return;
  uint64_t thr = tot / 8;
  const char* e = std::getenv("WMOM_POOL_RETAIN_GB");
  if (e) thr = (uint64_t)std::max(0.0, std::atof(e)) << 30;
  cudaMemPool_t pool = nullptr;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess)
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  cudaGetLastError();
}

namespace {

// Groups a sweep is split into so that the fill of one group (FP64 pipe) runs while
// the previous group factors (tensor pipe).  By default only a sweep of at least two
// groups of the tuned batch width is pipelined, at that width: splitting a batch
// narrower costs more than the overlap saves (12-frequency N = 8192 sweep, batch 12:
// 42.5 / 39.3 / 35.5 freq-solves/s for 1 / 2 / 3 groups -- half the parallelism of
// the latency-bound panels, 40 -> 68 ms per sweep), while full-width groups gain
// (256-frequency N = 2048 grid, batch 16: 209.5 -> 214.7).  WMOM_PIPELINE = 1 .. 8
// forces that many groups (1 = off).
int pipeline_groups(int nfreq, int batch) {
  const int v = env_int("WMOM_PIPELINE", 1, 8);
  if (v) return v;
  return nfreq >= 2 * batch ? (nfreq + batch - 1) / batch : 1;
}

// The cached factorisation shape for (n, mode), if a sweep of that order was tuned.
// Second-tier prediction inside one sweep.  The sweep's groups run from the highest
// frequency down (run_sweep orders them so).  The conditioning of these wire
// structures grows as the frequency falls (kappa ~ 1 / (ka)^2 below resonance), so
// once every matrix of a group has needed FP64-grade factors, the groups after it
// (lower frequencies) skip the FP32 factorisation and the refinement attempt that
// would fail, and go straight to the second tier.  A matrix's second-tier result does
// not depend on that attempt, so a predicted matrix gets the same answer, bit for
// bit, as it would after failing in tier 1; only its reported refinement steps
// differ.  A wrong prediction (a matrix that tier 1 would have served) costs time,
// not accuracy.  WMOM_TIER_PREDICT=0 turns it off.
//
// Within a group, structures with wire loops (Plan::loops; open wires keep a bounded
// kappa as the frequency falls) probe: the group's upper half gets FP32 factors and
// refines first, and if the lowest frequency of that half needs FP64-grade factors,
// the lower half joins it in the second tier without FP32 factors (solve_group's
// probe).  A group probes when it is the sweep's only group, or when the group before
// it had a matrix fall back (the sweep is then crossing into the ill-conditioned
// band); elsewhere the extra FP32 factorisation of the second half would cost more
// than a probe saves.
struct TierPrediction {
  bool on;
  bool all_fell_back = false, any_fell_back = false;
  explicit TierPrediction(int mode) {
    const char* e = std::getenv("WMOM_TIER_PREDICT");
    on = mode == WMOM_MODE_MIXED && !(e && e[0] == '0') && emul_gemm_hook() != nullptr;
  }
  bool direct() const { return on && all_fell_back; }
  int probe(const Plan& p, int bg, bool only_group) const {
    if (!on || all_fell_back || p.loops == 0 || bg < 4) return 0;
    return only_group || any_fell_back ? bg / 2 : 0;
  }
  void record(const wmom_report* rep, int bg) {
    bool all = bg > 0, any = false;
    for (int b = 0; b < bg; ++b) {
      if (rep[b].tier < 2) all = false;
      if (rep[b].tier >= 2) any = true;
    }
    all_fell_back = all;
    any_fell_back = any;
  }
};

bool cached_lu_config(int mode, int n, LuConfig* out) {
  if (env_int("WMOM_LU_BATCH", 1, kMaxLuBatch)) return false;  // an override goes through the tuner path
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tuned.find({(n + 255) / 256, mode});
  if (it == g_tuned.end()) return false;
  *out = it->second;
  return true;
}

struct StreamPair {
  cudaStream_t hi = nullptr, lo = nullptr;
  ~StreamPair() {
    if (hi) cudaStreamDestroy(hi);
    if (lo) cudaStreamDestroy(lo);
  }
};

// Pipelined sweep: the frequencies are split into G groups of width Bp; group g + 1 is
// filled on a second stream while group g is factored and solved on a
// higher-priority one, whose kernels the block scheduler serves first.  Results are
// those of the plain sweep bit for bit: the same fill per matrix and factorisations
// that do not depend on the batch width.
wmom_status run_sweep_pipelined(const SweepArgs& a, const LuConfig& cfg, int G) {
  use_shape(a.ws, cfg);
  const Plan& p = *a.plan;
  const int n = p.npls;
  const bool mixed = a.mode == WMOM_MODE_MIXED;
  const size_t nn = (size_t)n * n;
  const size_t mat64 = sizeof(double2) * nn;
  const int Bp = std::min(cfg.batch, (a.nfreq + G - 1) / G);
  StreamPair sp;
  int lo_pri = 0, hi_pri = 0;
  SWEEP_TRY(cudaDeviceGetStreamPriorityRange(&lo_pri, &hi_pri));
  SWEEP_TRY(cudaStreamCreateWithPriority(&sp.hi, cudaStreamNonBlocking, hi_pri));
  SWEEP_TRY(cudaStreamCreateWithPriority(&sp.lo, cudaStreamNonBlocking, lo_pri));
  cudaEvent_t start = nullptr;
  SWEEP_TRY(cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
  std::vector<cudaEvent_t> filled((a.nfreq + Bp - 1) / Bp, nullptr);
  auto cleanup = [&]() {
    if (start) cudaEventDestroy(start);
    for (cudaEvent_t e : filled)
      if (e) cudaEventDestroy(e);
  };
  struct Guard {
    std::function<void()> f;
    ~Guard() { f(); }
  } guard{cleanup};
  for (auto& e : filled) SWEEP_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  // both internal streams start after the caller's stream work so far
  SWEEP_TRY(cudaEventRecord(start, a.stream));
  SWEEP_TRY(cudaStreamWaitEvent(sp.hi, start, 0));
  SWEEP_TRY(cudaStreamWaitEvent(sp.lo, start, 0));
  DevBuf zall, lu, piv;
  SWEEP_TRY(zall.alloc(mat64 * a.nfreq, sp.hi));
  SWEEP_TRY(lu.alloc((mixed ? sizeof(float2) : sizeof(double2)) * nn * Bp, sp.hi));
  SWEEP_TRY(piv.alloc(sizeof(int) * (size_t)n * Bp, sp.hi));
  // the buffers come from the high-priority stream's pool: the fill stream waits for them
  cudaEvent_t alloc_done = nullptr;
  SWEEP_TRY(cudaEventCreateWithFlags(&alloc_done, cudaEventDisableTiming));
  SWEEP_TRY(cudaEventRecord(alloc_done, sp.hi));
  SWEEP_TRY(cudaStreamWaitEvent(sp.lo, alloc_done, 0));
  cudaEventDestroy(alloc_done);
  const int ngroups = (int)filled.size();
  auto launch_fill = [&](int gi) -> wmom_status {
    const int f0 = gi * Bp, nb = std::min(Bp, a.nfreq - f0);
    const wmom_status st = fill_batch(p, a.freq_mhz + f0, nb, zall.as<double2>() + (size_t)f0 * nn, sp.lo, false);
    if (st != WMOM_OK) return st;
    SWEEP_TRY(cudaEventRecord(filled[gi], sp.lo));
    return WMOM_OK;
  };
  wmom_status st = launch_fill(0);
  if (st != WMOM_OK) return st;
  GroupScratch g;
  st = scratch_init(&g, n, Bp, a.ngap, a.ampl, a.phas_deg, sp.hi);
  if (st != WMOM_OK) return st;
  FactorGraph graph;
  std::vector<wmom_report> rep(kMaxLuBatch);
  wmom_status overall = WMOM_OK;
  TierPrediction predict(a.mode);
  for (int gi = 0; gi < ngroups; ++gi) {
    // the next group's fill goes in before this group's factorisation: it runs on the
    // SMs the factorisation leaves
    if (gi + 1 < ngroups) {
      st = launch_fill(gi + 1);
      if (st != WMOM_OK) return st;
    }
    const int f0 = gi * Bp, bg = std::min(Bp, a.nfreq - f0);
    SWEEP_TRY(cudaStreamWaitEvent(sp.hi, filled[gi], 0));
    const double2* Zg = zall.as<double2>() + (size_t)f0 * nn;
    int info[kMaxLuBatch] = {};
    const bool direct = predict.direct();
    const int probe = direct ? 0 : predict.probe(p, bg, ngroups == 1);
    const std::function<wmom_status(int, int, int*)> rest = [&](int b0, int cnt, int* inf) {
      return factor_group(a.mode, n, Zg + (size_t)b0 * nn, cnt, lu.as<float2>() + (size_t)b0 * nn, nullptr,
                          piv.as<int>() + (size_t)b0 * n, a.ws, sp.hi, inf, nullptr, nullptr, cfg.span);
    };
    if (!direct) {
      st = factor_group(a.mode, n, Zg, probe ? probe : bg, lu.as<float2>(), lu.as<double2>(), piv.as<int>(), a.ws,
                        sp.hi, info, nullptr, &graph, cfg.span);
      if (st != WMOM_OK) return st;
    }
    st = solve_group(a.mode, n, Zg, bg, lu.as<float2>(), lu.as<double2>(), piv.as<int>(), info, a.tol, a.ws, g,
                     rep.data(), a.condest, n, direct, probe, &rest);
    if (st != WMOM_OK) return st;
    predict.record(rep.data(), bg);
    st = group_results(g, bg, a.ngap, rep.data(), f0, a.currents, a.zin, a.reports, &overall);
    if (st != WMOM_OK) return st;
  }
  SWEEP_TRY(cudaStreamSynchronize(sp.lo));
  SWEEP_TRY(cudaStreamSynchronize(sp.hi));
  return overall;
}

}  // namespace

namespace {

wmom_status run_sweep_ordered(const SweepArgs& a) {
  retain_pool_memory();
  {
    // pipelined when the shape is already tuned, the sweep has more than one group
    // and all its matrices fit
    LuConfig cfg;
    size_t fr = 0, tot = 0;
    int G = 1;
    if (cached_lu_config(a.mode, a.plan->npls, &cfg)) G = pipeline_groups(a.nfreq, cfg.batch);
    if (G > 1 && a.nfreq >= 2 * G && cudaMemGetInfo(&fr, &tot) == cudaSuccess) {
      const size_t nn = (size_t)a.plan->npls * a.plan->npls;
      const size_t need = nn * (sizeof(double2) * a.nfreq + sizeof(double2) * cfg.batch);
      const size_t budget = a.mem_budget ? a.mem_budget : fr / 2;
      if (need < budget) return run_sweep_pipelined(a, cfg, G);
    }
  }
  const Plan& p = *a.plan;
  const int n = p.npls;
  cudaStream_t s = a.stream;
  const bool mixed = a.mode == WMOM_MODE_MIXED;
  const size_t nn = (size_t)n * n;
  const size_t mat64 = sizeof(double2) * nn;
  const size_t mat32 = sizeof(float2) * nn;
  size_t budget = a.mem_budget;
  if (budget == 0) {
    size_t fr = 0, tot = 0;
    SWEEP_TRY(cudaMemGetInfo(&fr, &tot));
    budget = fr / 2;
  }
  // first fill batch: at least one matrix, so the batch width can be tuned on it
  const size_t reserve = (size_t)kMaxLuBatch * (mixed ? mat32 : mat64);
  if (budget < reserve + 2 * mat64) return WMOM_ERR_NOMEM;
  int nbf = (int)std::max<size_t>(1, std::min<size_t>((size_t)a.nfreq, (budget - reserve) / mat64));
  DevBuf zall;
  SWEEP_TRY(zall.alloc(mat64 * nbf, s));
  wmom_status overall = WMOM_OK;
  int B = 0;
  LuConfig cfg;
  std::vector<wmom_report> rep(kMaxLuBatch);
  DevBuf lu, piv;
  GroupScratch g;
  FactorGraph graph;
  TierPrediction predict(a.mode);
  for (int f0 = 0; f0 < a.nfreq; f0 += nbf) {
    const int nb = std::min(nbf, a.nfreq - f0);
    wmom_status st = fill_batch(p, a.freq_mhz + f0, nb, zall.as<double2>(), s);
    if (st != WMOM_OK) return st;
    if (B == 0) {
      st = choose_lu_config(a.mode, n, a.nfreq, zall.as<double2>(), a.ws, s, budget, &cfg, true);
      if (st != WMOM_OK) return st;
      use_shape(a.ws, cfg);
      B = cfg.batch;
      SWEEP_TRY(lu.alloc((mixed ? mat32 : mat64) * B, s));
      SWEEP_TRY(piv.alloc(sizeof(int) * (size_t)n * B, s));
      st = scratch_init(&g, n, B, a.ngap, a.ampl, a.phas_deg, s);
      if (st != WMOM_OK) return st;
    }
    for (int g0 = 0; g0 < nb; g0 += B) {
      const int bg = std::min(B, nb - g0);
      const double2* Zg = zall.as<double2>() + (size_t)g0 * nn;
      int info[kMaxLuBatch] = {};
      const bool direct = predict.direct();
      const int probe = direct ? 0 : predict.probe(p, bg, a.nfreq <= B);
      const std::function<wmom_status(int, int, int*)> rest = [&](int b0, int cnt, int* inf) {
        return factor_group(a.mode, n, Zg + (size_t)b0 * nn, cnt, lu.as<float2>() + (size_t)b0 * nn, nullptr,
                            piv.as<int>() + (size_t)b0 * n, a.ws, s, inf, nullptr, nullptr, cfg.span);
      };
      if (!direct) {
        st = factor_group(a.mode, n, Zg, probe ? probe : bg, lu.as<float2>(), lu.as<double2>(), piv.as<int>(),
                          a.ws, s, info, nullptr, &graph, cfg.span);
        if (st != WMOM_OK) return st;
      }
      st = solve_group(a.mode, n, Zg, bg, lu.as<float2>(), lu.as<double2>(), piv.as<int>(), info, a.tol, a.ws, g,
                       rep.data(), a.condest, n, direct, probe, &rest);
      if (st != WMOM_OK) return st;
      predict.record(rep.data(), bg);
      st = group_results(g, bg, a.ngap, rep.data(), f0 + g0, a.currents, a.zin, a.reports, &overall);
      if (st != WMOM_OK) return st;
    }
  }
  SWEEP_TRY(cudaStreamSynchronize(s));
  return overall;
}

}  // namespace

// The sweep in the order its second-tier prediction wants: frequencies from the
// highest down (TierPrediction).  The frequencies are permuted into that order, the
// sweep runs, and currents, Z_in and reports go back to the caller's order.  Each
// matrix is factored and solved on its own (batched launches keep the matrices
// independent), so the order changes no result.
wmom_status run_sweep(const SweepArgs& a) {
  const TierPrediction predict(a.mode);
  if (!predict.on || a.nfreq < 2) return run_sweep_ordered(a);
  std::vector<int> ord(a.nfreq);
  for (int i = 0; i < a.nfreq; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return a.freq_mhz[x] > a.freq_mhz[y]; });
  bool same = true;
  for (int i = 0; i < a.nfreq; ++i) same = same && ord[i] == i;
  if (same) return run_sweep_ordered(a);
  const size_t n = (size_t)a.plan->npls;
  std::vector<float> f(a.nfreq);
  for (int i = 0; i < a.nfreq; ++i) f[i] = a.freq_mhz[ord[i]];
  std::vector<double> cur(a.currents ? 2 * n * a.nfreq : 0), zin(a.zin ? 2 * (size_t)a.nfreq : 0);
  std::vector<wmom_report> rep(a.reports ? a.nfreq : 0);
  SweepArgs b = a;
  b.freq_mhz = f.data();
  b.currents = a.currents ? cur.data() : nullptr;
  b.zin = a.zin ? zin.data() : nullptr;
  b.reports = a.reports ? rep.data() : nullptr;
  const wmom_status st = run_sweep_ordered(b);
  for (int i = 0; i < a.nfreq; ++i) {
    const int k = ord[i];
    if (a.currents) std::copy(cur.begin() + 2 * n * i, cur.begin() + 2 * n * (i + 1), a.currents + 2 * n * k);
    if (a.zin) {
      a.zin[2 * k] = zin[2 * i];
      a.zin[2 * k + 1] = zin[2 * i + 1];
    }
    if (a.reports) a.reports[k] = rep[i];
  }
  return st;
}

// ----------------------------------------------- geometries of uneven order ----
// A batch of geometries of different orders is factored in size classes: each
// matrix is stored at the padded order of its class, padded_order(n), with an
// identity block beyond n.  Z_pad = [[Z, 0], [0, I]] factors as the LU of Z beside an
// identity (the padding rows are zero in Z's columns and never become pivots), so the
// leading n x n block of the factors and the first n entries of every solution are
// those of Z.  The class depends on n alone, so a geometry's factors are the same
// alone and in any batch: the same order, panel widths and reduction orders.  The
// classes are four per octave (P <= 1.25 n).

int padded_order(int n) {
  if (n <= 256) return ((n + 63) / 64) * 64;
  int p2 = 256;
  while (2 * p2 <= n) p2 *= 2;
  const int step = p2 / 4;
  return ((n + step - 1) / step) * step;
}

namespace {

// Z of matrix b (order P, zstride apart): rows nreal[b].. of its first nreal[b]
// columns and every other column set to the identity's
__global__ void pad_identity_kernel(double2* __restrict__ Z, int P, long long zstride,
                                    const int* __restrict__ nreal) {
  const int j = blockIdx.y, b = blockIdx.z;
  const int nb = nreal[b];
  double2* col = Z + (size_t)b * zstride + (size_t)j * P;
  const int i0 = j < nb ? nb : 0;
  for (int i = i0 + threadIdx.x; i < P; i += blockDim.x)
    col[i] = make_double2(i == j ? 1.0 : 0.0, 0.0);
}

}  // namespace

LuConfig tuned_shape(int n, int mode) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tuned.find({(n + 255) / 256, mode});
  LuConfig c{1, 2, 0, 0};
  if (it != g_tuned.end()) {
    c = it->second;
    if (c.span <= 0) c.span = 2;
  }
  return c;
}

wmom_status factor_class(int mode, int P, const Plan* const* plans, const float* freq, int count, double2* z64,
                         void* lu, int* ipiv, int* info, LuWorkspace* ws, int span, cudaStream_t s) {
  const size_t nn = (size_t)P * P;
  std::vector<double> ka(count);
  std::vector<double2*> zp(count);
  std::vector<long long> ld(count, P);
  std::vector<int> nreal(count);
  for (int i = 0; i < count; ++i) {
    ka[i] = ka_from_mhz(freq[i]);
    zp[i] = z64 + (size_t)i * nn;
    nreal[i] = plans[i]->npls;
  }
  SWEEP_TRY(launch_fill_geometries(plans, ka.data(), zp.data(), ld.data(), count, s));
  for (int i = 0; i < count; ++i) {
    const Plan& p = *plans[i];
    if (p.load_idx.empty()) continue;
    // R + j*2*pi*f[MHz]*L[uH] on the loaded diagonal entries (REF/Wire_MoM.cu:346-363)
    const int nl = (int)p.load_idx.size();
    const double pi = std::acos(-1.0);
    std::vector<double2> lv(nl);
    for (int l = 0; l < nl; ++l) lv[l] = make_double2(p.load_r[l], 2. * pi * freq[i] * p.load_l_uh[l]);
    DevBuf li, lvd;
    SWEEP_TRY(li.alloc(sizeof(int) * nl, s));
    SWEEP_TRY(lvd.alloc(sizeof(double2) * nl, s));
    SWEEP_TRY(cudaMemcpyAsync(li.p, p.load_idx.data(), sizeof(int) * nl, cudaMemcpyHostToDevice, s));
    SWEEP_TRY(cudaMemcpyAsync(lvd.p, lv.data(), sizeof(double2) * nl, cudaMemcpyHostToDevice, s));
    stats::count(stats::kMisc);
    add_loads_kernel<<<1, 128, 0, s>>>(zp[i], P, (long long)nn, li.as<int>(), lvd.as<double2>(), nl, 1);
    SWEEP_TRY(cudaGetLastError());
    SWEEP_TRY(cudaStreamSynchronize(s));  // the host staging vectors end with this scope
  }
  DevBuf dn;
  SWEEP_TRY(dn.alloc(sizeof(int) * count, s));
  SWEEP_TRY(cudaMemcpyAsync(dn.p, nreal.data(), sizeof(int) * count, cudaMemcpyHostToDevice, s));
  stats::count(stats::kMisc);
  pad_identity_kernel<<<dim3(1, P, count), 256, 0, s>>>(z64, P, (long long)nn, dn.as<int>());
  SWEEP_TRY(cudaGetLastError());
  const bool mixed = mode == WMOM_MODE_MIXED;
  const wmom_status st = factor_group(mode, P, z64, count, mixed ? reinterpret_cast<float2*>(lu) : nullptr,
                                      mixed ? nullptr : reinterpret_cast<double2*>(lu), ipiv, ws, s, info, nullptr,
                                      nullptr, span);
  SWEEP_TRY(cudaStreamSynchronize(s));
  return st;
}

// ------------------------------------------------------- resident factors ----
wmom_status factors_build(FactorSet* fs, cudaStream_t s) {
  const Plan& p = *fs->plan;
  const int n = p.npls;
  const size_t nn = (size_t)n * n;
  const bool mixed = fs->mode == WMOM_MODE_MIXED;
  const int nf = (int)fs->freq.size();
  // from the stream-ordered pool: a serving loop creates and evicts sets while other
  // streams run, and cudaMalloc / cudaFree may wait for the whole device
  retain_pool_memory();
  fs->pooled = true;
  SWEEP_TRY(cudaMallocAsync(reinterpret_cast<void**>(&fs->z64), sizeof(double2) * nn * nf, s));
  SWEEP_TRY(cudaMallocAsync(&fs->lu, (mixed ? sizeof(float2) : sizeof(double2)) * nn * nf, s));
  SWEEP_TRY(cudaMallocAsync(reinterpret_cast<void**>(&fs->ipiv), sizeof(int) * (size_t)n * nf, s));
  fs->info.assign(nf, 0);
  wmom_status st = fill_batch(p, fs->freq.data(), nf, fs->z64, s);
  if (st != WMOM_OK) return st;
  size_t fr = 0, tot = 0;
  SWEEP_TRY(cudaMemGetInfo(&fr, &tot));
  LuConfig cfg;
  st = choose_lu_config(fs->mode, n, nf, fs->z64, fs->ws, s, fr / 2, &cfg, false);
  if (st != WMOM_OK) return st;
  use_shape(fs->ws, cfg);
  fs->batch = cfg.batch;
  fs->span = cfg.span;
  for (int g0 = 0; g0 < nf; g0 += fs->batch) {
    const int bg = std::min(fs->batch, nf - g0);
    float2* l32 = reinterpret_cast<float2*>(fs->lu) + (size_t)g0 * nn;
    double2* l64 = reinterpret_cast<double2*>(fs->lu) + (size_t)g0 * nn;
    st = factor_group(fs->mode, n, fs->z64 + (size_t)g0 * nn, bg, l32, l64, fs->ipiv + (size_t)g0 * n, fs->ws, s,
                      fs->info.data() + g0, nullptr, nullptr, fs->span);
    if (st != WMOM_OK) return st;
  }
  SWEEP_TRY(cudaStreamSynchronize(s));
  return WMOM_OK;
}

wmom_status factors_solve(FactorSet* fs, int first, int count, int ngap, float ampl, float phas, double tol,
                          double* currents, double* zin, wmom_report* reports, cudaStream_t s) {
  const int nreal = fs->plan->npls;
  const int n = fs->order > 0 ? fs->order : nreal;  // storage order (padded for geometry batches)
  const size_t nn = (size_t)n * n;
  const bool mixed = fs->mode == WMOM_MODE_MIXED;
  const int B = std::max(1, fs->batch);
  GroupScratch g;
  wmom_status st = scratch_init(&g, n, B, ngap, ampl, phas, s);
  if (st != WMOM_OK) return st;
  wmom_status overall = WMOM_OK;
  std::vector<wmom_report> rep(kMaxLuBatch);
  // groups aligned with the factorisation's, so each group's factors are contiguous
  for (int f = first; f < first + count;) {
    const int bg = std::min(B, first + count - f);
    const float2* l32 = reinterpret_cast<const float2*>(fs->lu) + (size_t)f * nn;
    const double2* l64 = reinterpret_cast<const double2*>(fs->lu) + (size_t)f * nn;
    st = solve_group(fs->mode, n, fs->z64 + (size_t)f * nn, bg, mixed ? l32 : nullptr, mixed ? nullptr : l64,
                     fs->ipiv + (size_t)f * n, fs->info.data() + f, tol, fs->ws, g, rep.data(), fs->condest,
                     nreal, false);
    if (st != WMOM_OK) return st;
    // results are indexed from `first` in the caller's arrays
    st = group_results(g, bg, ngap, rep.data(), f - first, currents, zin, reports, &overall, nreal);
    if (st != WMOM_OK) return st;
    f += bg;
  }
  SWEEP_TRY(cudaStreamSynchronize(s));
  return overall;
}

}  // namespace wmom

extern "C" wmom_status wmom_tuned_config(int n, int mode, int* batch, int* span) {
  if (n <= 0 || (mode != WMOM_MODE_FP64 && mode != WMOM_MODE_MIXED)) return WMOM_ERR_ARG;
  std::lock_guard<std::mutex> lk(wmom::g_tune_mu);
  auto it = wmom::g_tuned.find({(n + 255) / 256, mode});
  if (it == wmom::g_tuned.end()) return WMOM_ERR_ARG;
  if (batch) *batch = it->second.batch;
  if (span) *span = it->second.span;
  return WMOM_OK;
}

extern "C" wmom_status wmom_tuned_shape(int n, int mode, int* tile_n, int* panel_w) {
  if (n <= 0 || (mode != WMOM_MODE_FP64 && mode != WMOM_MODE_MIXED)) return WMOM_ERR_ARG;
  std::lock_guard<std::mutex> lk(wmom::g_tune_mu);
  auto it = wmom::g_tuned.find({(n + 255) / 256, mode});
  if (it == wmom::g_tuned.end()) return WMOM_ERR_ARG;
  if (tile_n) *tile_n = it->second.tile_n ? it->second.tile_n : 256;
  if (panel_w) *panel_w = it->second.panel_w;
  return WMOM_OK;
}
