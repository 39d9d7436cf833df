// condest.cu -- condition estimates of the factored impedance matrices.
//
// kappa_1(Z) = ||Z||_1 * ||Z^-1||_1, with ||Z^-1||_1 estimated from the LU factors
// by Higham's refinement of Hager's method, the algorithm of LAPACK's zlacn2 /
// zgecon (N. J. Higham, "FORTRAN codes for estimating the one-norm of a real or
// complex matrix", ACM TOMS 14, 1988): a few solves with Z and with Z^H, each
// moving a unit vector to the column where ||Z^-1 x||_1 grows fastest, and a final
// alternating-sign test vector.  The reference never estimates a condition number:
// it checks the info of LAPACKE_zgetrf only ("wersja referencyjna/Wire_MoM.cu":372-377).
//
// Every matrix of a batch follows its own sequence of steps; each round solves,
// in one batched launch sequence per kind, the matrices whose next step is a solve
// with Z and those whose next step is a solve with Z^H, then reads four numbers
// per vector (sum of moduli, first index of the largest modulus, that modulus,
// and the modulus at the previous index).  At most 11 rounds.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "lu_common.cuh"
#include "solve_internal.h"
#include "stats.h"

namespace wmom {

namespace {

constexpr int kCondThreads = 256;

// out[4c + 0..3] for the vector of slot c (vector sel[c] of a batch n apart, its
// first nreal entries): sum_i |x_i|, the first index of max_i |x_i|, that maximum,
// |x_jprev[c]|.  |.| is the modulus (LAPACK's dzsum1 / izmax1); fixed reduction order.
template <typename C>
__global__ void __launch_bounds__(kCondThreads) cond_stats_kernel(const C* __restrict__ X, int n, int nreal,
                                                                  const int* __restrict__ sel,
                                                                  const int* __restrict__ jprev,
                                                                  double* __restrict__ out) {
  __shared__ double ssum[kCondThreads], smax[kCondThreads];
  __shared__ int sidx[kCondThreads];
  const int c = blockIdx.x, t = threadIdx.x;
  const C* x = X + (size_t)sel[c] * n;
  double sum = 0.0, mx = -1.0;
  int mi = 0x7fffffff;
  for (int i = t; i < nreal; i += kCondThreads) {
    const double a = hypot((double)x[i].x, (double)x[i].y);
    sum += a;
    if (a > mx) {  // increasing i: the first index of a tie stays
      mx = a;
      mi = i;
    }
  }
  ssum[t] = sum;
  smax[t] = mx;
  sidx[t] = mi;
  __syncthreads();
  for (int h = kCondThreads / 2; h > 0; h >>= 1) {
    if (t < h) {
      ssum[t] += ssum[t + h];
      const double ov = smax[t + h];
      const int oi = sidx[t + h];
      if (ov > smax[t] || (ov == smax[t] && oi < sidx[t])) {
        smax[t] = ov;
        sidx[t] = oi;
      }
    }
    __syncthreads();
  }
  if (t == 0) {
    const int jp = jprev[c];
    out[4 * c + 0] = ssum[0];
    out[4 * c + 1] = (double)sidx[0];
    out[4 * c + 2] = smax[0];
    out[4 * c + 3] = (jp >= 0 && jp < nreal) ? hypot((double)x[jp].x, (double)x[jp].y) : 0.0;
  }
}

// Sets the first nreal entries of the vector of slot c: action 0 x_i / |x_i| (1 where
// |x_i| is below the smallest normal), 1 the unit vector e_arg, 2 (-1)^i (1 + i /
// (nreal - 1)), 3 1/nreal; entries from nreal to n (the padding of a matrix stored at
// a larger order, an identity block) are 0.
template <typename C>
__global__ void cond_setup_kernel(C* __restrict__ X, int n, int nreal, const int* __restrict__ sel,
                                  const int* __restrict__ action, const int* __restrict__ arg) {
  using R = decltype(C{}.x);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i >= n) return;
  C* x = X + (size_t)sel[c] * n;
  double re = 0.0, im = 0.0;
  if (i >= nreal) {
    x[i] = cmake<C>((R)0, (R)0);
    return;
  }
  switch (action[c]) {
    case 0: {
      const double a = hypot((double)x[i].x, (double)x[i].y);
      if (a > DBL_MIN) {
        re = (double)x[i].x / a;
        im = (double)x[i].y / a;
      } else {
        re = 1.0;
      }
      break;
    }
    case 1:
      re = i == arg[c] ? 1.0 : 0.0;
      break;
    case 2:
      re = (i & 1 ? -1.0 : 1.0) * (1.0 + (nreal > 1 ? (double)i / (double)(nreal - 1) : 0.0));
      break;
    default:
      re = 1.0 / (double)nreal;
  }
  x[i] = cmake<C>((R)re, (R)im);
}

// out[b] (as the bits of a non-negative double) = max over the columns of matrix b
// of sum_i |Z_ij|, |.| the modulus computed in FP32 (a norm for a condition
// estimate, good to 1e-7); one warp per column, fixed order within a column, the
// maximum over columns by an integer atomic (order-independent).
__global__ void __launch_bounds__(256) norm1_kernel(const double2* __restrict__ Z, int n, long long lda,
                                                    long long zstride, unsigned long long* __restrict__ out) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * 8 + w;
  if (j >= n) return;
  const double2* col = Z + (size_t)blockIdx.y * zstride + (size_t)j * lda;
  double sum = 0.0;
  for (int i = lane; i < n; i += 32) {
    const double2 a = col[i];
    const float re = (float)a.x, im = (float)a.y;
    sum += (double)sqrtf(fmaf(re, re, im * im));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) atomicMax(&out[blockIdx.y], (unsigned long long)__double_as_longlong(sum));
}

struct Scratch {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  ~Scratch() {
    if (p) cudaFreeAsync(p, s);
  }
};

#define COND_TRY(call)                                       \
  do {                                                       \
    cudaError_t _e = (call);                                 \
    if (_e != cudaSuccess) return wmom_fail_cuda(_e, #call); \
  } while (0)

// zlacn2's steps: what the vector holds when the next solve has run
enum CondStep { kFirstA = 0, kFirstH, kStepA, kStepH, kAltA, kDone };

}  // namespace

cudaError_t norm1_batch(const double2* Z, int n, long long lda, long long zstride, int nmat, double* out_dev,
                        cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out_dev, 0, sizeof(double) * nmat, s);
  if (e != cudaSuccess) return e;
  stats::count(stats::kMisc);
  norm1_kernel<<<dim3((n + 7) / 8, nmat), 256, 0, s>>>(Z, n, lda, zstride,
                                                      reinterpret_cast<unsigned long long*>(out_dev));
  return cudaGetLastError();
}

template <typename C>
wmom_status condest_t(int n, int nreal, const C* lu, long long lda, long long astride, const int* ipiv,
                      const int* slots, int m, C* X, LuWorkspace* ws, cudaStream_t s, double* est) {
  if (m <= 0) return WMOM_OK;
  if (m > kMaxLuBatch || n < 1 || nreal < 1 || nreal > n) return WMOM_ERR_ARG;
  // device lists: [0] Z-solves, [1] Z^H-solves, [2] all, [3] previous index,
  // [4] setup slots, [5] actions, [6] unit-vector indices; then 4 doubles per slot
  constexpr int L = kMaxLuBatch;
  Scratch sb;
  sb.s = s;
  COND_TRY(cudaMallocAsync(&sb.p, sizeof(int) * 7 * L + sizeof(double) * 4 * L, s));
  int* di = reinterpret_cast<int*>(sb.p);
  double* dstat = reinterpret_cast<double*>(di + 7 * L);
  std::vector<int> hi(7 * L, 0);
  std::vector<double> hstat(4 * L, 0.0);
  struct State {
    int step;
    double est;
    int j;
    int iter;
  };
  std::vector<State> st(m, State{kFirstA, 0.0, 0, 1});
  const unsigned vgrid = (unsigned)((n + 255) / 256);
  auto setup = [&](const std::vector<int>& ks, const std::vector<int>& act, const std::vector<int>& arg)
      -> wmom_status {
    if (ks.empty()) return WMOM_OK;
    for (size_t q = 0; q < ks.size(); ++q) {
      hi[4 * L + q] = slots[ks[q]];
      hi[5 * L + q] = act[q];
      hi[6 * L + q] = arg[q];
    }
    COND_TRY(cudaMemcpyAsync(di + 4 * L, hi.data() + 4 * L, sizeof(int) * 3 * L, cudaMemcpyHostToDevice, s));
    stats::count(stats::kMisc);
    cond_setup_kernel<C><<<dim3(vgrid, (unsigned)ks.size()), 256, 0, s>>>(X, n, nreal, di + 4 * L, di + 5 * L,
                                                                        di + 6 * L);
    COND_TRY(cudaGetLastError());
    // the host lists are reused before the copy above has run
    COND_TRY(cudaStreamSynchronize(s));
    return WMOM_OK;
  };
  {
    std::vector<int> ks(m), act(m, 3), arg(m, 0);
    for (int k = 0; k < m; ++k) ks[k] = k;
    const wmom_status ss = setup(ks, act, arg);
    if (ss != WMOM_OK) return ss;
  }
  for (int round = 0; round < 16; ++round) {
    std::vector<int> ka, kh, kall;
    for (int k = 0; k < m; ++k) {
      if (st[k].step == kDone) continue;
      (st[k].step == kFirstH || st[k].step == kStepH ? kh : ka).push_back(k);
      kall.push_back(k);
    }
    if (kall.empty()) break;
    for (size_t q = 0; q < ka.size(); ++q) hi[0 * L + q] = slots[ka[q]];
    for (size_t q = 0; q < kh.size(); ++q) hi[1 * L + q] = slots[kh[q]];
    for (size_t q = 0; q < kall.size(); ++q) {
      hi[2 * L + q] = slots[kall[q]];
      hi[3 * L + q] = st[kall[q]].j;
    }
    COND_TRY(cudaMemcpyAsync(di, hi.data(), sizeof(int) * 4 * L, cudaMemcpyHostToDevice, s));
    if (!ka.empty())
      COND_TRY(lu_solve_t<C>(lu, lda, n, ipiv, X, n, 1, ws, s, (int)ka.size(), astride, di));
    if (!kh.empty())
      COND_TRY(lu_solve_h_t<C>(lu, lda, n, ipiv, X, ws, s, (int)kh.size(), astride, di + L));
    stats::count(stats::kMisc);
    cond_stats_kernel<C><<<(unsigned)kall.size(), kCondThreads, 0, s>>>(X, n, nreal, di + 2 * L, di + 3 * L,
                                                                        dstat);
    COND_TRY(cudaGetLastError());
    COND_TRY(cudaMemcpyAsync(hstat.data(), dstat, sizeof(double) * 4 * kall.size(), cudaMemcpyDeviceToHost, s));
    COND_TRY(cudaStreamSynchronize(s));
    std::vector<int> ks, act, arg;
    for (size_t q = 0; q < kall.size(); ++q) {
      State& z = st[kall[q]];
      const double sum = hstat[4 * q], amax = hstat[4 * q + 2], aprev = hstat[4 * q + 3];
      const int jmax = (int)hstat[4 * q + 1];
      switch (z.step) {
        case kFirstA:  // x = Z^-1 (1/n, ..., 1/n)
          z.est = sum;
          if (nreal == 1) {
            z.step = kDone;
          } else {
            z.step = kFirstH;
            ks.push_back(kall[q]);
            act.push_back(0);
            arg.push_back(0);
          }
          break;
        case kFirstH:  // x = Z^-H sign(...)
          z.j = jmax;
          z.iter = 2;
          z.step = kStepA;
          ks.push_back(kall[q]);
          act.push_back(1);
          arg.push_back(z.j);
          break;
        case kStepA: {  // x = Z^-1 e_j
          const double old = z.est;
          z.est = sum;
          ks.push_back(kall[q]);
          if (z.est <= old) {  // no growth: the iteration cycles
            z.step = kAltA;
            act.push_back(2);
          } else {
            z.step = kStepH;
            act.push_back(0);
          }
          arg.push_back(0);
          break;
        }
        case kStepH: {  // x = Z^-H sign(...)
          const int jlast = z.j;
          z.j = jmax;
          ks.push_back(kall[q]);
          if (aprev != amax && z.iter < 5) {
            ++z.iter;
            z.step = kStepA;
            act.push_back(1);
            arg.push_back(z.j);
          } else {
            z.step = kAltA;
            act.push_back(2);
            arg.push_back(0);
          }
          (void)jlast;
          break;
        }
        case kAltA: {  // x = Z^-1 (alternating test vector)
          const double temp = 2.0 * (sum / (3.0 * nreal));
          if (temp > z.est) z.est = temp;
          z.step = kDone;
          break;
        }
        default:
          break;
      }
    }
    const wmom_status ss = setup(ks, act, arg);
    if (ss != WMOM_OK) return ss;
  }
  if (lu_workspace_read_status(ws, nullptr, s, 1)) return WMOM_ERR_TIMEOUT;
  for (int k = 0; k < m; ++k) est[k] = st[k].est;
  return WMOM_OK;
}

template wmom_status condest_t<double2>(int, int, const double2*, long long, long long, const int*, const int*,
                                        int, double2*, LuWorkspace*, cudaStream_t, double*);
template wmom_status condest_t<float2>(int, int, const float2*, long long, long long, const int*, const int*, int,
                                       float2*, LuWorkspace*, cudaStream_t, double*);

}  // namespace wmom
