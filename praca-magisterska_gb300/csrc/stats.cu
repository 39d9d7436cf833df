// stats.cu -- see stats.h.
#include "lu_internal.h"
#include "stats.h"

#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "../../include/wmom.h"

namespace wmom {
namespace stats {
namespace {

struct Rec {
  int c;
  cudaEvent_t e0, e1;
  double work;
};

std::atomic<bool> g_timing{false};
std::atomic<long long> g_launches[kNumCls];
std::mutex g_mu;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;
double g_ms[kNumCls];
double g_work[kNumCls];
long long g_timed[kNumCls];

cudaEvent_t get_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Moves finished records into the totals (caller holds g_mu).
void drain(bool wait) {
  std::vector<Rec> keep;
  for (Rec& r : g_recs) {
    if (wait) cudaEventSynchronize(r.e1);
    if (cudaEventQuery(r.e1) == cudaSuccess) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, r.e0, r.e1);
      g_ms[r.c] += ms;
      g_work[r.c] += r.work;
      g_timed[r.c] += 1;
      g_pool.push_back(r.e0);
      g_pool.push_back(r.e1);
    } else {
      keep.push_back(r);
    }
  }
  g_recs.swap(keep);
}

}  // namespace

bool timing_enabled() { return g_timing.load(std::memory_order_relaxed); }

void count(Cls c, int launches) { g_launches[c].fetch_add(launches, std::memory_order_relaxed); }

void snapshot(long long out[kNumCls]) {
  for (int i = 0; i < kNumCls; ++i) out[i] = g_launches[i].load(std::memory_order_relaxed);
}

void add_counts(const long long delta[kNumCls]) {
  for (int i = 0; i < kNumCls; ++i) g_launches[i].fetch_add(delta[i], std::memory_order_relaxed);
}

Scope::Scope(Cls c, cudaStream_t s, double work, int launches) : c_(c), s_(s), work_(work) {
  count(c, launches);
  // no timing inside a stream capture: the events would become graph nodes
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (timing_enabled() && cudaStreamIsCapturing(s_, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone) {
    std::lock_guard<std::mutex> lk(g_mu);
    e0_ = get_event();
    cudaEventRecord(e0_, s_);
  }
}

Scope::~Scope() {
  if (!e0_) return;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaEvent_t e1 = get_event();
  cudaEventRecord(e1, s_);
  g_recs.push_back(Rec{c_, e0_, e1, work_});
  if (g_recs.size() > 4096) drain(false);
}

// CH independent FMA chains per thread; the loop count is a kernel argument, so the
// kernel always ends.
template <int CH>
__global__ void fp64_fma_probe_kernel(double* out, double a, double b, int iters) {
  double x[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) x[c] = threadIdx.x + c;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < CH; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace stats
}  // namespace wmom

using namespace wmom::stats;

namespace {

template <int CH>
double probe_once(double* buf, int blocks, int threads, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1) {
  const int iters = 4096;
  fp64_fma_probe_kernel<CH><<<blocks, threads, 0, s>>>(buf, 1.0000001, 1e-9, iters);  // warm-up
  cudaEventRecord(e0, s);
  fp64_fma_probe_kernel<CH><<<blocks, threads, 0, s>>>(buf, 1.0000001, 1e-9, iters);
  cudaEventRecord(e1, s);
  if (cudaEventSynchronize(e1) != cudaSuccess) return 0.0;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  return ms > 0.f ? 2.0 * CH * iters * double(blocks) * threads / (ms * 1e-3) / 1e12 : 0.0;
}

}  // namespace

extern "C" {

void wmom_stats_enable(int on) { g_timing.store(on != 0); }

void wmom_stats_reset(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  drain(true);
  for (int i = 0; i < kNumCls; ++i) {
    g_launches[i].store(0);
    g_ms[i] = 0.0;
    g_work[i] = 0.0;
    g_timed[i] = 0;
  }
}

int wmom_stats_read(double* ms, long long* launches, long long* timed, double* work, int n) {
  std::lock_guard<std::mutex> lk(g_mu);
  drain(true);
  const int m = n < kNumCls ? n : kNumCls;
  for (int i = 0; i < m; ++i) {
    if (ms) ms[i] = g_ms[i];
    if (launches) launches[i] = g_launches[i].load();
    if (timed) timed[i] = g_timed[i];
    if (work) work[i] = g_work[i];
  }
  return kNumCls;
}

wmom_status wmom_probe_fp64_tflops(double* tflops) {
  if (!tflops) return WMOM_ERR_ARG;
  *tflops = 0.0;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0)
    return WMOM_ERR_CUDA;
  const int max_blocks = nsm * 8, max_threads = 256;
  double* buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double) * max_blocks * max_threads) != cudaSuccess) return WMOM_ERR_NOMEM;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0.0;
  best = std::max(best, probe_once<8>(buf, nsm * 4, 256, s, e0, e1));
  best = std::max(best, probe_once<16>(buf, nsm * 4, 256, s, e0, e1));
  best = std::max(best, probe_once<16>(buf, nsm * 8, 128, s, e0, e1));
  best = std::max(best, probe_once<32>(buf, nsm * 2, 256, s, e0, e1));
  // FMA chains stop short of the pipe's rate on this GPU (about 1.05 against the
  // 1.24 TFLOP/s a register-tiled GEMM sustains with the FP64 pipe 99% busy, ncu), so
  // the FP64 complex GEMM of the plain form is timed as well, on a compute-bound shape
  // (C 4096 x 4096 += A 4096 x 256 B: 64 flops per byte of C), and the faster wins --
  // as the bf16 denominator is a measured GEMM
  {
    const int m = 4096, k = 256;
    double2 *a = nullptr, *bm = nullptr, *c = nullptr;
    if (cudaMalloc(&a, sizeof(double2) * (size_t)m * k) == cudaSuccess &&
        cudaMalloc(&bm, sizeof(double2) * (size_t)m * k) == cudaSuccess &&
        cudaMalloc(&c, sizeof(double2) * (size_t)m * m) == cudaSuccess) {
      cudaMemsetAsync(a, 0, sizeof(double2) * (size_t)m * k, s);
      cudaMemsetAsync(bm, 0, sizeof(double2) * (size_t)m * k, s);
      cudaMemsetAsync(c, 0, sizeof(double2) * (size_t)m * m, s);
      for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(e0, s);
        const cudaError_t ge = wmom::zgemm_sub_simt(a, m, bm, k, c, m, m, m, k, s, 1, 0);
        cudaEventRecord(e1, s);
        float ms = 0.f;
        if (ge == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess &&
            cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0.f && rep > 0)
          best = std::max(best, 8.0 * m * (double)m * k / (ms * 1e-3) / 1e12);
      }
    }
    cudaStreamSynchronize(s);
    if (a) cudaFree(a);
    if (bm) cudaFree(bm);
    if (c) cudaFree(c);
    cudaGetLastError();
  }
  const cudaError_t err = cudaStreamSynchronize(s);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  cudaFree(buf);
  if (err != cudaSuccess || best <= 0.0) return WMOM_ERR_CUDA;
  *tflops = best;
  return WMOM_OK;
}

}  // extern "C"
