// api.cu -- the C ABI of libwmom (include/wmom.h): plans, fill, LU, solves and the
// batched frequency-sweep solver with the FP64 (plain) and mixed-precision
// (FP32 tensor-core LU + FP64 iterative refinement) forms.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <set>
#include <thread>
#include <utility>
#include <vector>

#include "lu_common.cuh"
#include "lu_internal.h"
#include "solve_internal.h"
#include "wmom_internal.h"

namespace {
thread_local char g_last_error[256] = "";
}

wmom_status wmom_fail_cuda(cudaError_t e, const char* what) {
  std::snprintf(g_last_error, sizeof(g_last_error), "%s failed: %s", what, cudaGetErrorString(e));
  if (std::getenv("WMOM_VERBOSE")) std::fprintf(stderr, "wmom: %s\n", g_last_error);
  if (e == cudaErrorMemoryAllocation) return WMOM_ERR_NOMEM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorNoKernelImageForDevice)
    return WMOM_ERR_UNSUPPORTED;
  return WMOM_ERR_CUDA;
}

namespace wmom {

cudaError_t allow_dynamic_smem(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::set<std::pair<int, const void*>> raised;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  if (raised.count({dev, func})) return cudaSuccess;
  int optin = 0;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  cudaFuncAttributes fa{};
  e = cudaFuncGetAttributes(&fa, func);
  if (e != cudaSuccess) return e;
  const int cap = optin - (int)fa.sharedSizeBytes;  // static shared memory counts against it
  if (bytes > (size_t)std::max(cap, 0)) return cudaErrorInvalidValue;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
  if (e != cudaSuccess) return e;
  raised.insert({dev, func});
  return cudaSuccess;
}

// ---------------------------------------------------------- workspace ----
namespace {

cudaError_t ws_alloc(const LuWorkspace* ws, void** p, size_t bytes, cudaStream_t s) {
  return ws->pooled ? cudaMallocAsync(p, bytes, s) : cudaMalloc(p, bytes);
}

cudaError_t ws_zero(const LuWorkspace* ws, void* p, size_t bytes, cudaStream_t s) {
  return ws->pooled ? cudaMemsetAsync(p, 0, bytes, s) : cudaMemset(p, 0, bytes);
}

cudaError_t workspace_create(LuWorkspace* ws, int nmax, int nrhs_max, int max_batch, bool pooled, cudaStream_t s) {
  *ws = LuWorkspace{};
  ws->pooled = pooled;
  max_batch = std::max(max_batch, 1);
  const size_t off = lu_stage_offset(max_batch);
  const size_t bytes = off + lu_stage_bytes(max_batch);
  void* p = nullptr;
  cudaError_t e = ws_alloc(ws, &p, bytes, s);
  if (e != cudaSuccess) return e;
  ws->max_batch = max_batch;
  ws->barrier = reinterpret_cast<GridBarrier*>(p);
  ws->stage = reinterpret_cast<char*>(p) + off;
  e = ws_zero(ws, p, bytes, s);
  if (e != cudaSuccess) return e;
  e = ws_alloc(ws, reinterpret_cast<void**>(&ws->perm), sizeof(int) * (size_t)std::max(nmax, 1) * max_batch, s);
  if (e != cudaSuccess) return e;
  ws->perm_cap = nmax;
  ws->rhs_bytes =
      sizeof(double2) * (size_t)std::max(nmax, 1) * (size_t)std::max(std::max(nrhs_max, 1), max_batch);
  e = ws_alloc(ws, &ws->rhs, ws->rhs_bytes, s);
  if (e != cudaSuccess) return e;
  ws->flag_cap = (std::max(nmax, 1) + 63) / 64 + 1;
  const size_t fbytes = sizeof(int) * ((size_t)ws->flag_cap * max_batch + max_batch);
  e = ws_alloc(ws, reinterpret_cast<void**>(&ws->flags), fbytes, s);
  if (e != cudaSuccess) return e;
  e = ws_zero(ws, ws->flags, fbytes, s);
  if (e != cudaSuccess) return e;
  ws->ticket = reinterpret_cast<unsigned int*>(ws->flags + (size_t)ws->flag_cap * max_batch);
  ws->epoch = 0;
  e = ws_alloc(ws, reinterpret_cast<void**>(&ws->tc_err), sizeof(int), s);
  if (e != cudaSuccess) return e;
  return ws_zero(ws, ws->tc_err, sizeof(int), s);
}

}  // namespace

cudaError_t lu_workspace_create(LuWorkspace* ws, int nmax, int nrhs_max, int max_batch) {
  return workspace_create(ws, nmax, nrhs_max, max_batch, false, nullptr);
}

cudaError_t lu_workspace_create_async(LuWorkspace* ws, int nmax, int nrhs_max, int max_batch, cudaStream_t s) {
  return workspace_create(ws, nmax, nrhs_max, max_batch, true, s);
}

void lu_workspace_destroy(LuWorkspace* ws) {
  const bool pooled = ws->pooled;
  auto release = [pooled](void* p) {
    if (!p) return;
    if (pooled)
      cudaFreeAsync(p, cudaStreamPerThread);
    else
      cudaFree(p);
  };
  release(ws->barrier);
  release(ws->perm);
  release(ws->rhs);
  release(ws->flags);
  release(ws->tc_buf);
  release(ws->tc_err);
  *ws = LuWorkspace{};
}

cudaError_t lu_workspace_reset_barrier(LuWorkspace* ws, cudaStream_t s) {
  return cudaMemsetAsync(ws->barrier, 0, sizeof(GridBarrier) * ws->max_batch, s);
}

// Returns 0 when the last factorisation finished its waits; info[b] = first zero pivot.
int lu_workspace_read_status(LuWorkspace* ws, int* info, cudaStream_t s, int batch) {
  std::vector<GridBarrier> h(std::max(batch, 1));
  cudaMemcpyAsync(h.data(), ws->barrier, sizeof(GridBarrier) * h.size(), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  int err = 0;
  for (size_t b = 0; b < h.size(); ++b) {
    if (info) info[b] = h[b].info;
    err |= h[b].err;
  }
  return err;
}

namespace {

// A lazily created workspace per device for the stateless LAPACK-style entry points.
struct DefaultWs {
  std::mutex mu;
  std::vector<LuWorkspace> ws;
  std::vector<int> cap_n, cap_rhs;
};
DefaultWs& default_ws() {
  static DefaultWs* d = new DefaultWs();
  return *d;
}

cudaError_t get_default_ws(int n, int nrhs, LuWorkspace** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  DefaultWs& d = default_ws();
  if ((int)d.ws.size() <= dev) {
    d.ws.resize(dev + 1);
    d.cap_n.resize(dev + 1, 0);
    d.cap_rhs.resize(dev + 1, 0);
  }
  if (d.cap_n[dev] < n || d.cap_rhs[dev] < nrhs) {
    if (d.cap_n[dev] > 0) {
      cudaDeviceSynchronize();
      lu_workspace_destroy(&d.ws[dev]);
    }
    const int cn = std::max(n, d.cap_n[dev]);
    const int cr = std::max(nrhs, d.cap_rhs[dev]);
    e = lu_workspace_create(&d.ws[dev], cn, cr);
    if (e != cudaSuccess) {
      d.cap_n[dev] = 0;
      return e;
    }
    d.cap_n[dev] = cn;
    d.cap_rhs[dev] = cr;
  }
  *out = &d.ws[dev];
  return cudaSuccess;
}


}  // namespace
}  // namespace wmom

using namespace wmom;

struct wmom_plan_s {
  Plan p;
  std::mutex mu;
  FreqParams* d_fp = nullptr;
  int fp_cap = 0;
  LuWorkspace ws{};
  int ws_n = 0;
  size_t tile_bytes = 0;
};

extern "C" {

const char* wmom_last_error(void) { return g_last_error; }

const char* wmom_status_string(wmom_status s) {
  switch (s) {
    case WMOM_OK: return "ok";
    case WMOM_ERR_ARG: return "invalid argument";
    case WMOM_ERR_CUDA: return "CUDA error";
    case WMOM_ERR_SINGULAR: return "singular matrix (zero pivot)";
    case WMOM_ERR_TIMEOUT: return "device-side wait timed out";
    case WMOM_ERR_NOMEM: return "out of device memory";
    case WMOM_ERR_NOT_CONVERGED: return "iterative refinement did not converge";
    case WMOM_ERR_GEOMETRY: return "invalid geometry";
    case WMOM_ERR_UNSUPPORTED: return "unsupported device";
  }
  return "unknown";
}

double wmom_ka(float freq_mhz) { return ka_from_mhz(freq_mhz); }

wmom_status wmom_excitation(int npls, int ngap, float ampl, float phas_deg, double* v) {
  if (npls <= 0 || !v || ngap < 1 || ngap > npls) return WMOM_ERR_ARG;
  const double pi = std::acos(-1.);
  std::memset(v, 0, sizeof(double) * 2 * (size_t)npls);
  const double arg = pi * phas_deg / 180.;
  const double a = std::fabs((double)ampl);
  // (a, 0) * (cos, sin), as Z_MUL does it (REF/Wire_MoM.cu:307-309)
  const double c = std::cos(arg), s = std::sin(arg);
  v[2 * (ngap - 1)] = a * c - 0.0 * s;
  v[2 * (ngap - 1) + 1] = a * s + 0.0 * c;
  return WMOM_OK;
}

wmom_status wmom_plan_create(const float* x, const float* y, const float* z, const float* rad,
                             const int* ipc, const int* ips, const int* ise, int nsmax, int npls,
                             int ienv, float sgnx, float sgny, float sgnz, float sgnenv,
                             wmom_plan* out) {
  if (!out) return WMOM_ERR_ARG;
  *out = nullptr;
  if (!x || !y || !z || !rad || !ipc || !ips || !ise || nsmax <= 0 || npls <= 0 || npls > nsmax ||
      (ienv != 1 && ienv != 2))
    return WMOM_ERR_ARG;
  wmom_plan_s* h = new (std::nothrow) wmom_plan_s();
  if (!h) return WMOM_ERR_NOMEM;
  Plan& p = h->p;
  p.npls = npls;
  p.nsmax = nsmax;
  p.ienv = ienv;
  p.sgnx = sgnx;
  p.sgny = sgny;
  p.sgnz = sgnz;
  p.sgnenv = sgnenv;
  int st = plan_build_tables(&p, x, y, z, rad, ipc, ips, ise);
  if (st != WMOM_OK) {
    delete h;
    return (wmom_status)st;
  }
  cudaError_t e = cudaGetDevice(&p.device);
  if (e == cudaSuccess) e = cudaMalloc(&p.d_obs, sizeof(ObsHalf) * p.h_obs.size());
  if (e == cudaSuccess) e = cudaMalloc(&p.d_src, sizeof(SrcHalf) * p.h_src.size());
  if (e == cudaSuccess)
    e = cudaMemcpy(p.d_obs, p.h_obs.data(), sizeof(ObsHalf) * p.h_obs.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(p.d_src, p.h_src.data(), sizeof(SrcHalf) * p.h_src.size(), cudaMemcpyHostToDevice);
  // pair-tiled fill tables (free space)
  plan_build_pair_tiles(&p, x, y, z, rad, ipc, ips, ise);
  if (e == cudaSuccess && p.pt.ok) {
    const PairTiles& t = p.pt;
    std::vector<int> ints;
    ints.insert(ints.end(), t.rt_off.begin(), t.rt_off.end());
    p.off_rt_ids = (int)ints.size();
    ints.insert(ints.end(), t.rt_ids.begin(), t.rt_ids.end());
    p.off_ct_off = (int)ints.size();
    ints.insert(ints.end(), t.ct_off.begin(), t.ct_off.end());
    p.off_ct_ids = (int)ints.size();
    ints.insert(ints.end(), t.ct_ids.begin(), t.ct_ids.end());
    p.off_row_local = (int)ints.size();
    ints.insert(ints.end(), t.row_local.begin(), t.row_local.end());
    p.off_col_local = (int)ints.size();
    ints.insert(ints.end(), t.col_local.begin(), t.col_local.end());
    e = cudaMalloc(&p.d_oi, sizeof(ObsInst) * t.obs.size());
    if (e == cudaSuccess) e = cudaMalloc(&p.d_si, sizeof(SrcInst) * t.src.size());
    if (e == cudaSuccess) e = cudaMalloc(&p.d_tiles, sizeof(int) * ints.size());
    if (e == cudaSuccess)
      e = cudaMemcpy(p.d_oi, t.obs.data(), sizeof(ObsInst) * t.obs.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(p.d_si, t.src.data(), sizeof(SrcInst) * t.src.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(p.d_tiles, ints.data(), sizeof(int) * ints.size(), cudaMemcpyHostToDevice);
    h->tile_bytes = sizeof(ObsInst) * t.obs.size() + sizeof(SrcInst) * t.src.size() + sizeof(int) * ints.size();
  }
  if (e != cudaSuccess) {
    if (p.d_obs) cudaFree(p.d_obs);
    if (p.d_src) cudaFree(p.d_src);
    if (p.d_oi) cudaFree(p.d_oi);
    if (p.d_si) cudaFree(p.d_si);
    if (p.d_tiles) cudaFree(p.d_tiles);
    delete h;
    return wmom_fail_cuda(e, "plan upload");
  }
  *out = h;
  return WMOM_OK;
}

wmom_status wmom_plan_destroy(wmom_plan h) {
  if (!h) return WMOM_ERR_ARG;
  cudaDeviceSynchronize();
  if (h->p.d_obs) cudaFree(h->p.d_obs);
  if (h->p.d_src) cudaFree(h->p.d_src);
  if (h->p.d_oi) cudaFree(h->p.d_oi);
  if (h->p.d_si) cudaFree(h->p.d_si);
  if (h->p.d_tiles) cudaFree(h->p.d_tiles);
  if (h->d_fp) cudaFree(h->d_fp);
  if (h->ws_n) lu_workspace_destroy(&h->ws);
  delete h;
  return WMOM_OK;
}

int wmom_plan_npls(wmom_plan h) { return h ? h->p.npls : -1; }

int wmom_plan_fill_variant(wmom_plan h) {
  if (!h) return -1;
  if (!h->p.pt.ok) return 0;
  return fill_multi_fits(h->p) ? 2 : 1;
}

wmom_status wmom_plan_set_loads(wmom_plan h, int nloads, const int* idx, const double* r_ohm,
                                const double* l_uh) {
  if (!h || nloads < 0 || (nloads > 0 && (!idx || !r_ohm || !l_uh))) return WMOM_ERR_ARG;
  for (int i = 0; i < nloads; ++i)
    if (idx[i] < 1 || idx[i] > h->p.npls || !std::isfinite(r_ohm[i]) || !std::isfinite(l_uh[i]))
      return WMOM_ERR_ARG;
  std::lock_guard<std::mutex> lk(h->mu);
  h->p.load_idx.assign(idx, idx + nloads);
  h->p.load_r.assign(r_ohm, r_ohm + nloads);
  h->p.load_l_uh.assign(l_uh, l_uh + nloads);
  return WMOM_OK;
}

long long wmom_plan_upload_bytes(wmom_plan h) {
  if (!h) return -1;
  return (long long)(sizeof(ObsHalf) * h->p.h_obs.size() + sizeof(SrcHalf) * h->p.h_src.size() + h->tile_bytes);
}

long long wmom_plan_fill_pairs(wmom_plan h) {
  if (!h) return -1;
  if (!h->p.pt.ok) return 0;
  // distinct (observation, source) instance pairs the pair-tiled fill evaluates per
  // frequency: every row tile meets every column tile
  return (long long)h->p.pt.rt_ids.size() * (long long)h->p.pt.ct_ids.size();
}

int wmom_plan_loops(wmom_plan h) { return h ? h->p.loops : -1; }

wmom_status wmom_fill(wmom_plan h, const double* ka, int nk, void* z_dev, long long ldz,
                      long long zstride, void* stream) {
  if (!h || !ka || nk <= 0 || !z_dev || ldz < h->p.npls || (nk > 1 && zstride < ldz * h->p.npls))
    return WMOM_ERR_ARG;
  for (int i = 0; i < nk; ++i)
    if (!(ka[i] > 0.0) || !std::isfinite(ka[i])) return WMOM_ERR_ARG;
  std::lock_guard<std::mutex> lk(h->mu);
  cudaStream_t s = (cudaStream_t)stream;
  if (h->fp_cap < nk) {
    if (h->d_fp) {
      cudaStreamSynchronize(s);
      cudaFree(h->d_fp);
      h->d_fp = nullptr;
      h->fp_cap = 0;  // a failed allocation below leaves no stale capacity
    }
    WMOM_CUDA_TRY(cudaMalloc(&h->d_fp, sizeof(FreqParams) * nk));
    h->fp_cap = nk;
  }
  std::vector<FreqParams> fp(nk);
  for (int i = 0; i < nk; ++i) fp[i] = freq_params(ka[i]);
  WMOM_CUDA_TRY(cudaMemcpyAsync(h->d_fp, fp.data(), sizeof(FreqParams) * nk, cudaMemcpyHostToDevice, s));
  WMOM_CUDA_TRY(launch_fill(h->p, reinterpret_cast<const double*>(h->d_fp), nk,
                            reinterpret_cast<double2*>(z_dev), ldz, zstride, s));
  // the parameter upload is from pageable memory: finish before the vector dies
  WMOM_CUDA_TRY(cudaStreamSynchronize(s));
  return WMOM_OK;
}

wmom_status wmom_fill_geometries(const wmom_plan* plans, int count, const double* ka, void* const* z_dev,
                                 const long long* ldz, void* stream) {
  if (count <= 0 || !plans || !ka || !z_dev || !ldz) return WMOM_ERR_ARG;
  std::vector<const Plan*> ps(count);
  for (int i = 0; i < count; ++i) {
    if (!plans[i] || !z_dev[i] || ldz[i] < plans[i]->p.npls || !(ka[i] > 0.0) || !std::isfinite(ka[i]))
      return WMOM_ERR_ARG;
    ps[i] = &plans[i]->p;
  }
  cudaStream_t s = (cudaStream_t)stream;
  WMOM_CUDA_TRY(launch_fill_geometries(ps.data(), ka, reinterpret_cast<double2* const*>(z_dev), ldz, count, s));
  // the job list is uploaded from pageable memory: finish before it dies
  WMOM_CUDA_TRY(cudaStreamSynchronize(s));
  return WMOM_OK;
}

wmom_status wmom_zgetrf(int n, void* a_dev, long long lda, int* ipiv_dev, int* info, void* stream) {
  if (n <= 0 || !a_dev || lda < n || !ipiv_dev) return WMOM_ERR_ARG;
  if ((size_t)n * sizeof(int) > 200 * 1024) return WMOM_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(default_ws().mu);
  LuWorkspace* ws = nullptr;
  WMOM_CUDA_TRY(get_default_ws(n, 1, &ws));
  WMOM_CUDA_TRY(lu_workspace_reset_barrier(ws, s));
  WMOM_CUDA_TRY(lu_factor_t<double2>(reinterpret_cast<double2*>(a_dev), lda, n, ipiv_dev, ws, s, nullptr));
  int inf = 0;
  const int err = lu_workspace_read_status(ws, &inf, s);
  WMOM_CUDA_TRY(cudaGetLastError());
  if (info) *info = inf;
  if (err) return WMOM_ERR_TIMEOUT;
  return inf ? WMOM_ERR_SINGULAR : WMOM_OK;
}

wmom_status wmom_zlange1(int n, const void* a_dev, long long lda, double* anorm, void* stream) {
  if (n <= 0 || !a_dev || lda < n || !anorm) return WMOM_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  double* d = nullptr;
  WMOM_CUDA_TRY(cudaMallocAsync(&d, sizeof(double), s));
  cudaError_t e = norm1_batch(reinterpret_cast<const double2*>(a_dev), n, lda, 0, 1, d, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(anorm, d, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return wmom_fail_cuda(e, "wmom_zlange1");
  return WMOM_OK;
}

wmom_status wmom_zgecon(int n, const void* a_dev, long long lda, const int* ipiv_dev, double anorm, double* rcond,
                        void* stream) {
  if (n <= 0 || !a_dev || lda < n || !ipiv_dev || !rcond || !(anorm >= 0.0)) return WMOM_ERR_ARG;
  if ((size_t)n * sizeof(int) > 200 * 1024) return WMOM_ERR_ARG;
  *rcond = 0.0;
  if (anorm == 0.0) return WMOM_OK;  // LAPACK: rcond = 0 for a zero matrix
  cudaStream_t s = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(default_ws().mu);
  LuWorkspace* ws = nullptr;
  WMOM_CUDA_TRY(get_default_ws(n, 1, &ws));
  WMOM_CUDA_TRY(lu_workspace_reset_barrier(ws, s));
  double2* x = nullptr;
  WMOM_CUDA_TRY(cudaMallocAsync(&x, sizeof(double2) * n, s));
  const int slot = 0;
  double est = 0.0;
  const wmom_status st = condest_t<double2>(n, n, reinterpret_cast<const double2*>(a_dev), lda, 0, ipiv_dev, &slot,
                                            1, x, ws, s, &est);
  cudaFreeAsync(x, s);
  if (st != WMOM_OK) return st;
  if (est > 0.0) *rcond = (1.0 / est) / anorm;
  return WMOM_OK;
}

void wmom_debug_panel_missing_arrivals(int count) {
  g_panel_missing_arrivals.store(count > 0 ? (unsigned)count : 0u, std::memory_order_relaxed);
}

wmom_status wmom_cgetrf(int n, void* a_dev, long long lda, int* ipiv_dev, int* info, void* stream) {
  if (n <= 0 || !a_dev || lda < n || !ipiv_dev) return WMOM_ERR_ARG;
  if ((size_t)n * sizeof(int) > 200 * 1024) return WMOM_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(default_ws().mu);
  LuWorkspace* ws = nullptr;
  WMOM_CUDA_TRY(get_default_ws(n, 1, &ws));
  WMOM_CUDA_TRY(lu_workspace_reset_barrier(ws, s));
  const GemmHook<float2> hook = tc_gemm_hook();
  WMOM_CUDA_TRY(lu_factor_t<float2>(reinterpret_cast<float2*>(a_dev), lda, n, ipiv_dev, ws, s, hook));
  int inf = 0;
  int err = lu_workspace_read_status(ws, &inf, s);
  if (hook) err |= tc::read_and_clear_error(ws, s);
  WMOM_CUDA_TRY(cudaGetLastError());
  if (info) *info = inf;
  if (err) return WMOM_ERR_TIMEOUT;
  return inf ? WMOM_ERR_SINGULAR : WMOM_OK;
}

wmom_status wmom_zgetrs(int n, int nrhs, const void* a_dev, long long lda, const int* ipiv_dev,
                        void* b_dev, long long ldb, void* stream) {
  if (n <= 0 || nrhs <= 0 || !a_dev || lda < n || !ipiv_dev || !b_dev || ldb < n) return WMOM_ERR_ARG;
  if ((size_t)n * sizeof(int) > 200 * 1024) return WMOM_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(default_ws().mu);
  LuWorkspace* ws = nullptr;
  WMOM_CUDA_TRY(get_default_ws(n, nrhs, &ws));
  WMOM_CUDA_TRY(lu_solve_t<double2>(reinterpret_cast<const double2*>(a_dev), lda, n, ipiv_dev,
                                    reinterpret_cast<double2*>(b_dev), ldb, nrhs, ws, s));
  WMOM_CUDA_TRY(cudaStreamSynchronize(s));
  return WMOM_OK;
}

wmom_status wmom_zgesv_like(int n, double* z, const double* v, double* i_out, int* ipiv, int* info) {
  if (n <= 0 || !z || !v || !i_out || !ipiv) return WMOM_ERR_ARG;
  double2* dz = nullptr;
  double2* db = nullptr;
  int* dp = nullptr;
  wmom_status st = WMOM_OK;
  int inf = 0;
  cudaError_t e = cudaMalloc(&dz, sizeof(double2) * (size_t)n * n);
  if (e == cudaSuccess) e = cudaMalloc(&db, sizeof(double2) * (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc(&dp, sizeof(int) * (size_t)n);
  if (e == cudaSuccess) e = cudaMemcpy(dz, z, sizeof(double2) * (size_t)n * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(db, v, sizeof(double2) * (size_t)n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    st = wmom_fail_cuda(e, "zgesv_like upload");
  } else {
    st = wmom_zgetrf(n, dz, n, dp, &inf, nullptr);
    if (st == WMOM_OK || st == WMOM_ERR_SINGULAR) {
      const wmom_status st2 = wmom_zgetrs(n, 1, dz, n, dp, db, n, nullptr);
      if (st == WMOM_OK) st = st2;
      e = cudaMemcpy(z, dz, sizeof(double2) * (size_t)n * n, cudaMemcpyDeviceToHost);
      if (e == cudaSuccess) e = cudaMemcpy(i_out, db, sizeof(double2) * (size_t)n, cudaMemcpyDeviceToHost);
      if (e == cudaSuccess) e = cudaMemcpy(ipiv, dp, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess && st == WMOM_OK) st = wmom_fail_cuda(e, "zgesv_like download");
    }
  }
  if (info) *info = inf;
  if (dz) cudaFree(dz);
  if (db) cudaFree(db);
  if (dp) cudaFree(dp);
  return st;
}

wmom_status wmom_solve_sweep(wmom_plan h, const float* freq_mhz, int nfreq, int ngap, float ampl,
                             float phas_deg, int mode, double tol, double* currents, double* zin,
                             wmom_report* reports, void* stream) {
  const bool condest = (mode & WMOM_SOLVE_CONDEST) != 0;
  mode &= ~WMOM_SOLVE_CONDEST;
  if (!h || !freq_mhz || nfreq <= 0 || ngap < 1 || ngap > h->p.npls ||
      (mode != WMOM_MODE_FP64 && mode != WMOM_MODE_MIXED))
    return WMOM_ERR_ARG;
  for (int i = 0; i < nfreq; ++i)
    if (!(freq_mhz[i] > 0.f) || !std::isfinite(freq_mhz[i])) return WMOM_ERR_ARG;
  SweepArgs a;
  a.condest = condest;
  a.plan = &h->p;
  a.freq_mhz = freq_mhz;
  a.nfreq = nfreq;
  a.ngap = ngap;
  a.ampl = ampl;
  a.phas_deg = phas_deg;
  a.mode = mode;
  a.tol = tol > 0 ? tol : 1e-12;
  a.currents = currents;
  a.zin = zin;
  a.reports = reports;
  a.stream = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(h->mu);
  if (h->ws_n < h->p.npls) {
    if (h->ws_n) lu_workspace_destroy(&h->ws);
    h->ws_n = 0;
    WMOM_CUDA_TRY(lu_workspace_create(&h->ws, h->p.npls, 1, kMaxLuBatch));
    h->ws_n = h->p.npls;
  }
  a.ws = &h->ws;
  return run_sweep(a);
}

}  // extern "C"

// ----------------------------------------------------------- resident factors ----
struct wmom_factors_s {
  wmom::FactorSet fs;
  wmom::LuWorkspace ws{};
  wmom_plan plan = nullptr;
  size_t bytes = 0;
  std::mutex mu;
  // sets made by one geometry batch share one allocation of their class's matrices,
  // freed with the last of them
  std::shared_ptr<void> shared;
};

namespace {

// Matrices, factors and pivots of one class of a geometry batch.
// They come from the stream-ordered pool and go back to it on the releasing thread's
// default stream, after every call that used them has synchronised its stream.
struct ClassStore {
  void* z64 = nullptr;
  void* lu = nullptr;
  int* ipiv = nullptr;
  ~ClassStore() {
    if (z64) cudaFreeAsync(z64, cudaStreamPerThread);
    if (lu) cudaFreeAsync(lu, cudaStreamPerThread);
    if (ipiv) cudaFreeAsync(ipiv, cudaStreamPerThread);
  }
};

}  // namespace

extern "C" {

wmom_status wmom_factor(wmom_plan h, const float* freq_mhz, int nfreq, int mode, wmom_factors* out, void* stream) {
  if (!out) return WMOM_ERR_ARG;
  *out = nullptr;
  const bool condest = (mode & WMOM_SOLVE_CONDEST) != 0;
  mode &= ~WMOM_SOLVE_CONDEST;
  if (!h || !freq_mhz || nfreq <= 0 || (mode != WMOM_MODE_FP64 && mode != WMOM_MODE_MIXED)) return WMOM_ERR_ARG;
  for (int i = 0; i < nfreq; ++i)
    if (!(freq_mhz[i] > 0.f) || !std::isfinite(freq_mhz[i])) return WMOM_ERR_ARG;
  const int n = h->p.npls;
  const size_t nn = (size_t)n * n;
  const size_t need = (size_t)nfreq * nn * (sizeof(double2) + (mode == WMOM_MODE_MIXED ? sizeof(float2) : sizeof(double2)));
  size_t fr = 0, tot = 0;
  WMOM_CUDA_TRY(cudaMemGetInfo(&fr, &tot));
  if (need > fr) return WMOM_ERR_NOMEM;
  wmom_factors_s* f = new (std::nothrow) wmom_factors_s();
  if (!f) return WMOM_ERR_NOMEM;
  cudaError_t e = lu_workspace_create_async(&f->ws, n, 1, kMaxLuBatch, (cudaStream_t)stream);
  if (e != cudaSuccess) {
    cudaStreamSynchronize((cudaStream_t)stream);
    lu_workspace_destroy(&f->ws);
    delete f;
    return wmom_fail_cuda(e, "factor workspace");
  }
  f->plan = h;
  f->fs.plan = &h->p;
  f->fs.mode = mode;
  f->fs.condest = condest;
  f->fs.freq.assign(freq_mhz, freq_mhz + nfreq);
  f->fs.ws = &f->ws;
  f->bytes = need + (size_t)nfreq * n * sizeof(int);
  wmom_status st;
  {
    std::lock_guard<std::mutex> lk(h->mu);  // the fill reads the plan's loads
    st = factors_build(&f->fs, (cudaStream_t)stream);
  }
  if (st != WMOM_OK) {
    cudaStreamSynchronize((cudaStream_t)stream);  // nothing of the set still queued
    wmom_factors_destroy(f);
    return st;
  }
  *out = f;
  return WMOM_OK;
}

wmom_status wmom_factors_solve(wmom_factors f, int first, int count, int ngap, float ampl, float phas_deg,
                               double tol, double* currents, double* zin, wmom_report* reports, void* stream) {
  if (!f || first < 0 || count <= 0 || first + count > (int)f->fs.freq.size() || ngap < 1 ||
      ngap > f->fs.plan->npls)
    return WMOM_ERR_ARG;
  std::lock_guard<std::mutex> lk(f->mu);
  return factors_solve(&f->fs, first, count, ngap, ampl, phas_deg, tol > 0 ? tol : 1e-12, currents, zin, reports,
                       (cudaStream_t)stream);
}

long long wmom_factors_device_bytes(wmom_factors f) { return f ? (long long)f->bytes : -1; }

wmom_status wmom_factors_destroy(wmom_factors f) {
  if (!f) return WMOM_ERR_ARG;
  // Every call on the set synchronised its stream before it returned, so nothing of
  // the set is still queued: its pooled memory goes back to the pool in the order of
  // this thread's default stream, without waiting for other streams' work.
  if (f->shared) {
    f->shared.reset();  // the class's storage goes with its last set
  } else if (f->fs.pooled) {
    if (f->fs.z64) cudaFreeAsync(f->fs.z64, cudaStreamPerThread);
    if (f->fs.lu) cudaFreeAsync(f->fs.lu, cudaStreamPerThread);
    if (f->fs.ipiv) cudaFreeAsync(f->fs.ipiv, cudaStreamPerThread);
  } else {
    if (f->fs.z64) cudaFree(f->fs.z64);
    if (f->fs.lu) cudaFree(f->fs.lu);
    if (f->fs.ipiv) cudaFree(f->fs.ipiv);
  }
  lu_workspace_destroy(&f->ws);
  delete f;
  return WMOM_OK;
}

int wmom_padded_order(int npls) { return npls > 0 ? padded_order(npls) : 0; }

wmom_status wmom_factor_geometries(const wmom_plan* plans, int count, const float* freq_mhz, int mode,
                                   wmom_factors* out, void* stream) {
  if (!out || count <= 0) return WMOM_ERR_ARG;
  for (int i = 0; i < count; ++i) out[i] = nullptr;
  const bool condest = (mode & WMOM_SOLVE_CONDEST) != 0;
  mode &= ~WMOM_SOLVE_CONDEST;
  if (!plans || !freq_mhz || (mode != WMOM_MODE_FP64 && mode != WMOM_MODE_MIXED)) return WMOM_ERR_ARG;
  for (int i = 0; i < count; ++i)
    if (!plans[i] || !(freq_mhz[i] > 0.f) || !std::isfinite(freq_mhz[i])) return WMOM_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const bool mixed = mode == WMOM_MODE_MIXED;
  const size_t elem = mixed ? sizeof(float2) : sizeof(double2);
  // size classes, members in input order, batches of up to kMaxLuBatch
  std::map<int, std::vector<int>> cls;
  size_t need = 0;
  for (int i = 0; i < count; ++i) {
    const int P = padded_order(plans[i]->p.npls);
    cls[P].push_back(i);
    need += (size_t)P * P * (sizeof(double2) + elem) + sizeof(int) * (size_t)P;
  }
  size_t fr = 0, tot = 0;
  WMOM_CUDA_TRY(cudaMemGetInfo(&fr, &tot));
  if (need > fr) return WMOM_ERR_NOMEM;
  // the fill reads every plan's loads: hold each distinct plan's lock, in address order
  std::set<wmom_plan> uniq(plans, plans + count);
  std::vector<std::unique_lock<std::mutex>> locks;
  for (wmom_plan h : uniq) locks.emplace_back(h->mu);
  retain_pool_memory();
  auto fail = [&](wmom_status st) {
    cudaStreamSynchronize(s);  // allocations and clears of the sets queued on s
    for (int i = 0; i < count; ++i)
      if (out[i]) {
        wmom_factors_destroy(out[i]);
        out[i] = nullptr;
      }
    return st;
  };
  // every class chunk's storage and sets first (allocations on this thread), then the
  // chunks' fills and factorisations concurrently: one host thread and stream each,
  // so that one chunk's fill overlaps another's latency-bound panels
  struct Chunk {
    int P = 0, bg = 0;
    std::vector<int> mem;
    std::shared_ptr<ClassStore> store;
    std::vector<wmom_factors_s*> sets;
    std::vector<int> info;
    wmom_status st = WMOM_OK;
  };
  std::vector<Chunk> chunks;
  for (auto& kv : cls) {
    const int P = kv.first;
    const size_t nn = (size_t)P * P;
    for (size_t c0 = 0; c0 < kv.second.size(); c0 += kMaxLuBatch) {
      Chunk ch;
      ch.P = P;
      ch.bg = (int)std::min<size_t>(kMaxLuBatch, kv.second.size() - c0);
      ch.mem.assign(kv.second.begin() + c0, kv.second.begin() + c0 + ch.bg);
      ch.store = std::make_shared<ClassStore>();
      cudaError_t e = cudaMallocAsync(&ch.store->z64, sizeof(double2) * nn * ch.bg, s);
      if (e == cudaSuccess) e = cudaMallocAsync(&ch.store->lu, elem * nn * ch.bg, s);
      if (e == cudaSuccess) e = cudaMallocAsync(reinterpret_cast<void**>(&ch.store->ipiv), sizeof(int) * (size_t)P * ch.bg, s);
      if (e != cudaSuccess) return fail(wmom_fail_cuda(e, "geometry batch storage"));
      ch.sets.assign(ch.bg, nullptr);
      ch.info.assign(ch.bg, 0);
      for (int j = 0; j < ch.bg; ++j) {
        wmom_factors_s* f = new (std::nothrow) wmom_factors_s();
        if (!f) return fail(WMOM_ERR_NOMEM);
        out[ch.mem[j]] = f;
        ch.sets[j] = f;
        e = lu_workspace_create_async(&f->ws, P, 1, kMaxLuBatch, s);
        if (e != cudaSuccess) return fail(wmom_fail_cuda(e, "factor workspace"));
        wmom_plan h = plans[ch.mem[j]];
        f->plan = h;
        f->shared = ch.store;
        f->fs.plan = &h->p;
        f->fs.mode = mode;
        f->fs.condest = condest;
        f->fs.freq.assign(1, freq_mhz[ch.mem[j]]);
        f->fs.ws = &f->ws;
        f->fs.batch = 1;
        const LuConfig shape = tuned_shape(P, mode);
        f->fs.span = shape.span;
        use_shape(&f->ws, shape);
        f->fs.order = P;
        f->fs.z64 = reinterpret_cast<double2*>(ch.store->z64) + (size_t)j * nn;
        f->fs.lu = reinterpret_cast<unsigned char*>(ch.store->lu) + elem * nn * j;
        f->fs.ipiv = ch.store->ipiv + (size_t)j * P;
        f->fs.info.assign(1, 0);
        f->bytes = nn * (sizeof(double2) + elem) + sizeof(int) * (size_t)P;
      }
      chunks.push_back(std::move(ch));
    }
  }
  cudaEvent_t start = nullptr;
  WMOM_CUDA_TRY(cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
  cudaError_t se = cudaEventRecord(start, s);  // the chunks' streams follow the caller's
  if (se != cudaSuccess) {
    cudaEventDestroy(start);
    return fail(wmom_fail_cuda(se, "cudaEventRecord"));
  }
  int dev = 0;
  cudaGetDevice(&dev);
  std::atomic<int> next{0};
  auto worker = [&]() {
    cudaSetDevice(dev);
    cudaStream_t cs = nullptr;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess || cudaStreamWaitEvent(cs, start, 0)) {
      for (int c; (c = next.fetch_add(1)) < (int)chunks.size();) chunks[c].st = WMOM_ERR_CUDA;
      if (cs) cudaStreamDestroy(cs);
      return;
    }
    for (int c; (c = next.fetch_add(1)) < (int)chunks.size();) {
      Chunk& ch = chunks[c];
      std::vector<const Plan*> ps(ch.bg);
      std::vector<float> fq(ch.bg);
      for (int j = 0; j < ch.bg; ++j) {
        ps[j] = &plans[ch.mem[j]]->p;
        fq[j] = freq_mhz[ch.mem[j]];
      }
      ch.st = factor_class(mode, ch.P, ps.data(), fq.data(), ch.bg, reinterpret_cast<double2*>(ch.store->z64),
                           ch.store->lu, ch.store->ipiv, ch.info.data(), &ch.sets[0]->ws, ch.sets[0]->fs.span, cs);
    }
    cudaStreamSynchronize(cs);
    cudaStreamDestroy(cs);
  };
  const int nthreads = std::min<int>((int)chunks.size(), 6);
  std::vector<std::thread> pool;
  for (int t = 1; t < nthreads; ++t) pool.emplace_back(worker);
  worker();
  for (auto& t : pool) t.join();
  cudaEventDestroy(start);
  for (Chunk& ch : chunks) {
    if (ch.st != WMOM_OK) return fail(ch.st);
    for (int j = 0; j < ch.bg; ++j) ch.sets[j]->fs.info[0] = ch.info[j];
  }
  return WMOM_OK;
}

}  // extern "C"
