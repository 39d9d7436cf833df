// noalloc.cu -- an FP64 LU entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host application that hands this library
// device buffers from its own memory pool and forbids any other allocation on the
// device, or a serving process that must not take cudaMalloc's implicit device-wide
// synchronisation (or risk an out-of-memory failure) once it is running.
// wmom_zgetrf_noalloc gives them the FP64 LU of wmom_zgetrf with the factorisation's
// scratch -- the panel kernel's grid-barrier word and its candidate-row staging --
// held in a file-scope __device__ array of fixed size instead of cudaMalloc'd memory.
// The caller still owns the matrix and pivot buffers.
//
// The array is part of the library's device image: every GPU that loads the library
// keeps it (kScratchBytes) until the process exits.  Every call shares it, so calls
// whose work overlaps on the GPU (different streams, different host threads) race on
// it and must be serialised by the caller.  It keeps the last call's contents; the
// parts that must start at zero (the barrier word, error flag and pivot info) are
// cleared by each call with cudaMemsetAsync on the caller's stream.
//
// Host code cannot pass the array's name to a kernel (in host code it names a
// host-side stand-in), so every call asks the runtime for its device address on the
// current device with cudaGetSymbolAddress, which allocates nothing.  Asking on every
// call rather than once keeps the address right after a cudaDeviceReset, which may
// reload the library's device image at another address.
#include <cuda_runtime.h>

#include <cstdio>

#include "lu_common.cuh"
#include "lu_internal.h"
#include "wmom_internal.h"

namespace wmom {
namespace {

// 576 KiB: the barrier header (256 B) plus the FP64 panel kernel's double-buffered
// candidate staging for up to kMaxPanelBlocks blocks (about 520 KiB).
constexpr size_t kScratchBytes = 576 * 1024;

static __device__ __align__(256) unsigned char g_lu_scratch[kScratchBytes];

}  // namespace
}  // namespace wmom

using namespace wmom;

extern "C" wmom_status wmom_zgetrf_noalloc(int n, void* a_dev, long long lda, int* ipiv_dev, int* info,
                                           void* stream) {
  if (info) *info = 0;
  if (n <= 0 || !a_dev || lda < n || !ipiv_dev) return WMOM_ERR_ARG;
  if (n > WMOM_NOALLOC_MAX_N) {
    std::fprintf(stderr, "wmom_zgetrf_noalloc: n = %d exceeds WMOM_NOALLOC_MAX_N = %d\n", n, WMOM_NOALLOC_MAX_N);
    return WMOM_ERR_ARG;
  }
  if (lu_workspace_bytes(16) > kScratchBytes) return WMOM_ERR_UNSUPPORTED;
  // the array's device address on the current device (see the file comment)
  void* scratch = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&scratch, g_lu_scratch);
  if (e != cudaSuccess) return wmom_fail_cuda(e, "cudaGetSymbolAddress(g_lu_scratch)");
  cudaStream_t s = (cudaStream_t)stream;
  LuWorkspace ws{};
  ws.barrier = reinterpret_cast<GridBarrier*>(scratch);
  ws.stage = reinterpret_cast<unsigned char*>(scratch) + 256;
  // the barrier counters, error flag and pivot info must start at zero
  e = cudaMemsetAsync(ws.barrier, 0, sizeof(GridBarrier), s);
  if (e != cudaSuccess) return wmom_fail_cuda(e, "cudaMemsetAsync(scratch)");
  e = lu_factor_t<double2>(reinterpret_cast<double2*>(a_dev), lda, n, ipiv_dev, &ws, s, nullptr);
  if (e != cudaSuccess) return wmom_fail_cuda(e, "lu_factor (no-alloc)");
  GridBarrier h{};
  e = cudaMemcpyAsync(&h, ws.barrier, sizeof(GridBarrier), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return wmom_fail_cuda(e, "zgetrf_noalloc status");
  if (info) *info = h.info;
  if (h.err) return WMOM_ERR_TIMEOUT;
  return h.info ? WMOM_ERR_SINGULAR : WMOM_OK;
}
