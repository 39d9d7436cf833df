// stats.h -- per-kernel-class launch counters and (optional) CUDA-event timing.
//
// Every kernel launch of the library is counted by class.  When timing is enabled
// (wmom_stats_enable), each launch is also bracketed by a pair of CUDA events
// recorded on the launching stream, so that the caller can read the device time
// of each class and its algorithmic work (flops or bytes, see each call site).
#pragma once

#include <cuda_runtime.h>

namespace wmom {
namespace stats {

enum Cls : int {
  kFill = 0,   // impedance-matrix fill (work: 384 flop-eq per entry)
  kPanel,      // cooperative panel factorisation (work: complex panel flops)
  kTcGemm,     // tcgen05 trailing update (work: 8*M*N*K real flops)
  kGemm,       // SIMT complex GEMM (trailing update / blocked solve; 8*M*N*K flops)
  kTrsm,       // triangular block solves
  kLaswp,      // row interchanges
  kResidual,   // FP64 residual GEMV (work: bytes of Z read)
  kMisc,       // conversions, norms, packing, permutations
  kEmulGemm,   // FP64-grade trailing update on the bf16 tensor cores (8*M*N*K real flops)
  kTrsv,       // triangular solves of one right-hand side per matrix (the refinement's)
  kNumCls
};

bool timing_enabled();
void count(Cls c, int launches = 1);
// Launch counters, for crediting the launches of a replayed CUDA graph.
void snapshot(long long out[kNumCls]);
void add_counts(const long long delta[kNumCls]);

// Brackets the launches issued in its lifetime on `s` with events (when enabled).
class Scope {
 public:
  Scope(Cls c, cudaStream_t s, double work, int launches = 1);
  ~Scope();
  Scope(const Scope&) = delete;
  Scope& operator=(const Scope&) = delete;

 private:
  Cls c_;
  cudaStream_t s_;
  double work_;
  cudaEvent_t e0_ = nullptr;
};

}  // namespace stats
}  // namespace wmom
