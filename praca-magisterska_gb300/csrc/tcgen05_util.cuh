// tcgen05_util.cuh -- inline-PTX helpers shared by the tensor-core trailing updates
// (lu_tc.cu: complex FP32 via 3xTF32; lu_emul.cu: complex FP64 via bf16 slices):
// mbarriers, TMA tiled loads, shared-memory matrix descriptors, MMA commits and the
// bounded waits every role of those kernels uses.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "lu_common.cuh"
#include "lu_internal.h"

namespace wmom {
namespace tc {

// Host side (lu_tc.cu): the driver's tensor-map encoder, and the growth of a
// workspace's operand scratch (ws->tc_buf, in floats; refused inside a capture).
using EncodeFn = PFN_cuTensorMapEncodeTiled_v12000;
EncodeFn encode_fn();
cudaError_t tc_scratch(LuWorkspace* ws, size_t floats, cudaStream_t s);

constexpr unsigned long long kWaitNs = 1000000000ull;  // 1 s per wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred P1;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, P1;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// 3-D tiled TMA load (x = K element, y = row, z = matrix of the batch).
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

// 4-D tiled TMA load (x = K element, y = row, z = matrix of the batch, w = plane).
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int x, int y, int z, int w,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor of a K-major operand tile whose rows are
// `row_bytes` long (128 or 64) and swizzled over that length: 8-row groups
// 8 * row_bytes apart (stride byte offset), descriptor version 1, layout type
// 2 (128-byte swizzle) or 4 (64-byte swizzle).
template <int ROW_BYTES>
__device__ __forceinline__ uint64_t sdesc_sw(uint32_t addr) {
  static_assert(ROW_BYTES == 128 || ROW_BYTES == 64, "swizzle width");
  constexpr uint64_t layout = ROW_BYTES == 128 ? 2 : 4;
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(16u >> 4) << 16;
  d |= (uint64_t)((8u * ROW_BYTES) >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= layout << 61;
  return d;
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

// Bounded wait that also ends when this CTA has failed (s_fail) or, through err,
// another CTA of the launch.
__device__ __forceinline__ bool role_wait(uint32_t bar, uint32_t parity, const int* err, const volatile int* s_fail) {
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (*s_fail || *reinterpret_cast<const volatile int*>(err)) return false;
    if (global_ns() - t0 > kWaitNs) return false;
  }
  return true;
}

}  // namespace tc
}  // namespace wmom
