// lu_common.cuh -- complex arithmetic and the bounded grid barrier shared by the
// LU kernels (FP64 plain form and FP32 precision form).
#pragma once

#include <cuda_runtime.h>

namespace wmom {

template <typename R>
struct CplxOf;
template <>
struct CplxOf<double> {
  using type = double2;
};
template <>
struct CplxOf<float> {
  using type = float2;
};

template <typename C>
__device__ __forceinline__ C cmake(decltype(C{}.x) r, decltype(C{}.x) i) {
  C z;
  z.x = r;
  z.y = i;
  return z;
}
template <typename C>
__device__ __forceinline__ C cadd(C a, C b) {
  return cmake<C>(a.x + b.x, a.y + b.y);
}
template <typename C>
__device__ __forceinline__ C csub(C a, C b) {
  return cmake<C>(a.x - b.x, a.y - b.y);
}
template <typename C>
__device__ __forceinline__ C cmul(C a, C b) {
  return cmake<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// c - a*b
template <typename C>
__device__ __forceinline__ C cfms(C c, C a, C b) {
  C r;
  r.x = fma(-a.y, -b.y, fma(-a.x, b.x, c.x));
  r.y = fma(-a.y, b.x, fma(-a.x, b.y, c.y));
  return r;
}
template <typename C>
__device__ __forceinline__ decltype(C{}.x) cabs1(C a) {
  return fabs(a.x) + fabs(a.y);
}
// 1/a by Smith's scaled formula.
template <typename C>
__device__ __forceinline__ C crecip(C a) {
  using R = decltype(C{}.x);
  if (fabs(a.x) >= fabs(a.y)) {
    R r = a.y / a.x;
    R d = a.x + a.y * r;
    return cmake<C>(R(1) / d, -r / d);
  } else {
    R r = a.x / a.y;
    R d = a.y + a.x * r;
    return cmake<C>(r / d, R(-1) / d);
  }
}
// a/b by Smith's scaled formula.
template <typename C>
__device__ __forceinline__ C cdiv(C a, C b) {
  using R = decltype(C{}.x);
  if (fabs(b.x) >= fabs(b.y)) {
    R r = b.y / b.x;
    R d = b.x + b.y * r;
    return cmake<C>((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  } else {
    R r = b.x / b.y;
    R d = b.y + b.x * r;
    return cmake<C>((a.x * r + a.y) / d, (a.y * r - a.x) / d);
  }
}

// State of a software grid barrier for one cooperative launch.  `gen` only ever
// increases; `count` is reset by the last arriving block.  Waits are bounded: a
// block that waits longer than kBarrierTimeoutNs records an error and every block
// leaves the kernel at its next barrier (no trap, no unbounded spin).
struct GridBarrier {
  unsigned int count;
  unsigned int gen;
  int err;     // 1 = a wait timed out
  int info;    // first exactly-zero pivot (1-based global column), 0 if none
};

constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;  // 2 s

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_volatile_i32(const int* p) {
  return *reinterpret_cast<const volatile int*>(p);
}

// Counting barrier: the counter only grows, so arriving is one release reduction and
// waiting is polling the counter with acquire loads until it reaches `target` (= the
// caller's running total of arrivals expected so far).  The acquire that reads the
// final count synchronises with every block's release, and the closing
// __syncthreads passes that on to the rest of the block.  The error word and the
// clock are looked at every 64 polls only, so a poll is one L2 round trip.  Returns
// false on timeout, or when another block has recorded one.
__device__ __forceinline__ bool grid_barrier_count(GridBarrier* gb, unsigned int target) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    // arrive, ordered after the block's writes (which __syncthreads ordered before
    // this thread's release)
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(&gb->count) : "memory");
    if (ld_acquire_u32(&gb->count) < target) {
      const unsigned long long t0 = global_ns();
      unsigned int polls = 0;
      while (ld_acquire_u32(&gb->count) < target) {
        if ((++polls & 63u) == 0) {
          if (ld_volatile_i32(&gb->err)) {
            ok = 0;
            break;
          }
          if (global_ns() - t0 > kBarrierTimeoutNs) {
            atomicExch(&gb->err, 1);
            ok = 0;
            break;
          }
        }
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Returns false when the barrier timed out (here or in another block).
__device__ __forceinline__ bool grid_barrier(GridBarrier* gb, unsigned int nblocks,
                                             unsigned int* gen_local) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned int g = *gen_local;
    __threadfence();
    const unsigned int prev = atomicAdd(&gb->count, 1u);
    if (prev == nblocks - 1) {
      atomicExch(&gb->count, 0u);
      __threadfence();
      atomicExch(&gb->gen, g + 1u);
    } else {
      const unsigned long long t0 = global_ns();
      while (ld_acquire_u32(&gb->gen) == g) {
        if (ld_volatile_i32(&gb->err)) break;
        if (global_ns() - t0 > kBarrierTimeoutNs) {
          atomicExch(&gb->err, 1);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    if (ld_volatile_i32(&gb->err)) ok = 0;
    *gen_local = g + 1u;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

}  // namespace wmom
