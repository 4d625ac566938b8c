// Device-side helpers shared by the stencil and reduction kernels:
// mbarrier + TMA (cp.async.bulk.tensor) wrappers written as inline PTX for
// sm_103a, bounded waits, and round-to-nearest arithmetic that the compiler
// may not contract into FMAs (so results match the REF target bit for bit).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "ps_arith.cuh"

namespace psg {

// Error bits written into the runtime's device error word.
enum : int {
  kDevErrWaitTimeout = 1,  // an mbarrier wait ran past its iteration limit
  kDevErrBadLaunch = 2,    // a kernel found inconsistent launch parameters
};

// Iteration limit for every spin-wait in this library.  One iteration is a
// try_wait (returns at once or after a short hardware window) plus a short
// sleep after the first few, so the limit bounds a wait to well under a
// second of wall time.
constexpr uint32_t kWaitLimit = 1u << 22;

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}

// Makes initialised mbarriers visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar,
                                                      uint32_t bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
          smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase with the given parity to complete.  Returns
// false (and sets kDevErrWaitTimeout in *err) if the limit runs out.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity,
                                          int *err, uint32_t limit = kWaitLimit) {
  for (uint32_t i = 0; i < limit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i >= 8) __nanosleep(64);
  }
  if (err) atomicOr(err, kDevErrWaitTimeout);
  return false;
}

// 3D tiled TMA load of box {w,h,1} at element coordinates (x,y,z) into
// shared memory, completing on `bar`.  x * sizeof(element) must be a
// multiple of 16 bytes (callers keep x a multiple of 16/sizeof(T)).
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map,
                                            int x, int y, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z),
      "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void prefetch_tmap(const CUtensorMap *map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map))
               : "memory");
}

// 16-byte vector of T held as VEC scalars.
template <typename T>
struct V16 {
  static constexpr int N = 16 / sizeof(T);
  T v[N];
};

template <typename T>
__device__ __forceinline__ void ld16_shared(T (&dst)[16 / sizeof(T)], const T *src) {
  uint4 u = *reinterpret_cast<const uint4 *>(src);
  union { uint4 u; T t[16 / sizeof(T)]; } cvt;
  cvt.u = u;
#pragma unroll
  for (int i = 0; i < (int)(16 / sizeof(T)); ++i) dst[i] = cvt.t[i];
}

template <typename T>
__device__ __forceinline__ void st16_global(T *dst, const T (&src)[16 / sizeof(T)]) {
  union { uint4 u; T t[16 / sizeof(T)]; } cvt;
#pragma unroll
  for (int i = 0; i < (int)(16 / sizeof(T)); ++i) cvt.t[i] = src[i];
  *reinterpret_cast<uint4 *>(dst) = cvt.u;
}

// v = *addr if pred, else v unchanged: a predicated shared load with no
// branch (the edge lanes of a warp fetch their halo cell this way).  The
// volatile asm stays after the mbarrier wait (also volatile asm) that made
// the data visible.
__device__ __forceinline__ void ld_shared_if(bool pred, const float *addr, float &v) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %1, 0;\n\t@p ld.shared.f32 %0, [%2];\n\t}"
      : "+f"(v)
      : "r"((unsigned)pred), "r"(smem_u32(addr)));
}
__device__ __forceinline__ void ld_shared_if(bool pred, const double *addr, double &v) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %1, 0;\n\t@p ld.shared.f64 %0, [%2];\n\t}"
      : "+d"(v)
      : "r"((unsigned)pred), "r"(smem_u32(addr)));
}
__device__ __forceinline__ void ld_shared_if(bool pred, const int *addr, int &v) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %1, 0;\n\t@p ld.shared.s32 %0, [%2];\n\t}"
      : "+r"(v)
      : "r"((unsigned)pred), "r"(smem_u32(addr)));
}
__device__ __forceinline__ void ld_shared_if(bool pred, const long long *addr, long long &v) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %1, 0;\n\t@p ld.shared.s64 %0, [%2];\n\t}"
      : "+l"(v)
      : "r"((unsigned)pred), "r"(smem_u32(addr)));
}

template <typename T>
__device__ __forceinline__ T shfl_up1(T v) { return __shfl_up_sync(0xffffffffu, v, 1); }
template <typename T>
__device__ __forceinline__ T shfl_down1(T v) { return __shfl_down_sync(0xffffffffu, v, 1); }

}  // namespace psg
