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
