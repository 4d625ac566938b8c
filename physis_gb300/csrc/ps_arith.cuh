// Device helpers with no header dependencies, shared by the kernels built
// with nvcc and the kernels compiled at run time by NVRTC (which sees this
// file as an in-memory header): shared-memory addresses, round-to-nearest
// arithmetic that is never contracted into an FMA (so results match the REF
// target bit for bit), and cp.async copies.
#pragma once

namespace psg {

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// Round-to-nearest arithmetic that is never fused into an FMA.
template <typename T>
struct RN {
  static __device__ __forceinline__ T add(T a, T b) { return a + b; }
  static __device__ __forceinline__ T sub(T a, T b) { return a - b; }
  static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
};
template <>
struct RN<float> {
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
};
template <>
struct RN<double> {
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
};
// Integer grids wrap modulo 2^32 / 2^64 like the REF target's C arithmetic
// on two's-complement hosts; compute in unsigned to keep that defined.
template <>
struct RN<int> {
  static __device__ __forceinline__ int add(int a, int b) { return (int)((unsigned)a + (unsigned)b); }
  static __device__ __forceinline__ int sub(int a, int b) { return (int)((unsigned)a - (unsigned)b); }
  static __device__ __forceinline__ int mul(int a, int b) { return (int)((unsigned)a * (unsigned)b); }
};
template <>
struct RN<long long> {
  typedef unsigned long long U;
  static __device__ __forceinline__ long long add(long long a, long long b) { return (long long)((U)a + (U)b); }
  static __device__ __forceinline__ long long sub(long long a, long long b) { return (long long)((U)a - (U)b); }
  static __device__ __forceinline__ long long mul(long long a, long long b) { return (long long)((U)a * (U)b); }
};

// cp.async (global -> shared, asynchronous, completion per commit group).
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)),
               "l"(__cvta_generic_to_global(src))
               : "memory");
}
template <int B>
__device__ __forceinline__ void cp_async_small(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_u32(dst)),
               "l"(__cvta_generic_to_global(src)), "n"(B)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

}  // namespace psg
