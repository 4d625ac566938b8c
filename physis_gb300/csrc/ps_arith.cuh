// Device helpers with no header dependencies, shared by the kernels built
// with nvcc and the kernels compiled at run time by NVRTC (which sees this
// file as an in-memory header): shared-memory addresses, round-to-nearest
// arithmetic that is never contracted into an FMA (so results match the REF
// target bit for bit), bounded mbarrier waits, TMA box loads and cp.async
// copies, all as inline PTX for sm_103a.
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
  // a * b + c rounded once (kernels that may contract)
  static __device__ __forceinline__ float fma(float a, float b, float c) {
    return __fmaf_rn(a, b, c);
  }
};
template <>
struct RN<double> {
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double fma(double a, double b, double c) {
    return __fma_rn(a, b, c);
  }
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

// Error bits written into the runtime's device error word.
enum : int {
  kDevErrWaitTimeout = 1,  // an mbarrier wait ran past its iteration limit
  kDevErrBadLaunch = 2,    // a kernel found inconsistent launch parameters
};

// Iteration limit for every spin-wait in this library.  One iteration is a
// try_wait (returns at once or after a short hardware window) plus a short
// sleep after the first few, so the limit bounds a wait to well under a
// second of wall time.
constexpr unsigned kWaitLimit = 1u << 22;

__device__ __forceinline__ void mbar_init(void *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}

// Makes initialised mbarriers visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(void *bar,
                                                      unsigned bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
          smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(void *bar, unsigned parity) {
  unsigned ok;
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
__device__ __forceinline__ bool mbar_wait(void *bar, unsigned parity,
                                          int *err, unsigned limit = kWaitLimit) {
  for (unsigned i = 0; i < limit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i >= 8) __nanosleep(64);
  }
  if (err) atomicOr(err, kDevErrWaitTimeout);
  return false;
}

// 3D tiled TMA load of box {w,h,1} at element coordinates (x,y,z) into
// shared memory, completing on `bar`.  x * sizeof(element) must be a
// multiple of 16 bytes (callers keep x a multiple of 16/sizeof(T)).
__device__ __forceinline__ void tma_load_3d(void *dst, const void *map,
                                            int x, int y, int z, void *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z),
      "r"(smem_u32(bar))
      : "memory");
}

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
