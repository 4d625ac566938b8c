// PSReduce over a whole pitched grid on GB300 (sm_103a).
//
// Replaces the reference's Thrust call (runtime/reduce_cuda.h:19-40,
// runtime/reduce_cuda.cu:14-40) and plays the role of its CUB block reduce
// (runtime/reduce_grid_mpi_cuda_exp.cu:177-330).  Semantics follow the REF
// target: every element of the grid, operators max/min/sum/prod
// (runtime/reduce.h:14-49).
//
// One pass: warps stride over x-rows; lanes read 16-byte vectors (a warp
// reads 512 contiguous bytes per load) and accumulate in the element type
// (FP32 for float grids; a float PS_PROD accumulates in FP64, because a long
// FP32 product loses about sqrt(n) ulps whatever the order), then warp
// shuffles and a shared-memory tree give one partial per CTA.  Each lane
// issues kLoadsInFlight vector loads of a row before it combines any of them,
// so every warp keeps 2 KiB in flight; four CTAs of 256 threads per SM then
// cover the HBM latency.  Partials are stored as 8-byte values (FP64 for
// float/double grids, 64-bit integers for int/long grids) and the last CTA to
// finish (atomic ticket) combines them in a fixed order, all 256 threads
// strided over the partials: FP64 for floating grids, wrapping integer
// arithmetic for integer grids (the REF fold wraps the same way).  The result
// is deterministic run to run.
#include <atomic>
#include <mutex>
#include <type_traits>

#include <cuda.h>

#include "physis_gb300/physis_gb300.h"
#include "ps_device.cuh"
#include "ps_internal.h"

namespace psg {
namespace {

constexpr int kReduceThreads = 256;
constexpr int kLoadsInFlight = 4;  // 16-byte loads per lane before combining
constexpr int kReduceCtasPerSm = 4;

template <typename T> struct RTraits;
template <> struct RTraits<float> {
  typedef float Acc;      // per-thread / per-CTA accumulation
  typedef double Comb;    // final combine
};
template <> struct RTraits<double> {
  typedef double Acc;
  typedef double Comb;
};
template <> struct RTraits<int> {
  typedef unsigned Acc;   // wraps modulo 2^32 for sum/prod
  typedef unsigned Comb;
};
template <> struct RTraits<long long> {
  typedef unsigned long long Acc;
  typedef unsigned long long Comb;
};

template <typename T, typename A>
__device__ __forceinline__ A identity(int op) {
  switch (op) {
    case kSum: return (A)0;
    case kProd: return (A)1;
  }
  return (A)0;  // min/max start from the first element seen (see below)
}

// Combine for floating accumulators (min/max by value).
template <typename A>
__device__ __forceinline__ A combine_f(int op, A a, A b) {
  switch (op) {
    case kMax: return (a > b) ? a : b;
    case kMin: return (a < b) ? a : b;
    case kSum: return RN<A>::add(a, b);
    default: return RN<A>::mul(a, b);
  }
}

// Integers: min/max compare as signed T, sum/prod wrap in unsigned A.
template <typename T, typename A>
__device__ __forceinline__ A combine_i(int op, A a, A b) {
  switch (op) {
    case kMax: return ((T)a > (T)b) ? a : b;
    case kMin: return ((T)a < (T)b) ? a : b;
    case kSum: return a + b;
    default: return a * b;
  }
}

template <typename T, typename A>
__device__ __forceinline__ A combine(int op, A a, A b) {
  if constexpr (std::is_integral<T>::value) {
    return combine_i<T, A>(op, a, b);
  } else {
    return combine_f<A>(op, a, b);
  }
}

// Integers keep their bit pattern in the unsigned accumulator.
template <typename T, typename A>
__device__ __forceinline__ A to_acc(T v) { return (A)v; }

template <typename A>
__device__ __forceinline__ A shfl_x(A v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }

template <typename T, typename A, typename C>
__global__ void __launch_bounds__(kReduceThreads)
reduce_kernel(const char *__restrict__ base, int64_t pitch, int nx, int ny, int nz,
              int op, uint64_t *partials, unsigned *ticket, uint64_t *result) {
  constexpr int VEC = 16 / (int)sizeof(T);
  constexpr int U = kLoadsInFlight;
  __shared__ A red[kReduceThreads / 32];
  __shared__ bool red_has[kReduceThreads / 32];
  __shared__ C redc[kReduceThreads / 32];
  __shared__ bool redc_has[kReduceThreads / 32];
  __shared__ int last_cta;

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t rows = (int64_t)ny * nz;
  const int64_t gw = (int64_t)blockIdx.x * (kReduceThreads / 32) + warp;
  const int64_t nw = (int64_t)gridDim.x * (kReduceThreads / 32);
  const int nvec = nx / VEC;
  const int tail = nx - nvec * VEC;

  // min/max have no identity that is exact for every type; track whether
  // this thread has seen an element instead.
  A acc = identity<T, A>(op);
  bool has = false;
  for (int64_t r = gw; r < rows; r += nw) {
    // Row r of plane r / ny starts at ((r / ny) * ny + r % ny) * pitch.
    const char *rp = base + r * pitch;
    const uint4 *vp = reinterpret_cast<const uint4 *>(rp);
    // A lane takes vectors lane, lane + 32, lane + 64, ... in that order.
    for (int v0 = 0; v0 < nvec; v0 += 32 * U) {
      uint4 u[U];
#pragma unroll
      for (int j = 0; j < U; ++j) {
        const int v = v0 + lane + 32 * j;
        u[j] = (v < nvec) ? __ldcs(vp + v) : make_uint4(0u, 0u, 0u, 0u);
      }
#pragma unroll
      for (int j = 0; j < U; ++j) {
        if (v0 + lane + 32 * j >= nvec) break;
        union { uint4 u; T t[VEC]; } cvt;
        cvt.u = u[j];
#pragma unroll
        for (int i = 0; i < VEC; ++i) {
          const A e = to_acc<T, A>(cvt.t[i]);
          acc = has ? combine<T, A>(op, acc, e)
                    : ((op == kSum || op == kProd) ? combine<T, A>(op, acc, e) : e);
          has = true;
        }
      }
    }
    if (lane < tail) {
      const A e = to_acc<T, A>(reinterpret_cast<const T *>(rp)[nvec * VEC + lane]);
      acc = has ? combine<T, A>(op, acc, e)
                : ((op == kSum || op == kProd) ? combine<T, A>(op, acc, e) : e);
      has = true;
    }
  }
  // warp tree
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const A other = shfl_x(acc, o);
    const bool ohas = __shfl_xor_sync(0xffffffffu, (int)has, o) != 0;
    if (ohas) acc = has ? combine<T, A>(op, acc, other) : other;
    has = has || ohas;
  }
  if (lane == 0) {
    red[warp] = acc;
    red_has[warp] = has;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    A b = identity<T, A>(op);
    bool bh = false;
    for (int w = 0; w < kReduceThreads / 32; ++w) {
      if (!red_has[w]) continue;
      b = bh ? combine<T, A>(op, b, red[w]) : red[w];
      bh = true;
    }
    // Partial as an 8-byte slot; an empty CTA stores the op's identity
    // (only possible for sum/prod shapes, min/max CTAs always see data
    // because the host sizes the grid to the row count).
    C cb = bh ? (C)b : (C)identity<T, A>(op);
    uint64_t bits = 0;
    if constexpr (sizeof(C) == 8) {
      bits = *reinterpret_cast<uint64_t *>(&cb);
    } else {
      bits = (uint64_t)(uint32_t)cb;
    }
    partials[blockIdx.x] = bits;
    __threadfence();
    const unsigned prev = atomicAdd(ticket, 1u);
    last_cta = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (last_cta) {  // uniform across the CTA (shared flag after the barrier)
    __threadfence();
    C v = (C)identity<T, A>(op);
    bool vh = false;
    for (unsigned i = threadIdx.x; i < gridDim.x; i += kReduceThreads) {
      const uint64_t bits = __ldcg(reinterpret_cast<const unsigned long long *>(partials) + i);
      C e;
      if constexpr (sizeof(C) == 8) {
        e = *reinterpret_cast<const C *>(&bits);
      } else {
        e = (C)(uint32_t)bits;
      }
      v = vh ? combine<T, C>(op, v, e) : e;
      vh = true;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const C other = shfl_x(v, o);
      const bool oh = __shfl_xor_sync(0xffffffffu, (int)vh, o) != 0;
      if (oh) v = vh ? combine<T, C>(op, v, other) : other;
      vh = vh || oh;
    }
    if (lane == 0) {
      redc[warp] = v;
      redc_has[warp] = vh;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      v = (C)identity<T, A>(op);
      vh = false;
      for (int w = 0; w < kReduceThreads / 32; ++w) {
        if (!redc_has[w]) continue;
        v = vh ? combine<T, C>(op, v, redc[w]) : redc[w];
        vh = true;
      }
      uint64_t bits;
      if constexpr (sizeof(C) == 8) {
        bits = *reinterpret_cast<uint64_t *>(&v);
      } else {
        bits = (uint64_t)(int64_t)(int32_t)v;  // int grids: sign-extend
      }
      *result = bits;
      *ticket = 0u;
    }
  }
}

// One CTA waiting on an mbarrier that nothing arrives at: the bounded wait
// gives up after `limit` tries and records kDevErrWaitTimeout.
__global__ void wait_timeout_probe_kernel(int *err, uint32_t limit) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_wait(&bar, 0, err, limit);
}

template <typename T, typename A = typename RTraits<T>::Acc,
          typename C = typename RTraits<T>::Comb>
cudaError_t launch_t(const GridView &g, int op, uint64_t *partials, int num_ctas,
                     unsigned *ticket, uint64_t *result, cudaStream_t s) {
  reduce_kernel<T, A, C><<<num_ctas, kReduceThreads, 0, s>>>(
      static_cast<const char *>(g.ptr), g.pitch, g.nx, g.ny, g.nz, op, partials,
      ticket, result);
  return cudaGetLastError();
}

}  // namespace

int reduce_num_ctas(const GridView &g, int sm_count) {
  const int64_t rows = (int64_t)g.ny * g.nz;
  const int64_t warps = kReduceThreads / 32;
  int64_t n = (rows + warps - 1) / warps;
  const int64_t cap = (int64_t)sm_count * kReduceCtasPerSm;
  if (n > cap) n = cap;
  if (n < 1) n = 1;
  return (int)n;
}

cudaError_t launch_reduce(const GridView &g, int op, uint64_t *partials,
                          int num_ctas, unsigned *ticket, uint64_t *result,
                          int *dev_err, cudaStream_t s) {
  (void)dev_err;
  if (op < kMax || op > kProd) return cudaErrorInvalidValue;
  switch (g.type) {
    case kFloat:
      if (op == kProd)
        return launch_t<float, double, double>(g, op, partials, num_ctas, ticket, result, s);
      return launch_t<float>(g, op, partials, num_ctas, ticket, result, s);
    case kDouble: return launch_t<double>(g, op, partials, num_ctas, ticket, result, s);
    case kInt: return launch_t<int>(g, op, partials, num_ctas, ticket, result, s);
    case kLong: return launch_t<long long>(g, op, partials, num_ctas, ticket, result, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_wait_timeout_probe(int *dev_err, uint32_t limit,
                                      cudaStream_t s) {
  wait_timeout_probe_kernel<<<1, 32, 0, s>>>(dev_err, limit);
  return cudaGetLastError();
}

// ---- PSReduceNoAlloc: the same reduction with statically placed scratch ----
//
// For callers that must not allocate device memory (see the declaration in
// physis_gb300.h).  The per-CTA partials and the last-CTA ticket live in this
// file-scope array instead of runtime-allocated buffers; it belongs to the
// loaded module, so every GPU that loads the library holds these 16 KiB
// until the process exits.  All calls share it: calls whose work overlaps on
// the GPU (other streams, or the same array from another host thread) race.
constexpr int kNoAllocMaxPartials = 2048;
static __device__ __align__(256) uint64_t g_noalloc_scratch[kNoAllocMaxPartials + 2];

namespace {

// Device address of g_noalloc_scratch and the SM count, per device ordinal,
// for the CUDA context that was current when they were looked up.  A device
// reset destroys that context and the module with it; the array may then
// sit elsewhere, so the entry is keyed by the context's process-unique id
// (cuCtxGetId) and looked up again when the current context differs.
struct NoAllocDevice {
  std::atomic<unsigned long long> ctx_id{0};  // 0: not set up
  uint64_t *scratch = nullptr;
  int sm_count = 0;
};
constexpr int kNoAllocMaxDevices = 64;
NoAllocDevice g_noalloc_dev[kNoAllocMaxDevices];
std::mutex g_noalloc_setup;  // first calls from several host threads

// The current context's id through the driver entry points the runtime
// exposes (the library does not link libcuda).  0 when unavailable.
unsigned long long current_context_id() {
  typedef CUresult (*GetCurrent)(CUcontext *);
  typedef CUresult (*GetId)(CUcontext, unsigned long long *);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(fn);
    fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(fn);
    cudaGetLastError();
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx ||
      get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

}  // namespace

int reduce_noalloc(const void *data, size_t pitch, int nx, int ny, int nz, int type,
                   int op, void *result, cudaStream_t stream, const char **why) {
  // Arguments first: these checks need no GPU.
  const int esz = (type == kFloat || type == kInt) ? 4 : (type == kDouble || type == kLong) ? 8 : 0;
  if (!esz) { *why = "unknown element type"; return PS_ERR_INVALID_ARGUMENT; }
  if (op < kMax || op > kProd) { *why = "unknown reduction op"; return PS_ERR_INVALID_ARGUMENT; }
  if (!data || !result) { *why = "NULL data or result pointer"; return PS_ERR_INVALID_ARGUMENT; }
  if (nx <= 0 || ny <= 0 || nz <= 0) { *why = "grid sizes must be positive"; return PS_ERR_INVALID_ARGUMENT; }
  if (pitch < (size_t)nx * esz || pitch % 16 != 0) {
    *why = "pitch must cover a row and be a multiple of 16 bytes";
    return PS_ERR_INVALID_ARGUMENT;
  }
  if ((reinterpret_cast<uintptr_t>(data) & 15u) != 0 ||
      (reinterpret_cast<uintptr_t>(result) & 7u) != 0) {
    *why = "data must be 16-byte and result 8-byte aligned";
    return PS_ERR_INVALID_ARGUMENT;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) {
    cudaGetLastError();
    *why = "no usable current CUDA device";
    return PS_ERR_NO_DEVICE;
  }
  NoAllocDevice &d = g_noalloc_dev[dev];
  unsigned long long ctx = current_context_id();
  if (ctx == 0 || d.ctx_id.load(std::memory_order_acquire) != ctx) {
    std::lock_guard<std::mutex> lock(g_noalloc_setup);
    // Set-up with the device current: the host-side name g_noalloc_scratch
    // is not a device address, so look the address up.  This also loads
    // the module into the context, and creates the primary context if none
    // exists yet (so the id is read again afterwards).
    uint64_t *ptr = nullptr;
    if (cudaGetSymbolAddress(reinterpret_cast<void **>(&ptr), g_noalloc_scratch) !=
        cudaSuccess) {
      cudaGetLastError();
      *why = "cudaGetSymbolAddress failed for the static scratch array";
      return PS_ERR_CUDA;
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
      cudaGetLastError();
      *why = "cannot query the SM count";
      return PS_ERR_CUDA;
    }
    d.scratch = ptr;
    d.sm_count = sms;
    // Without a context id (driver entry points unavailable) the lookup is
    // simply repeated on every call.
    d.ctx_id.store(current_context_id(), std::memory_order_release);
  }
  GridView g;
  g.ptr = const_cast<void *>(data);
  g.pitch = (int64_t)pitch;
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.type = type;
  g.esz = esz;
  // Same CTA count as the allocating entry point, so both give the same bits.
  const int n = reduce_num_ctas(g, d.sm_count);
  if (n > kNoAllocMaxPartials) {
    *why = "the launch needs more per-CTA partial slots than the static scratch holds (2048)";
    return PS_ERR_UNSUPPORTED;
  }
  uint64_t *partials = d.scratch;
  unsigned *ticket = reinterpret_cast<unsigned *>(d.scratch + kNoAllocMaxPartials);
  // The ticket must start at zero; an interrupted earlier call could have
  // left it set.  cudaMemsetAsync allocates nothing.
  if (cudaMemsetAsync(ticket, 0, sizeof(unsigned), stream) != cudaSuccess) {
    cudaGetLastError();
    *why = "cudaMemsetAsync of the ticket failed";
    return PS_ERR_CUDA;
  }
  cudaError_t e = launch_reduce(g, op, partials, n, ticket, static_cast<uint64_t *>(result),
                                nullptr, stream);
  if (e != cudaSuccess) {
    *why = cudaGetErrorString(e);
    return PS_ERR_CUDA;
  }
  return PS_OK;
}

}  // namespace psg
