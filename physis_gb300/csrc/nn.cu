// Kernels of the learned warm start for the 19-point Jacobi (Himeno) solve:
// a 3D convolutional network of 3x3x3 layers with 16 channels, BF16 weights
// and activations, FP32 accumulation, trained on the GPU.  No counterpart in
// the reference.
//
// Tensors are channels-last, [batch, z, y, x, 16] BF16 (16 channels: 32
// bytes per voxel).  A convolution is an implicit GEMM per tap: rows are
// voxels, K the 16 input channels, N the 16 output channels.  Tensor cores
// via mma.sync.m16n8k16 (BF16 in, FP32 accumulate): each warp owns 16
// voxels and accumulates 27 taps x 2 n-tiles; the layer's weights sit in
// shared memory in the fragment-friendly [tap][out][in] order.  The
// backward-data pass is the same kernel with the weights flipped in space
// and transposed in channels; the weight gradient is a K = voxels GEMM per
// tap, split over CTAs and reduced in a fixed order (deterministic).
// Pooling (fine grids -> coarse network input), the MSE gradient, Adam and
// cubic upsampling (coarse prediction -> fine warm start) complete the
// set.  Every kernel is checked against oracle/nn_oracle.py.
#include <cuda_bf16.h>
#include <stdlib.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "ps_arith.cuh"
#include "ps_internal.h"

namespace psg {
namespace {

int *g_err = nullptr;  // the runtime's device error word (bounded waits)

constexpr int kC = 16;       // channels
constexpr int kTaps = 27;
constexpr int kPoolChannels = 9;  // network input channels in use
constexpr int kConvWarps = 8;

__device__ __forceinline__ void mma_16816(float (&d)[4], const uint32_t (&a)[4],
                                          uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

struct Dims {
  int B, Z, Y, X;
  long long nvox;
};

// Voxel coordinates of flattened index v (x fastest).
struct Vox {
  int b, z, y, x;
  bool ok;
};
__device__ __forceinline__ Vox vox_of(long long v, const Dims &d) {
  Vox r;
  r.ok = v < d.nvox;
  if (!r.ok) v = 0;
  r.x = (int)(v % d.X);
  long long t = v / d.X;
  r.y = (int)(t % d.Y);
  t /= d.Y;
  r.z = (int)(t % d.Z);
  r.b = (int)(t / d.Z);
  return r;
}

// Flattened index of the neighbour of `p` at tap t, or -1 outside.
__device__ __forceinline__ long long nbr(const Vox &p, int t, const Dims &d) {
  const int dz = t / 9 - 1, dy = (t / 3) % 3 - 1, dx = t % 3 - 1;
  const int z = p.z + dz, y = p.y + dy, x = p.x + dx;
  if (!p.ok || z < 0 || z >= d.Z || y < 0 || y >= d.Y || x < 0 || x >= d.X) return -1;
  return (((long long)p.b * d.Z + z) * d.Y + y) * d.X + x;
}

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16 *base, long long v, int c) {
  return v < 0 ? 0u : *reinterpret_cast<const uint32_t *>(base + v * kC + c);
}
__device__ __forceinline__ uint32_t pack2(const __nv_bfloat16 *base, long long v0, long long v1,
                                          int c) {
  const uint16_t lo = v0 < 0 ? 0 : reinterpret_cast<const uint16_t *>(base)[v0 * kC + c];
  const uint16_t hi = v1 < 0 ? 0 : reinterpret_cast<const uint16_t *>(base)[v1 * kC + c];
  return (uint32_t)lo | ((uint32_t)hi << 16);
}

// Y = epilogue(conv(X, W) + bias): relu, or times (mask > 0).  W is
// [27][out][in] BF16.  yf (optional) receives channel 0 in FP32.
__global__ void __launch_bounds__(32 * kConvWarps)
conv_kernel(const __nv_bfloat16 *__restrict__ x, const __nv_bfloat16 *__restrict__ w,
            const float *__restrict__ bias, const __nv_bfloat16 *__restrict__ mask,
            int relu, __nv_bfloat16 *__restrict__ y, float *__restrict__ yf, Dims d) {
  __shared__ __align__(16) __nv_bfloat16 ws[kTaps * kC * kC];
  for (int i = threadIdx.x; i < kTaps * kC * kC / 8; i += blockDim.x)
    reinterpret_cast<uint4 *>(ws)[i] = reinterpret_cast<const uint4 *>(w)[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, q = lane & 3;
  const long long v0 = ((long long)blockIdx.x * kConvWarps + warp) * 16;
  if (v0 >= d.nvox) return;
  const Vox pa = vox_of(v0 + g, d), pb = vox_of(v0 + g + 8, d);
  float acc0[4] = {0.f, 0.f, 0.f, 0.f}, acc1[4] = {0.f, 0.f, 0.f, 0.f};
  for (int t = 0; t < kTaps; ++t) {
    const long long na = nbr(pa, t, d), nb = nbr(pb, t, d);
    const uint32_t a[4] = {ld_pair(x, na, 2 * q), ld_pair(x, nb, 2 * q),
                           ld_pair(x, na, 2 * q + 8), ld_pair(x, nb, 2 * q + 8)};
    const uint32_t *wt = reinterpret_cast<const uint32_t *>(ws + t * kC * kC);
    // B (k = in, n = out) from ws[t][out][in]: two consecutive in-channels
    mma_16816(acc0, a, wt[(g * kC + 2 * q) / 2], wt[(g * kC + 2 * q + 8) / 2]);
    mma_16816(acc1, a, wt[((g + 8) * kC + 2 * q) / 2], wt[((g + 8) * kC + 2 * q + 8) / 2]);
  }
  // C: c0,c1 -> (voxel g, out 2q, 2q+1); c2,c3 -> (voxel g+8, ...)
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    const Vox &p = half ? pb : pa;
    if (!p.ok) continue;
    const long long v = v0 + g + 8 * half;
#pragma unroll
    for (int tile = 0; tile < 2; ++tile) {
      const float *acc = tile ? acc1 : acc0;
      const int co = 2 * q + 8 * tile;
      float r0 = acc[2 * half], r1 = acc[2 * half + 1];
      if (bias) {
        r0 += bias[co];
        r1 += bias[co + 1];
      }
      if (relu) {
        r0 = fmaxf(r0, 0.f);
        r1 = fmaxf(r1, 0.f);
      }
      if (mask) {
        const __nv_bfloat162 m = *reinterpret_cast<const __nv_bfloat162 *>(mask + v * kC + co);
        if (!(__bfloat162float(m.x) > 0.f)) r0 = 0.f;
        if (!(__bfloat162float(m.y) > 0.f)) r1 = 0.f;
      }
      *reinterpret_cast<__nv_bfloat162 *>(y + v * kC + co) = __floats2bfloat162_rn(r0, r1);
      if (yf && co == 0) yf[v] = r0;
    }
  }
}

// ---- tcgen05 implicit GEMM -------------------------------------------------
//
// One CTA: M = 128 consecutive voxels, N = 16 output channels, K = 27 taps x
// 16 input channels, in three phases of 9 taps (one z offset each).  Per
// phase all 256 threads gather the 9 A tiles (each voxel's neighbour row of
// 16 BF16 channels, zero outside) into shared memory in the canonical
// no-swizzle K-major layout of 8-row x 16-byte core matrices (K-adjacent core
// matrices 128 B apart, M-adjacent ones 256 B apart); one thread issues the 9
// tcgen05.mma (kind::f16, BF16 x BF16 -> FP32 in tensor memory) and commits
// them to an mbarrier; everyone waits (bounded) before the buffer is reused.
// The 27 B tiles (the layer's [tap][out][in] weights) are staged once.  After
// the last phase warps 0-3 and 4-7 read columns 0-7 and 8-15 of the 128 x 16
// accumulator with tcgen05.ld and apply the epilogue.  52 KB of shared
// memory: 4 CTAs per SM.  Tensor memory (32 columns) is allocated and freed
// by warp 0 on every path.
constexpr int kTcM = 128;
constexpr int kTcThreads = 256;
constexpr int kTcPhaseTaps = 9;
constexpr int kTcATile = kTcM * kC * 2;   // 4096 B per tap
constexpr int kTcBTile = kC * kC * 2;     // 512 B per tap
constexpr size_t kTcSmem = 1024 + (size_t)kTcPhaseTaps * kTcATile + (size_t)kTaps * kTcBTile + 64;

// Shared-memory matrix descriptor: start, leading (K) and stride (M/N) byte
// offsets >> 4, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor: FP32 accumulate, BF16 A and B, both K-major,
// N = 16, M = 128.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kC >> 3) << 17) |
                              ((uint32_t)(kTcM >> 4) << 24);

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__global__ void __launch_bounds__(kTcThreads, 4)
conv_tc_kernel(const __nv_bfloat16 *__restrict__ x, const __nv_bfloat16 *__restrict__ w,
               const float *__restrict__ bias, const __nv_bfloat16 *__restrict__ mask, int relu,
               __nv_bfloat16 *__restrict__ y, float *__restrict__ yf, Dims d, int *err) {
  extern __shared__ __align__(1024) unsigned char tc_raw[];
  unsigned char *smem = tc_raw + ((1024u - (smem_u32(tc_raw) & 1023u)) & 1023u);
  unsigned char *sa = smem;
  unsigned char *sb = sa + kTcPhaseTaps * kTcATile;
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(sb + kTaps * kTcBTile);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long v0 = (long long)blockIdx.x * kTcM;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(
                     smem_u32(tslot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_barrier_init();
  }
  // B tiles: row n (out channel) of 16 in-channels = two 16-byte halves
  for (int i = tid; i < kTaps * kC * 2; i += kTcThreads) {
    const int t = i / (kC * 2), n = (i / 2) % kC, c = i & 1;
    const uint4 v = *reinterpret_cast<const uint4 *>(w + (t * kC + n) * kC + c * 8);
    *reinterpret_cast<uint4 *>(sb + t * kTcBTile + (n >> 3) * 256 + c * 128 + (n & 7) * 16) = v;
  }
  // this thread's A row (voxel m, 16-byte half c) and its neighbour bounds
  const int m = tid & (kTcM - 1), c = tid >> 7;
  const Vox p = vox_of(v0 + m, d);
  const long long vm = v0 + m;
  const long long YX = (long long)d.Y * d.X;
  const bool ylo = p.y > 0, yhi = p.y < d.Y - 1, xlo = p.x > 0, xhi = p.x < d.X - 1;
  unsigned char *dst = sa + (m >> 3) * 256 + c * 128 + (m & 7) * 16;
  const __nv_bfloat16 *src = x + vm * kC + c * 8;

  bool ok = true;
  uint32_t tmem = 0;
  for (int g = 0; g < 3; ++g) {
    const int dz = g - 1;
    const bool zok = p.ok && (dz < 0 ? p.z > 0 : (dz > 0 ? p.z < d.Z - 1 : true));
#pragma unroll
    for (int k = 0; k < kTcPhaseTaps; ++k) {
      const int dy = k / 3 - 1, dx = k % 3 - 1;
      const bool in = zok && (dy < 0 ? ylo : (dy > 0 ? yhi : true)) &&
                      (dx < 0 ? xlo : (dx > 0 ? xhi : true));
      uint4 v = make_uint4(0, 0, 0, 0);
      if (in) v = *reinterpret_cast<const uint4 *>(src + (dz * YX + dy * d.X + dx) * kC);
      *reinterpret_cast<uint4 *>(dst + k * kTcATile) = v;
    }
    // make the generic-proxy writes visible to the tensor core (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    tmem = *tslot;
    if (tid == 0) {
      const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
      for (int k = 0; k < kTcPhaseTaps; ++k) {
        const int t = g * kTcPhaseTaps + k;
        const uint64_t ad = umma_desc(a0 + k * kTcATile, 128, 256);
        const uint64_t bd = umma_desc(b0 + t * kTcBTile, 128, 256);
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(kTcIdesc), "r"((uint32_t)(t > 0))
            : "memory");
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(bar))
          : "memory");
    }
    // the A buffer is reused by the next phase only after these MMAs are done
    if (!mbar_wait(bar, (uint32_t)(g & 1), err)) ok = false;
    tc_fence_after();
  }
  // epilogue: warp quadrant q = rows 32q..32q+31, column half h
  {
    const int q = warp & 3, h = warp >> 2;
    uint32_t r[8];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7])
        : "r"(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(8 * h)));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    const long long v = v0 + 32 * q + lane;
    if (ok && v < d.nvox) {
      float f[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int co = 8 * h + i;
        float a = __uint_as_float(r[i]);
        if (bias) a += bias[co];
        if (relu) a = fmaxf(a, 0.f);
        if (mask && !(__bfloat162float(mask[v * kC + co]) > 0.f)) a = 0.f;
        f[i] = a;
      }
      uint4 o;
      __nv_bfloat162 *ob = reinterpret_cast<__nv_bfloat162 *>(&o);
#pragma unroll
      for (int i = 0; i < 4; ++i) ob[i] = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
      *reinterpret_cast<uint4 *>(y + v * kC + 8 * h) = o;
      if (yf && h == 0) yf[v] = f[0];
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(tmem)
                 : "memory");
  }
}

// Partial weight gradients: block (t, s) sums over the s-th share of the
// 16-voxel chunks dW[t][in][out] = sum_v X[v + d_t][in] * dY[v][out] into
// part[s][t][in][out]; blocks of the centre tap also sum dY into
// bpart[s][out] (the bias gradient).
__global__ void __launch_bounds__(32 * kConvWarps)
wgrad_kernel(const __nv_bfloat16 *__restrict__ x, const __nv_bfloat16 *__restrict__ dy,
             float *__restrict__ part, float *__restrict__ bpart, Dims d) {
  __shared__ float red[kConvWarps][kC * kC];
  __shared__ float bred[kConvWarps][kC];
  const int t = blockIdx.x, s = blockIdx.y, S = gridDim.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, q = lane & 3;
  float acc0[4] = {0.f, 0.f, 0.f, 0.f}, acc1[4] = {0.f, 0.f, 0.f, 0.f};
  float bsum0 = 0.f, bsum1 = 0.f;
  const long long nchunks = (d.nvox + 15) / 16;
  for (long long c = (long long)s * kConvWarps + warp; c < nchunks; c += (long long)S * kConvWarps) {
    const long long k0 = c * 16 + 2 * q;  // this lane's voxels: k0, k0+1, k0+8, k0+9
    const long long vk[4] = {k0, k0 + 1, k0 + 8, k0 + 9};
    long long nb[4], dv[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const Vox p = vox_of(vk[i], d);
      nb[i] = nbr(p, t, d);
      dv[i] = p.ok ? vk[i] : -1;
    }
    // A = X^T (rows in-channel, k voxel)
    const uint32_t a[4] = {pack2(x, nb[0], nb[1], g), pack2(x, nb[0], nb[1], g + 8),
                           pack2(x, nb[2], nb[3], g), pack2(x, nb[2], nb[3], g + 8)};
    // B = dY (k voxel, n out-channel)
    const uint32_t b00 = pack2(dy, dv[0], dv[1], g), b01 = pack2(dy, dv[2], dv[3], g);
    const uint32_t b10 = pack2(dy, dv[0], dv[1], g + 8), b11 = pack2(dy, dv[2], dv[3], g + 8);
    mma_16816(acc0, a, b00, b01);
    mma_16816(acc1, a, b10, b11);
    if (t == 13) {
      const uint32_t bb[4] = {b00, b01, b10, b11};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float lo = __uint_as_float(bb[i] << 16), hi = __uint_as_float(bb[i] & 0xffff0000u);
        if (i < 2) bsum0 += lo + hi;
        else bsum1 += lo + hi;
      }
    }
  }
  // C tile layout: (row in g / g+8, col out 2q, 2q+1 [+8 for tile 1])
#pragma unroll
  for (int tile = 0; tile < 2; ++tile) {
    const float *acc = tile ? acc1 : acc0;
    const int co = 2 * q + 8 * tile;
    red[warp][g * kC + co] = acc[0];
    red[warp][g * kC + co + 1] = acc[1];
    red[warp][(g + 8) * kC + co] = acc[2];
    red[warp][(g + 8) * kC + co + 1] = acc[3];
  }
  bsum0 += __shfl_xor_sync(0xffffffffu, bsum0, 1);
  bsum0 += __shfl_xor_sync(0xffffffffu, bsum0, 2);
  bsum1 += __shfl_xor_sync(0xffffffffu, bsum1, 1);
  bsum1 += __shfl_xor_sync(0xffffffffu, bsum1, 2);
  if (q == 0) {
    bred[warp][g] = bsum0;
    bred[warp][g + 8] = bsum1;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kC * kC; i += blockDim.x) {
    float v = 0.f;
    for (int w = 0; w < kConvWarps; ++w) v += red[w][i];
    part[((long long)s * kTaps + t) * kC * kC + i] = v;
  }
  if (t == 13 && threadIdx.x < kC) {
    float v = 0.f;
    for (int w = 0; w < kConvWarps; ++w) v += bred[w][threadIdx.x];
    bpart[s * kC + threadIdx.x] = v;
  }
}

__global__ void wgrad_reduce_kernel(const float *__restrict__ part,
                                    const float *__restrict__ bpart, int S,
                                    float *__restrict__ dw, float *__restrict__ db) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = kTaps * kC * kC;
  if (i < n) {
    float v = 0.f;
    for (int s = 0; s < S; ++s) v += part[(long long)s * n + i];
    dw[i] = v;
  } else if (i < n + kC && db) {
    float v = 0.f;
    for (int s = 0; s < S; ++s) v += bpart[s * kC + (i - n)];
    db[i - n] = v;
  }
}

// FP32 master [27][in][out] -> BF16 forward [27][out][in] and backward-data
// [27][in][out] with taps reversed (the adjoint convolution).
__global__ void prep_weights_kernel(const float *__restrict__ w, __nv_bfloat16 *__restrict__ wf,
                                    __nv_bfloat16 *__restrict__ wb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kTaps * kC * kC) return;
  const int t = i / (kC * kC), ci = (i / kC) % kC, co = i % kC;
  const __nv_bfloat16 v = __float2bfloat16_rn(w[i]);
  wf[(t * kC + co) * kC + ci] = v;
  wb[((kTaps - 1 - t) * kC + ci) * kC + co] = v;
}

// Adam (Kingma & Ba 2015) with bias corrections c1 = 1/(1 - b1^t),
// c2 = 1/(1 - b2^t).
__global__ void adam_kernel(float *__restrict__ w, const float *__restrict__ g,
                            float *__restrict__ m, float *__restrict__ v, long long n, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

// dY (channel 0) = 2 (pred - target) / n; per-block FP64 sums of the
// squared error in part[blockIdx.x].
__global__ void mse_kernel(const float *__restrict__ pred, const float *__restrict__ tgt,
                           long long n, __nv_bfloat16 *__restrict__ dy,
                           double *__restrict__ part) {
  __shared__ double red[256];
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double e2 = 0.0;
  if (i < n) {
    const float e = pred[i] - tgt[i];
    e2 = (double)e * (double)e;
    uint4 z = make_uint4(0, 0, 0, 0);
    uint4 *row = reinterpret_cast<uint4 *>(dy + i * kC);
    row[0] = z;
    row[1] = z;
    dy[i * kC] = __float2bfloat16_rn(2.f * e / (float)n);
  }
  red[threadIdx.x] = e2;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// Fine stacked grids -> coarse network input.  Instance b sits at fine
// origin ((b % nsx) * inx, 0, (b / nsx) * inz) of float grids with row pitch
// `pitch` bytes and ny rows per plane; coarse cell (zc, yc, xc) averages the
// fine cells [zc f, zc f + f) x ... inside the instance.
//
// `flip` selects one of the 16 mirror images of an instance that are
// instances of the same problem family: bit 0/1/2 mirror x/y/z, bit 3 swaps
// x and y (with a2 and a1, the x and y coefficients; needs inx == iny).  The 19-point operator with
// c_i = a_i and b = 0 weighs both neighbours of a cell along an axis with
// that cell's own a_i, and the Dirichlet faces are symmetric, so the mirrored
// fields' solution is the mirrored solution: one solve gives 16 training
// pairs.  Coordinates below are those of the mirror image; vmap takes them
// back to the stored instance.
struct PoolArgs {
  const float *a0, *a1, *a2, *wrk1, *bnd, *p;
  long long pitch_e;  // row pitch in floats
  int ny;             // rows per plane of the stacked grids
  int inx, iny, inz;  // instance size
  int nsx;            // instances along x
  int f;              // pooling factor
  int zc, yc, xc;     // coarse size
  int batch;
  int flip;
  float wscale, pscale;
  const float *inst_scale;  // per-instance source/solution scale (NULL: 1)
  const float *p_sub;       // pool_target: subtract this grid from p (NULL: none)
};

__device__ __forceinline__ float inst_scale_of(const PoolArgs &a, int b) {
  return a.inst_scale ? a.inst_scale[b] : 1.f;
}

__device__ __forceinline__ long long fine_index(const PoolArgs &a, int b, int z, int y, int x) {
  const int ox = (b % a.nsx) * a.inx, oz = (b / a.nsx) * a.inz;
  return ((long long)(oz + z) * a.ny + y) * a.pitch_e + ox + x;
}

// Index of mirror-image cell (z, y, x) of instance b in the stored grids.
__device__ __forceinline__ long long vmap(const PoolArgs &a, int b, int z, int y, int x) {
  if (a.flip & 1) x = a.inx - 1 - x;
  if (a.flip & 2) y = a.iny - 1 - y;
  if (a.flip & 4) z = a.inz - 1 - z;
  if (a.flip & 8) {
    const int t = x;
    x = y;
    y = t;
  }
  return fine_index(a, b, z, y, x);
}

// Channels (means over the block): 0-2 ln a0, ln a1, ln a2; 3 wrk1 * wscale;
// 4 bnd; 5 wrk1 * 3 / (a0 + a1 + a2) * wscale (the source over the local
// coefficient, whose block mean the means of wrk1 and a do not give);
// 6-8 -ln mean(1 / a_i) (log harmonic means: a block's series
// conductance); 9-15 zeros.  a1/a2 are those of the mirror image.
__global__ void pool_inputs_kernel(PoolArgs a, __nv_bfloat16 *__restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)a.batch * a.zc * a.yc * a.xc;
  if (i >= n) return;
  const int xc = (int)(i % a.xc), yc = (int)((i / a.xc) % a.yc);
  const int zc = (int)((i / ((long long)a.xc * a.yc)) % a.zc);
  const int b = (int)(i / ((long long)a.xc * a.yc * a.zc));
  // a0 weighs the z neighbours, a1 the y and a2 the x neighbours
  const float *ay = (a.flip & 8) ? a.a2 : a.a1;
  const float *ax = (a.flip & 8) ? a.a1 : a.a2;
  float s[kPoolChannels] = {};
  int cnt = 0;
  for (int z = zc * a.f; z < min(zc * a.f + a.f, a.inz); ++z)
    for (int y = yc * a.f; y < min(yc * a.f + a.f, a.iny); ++y)
      for (int x = xc * a.f; x < min(xc * a.f + a.f, a.inx); ++x) {
        const long long k = vmap(a, b, z, y, x);
        const float c0 = a.a0[k], c1 = ay[k], c2 = ax[k], w = a.wrk1[k];
        s[0] += logf(c0);
        s[1] += logf(c1);
        s[2] += logf(c2);
        s[3] += w;
        s[4] += a.bnd[k];
        s[5] += w * 3.f / (c0 + c1 + c2);
        s[6] += 1.f / c0;
        s[7] += 1.f / c1;
        s[8] += 1.f / c2;
        ++cnt;
      }
  const float inv = 1.f / (float)cnt;
  const float ws = a.wscale * inst_scale_of(a, b);
  __nv_bfloat16 *row = out + i * kC;
  row[0] = __float2bfloat16_rn(s[0] * inv);
  row[1] = __float2bfloat16_rn(s[1] * inv);
  row[2] = __float2bfloat16_rn(s[2] * inv);
  row[3] = __float2bfloat16_rn(s[3] * inv * ws);
  row[4] = __float2bfloat16_rn(s[4] * inv);
  row[5] = __float2bfloat16_rn(s[5] * inv * ws);
  for (int c = 6; c < 9; ++c) row[c] = __float2bfloat16_rn(-logf(s[c] * inv));
  for (int c = kPoolChannels; c < kC; ++c) row[c] = __float2bfloat16_rn(0.f);
}

// Training target: p at each block's centre (c + 0.5) f - 0.5, the mean of
// the fine cells nearest to it (two per axis for even f), times pscale; in
// the mirror image's coordinates.
__global__ void pool_target_kernel(PoolArgs a, float *__restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)a.batch * a.zc * a.yc * a.xc;
  if (i >= n) return;
  const int xc = (int)(i % a.xc), yc = (int)((i / a.xc) % a.yc);
  const int zc = (int)((i / ((long long)a.xc * a.yc)) % a.zc);
  const int b = (int)(i / ((long long)a.xc * a.yc * a.zc));
  // nearest fine cells to the centre: lo = floor, hi = ceil of (c + 0.5) f - 0.5
  auto near = [&](int c, int nf, int &lo, int &hi) {
    lo = min((2 * c * a.f + a.f - 1) / 2, nf - 1);
    hi = min((2 * c * a.f + a.f) / 2, nf - 1);
  };
  int z0, z1, y0, y1, x0, x1;
  near(zc, a.inz, z0, z1);
  near(yc, a.iny, y0, y1);
  near(xc, a.inx, x0, x1);
  const int zs[2] = {z0, z1}, ys[2] = {y0, y1}, xs[2] = {x0, x1};
  float s = 0.f;
  for (int k = 0; k < 2; ++k)
    for (int j = 0; j < 2; ++j)
      for (int m = 0; m < 2; ++m) {
        const long long c = vmap(a, b, zs[k], ys[j], xs[m]);
        s += a.p_sub ? a.p[c] - a.p_sub[c] : a.p[c];
      }
  out[i] = s * 0.125f * a.pscale * inst_scale_of(a, b);
}

// Catmull-Rom weights of points -1, 0, 1, 2 at t in [0, 1] past point 0
// (Catmull & Rom 1974).
__device__ __forceinline__ void catmull_rom(float t, float (&w)[4]) {
  const float t2 = t * t, t3 = t2 * t;
  w[0] = 0.5f * (-t3 + 2.f * t2 - t);
  w[1] = 0.5f * (3.f * t3 - 5.f * t2 + 2.f);
  w[2] = 0.5f * (-3.f * t3 + 4.f * t2 + t);
  w[3] = 0.5f * (t3 - t2);
}

// Coarse prediction (FP32, one value per coarse cell) -> fine p:
// Catmull-Rom cubic interpolation per axis from coarse centres at
// (c + 0.5) f - 0.5 (positions clamped to [0, nc - 1], neighbour indices to
// the coarse grid), divided by pscale, times bnd.  Writes (or, with add,
// adds to) every fine cell of every instance.  With a mirror (flip != 0) the
// coarse grid is a prediction for that mirror image: stored cell (z, y, x)
// reads it at its mirror-image coordinates.
__global__ void upsample_kernel(PoolArgs a, const float *__restrict__ coarse,
                                float *__restrict__ p, bool add) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)a.batch * a.inz * a.iny * a.inx;
  if (i >= n) return;
  const int x = (int)(i % a.inx), y = (int)((i / a.inx) % a.iny);
  const int z = (int)((i / ((long long)a.inx * a.iny)) % a.inz);
  const int b = (int)(i / ((long long)a.inx * a.iny * a.inz));
  // mirror-image coordinates of stored cell (z, y, x): undo vmap
  int xm = (a.flip & 8) ? y : x, ym = (a.flip & 8) ? x : y, zm = z;
  if (a.flip & 1) xm = a.inx - 1 - xm;
  if (a.flip & 2) ym = a.iny - 1 - ym;
  if (a.flip & 4) zm = a.inz - 1 - zm;
  auto axis = [&](int j, int nc, int (&idx)[4], float (&w)[4]) {
    float pos = ((float)j + 0.5f) / (float)a.f - 0.5f;
    pos = fminf(fmaxf(pos, 0.f), (float)(nc - 1));
    const int i0 = min((int)floorf(pos), nc - 1);
    catmull_rom(pos - (float)i0, w);
    for (int k = 0; k < 4; ++k) idx[k] = min(max(i0 - 1 + k, 0), nc - 1);
  };
  int iz[4], iy[4], ix[4];
  float wz[4], wy[4], wx[4];
  axis(zm, a.zc, iz, wz);
  axis(ym, a.yc, iy, wy);
  axis(xm, a.xc, ix, wx);
  const float *c = coarse + (long long)b * a.zc * a.yc * a.xc;
  float v = 0.f;
  for (int kz = 0; kz < 4; ++kz) {
    float vy = 0.f;
    for (int ky = 0; ky < 4; ++ky) {
      const float *row = c + ((long long)iz[kz] * a.yc + iy[ky]) * a.xc;
      float vx = 0.f;
      for (int kx = 0; kx < 4; ++kx) vx += wx[kx] * row[ix[kx]];
      vy += wy[ky] * vx;
    }
    v += wz[kz] * vy;
  }
  const long long k = fine_index(a, b, z, y, x);
  const float sc = inst_scale_of(a, b);
  const float u = sc != 0.f ? v / (a.pscale * sc) * a.bnd[k] : 0.f;
  p[k] = add ? p[k] + u : u;
}

// Residual source of the current pressure p, for the correction problem:
// with c_i = a_i and b = 0 the 19-point Himeno residual is
// ss = (s0 a3 - p) bnd with s0 = sum_i a_i (p(x + e_i) + p(x - e_i)) + wrk1
// and a3 = 1 / (2 (a0 + a1 + a2)), so r = ss / a3 =
// (s0 - 2 (a0 + a1 + a2) p) bnd is the source (in wrk1's units) of the
// equation the error p* - p satisfies.  Cells on an instance's faces (and
// bnd = 0 cells) get r = 0 and read no neighbours.  r is written in the
// stacked layout of the fields.  Grid (G, batch): block (g, b) strides over
// instance b's cells and stores its FP64 partial sum of r^2 at
// part[b * G + g] (fixed assignment, so the per-instance sums are
// deterministic).
__global__ void residual_source_kernel(PoolArgs a, float *__restrict__ r,
                                       double *__restrict__ part) {
  const int b = blockIdx.y;
  const long long n = (long long)a.inz * a.iny * a.inx;
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % a.inx), y = (int)((i / a.inx) % a.iny);
    const int z = (int)(i / ((long long)a.inx * a.iny));
    const long long k = fine_index(a, b, z, y, x);
    float v = 0.f;
    const bool inner = x > 0 && x < a.inx - 1 && y > 0 && y < a.iny - 1 && z > 0 &&
                       z < a.inz - 1;
    if (inner && a.bnd[k] != 0.f) {
      const long long py = a.pitch_e, pz = (long long)a.ny * a.pitch_e;
      const float pc = a.p[k];
      const float c0 = a.a0[k], c1 = a.a1[k], c2 = a.a2[k];
      float s0 = c0 * (a.p[k + pz] + a.p[k - pz]);
      s0 += c1 * (a.p[k + py] + a.p[k - py]);
      s0 += c2 * (a.p[k + 1] + a.p[k - 1]);
      s0 += a.wrk1[k];
      v = (s0 - 2.f * (c0 + c1 + c2) * pc) * a.bnd[k];
    }
    r[k] = v;
    acc += (double)v * v;
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(long long)b * gridDim.x + blockIdx.x] = red[0];
}

// p = p_scale * p + delta at every cell of every instance (stored layout;
// delta may be NULL): one rounding of p per restart, whatever number of
// mirror predictions delta sums.
__global__ void add_correction_kernel(PoolArgs a, const float *__restrict__ delta,
                                      float p_scale, float *__restrict__ p) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)a.batch * a.inz * a.iny * a.inx;
  if (i >= n) return;
  const int x = (int)(i % a.inx), y = (int)((i / a.inx) % a.iny);
  const int z = (int)((i / ((long long)a.inx * a.iny)) % a.inz);
  const int b = (int)(i / ((long long)a.inx * a.iny * a.inz));
  const long long k = fine_index(a, b, z, y, x);
  const float v = p_scale == 1.f ? p[k] : __fmul_rn(p_scale, p[k]);
  p[k] = delta ? __fadd_rn(v, delta[k]) : v;
}

// scale[b] = target_rms / rms(r of instance b) over its interior cells
// (0 when r vanishes); the partials are summed in a fixed order.
__global__ void inst_scale_kernel(const double *__restrict__ part, int G, int batch,
                                  long long cells, float target_rms,
                                  float *__restrict__ scale) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  double s = 0.0;
  for (int g = 0; g < G; ++g) s += part[(long long)b * G + g];
  const double rms = sqrt(s / (double)cells);
  scale[b] = rms > 0.0 ? (float)(target_rms / rms) : 0.f;
}

}  // namespace

void nn_set_error_word(int *err) { g_err = err; }

static bool use_tcgen05() {
  const char *e = getenv("PS_WARMSTART_TC");
  return !(e && e[0] == '0');
}

int nn_conv(const void *x, const void *w, const float *bias, const void *mask, int relu,
            void *y, float *yf, int B, int Z, int Y, int X, cudaStream_t s) {
  Dims d{B, Z, Y, X, (long long)B * Z * Y * X};
  if (d.nvox <= 0) return 0;
  if (use_tcgen05()) {
    static bool attr = false;
    if (!attr) {
      const cudaError_t e = cudaFuncSetAttribute(
          conv_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
      if (e != cudaSuccess) return (int)e;
      attr = true;
    }
    const long long blocks = (d.nvox + kTcM - 1) / kTcM;
    conv_tc_kernel<<<(unsigned)blocks, kTcThreads, kTcSmem, s>>>(
        static_cast<const __nv_bfloat16 *>(x), static_cast<const __nv_bfloat16 *>(w), bias,
        static_cast<const __nv_bfloat16 *>(mask), relu, static_cast<__nv_bfloat16 *>(y), yf, d,
        g_err);
    return (int)cudaGetLastError();
  }
  const long long blocks = (d.nvox + 16 * kConvWarps - 1) / (16 * kConvWarps);
  conv_kernel<<<(unsigned)blocks, 32 * kConvWarps, 0, s>>>(
      static_cast<const __nv_bfloat16 *>(x), static_cast<const __nv_bfloat16 *>(w), bias,
      static_cast<const __nv_bfloat16 *>(mask), relu, static_cast<__nv_bfloat16 *>(y), yf, d);
  return (int)cudaGetLastError();
}

int nn_wgrad(const void *x, const void *dy, float *part, int S, float *dw, float *db, int B,
             int Z, int Y, int X, cudaStream_t s) {
  Dims d{B, Z, Y, X, (long long)B * Z * Y * X};
  if (S < 1) return -1;
  float *bpart = part + (long long)S * kTaps * kC * kC;
  wgrad_kernel<<<dim3(kTaps, S), 32 * kConvWarps, 0, s>>>(
      static_cast<const __nv_bfloat16 *>(x), static_cast<const __nv_bfloat16 *>(dy), part, bpart,
      d);
  const int n = kTaps * kC * kC + kC;
  wgrad_reduce_kernel<<<(n + 255) / 256, 256, 0, s>>>(part, bpart, S, dw, db);
  return (int)cudaGetLastError();
}

int nn_prep_weights(const float *w, void *wf, void *wb, cudaStream_t s) {
  prep_weights_kernel<<<(kTaps * kC * kC + 255) / 256, 256, 0, s>>>(
      w, static_cast<__nv_bfloat16 *>(wf), static_cast<__nv_bfloat16 *>(wb));
  return (int)cudaGetLastError();
}

int nn_adam(float *w, const float *g, float *m, float *v, long long n, float lr, float b1,
            float b2, float eps, int step, cudaStream_t s) {
  if (n <= 0 || step < 1) return -1;
  const float c1 = (float)(1.0 / (1.0 - pow((double)b1, step)));
  const float c2 = (float)(1.0 / (1.0 - pow((double)b2, step)));
  adam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(w, g, m, v, n, lr, b1, b2, eps, c1, c2);
  return (int)cudaGetLastError();
}

int nn_mse(const float *pred, const float *tgt, long long n, void *dy, double *part,
           cudaStream_t s) {
  if (n <= 0) return -1;
  mse_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(pred, tgt, n,
                                                         static_cast<__nv_bfloat16 *>(dy), part);
  return (int)cudaGetLastError();
}

static PoolArgs pool_args(const NNFields &f) {
  PoolArgs a{};
  a.a0 = f.a0;
  a.a1 = f.a1;
  a.a2 = f.a2;
  a.wrk1 = f.wrk1;
  a.bnd = f.bnd;
  a.p = f.p;
  a.pitch_e = f.pitch / 4;
  a.ny = f.ny;
  a.inx = f.inx;
  a.iny = f.iny;
  a.inz = f.inz;
  a.nsx = f.nsx;
  a.f = f.factor;
  a.zc = (f.inz + f.factor - 1) / f.factor;
  a.yc = (f.iny + f.factor - 1) / f.factor;
  a.xc = (f.inx + f.factor - 1) / f.factor;
  a.batch = f.batch;
  a.flip = f.flip;
  a.wscale = f.wscale;
  a.pscale = f.pscale;
  a.inst_scale = f.inst_scale;
  a.p_sub = f.p_sub;
  return a;
}

int nn_pool_inputs(const NNFields &f, void *out, cudaStream_t s) {
  const PoolArgs a = pool_args(f);
  const long long n = (long long)a.batch * a.zc * a.yc * a.xc;
  if (n <= 0) return -1;
  pool_inputs_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(
      a, static_cast<__nv_bfloat16 *>(out));
  return (int)cudaGetLastError();
}

int nn_pool_target(const NNFields &f, float *out, cudaStream_t s) {
  const PoolArgs a = pool_args(f);
  const long long n = (long long)a.batch * a.zc * a.yc * a.xc;
  if (n <= 0 || !a.p) return -1;
  pool_target_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(a, out);
  return (int)cudaGetLastError();
}

int nn_upsample(const NNFields &f, const float *coarse, float *p, bool add, cudaStream_t s) {
  const PoolArgs a = pool_args(f);
  const long long n = (long long)a.batch * a.inz * a.iny * a.inx;
  if (n <= 0) return -1;
  upsample_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, coarse, p, add);
  return (int)cudaGetLastError();
}

int nn_residual_source(const NNFields &f, float *r, float *inst_scale, float target_rms,
                       double *work, int work_len, cudaStream_t s) {
  const PoolArgs a = pool_args(f);
  if (!a.p || !r || !inst_scale || !work || a.batch < 1) return -1;
  const int G = work_len / a.batch;
  if (G < 1) return -1;
  const int g = G < 64 ? G : 64;
  residual_source_kernel<<<dim3((unsigned)g, (unsigned)a.batch), 256, 0, s>>>(a, r, work);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  const long long cells = (long long)(a.inz - 2) * (a.iny - 2) * (a.inx - 2);
  inst_scale_kernel<<<(unsigned)((a.batch + 127) / 128), 128, 0, s>>>(
      work, g, a.batch, cells > 0 ? cells : 1, target_rms, inst_scale);
  return (int)cudaGetLastError();
}

int nn_add_correction(const NNFields &f, const float *delta, float p_scale, float *p,
                      cudaStream_t s) {
  const PoolArgs a = pool_args(f);
  const long long n = (long long)a.batch * a.inz * a.iny * a.inx;
  if (n <= 0 || !p) return -1;
  add_correction_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, delta, p_scale, p);
  return (int)cudaGetLastError();
}

}  // namespace psg
