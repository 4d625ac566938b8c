// 7-point stencil sweeps on GB300 (sm_103a): 2.5D z-marching tiles.
//
// Replaces the translator-generated CUDA run kernel of the reference
// (translator/cuda_runtime_builder.cc:1099-1228, 1392-1410: one thread per
// (x,y), a z-loop, every neighbour a separate global load) for the builtin
// 7-point stencils:
//   DIFFUSION7  clamped diffusion, examples/diffusion-benchmark/diffusion3d_physis.c:29-58
//   SUM7        unclamped 7-point sum, tests/system_tests/test_cases/test_7-pt.c:12-20
//   COPY        out = in over the domain
//
// Design (one CTA = one 32*VEC x TY tile in x,y marching over zchunk planes):
// * each z-plane of the tile plus a one-cell halo in y and a 16-byte halo in
//   x (TMA wants 16-byte aligned x) is fetched by one TMA 3D box load into a
//   ring of `ns` shared-memory stages; an mbarrier per stage signals arrival;
// * one thread per 16-byte vector (VEC = 16/sizeof(T) cells): the z
//   neighbours come from a register queue (b = previous centre, c = centre,
//   t = next plane), the x neighbours from warp shuffles of the centre
//   vector, the y neighbours from the rows above and below in shared memory;
// * results leave as one 16-byte store per thread (a warp writes 512
//   contiguous bytes); edge vectors that straddle the domain use masked
//   scalar stores;
// * clamped faces (neighbour index outside the grid -> centre value) are
//   selects on the global coordinate, so the zero fill of out-of-range TMA
//   boxes is never used;
// * arithmetic is round-to-nearest without FMA contraction, in the REF
//   expression order, so every cell is bit-identical to the REF target.
#include "ps_device.cuh"
#include "ps_internal.h"

namespace psg {
namespace {

template <typename T>
struct S7Params {
  T *out;
  int64_t row;    // out pitch in elements
  int64_t plane;  // out elements per z-plane
  int nx, ny, nz;
  int dmin0, dmin1, dmin2, dmax0, dmax1, dmax2;
  int xbase;      // x of the first tile (multiple of VEC)
  int zchunk;
  int ns;
  T cc, cw, ce, cs, cn, cb, ct;  // expression order of DIFFUSION7
  int *err;
};

__host__ __device__ constexpr int s7_bar_bytes(int ns) { return 128 * ((8 * ns + 127) / 128); }
__host__ __device__ constexpr uint32_t s7_stage_bytes(uint32_t b) { return (b + 127u) & ~127u; }

template <typename T, int K>
__global__ void __launch_bounds__(512, 1)
s7_march_kernel(const __grid_constant__ CUtensorMap tin, const S7Params<T> p) {
  constexpr int VEC = 16 / (int)sizeof(T);
  constexpr int TX = 32 * VEC;
  constexpr int W = TX + 2 * VEC;  // shared row width in elements
  constexpr bool kClamp = (K == kKernelDiffusion7);
  typedef RN<T> R;

  const int TY = blockDim.y;
  // TMA writes a box of W x (TY+2) elements; each ring stage starts on a
  // 128-byte boundary (the alignment cp.async.bulk.tensor requires of its
  // shared-memory destination).
  const uint32_t plane_bytes = (uint32_t)(W * (TY + 2) * sizeof(T));
  const int plane_elems = (int)(s7_stage_bytes(plane_bytes) / sizeof(T));
  const int ns = p.ns;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);
  T *ring = reinterpret_cast<T *>(smem + s7_bar_bytes(ns));

  const int lane = threadIdx.x, row = threadIdx.y;
  const int tid = row * 32 + lane;
  const int x0 = p.xbase + blockIdx.x * TX;
  const int y0 = p.dmin1 + blockIdx.y * TY;
  const int zs = p.dmin2 + blockIdx.z * p.zchunk;
  const int ze = min(zs + p.zchunk, p.dmax2);
  const int nplanes = ze - zs + 2;  // planes zs-1 .. ze

  if (tid == 0) {
    prefetch_tmap(&tin);
    for (int s = 0; s < ns; ++s) mbar_init(&full[s], 1);
    fence_barrier_init();
  }
  __syncthreads();

  // Plane q of this CTA is global plane zs-1+q, held in stage q % ns.
  auto issue = [&](int q) {
    const int s = q % ns;
    mbar_arrive_expect_tx(&full[s], plane_bytes);
    tma_load_3d(ring + s * plane_elems, &tin, x0 - VEC, y0 - 1, zs - 1 + q, &full[s]);
  };
  if (tid == 0) {
    const int n0 = min(ns, nplanes);
    for (int q = 0; q < n0; ++q) issue(q);
  }
  bool ok = true;
  auto wait = [&](int q) -> const T * {
    const int s = q % ns;
    if (!mbar_wait(&full[s], (uint32_t)((q / ns) & 1), p.err)) ok = false;
    return ring + s * plane_elems;
  };

  const int cen = (row + 1) * W + VEC + lane * VEC;  // own vector, centre row
  T b[VEC], c[VEC], t[VEC];
  {
    const T *pm = wait(0);
    const T *pc = wait(1);
    ld16_shared<T>(c, pc + cen);
    ld16_shared<T>(b, pm + cen);
    if (kClamp && zs == 0) {
#pragma unroll
      for (int i = 0; i < VEC; ++i) b[i] = c[i];
    }
  }
  ok = __syncthreads_and(ok);
  if (!ok) return;
  if (tid == 0 && ns < nplanes) issue(ns);

  const int y = y0 + row;
  const int x = x0 + lane * VEC;
  const bool row_in = (y < p.dmax1);
  const bool vec_in = (x >= p.dmin0) && (x + VEC <= p.dmax0);

  for (int z = zs; z < ze; ++z) {
    const int q = z - zs + 1;
    const T *cur = ring + (q % ns) * plane_elems;
    const T *nxt = wait(q + 1);
    ld16_shared<T>(t, nxt + cen);
    if (kClamp && z == p.nz - 1) {
#pragma unroll
      for (int i = 0; i < VEC; ++i) t[i] = c[i];
    }
    T o[VEC];
    if (K == kKernelCopy) {
#pragma unroll
      for (int i = 0; i < VEC; ++i) o[i] = c[i];
    } else {
      T n[VEC], s[VEC];
      ld16_shared<T>(n, cur + cen - W);  // y-1
      ld16_shared<T>(s, cur + cen + W);  // y+1
      T left = shfl_up1(c[VEC - 1]);
      T right = shfl_down1(c[0]);
      if (lane == 0) left = cur[cen - 1];
      if (lane == 31) right = cur[cen + VEC];
      if (kClamp) {
        if (y == 0) {
#pragma unroll
          for (int i = 0; i < VEC; ++i) n[i] = c[i];
        }
        if (y == p.ny - 1) {
#pragma unroll
          for (int i = 0; i < VEC; ++i) s[i] = c[i];
        }
      }
#pragma unroll
      for (int i = 0; i < VEC; ++i) {
        T w = (i == 0) ? left : c[i - 1];
        T e = (i == VEC - 1) ? right : c[i + 1];
        if (kClamp) {
          if (x + i == 0) w = c[i];
          if (x + i == p.nx - 1) e = c[i];
          // cc*c + cw*w + ce*e + cs*s + cn*n + cb*b + ct*t, left to right
          T v = R::mul(p.cc, c[i]);
          v = R::add(v, R::mul(p.cw, w));
          v = R::add(v, R::mul(p.ce, e));
          v = R::add(v, R::mul(p.cs, s[i]));
          v = R::add(v, R::mul(p.cn, n[i]));
          v = R::add(v, R::mul(p.cb, b[i]));
          v = R::add(v, R::mul(p.ct, t[i]));
          o[i] = v;
        } else {
          // c + e + w + s + n + b + t, left to right
          T v = R::add(c[i], e);
          v = R::add(v, w);
          v = R::add(v, s[i]);
          v = R::add(v, n[i]);
          v = R::add(v, b[i]);
          v = R::add(v, t[i]);
          o[i] = v;
        }
      }
    }
    if (ok && row_in) {
      T *dst = p.out + (int64_t)z * p.plane + (int64_t)y * p.row + x;
      if (vec_in) {
        st16_global<T>(dst, o);
      } else {
#pragma unroll
        for (int i = 0; i < VEC; ++i)
          if (x + i >= p.dmin0 && x + i < p.dmax0) dst[i] = o[i];
      }
    }
#pragma unroll
    for (int i = 0; i < VEC; ++i) {
      b[i] = c[i];
      c[i] = t[i];
    }
    ok = __syncthreads_and(ok);
    if (!ok) break;
    if (tid == 0 && q + ns < nplanes) issue(q + ns);
  }
  if (!ok && tid == 0) {
    // Give copies still in flight a bounded chance to land before exit.
    for (int q = 0; q < nplanes; ++q) {
      const int s = q % ns;
      mbar_wait(&full[s], (uint32_t)((q / ns) & 1), nullptr, 1024);
    }
  }
}

template <typename T, int K>
cudaError_t launch_t(const Stencil7Args &a, const MarchConfig &cfg,
                     const CUtensorMap *tin, int *dev_err, cudaStream_t st) {
  constexpr int VEC = 16 / (int)sizeof(T);
  constexpr int TX = 32 * VEC;
  S7Params<T> p;
  p.out = static_cast<T *>(a.out.ptr);
  p.row = a.out.pitch / (int64_t)sizeof(T);
  p.plane = p.row * a.out.ny;
  p.nx = a.in.nx;
  p.ny = a.in.ny;
  p.nz = a.in.nz;
  p.dmin0 = a.dom.min[0];
  p.dmin1 = a.dom.min[1];
  p.dmin2 = a.dom.min[2];
  p.dmax0 = a.dom.max[0];
  p.dmax1 = a.dom.max[1];
  p.dmax2 = a.dom.max[2];
  p.xbase = (a.dom.min[0] / VEC) * VEC;
  p.zchunk = cfg.zchunk;
  p.ns = cfg.ns;
  // map argument order ce cw cn cs ct cb cc
  p.ce = (T)a.coef[0];
  p.cw = (T)a.coef[1];
  p.cn = (T)a.coef[2];
  p.cs = (T)a.coef[3];
  p.ct = (T)a.coef[4];
  p.cb = (T)a.coef[5];
  p.cc = (T)a.coef[6];
  p.err = dev_err;
  const int ex = a.dom.max[0] - p.xbase;
  const int ey = a.dom.max[1] - a.dom.min[1];
  const int ez = a.dom.max[2] - a.dom.min[2];
  if (ex <= 0 || ey <= 0 || ez <= 0) return cudaSuccess;
  dim3 grid((ex + TX - 1) / TX, (ey + cfg.ty - 1) / cfg.ty,
            (ez + cfg.zchunk - 1) / cfg.zchunk);
  if (grid.y > 65535 || grid.z > 65535 || cfg.ty < 1 || cfg.ty > 16 || cfg.ns < 2)
    return cudaErrorInvalidConfiguration;
  dim3 block(32, cfg.ty, 1);
  const size_t smem = stencil7_smem_bytes((int)sizeof(T), cfg);
  static size_t attr_set = 0;  // dynamic shared memory opted in so far
  if (smem > attr_set) {
    cudaError_t e = cudaFuncSetAttribute(s7_march_kernel<T, K>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = smem;
  }
  s7_march_kernel<T, K><<<grid, block, smem, st>>>(*tin, p);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_type(const Stencil7Args &a, const MarchConfig &cfg,
                        const CUtensorMap *tin, int *dev_err, cudaStream_t st) {
  switch (a.kernel) {
    case kKernelDiffusion7:
      return launch_t<T, kKernelDiffusion7>(a, cfg, tin, dev_err, st);
    case kKernelSum7:
      return launch_t<T, kKernelSum7>(a, cfg, tin, dev_err, st);
    case kKernelCopy:
      return launch_t<T, kKernelCopy>(a, cfg, tin, dev_err, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace

size_t stencil7_smem_bytes(int esz, const MarchConfig &cfg) {
  const int vec = 16 / esz;
  const int w = 32 * vec + 2 * vec;
  // 128 bytes of slack for aligning the dynamic shared-memory base
  return 128 + (size_t)s7_bar_bytes(cfg.ns) +
         (size_t)cfg.ns * s7_stage_bytes((uint32_t)(w * (cfg.ty + 2) * esz));
}

cudaError_t launch_stencil7(const Stencil7Args &a, const MarchConfig &cfg,
                            const CUtensorMap *tin, int *dev_err,
                            cudaStream_t s) {
  if (a.kernel == kKernelDiffusion7 &&
      (a.in.type == kInt || a.in.type == kLong))
    return cudaErrorInvalidValue;
  switch (a.in.type) {
    case kFloat: return launch_type<float>(a, cfg, tin, dev_err, s);
    case kDouble: return launch_type<double>(a, cfg, tin, dev_err, s);
    case kInt: return launch_type<int>(a, cfg, tin, dev_err, s);
    case kLong: return launch_type<long long>(a, cfg, tin, dev_err, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace psg
