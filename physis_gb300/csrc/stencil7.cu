// 7-point stencil sweeps on GB300 (sm_103a): persistent 2.5D z-marching tiles.
//
// Replaces the translator-generated CUDA run kernel of the reference
// (translator/cuda_runtime_builder.cc:1099-1228, 1392-1410: one thread per
// (x,y), a z-loop, every neighbour a separate global load) for the builtin
// 7-point stencils:
//   DIFFUSION7  clamped diffusion, examples/diffusion-benchmark/diffusion3d_physis.c:29-58
//   SUM7        unclamped 7-point sum, tests/system_tests/test_cases/test_7-pt.c:12-20
//   COPY        out = in over the domain
//
// Design.  A tile is 32 lanes x 16 bytes wide in x (128 floats, 64 doubles)
// and WARPS*RY rows high in y.  Work items are (z-chunk, tile) pairs in
// chunk-major order; a persistent grid of SMs x occupancy CTAs takes items
// round-robin, so the CTAs resident at any moment march the same z-chunk of
// neighbouring tiles side by side and every halo row or column a tile reads
// is read from L2 by its neighbour at about the same time (HBM sees each byte
// once).  The host picks the chunk length that fills whole rounds.
// * Each z-plane of the tile plus a one-row y halo and a 16-byte x halo
//   (TMA wants 16-byte aligned x) arrives by one TMA 3D box load into a
//   ring of `ns` shared-memory stages; one mbarrier per stage signals
//   arrival.  Stage and phase advance incrementally (no divisions).
// * Each thread owns one 16-byte vector column of RY rows: the z neighbours
//   come from a register queue (b, c, t), the y neighbours of inner rows from
//   the thread's own registers (only the rows above and below the column are
//   read from shared memory), the x neighbours from warp shuffles.
// * One 16-byte store per thread and row (a warp writes 512 contiguous
//   bytes); vectors that straddle the domain edge use masked scalar stores.
// * Clamped faces (neighbour outside the grid -> centre value) are selects
//   on the global coordinate, so the zero fill of out-of-range boxes is never
//   used.
// * Arithmetic is round-to-nearest without FMA contraction in the REF
//   expression order, so every cell is bit-identical to the REF target.
#include <type_traits>

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
  int tiles_x;    // tiles per y-band
  int tiles;      // tiles_x * tiles per x-column
  int zlen;       // planes per z-chunk
  int64_t items;  // tiles * chunks
  int ns;
  T cc, cw, ce, cs, cn, cb, ct;  // expression order of DIFFUSION7
  int *err;
};

__host__ __device__ constexpr int s7_bar_bytes(int ns) { return 128 * ((8 * ns + 127) / 128); }
__host__ __device__ constexpr uint32_t s7_stage_bytes(uint32_t b) { return (b + 127u) & ~127u; }

template <typename T, int K, int RY>
__global__ void __launch_bounds__(512, 1)
s7_march_kernel(const __grid_constant__ CUtensorMap tin, const S7Params<T> p) {
  constexpr int VEC = 16 / (int)sizeof(T);
  constexpr int TX = 32 * VEC;
  constexpr int W = TX + 2 * VEC;  // shared row width in elements
  constexpr bool kClamp = (K == kKernelDiffusion7);
  typedef RN<T> R;

  const int TY = blockDim.y * RY;
  // Each ring stage starts on a 128-byte boundary (required of the shared
  // destination of cp.async.bulk.tensor).
  const uint32_t plane_bytes = (uint32_t)(W * (TY + 2) * sizeof(T));
  const int plane_elems = (int)(s7_stage_bytes(plane_bytes) / sizeof(T));
  const int ns = p.ns;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);
  T *ring = reinterpret_cast<T *>(smem + s7_bar_bytes(ns));

  const int lane = threadIdx.x, warp = threadIdx.y;
  const int tid = warp * 32 + lane;
  if (tid == 0) {
    prefetch_tmap(&tin);
    for (int s = 0; s < ns; ++s) mbar_init(&full[s], 1);
    fence_barrier_init();
  }
  __syncthreads();

  // Producer state (thread 0) and consumer state (all threads): the stage
  // that the next issued / next awaited plane uses, and its phase parity.
  int pstage = 0;
  uint32_t pphase = 0;
  int cstage = 0;
  uint32_t cphase = 0;
  bool ok = true;

  const int rows0 = warp * RY;                          // first own row in the tile
  const int cen0 = (rows0 + 1) * W + VEC + lane * VEC;  // own first row, centre

  for (int64_t item = blockIdx.x; item < p.items && ok; item += gridDim.x) {
    const int chunk = (int)(item / p.tiles);
    const int tile = (int)(item - (int64_t)chunk * p.tiles);
    const int zs = p.dmin2 + chunk * p.zlen;
    const int ze = min(zs + p.zlen, p.dmax2);
    const int x0 = p.xbase + (tile % p.tiles_x) * TX;
    const int y0 = p.dmin1 + (tile / p.tiles_x) * TY;
    const int nplanes = ze - zs + 2;  // planes zs-1 .. ze

    // Issues plane q (global plane zs-1+q) into the producer's next stage.
    auto issue = [&](int q) {
      mbar_arrive_expect_tx(&full[pstage], plane_bytes);
      tma_load_3d(ring + pstage * plane_elems, &tin, x0 - VEC, y0 - 1, zs - 1 + q,
                  &full[pstage]);
      if (++pstage == ns) {
        pstage = 0;
        pphase ^= 1u;
      }
    };
    // Waits for the next plane in issue order; returns its stage.
    auto wait_next = [&]() -> const T * {
      if (!mbar_wait(&full[cstage], cphase, p.err)) ok = false;
      const T *pl = ring + cstage * plane_elems;
      if (++cstage == ns) {
        cstage = 0;
        cphase ^= 1u;
      }
      return pl;
    };

    if (tid == 0) {
      const int n0 = min(ns, nplanes);
      for (int q = 0; q < n0; ++q) issue(q);
    }
    T b[RY][VEC], c[RY][VEC], t[RY][VEC];
    const T *pm = wait_next();   // plane zs-1
    const T *cur = wait_next();  // plane zs
#pragma unroll
    for (int r = 0; r < RY; ++r) {
      ld16_shared<T>(c[r], cur + cen0 + r * W);
      ld16_shared<T>(b[r], pm + cen0 + r * W);
      if (kClamp && zs == 0) {
#pragma unroll
        for (int i = 0; i < VEC; ++i) b[r][i] = c[r][i];
      }
    }
    ok = __syncthreads_and(ok);
    if (!ok) break;
    if (tid == 0 && ns < nplanes) issue(ns);

    const int x = x0 + lane * VEC;
    const int y = y0 + rows0;  // first own row
    const bool vec_in = (x >= p.dmin0) && (x + VEC <= p.dmax0);
    const bool west_face = kClamp && (x == 0);            // element 0 clamps west
    const int east_elem = kClamp ? (p.nx - 1 - x) : -1;  // element clamping east

    for (int z = zs; z < ze; ++z) {
      const int q = z - zs + 1;  // plane index of z
      const T *nxt = wait_next();
      T n[VEC], s[VEC];
#pragma unroll
      for (int r = 0; r < RY; ++r) ld16_shared<T>(t[r], nxt + cen0 + r * W);
      if (K != kKernelCopy) {
        ld16_shared<T>(n, cur + cen0 - W);       // row above the column
        ld16_shared<T>(s, cur + cen0 + RY * W);  // row below the column
      }
      if (kClamp && z == p.nz - 1) {
#pragma unroll
        for (int r = 0; r < RY; ++r)
#pragma unroll
          for (int i = 0; i < VEC; ++i) t[r][i] = c[r][i];
      }
#pragma unroll
      for (int r = 0; r < RY; ++r) {
        T o[VEC];
        if (K == kKernelCopy) {
#pragma unroll
          for (int i = 0; i < VEC; ++i) o[i] = c[r][i];
        } else {
          T nn[VEC], ss[VEC];
#pragma unroll
          for (int i = 0; i < VEC; ++i) {
            nn[i] = (r == 0) ? n[i] : c[r - 1][i];
            ss[i] = (r == RY - 1) ? s[i] : c[r + 1][i];
          }
          if (kClamp) {
            if (y + r == 0) {
#pragma unroll
              for (int i = 0; i < VEC; ++i) nn[i] = c[r][i];
            }
            if (y + r == p.ny - 1) {
#pragma unroll
              for (int i = 0; i < VEC; ++i) ss[i] = c[r][i];
            }
          }
          T left = shfl_up1(c[r][VEC - 1]);
          T right = shfl_down1(c[r][0]);
          if (lane == 0) left = cur[cen0 + r * W - 1];
          if (lane == 31) right = cur[cen0 + r * W + VEC];
#pragma unroll
          for (int i = 0; i < VEC; ++i) {
            T w = (i == 0) ? left : c[r][i - 1];
            T e = (i == VEC - 1) ? right : c[r][i + 1];
            if (kClamp) {
              if (i == 0 && west_face) w = c[r][0];
              if (i == east_elem) e = c[r][i];
              // cc*c + cw*w + ce*e + cs*s + cn*n + cb*b + ct*t, left to right
              T v = R::mul(p.cc, c[r][i]);
              v = R::add(v, R::mul(p.cw, w));
              v = R::add(v, R::mul(p.ce, e));
              v = R::add(v, R::mul(p.cs, ss[i]));
              v = R::add(v, R::mul(p.cn, nn[i]));
              v = R::add(v, R::mul(p.cb, b[r][i]));
              v = R::add(v, R::mul(p.ct, t[r][i]));
              o[i] = v;
            } else {
              // c + e + w + s + n + b + t, left to right
              T v = R::add(c[r][i], e);
              v = R::add(v, w);
              v = R::add(v, ss[i]);
              v = R::add(v, nn[i]);
              v = R::add(v, b[r][i]);
              v = R::add(v, t[r][i]);
              o[i] = v;
            }
          }
        }
        if (ok && y + r < p.dmax1) {
          T *dst = p.out + (int64_t)z * p.plane + (int64_t)(y + r) * p.row + x;
          if (vec_in) {
            st16_global<T>(dst, o);
          } else {
#pragma unroll
            for (int i = 0; i < VEC; ++i)
              if (x + i >= p.dmin0 && x + i < p.dmax0) dst[i] = o[i];
          }
        }
      }
#pragma unroll
      for (int r = 0; r < RY; ++r)
#pragma unroll
        for (int i = 0; i < VEC; ++i) {
          b[r][i] = c[r][i];
          c[r][i] = t[r][i];
        }
      cur = nxt;
      ok = __syncthreads_and(ok);
      if (!ok) break;
      // Plane q is consumed by every thread: refill its stage with q + ns.
      if (tid == 0 && q + ns < nplanes) issue(q + ns);
    }
  }
  if (!ok && tid == 0) {
    // Give copies still in flight a bounded chance to land before exit.
    for (int s = 0; s < ns; ++s) mbar_wait(&full[s], 0, nullptr, 1024);
  }
}

template <typename T, int K, int RY>
cudaError_t launch_ry(S7Params<T> p, int tiles, int nzd, const MarchConfig &cfg,
                      const CUtensorMap *tin, int sm_count, cudaStream_t st) {
  const size_t smem = stencil7_smem_bytes((int)sizeof(T), cfg);
  static size_t attr_set = 0;     // dynamic shared memory opted in so far
  static int occ_cached[17][17];  // [warps][ns] -> CTAs per SM (0 = unknown)
  auto kern = s7_march_kernel<T, K, RY>;
  if (smem > attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = smem;
  }
  const int threads = 32 * cfg.warps;
  // The round-robin schedule assumes every CTA is resident: never launch
  // more per SM than fit.
  int &oc = occ_cached[cfg.warps][cfg.ns];
  if (oc == 0) {
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&oc, kern, threads, smem);
    if (e != cudaSuccess) return e;
    if (oc < 1) oc = 1;
  }
  const int per_sm = (cfg.ctas_per_sm > 0 && cfg.ctas_per_sm < oc) ? cfg.ctas_per_sm : oc;
  const int resident = sm_count * per_sm;
  p.tiles = tiles;
  p.zlen = choose_zchunk(tiles, nzd, resident);
  p.items = (int64_t)tiles * ((nzd + p.zlen - 1) / p.zlen);
  int64_t grid = resident;
  if (grid > p.items) grid = p.items;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, dim3(32, cfg.warps, 1), smem, st>>>(*tin, p);
  return cudaGetLastError();
}

template <typename T, int K>
cudaError_t launch_t(const Stencil7Args &a, const MarchConfig &cfg,
                     const CUtensorMap *tin, int *dev_err, int sm_count,
                     cudaStream_t st) {
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
  if (cfg.warps < 1 || cfg.warps > 16 || cfg.ns < 2 || cfg.ns > 16)
    return cudaErrorInvalidConfiguration;
  const int ty = cfg.warps * cfg.rows;
  p.tiles_x = (ex + TX - 1) / TX;
  const int tiles = p.tiles_x * ((ey + ty - 1) / ty);
  switch (cfg.rows) {
    case 1: return launch_ry<T, K, 1>(p, tiles, ez, cfg, tin, sm_count, st);
    case 2: return launch_ry<T, K, 2>(p, tiles, ez, cfg, tin, sm_count, st);
    case 4: return launch_ry<T, K, 4>(p, tiles, ez, cfg, tin, sm_count, st);
    case 8: return launch_ry<T, K, 8>(p, tiles, ez, cfg, tin, sm_count, st);
  }
  return cudaErrorInvalidConfiguration;
}

template <typename T>
cudaError_t launch_type(const Stencil7Args &a, const MarchConfig &cfg,
                        const CUtensorMap *tin, int *dev_err, int sm_count,
                        cudaStream_t st) {
  switch (a.kernel) {
    case kKernelDiffusion7:
      if constexpr (std::is_floating_point<T>::value)
        return launch_t<T, kKernelDiffusion7>(a, cfg, tin, dev_err, sm_count, st);
      return cudaErrorInvalidValue;
    case kKernelSum7:
      return launch_t<T, kKernelSum7>(a, cfg, tin, dev_err, sm_count, st);
    case kKernelCopy:
      return launch_t<T, kKernelCopy>(a, cfg, tin, dev_err, sm_count, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace

size_t stencil7_smem_bytes(int esz, const MarchConfig &cfg) {
  const int vec = 16 / esz;
  const int w = 32 * vec + 2 * vec;
  const int ty = cfg.warps * cfg.rows;
  // 128 bytes of slack for aligning the dynamic shared-memory base
  return 128 + (size_t)s7_bar_bytes(cfg.ns) +
         (size_t)cfg.ns * s7_stage_bytes((uint32_t)(w * (ty + 2) * esz));
}

cudaError_t launch_stencil7(const Stencil7Args &a, const MarchConfig &cfg,
                            const CUtensorMap *tin, int *dev_err, int sm_count,
                            cudaStream_t s) {
  switch (a.in.type) {
    case kFloat: return launch_type<float>(a, cfg, tin, dev_err, sm_count, s);
    case kDouble: return launch_type<double>(a, cfg, tin, dev_err, sm_count, s);
    case kInt: return launch_type<int>(a, cfg, tin, dev_err, sm_count, s);
    case kLong: return launch_type<long long>(a, cfg, tin, dev_err, sm_count, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace psg
