// Point-list stencils and red/black sweeps on GB300 (sm_103a).
//
// Replaces the translator-generated run kernels of the reference
// (translator/cuda_runtime_builder.cc:1099-1228, red/black offsets
// 1206-1226; REF loops translator/reference_runtime_builder.cc:585-664) for
// stencils of the form
//     out(x,y,z) = w0*in(p0) + w1*in(p1) + ... + w(n-1)*in(p(n-1))
// evaluated left to right, p_i = (x+dx_i, y+dy_i, z+dz_i) mapped per axis by a
// boundary rule (none / periodic (i + n) % n, include/physis/physis_cuda.h:
// 247-269 / clamp to the grid).  With unit weights this is exactly the
// neighbour sums of the reference's system tests (27-point, 9-point 2D,
// 3-point 1D, asymmetric, hole, periodic variants, red/black).
//
// Design.  A tile is 128 cells wide in x (32 lanes x 4 columns, lane-strided
// so that every shared-memory access of a warp is conflict-free) and
// warps*RY rows high; work items are (z-chunk, tile) pairs in chunk-major
// order taken round-robin by a persistent grid, as in the 7-point kernels.
// * Each z-plane of the tile plus its x/y halo is copied into a ring of
//   shared-memory planes with cp.async: 16-byte copies for the aligned chunks
//   inside the grid, element copies through the boundary map for the chunks
//   that cross an edge.  The boundary rule is applied once, at load time
//   (periodic halo cells are fetched from the opposite face, clamped ones
//   from the face), so the compute loop is the same for every rule.
//   (TMA box loads cannot wrap, hence cp.async here.)
// * The ring holds rzl + rzh + 1 planes for the stencil's z extent plus
//   kPrefetch planes in flight; one commit group per plane, and
//   cp.async.wait_group keeps kPrefetch planes outstanding.
// * The point table (shared-memory offset, plane lag, weight) is copied to
//   shared memory once per CTA; the compute loop walks it in order.
// * Arithmetic is round-to-nearest without FMA contraction in the point
//   order, so results are bit-identical to the REF loops.
// * Red/black (color 0/1) writes only cells with (x + y + z + color) even --
//   the cells the REF loop start min + ((min & 1) ^ ((y + z + color) % 2))
//   visits -- in place.  The host admits only stencils whose non-centre
//   points all have odd parity, so a pass never reads a cell it writes
//   (other than each cell's own centre) and the parallel result equals the
//   sequential REF one.
#include "ps_device.cuh"
#include "ps_internal.h"

namespace psg {
namespace {

constexpr int kTX = 128;      // tile width in cells
constexpr int kVX = 4;        // columns per lane (lane + 32*j)
constexpr int kPrefetch = 2;  // planes in flight ahead of the newest needed plane
// Point table in shared memory: offsets, plane lags, weights (8-byte slots).
constexpr int kTableBytes = kMaxPoints * (4 + 4 + 8);

template <typename T>
struct PtsParams {
  const T *in;
  T *out;          // may equal in (red/black)
  int64_t row;     // pitch in elements
  int64_t plane;   // elements per z-plane
  int nx, ny, nz;
  int dmin0, dmin1, dmin2, dmax0, dmax1, dmax2;
  int boundary;    // kBoundaryNone / Periodic / Clamp
  int color;       // -1 every cell, 0 red, 1 black
  int n;           // points
  int ryl, rzl, rzh;
  int lp, w, rows_h, nstage, plane_elems;
  int xbase, tiles_x, tiles, zlen;
  int64_t items;
  int off[kMaxPoints];  // shared offset of point i relative to the cell
  int lag[kMaxPoints];  // rzl + dz_i: the point's plane relative to z - rzl
  T wt[kMaxPoints];
};

// Grid index of coordinate i on an axis of n cells.  Periodic: i mod n, which
// equals the reference's (i + n) % n for every i >= -n (the host admits only
// offsets with |d| <= n, so every read that is used has i >= -n; halo cells
// that are never read may lie further out and still land inside the grid).
// Clamp, and the never-read halo of boundary "none": the nearest face.
__device__ __forceinline__ int map_axis(int i, int n, int boundary) {
  if (boundary == kBoundaryPeriodic) {
    const int m = i % n;
    return m < 0 ? m + n : m;
  }
  return min(max(i, 0), n - 1);
}

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

// Issues the copies of global plane zg (tile origin x0, y0) into `dst`.
template <typename T>
__device__ __forceinline__ void load_plane(const PtsParams<T> &p, T *dst, int zg, int x0,
                                           int y0) {
  constexpr int VEC = 16 / (int)sizeof(T);
  const T *src_plane = p.in + (int64_t)map_axis(zg, p.nz, p.boundary) * p.plane;
  const int nchunk = p.w / VEC;
  const int xs = x0 - p.lp;
  for (int r = threadIdx.y; r < p.rows_h; r += blockDim.y) {
    const T *src = src_plane + (int64_t)map_axis(y0 - p.ryl + r, p.ny, p.boundary) * p.row;
    T *d = dst + r * p.w;
    for (int c = threadIdx.x; c < nchunk; c += 32) {
      const int x = xs + c * VEC;
      if (x >= 0 && x + VEC <= p.nx) {
        cp_async16(d + c * VEC, src + x);
      } else {
#pragma unroll
        for (int i = 0; i < VEC; ++i)
          cp_async_small<sizeof(T)>(d + c * VEC + i, src + map_axis(x + i, p.nx, p.boundary));
      }
    }
  }
}

template <typename T, int RY, bool UNIT>
__global__ void __launch_bounds__(512, 1)
pts_kernel(const __grid_constant__ PtsParams<T> p) {
  typedef RN<T> R;
  extern __shared__ __align__(128) unsigned char smem[];
  int *s_off = reinterpret_cast<int *>(smem);
  int *s_lag = s_off + kMaxPoints;
  T *s_w = reinterpret_cast<T *>(smem + kMaxPoints * 8);
  T *ring = reinterpret_cast<T *>(smem + kTableBytes);

  const int lane = threadIdx.x, warp = threadIdx.y;
  const int tid = warp * 32 + lane;
  for (int i = tid; i < p.n; i += blockDim.x * blockDim.y) {
    s_off[i] = p.off[i];
    s_lag[i] = p.lag[i];
    s_w[i] = p.wt[i];
  }
  __syncthreads();

  const int TY = blockDim.y * RY;
  const int pre = p.nstage - 1;  // planes issued before the first compute step
  const int cell0 = warp * RY * p.w + lane;

  for (int64_t item = blockIdx.x; item < p.items; item += gridDim.x) {
    const int chunk = (int)(item / p.tiles);
    const int tile = (int)(item - (int64_t)chunk * p.tiles);
    const int zs = p.dmin2 + chunk * p.zlen;
    const int ze = min(zs + p.zlen, p.dmax2);
    const int x0 = p.xbase + (tile % p.tiles_x) * kTX;
    const int y0 = p.dmin1 + (tile / p.tiles_x) * TY;
    const int nplanes = ze - zs + p.rzl + p.rzh;  // planes zs-rzl .. ze+rzh-1

    int ld = 0;  // ring slot of the next plane to issue
    for (int q = 0; q < pre; ++q) {
      if (q < nplanes) load_plane(p, ring + ld * p.plane_elems, zs - p.rzl + q, x0, y0);
      cp_async_commit();
      if (++ld == p.nstage) ld = 0;
    }
    int cs = 0;  // ring slot of plane z - rzl
    for (int z = zs; z < ze; ++z) {
      const int q = z - zs + pre;
      if (q < nplanes) load_plane(p, ring + ld * p.plane_elems, zs - p.rzl + q, x0, y0);
      cp_async_commit();
      if (++ld == p.nstage) ld = 0;
      cp_async_wait<kPrefetch>();  // planes up to z + rzh have landed
      __syncthreads();

      T acc[RY][kVX];
      {
        int s = cs + s_lag[0];
        if (s >= p.nstage) s -= p.nstage;
        const T *src = ring + s * p.plane_elems + s_off[0] + cell0;
        const T wk = s_w[0];
#pragma unroll
        for (int r = 0; r < RY; ++r)
#pragma unroll
          for (int j = 0; j < kVX; ++j) {
            const T v = src[r * p.w + 32 * j];
            acc[r][j] = UNIT ? v : R::mul(wk, v);
          }
      }
      for (int k = 1; k < p.n; ++k) {
        int s = cs + s_lag[k];
        if (s >= p.nstage) s -= p.nstage;
        const T *src = ring + s * p.plane_elems + s_off[k] + cell0;
        const T wk = s_w[k];
#pragma unroll
        for (int r = 0; r < RY; ++r)
#pragma unroll
          for (int j = 0; j < kVX; ++j) {
            const T v = src[r * p.w + 32 * j];
            acc[r][j] = R::add(acc[r][j], UNIT ? v : R::mul(wk, v));
          }
      }

#pragma unroll
      for (int r = 0; r < RY; ++r) {
        const int y = y0 + warp * RY + r;
        if (y >= p.dmax1) continue;
        T *dst = p.out + (int64_t)z * p.plane + (int64_t)y * p.row;
#pragma unroll
        for (int j = 0; j < kVX; ++j) {
          const int x = x0 + lane + 32 * j;
          const bool in_dom = x >= p.dmin0 && x < p.dmax0;
          const bool colored = p.color < 0 || ((x + y + z + p.color) & 1) == 0;
          if (in_dom && colored) dst[x] = acc[r][j];
        }
      }
      if (++cs == p.nstage) cs = 0;
      __syncthreads();  // the slot of plane z - rzl is refilled next step
    }
    cp_async_wait<0>();  // only empty groups can remain
  }
}

struct Shape {
  int warps, ry;
};

template <typename T>
size_t smem_for(int rows_h, int w, int nstage) {
  return (size_t)kTableBytes + (size_t)nstage * rows_h * w * sizeof(T);
}

template <typename T, int RY, bool UNIT>
cudaError_t launch_t(const PointsArgs &a, int warps, int sm_count, cudaStream_t s) {
  constexpr int VEC = 16 / (int)sizeof(T);
  PtsParams<T> p;
  p.in = static_cast<const T *>(a.in.ptr);
  p.out = static_cast<T *>(a.out.ptr);
  p.row = a.in.pitch / (int64_t)sizeof(T);
  p.plane = p.row * a.in.ny;
  p.nx = a.in.nx;
  p.ny = a.in.ny;
  p.nz = a.in.nz;
  p.dmin0 = a.dom.min[0];
  p.dmin1 = a.dom.min[1];
  p.dmin2 = a.dom.min[2];
  p.dmax0 = a.dom.max[0];
  p.dmax1 = a.dom.max[1];
  p.dmax2 = a.dom.max[2];
  p.boundary = a.boundary;
  p.color = a.color;
  p.n = a.n;
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (int i = 0; i < a.n; ++i)
    for (int d = 0; d < 3; ++d) {
      lo[d] = min(lo[d], a.d[i][d]);
      hi[d] = max(hi[d], a.d[i][d]);
    }
  p.ryl = -lo[1];
  p.rzl = -lo[2];
  p.rzh = hi[2];
  p.lp = (-lo[0] + VEC - 1) / VEC * VEC;
  const int rp = (hi[0] + VEC - 1) / VEC * VEC;
  p.w = p.lp + kTX + rp;
  const int TY = warps * RY;
  p.rows_h = TY + p.ryl + hi[1];
  p.nstage = p.rzl + p.rzh + 1 + kPrefetch;
  p.plane_elems = p.rows_h * p.w;
  for (int i = 0; i < a.n; ++i) {
    p.off[i] = (p.ryl + a.d[i][1]) * p.w + p.lp + a.d[i][0];
    p.lag[i] = p.rzl + a.d[i][2];
    p.wt[i] = (T)a.w[i];
  }
  p.xbase = a.dom.min[0] / VEC * VEC;
  p.tiles_x = (a.dom.max[0] - p.xbase + kTX - 1) / kTX;
  const int tiles_y = (a.dom.max[1] - a.dom.min[1] + TY - 1) / TY;
  p.tiles = p.tiles_x * tiles_y;

  const size_t smem = smem_for<T>(p.rows_h, p.w, p.nstage);
  auto kern = pts_kernel<T, RY, UNIT>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  int occ = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32 * warps, smem);
  if (e != cudaSuccess) return e;
  if (occ < 1) return cudaErrorInvalidConfiguration;
  const int resident = sm_count * occ;
  const int nzd = a.dom.max[2] - a.dom.min[2];
  p.zlen = choose_zchunk_overhead(p.tiles, nzd, resident, p.rzl + p.rzh + 1);
  const int chunks = (nzd + p.zlen - 1) / p.zlen;
  p.items = (int64_t)p.tiles * chunks;
  const int grid = (int)(p.items < resident ? p.items : resident);
  kern<<<grid, dim3(32, warps, 1), smem, s>>>(p);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_type(const PointsArgs &a, const MarchConfig &cfg, int sm_count,
                        cudaStream_t s) {
  const int warps = cfg.warps;
  if (cfg.rows >= 2)
    return a.unit ? launch_t<T, 2, true>(a, warps, sm_count, s)
                  : launch_t<T, 2, false>(a, warps, sm_count, s);
  return a.unit ? launch_t<T, 1, true>(a, warps, sm_count, s)
                : launch_t<T, 1, false>(a, warps, sm_count, s);
}

}  // namespace

size_t points_smem_bytes(const PointsArgs &a, const MarchConfig &cfg) {
  const int esz = a.in.esz;
  const int vec = 16 / esz;
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (int i = 0; i < a.n; ++i)
    for (int d = 0; d < 3; ++d) {
      lo[d] = lo[d] < a.d[i][d] ? lo[d] : a.d[i][d];
      hi[d] = hi[d] > a.d[i][d] ? hi[d] : a.d[i][d];
    }
  const int w = (-lo[0] + vec - 1) / vec * vec + kTX + (hi[0] + vec - 1) / vec * vec;
  const int rows_h = cfg.warps * (cfg.rows >= 2 ? 2 : 1) - lo[1] + hi[1];
  const int nstage = -lo[2] + hi[2] + 1 + kPrefetch;
  return (size_t)kTableBytes + (size_t)nstage * rows_h * w * esz;
}

cudaError_t launch_points(const PointsArgs &a, const MarchConfig &cfg, int sm_count,
                          cudaStream_t s) {
  if (a.n < 1 || a.n > kMaxPoints || cfg.warps < 1 || cfg.warps > 16)
    return cudaErrorInvalidValue;
  if (a.dom.min[0] >= a.dom.max[0] || a.dom.min[1] >= a.dom.max[1] ||
      a.dom.min[2] >= a.dom.max[2])
    return cudaSuccess;
  switch (a.in.type) {
    case kFloat: return launch_type<float>(a, cfg, sm_count, s);
    case kDouble: return launch_type<double>(a, cfg, sm_count, s);
    case kInt: return launch_type<int>(a, cfg, sm_count, s);
    default: return launch_type<long long>(a, cfg, sm_count, s);
  }
}

}  // namespace psg
