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
// * Each z-plane of the tile plus its x/y halo arrives in a ring of
//   shared-memory planes by one TMA 3D box load (mbarrier per stage, bounded
//   waits).  A box cannot wrap and fills cells outside the grid with zeros,
//   so on the edge tiles of periodic and clamped stencils those halo cells
//   are then rewritten through the boundary map (periodic cells from the
//   opposite face, clamped ones from the face); the compute loop is the same
//   for every rule.  Grids without a tensor map are staged with cp.async
//   through the boundary map instead (16-byte copies inside the grid,
//   element copies across an edge).
// * The ring holds rzl + rzh + 1 planes for the stencil's z extent plus
//   planes in flight ahead of the newest one a step reads.
// * The sweep body (points_body.cuh) is compiled two ways: here with the
//   point table (shared-memory offset, plane lag, weight) copied to shared
//   memory once per CTA and walked in order, and by jit.cpp with NVRTC per
//   stencil, the table baked in as constants.  The runtime uses the compiled
//   form when NVRTC is present (PS_POINTS_JIT=0 forces the table form).
// * Arithmetic is round-to-nearest without FMA contraction in the point
//   order, so results are bit-identical to the REF loops.
// * Red/black (color 0/1) writes only cells with (x + y + z + color) even --
//   the cells the REF loop start min + ((min & 1) ^ ((y + z + color) % 2))
//   visits -- in place.  The host admits only stencils whose non-centre
//   points all have odd parity, so a pass never reads a cell it writes
//   (other than each cell's own centre) and the parallel result equals the
//   sequential REF one.
#include <cstdlib>
#include <cstring>

#include "points_body.cuh"
#include "ps_internal.h"

namespace psg {
namespace {

template <typename T, int RY, bool UNIT>
__global__ void __launch_bounds__(512, 1)
pts_kernel(const __grid_constant__ PtsParams<T> p, const __grid_constant__ PtsTmap tm) {
  extern __shared__ __align__(128) unsigned char smem[];
  pts_body<T, RY, UNIT, PtsTableSpec>(p, &tm, smem);
}

// Planes in flight ahead of the newest plane a step reads: the cp.async ring
// waits with wait_group<kPtsPrefetch>; a TMA plane lands in one copy, and one
// plane ahead is enough (measured at 512^3: two or three planes ahead run the
// 7-point stencil 4-15 % and the 27-point 1-2 % slower, whatever the tile).
// PS_POINTS_PREFETCH=<1..4> overrides the TMA depth (a tuning knob).
int points_prefetch(bool tma) {
  if (!tma) return kPtsPrefetch;
  static const int depth = [] {
    const char *e = getenv("PS_POINTS_PREFETCH");
    const int v = e ? atoi(e) : 0;
    return (v >= 1 && v <= 4) ? v : 1;
  }();
  return depth;
}

// Offsets' extent per axis: lo <= 0 <= hi.
void extents(const PointsArgs &a, int lo[3], int hi[3]) {
  for (int d = 0; d < 3; ++d) lo[d] = hi[d] = 0;
  for (int i = 0; i < a.n; ++i)
    for (int d = 0; d < 3; ++d) {
      lo[d] = a.d[i][d] < lo[d] ? a.d[i][d] : lo[d];
      hi[d] = a.d[i][d] > hi[d] ? a.d[i][d] : hi[d];
    }
}

// Fills everything but zlen / items (those need the occupancy).
template <typename T>
void fill_params(const PointsArgs &a, int warps, int ry, PtsParams<T> *pp) {
  constexpr int VEC = 16 / (int)sizeof(T);
  PtsParams<T> &p = *pp;
  memset(&p, 0, sizeof(p));
  p.in = static_cast<const T *>(a.in.ptr);
  p.out = static_cast<T *>(a.out.ptr);
  p.row = a.in.pitch / (long long)sizeof(T);
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
  int lo[3], hi[3];
  extents(a, lo, hi);
  p.ryl = -lo[1];
  p.rzl = -lo[2];
  p.rzh = hi[2];
  p.lp = (-lo[0] + VEC - 1) / VEC * VEC;
  const int rp = (hi[0] + VEC - 1) / VEC * VEC;
  p.w = p.lp + kPtsTX + rp;
  const int TY = warps * ry;
  p.rows_h = TY + p.ryl + hi[1];
  p.nstage = p.rzl + p.rzh + 1 + points_prefetch(a.has_tmap);
  p.plane_elems = p.rows_h * p.w;
  p.pstride = (int)(((size_t)p.plane_elems * sizeof(T) + 127) / 128 * 128 / sizeof(T));
  p.use_tma = a.has_tmap ? 1 : 0;
  p.err = a.err;
  for (int i = 0; i < a.n; ++i) {
    p.off[i] = (p.ryl + a.d[i][1]) * p.w + p.lp + a.d[i][0];
    p.lag[i] = p.rzl + a.d[i][2];
    p.wt[i] = (T)a.w[i];
  }
  p.xbase = a.dom.min[0] / VEC * VEC;
  p.tiles_x = (a.dom.max[0] - p.xbase + kPtsTX - 1) / kPtsTX;
  const int tiles_y = (a.dom.max[1] - a.dom.min[1] + TY - 1) / TY;
  p.tiles = p.tiles_x * tiles_y;
}

// zlen, items and the grid size for `occ` resident CTAs per SM.
template <typename T>
int schedule(PtsParams<T> *p, int occ, int sm_count) {
  const int resident = sm_count * occ;
  const int nzd = p->dmax2 - p->dmin2;
  p->zlen = choose_zchunk_overhead(p->tiles, nzd, resident, p->rzl + p->rzh + 1);
  const int chunks = (nzd + p->zlen - 1) / p->zlen;
  p->items = (long long)p->tiles * chunks;
  return (int)(p->items < resident ? p->items : resident);
}

template <typename T>
size_t smem_for(const PtsParams<T> &p) {
  return 128 + (size_t)kPtsRingOffset + (size_t)p.nstage * p.pstride * sizeof(T);
}

bool jit_enabled() {
  const char *e = getenv("PS_POINTS_JIT");
  return !(e && e[0] == '0');
}

template <typename T, int RY, bool UNIT>
cudaError_t launch_t(const PointsArgs &a, int warps, int sm_count, cudaStream_t s) {
  PtsParams<T> p;
  fill_params<T>(a, warps, RY, &p);
  const size_t smem = smem_for(p);
  PtsTmap tm;
  memset(&tm, 0, sizeof(tm));
  static_assert(sizeof(PtsTmap) == sizeof(CUtensorMap), "tensor map layout");
  if (a.has_tmap) memcpy(&tm, &a.tmap, sizeof(tm));
  if (jit_enabled()) {
    // The stencil compiled with its table as constants (cached per stencil,
    // type and tile shape); on any failure the table kernel below runs.
    PtsJitKey key;
    memset(&key, 0, sizeof(key));
    key.type = a.in.type;
    key.ry = RY;
    key.warps = warps;
    key.n = a.n;
    key.unit = UNIT;
    key.w = p.w;
    key.nstage = p.nstage;
    key.pstride = p.pstride;
    for (int i = 0; i < a.n; ++i) {
      key.off[i] = p.off[i];
      key.lag[i] = p.lag[i];
      key.wt[i] = UNIT ? 1.0 : a.w[i];
    }
    void *fn = jit_points_function(key);
    int occ = 0;
    if (fn && jit_prepare(fn, 32 * warps, smem, &occ) && occ >= 1) {
      const int grid = schedule(&p, occ, sm_count);
      void *args[2] = {&p, &tm};
      return jit_launch_raw(fn, grid, dim3(32, warps, 1), smem, s, args);
    }
  }
  auto kern = pts_kernel<T, RY, UNIT>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  int occ = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 32 * warps, smem);
  if (e != cudaSuccess) return e;
  if (occ < 1) return cudaErrorInvalidConfiguration;
  const int grid = schedule(&p, occ, sm_count);
  kern<<<grid, dim3(32, warps, 1), smem, s>>>(p, tm);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_type(const PointsArgs &a, const MarchConfig &cfg, int sm_count,
                        cudaStream_t s) {
  const int warps = cfg.warps;
  if (cfg.rows >= 4)
    return a.unit ? launch_t<T, 4, true>(a, warps, sm_count, s)
                  : launch_t<T, 4, false>(a, warps, sm_count, s);
  if (cfg.rows >= 2)
    return a.unit ? launch_t<T, 2, true>(a, warps, sm_count, s)
                  : launch_t<T, 2, false>(a, warps, sm_count, s);
  return a.unit ? launch_t<T, 1, true>(a, warps, sm_count, s)
                : launch_t<T, 1, false>(a, warps, sm_count, s);
}

}  // namespace

int points_rows(const MarchConfig &cfg) { return cfg.rows >= 4 ? 4 : (cfg.rows >= 2 ? 2 : 1); }

void points_box(const PointsArgs &a, const MarchConfig &cfg, int *w, int *h) {
  const int vec = 16 / a.in.esz;
  int lo[3], hi[3];
  extents(a, lo, hi);
  *w = (-lo[0] + vec - 1) / vec * vec + kPtsTX + (hi[0] + vec - 1) / vec * vec;
  *h = cfg.warps * points_rows(cfg) - lo[1] + hi[1];
}

size_t points_smem_bytes(const PointsArgs &a, const MarchConfig &cfg) {
  int lo[3], hi[3], w, h;
  extents(a, lo, hi);
  points_box(a, cfg, &w, &h);
  const int nstage = -lo[2] + hi[2] + 1 + points_prefetch(a.has_tmap);
  const size_t stage = ((size_t)w * h * a.in.esz + 127) / 128 * 128;
  return 128 + (size_t)kPtsRingOffset + (size_t)nstage * stage;
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
