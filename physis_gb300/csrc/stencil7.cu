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

#include "s7_body.cuh"

namespace psg {
namespace {

template <typename T, int K, int RY>
__global__ void __launch_bounds__(512, 1)
s7_march_kernel(const __grid_constant__ CUtensorMap tin, const S7Params<T> p) {
  constexpr int VEC = 16 / (int)sizeof(T);
  constexpr int W = 34 * VEC;  // shared row width in elements
  const int TY = blockDim.y * RY;
  // Each ring stage starts on a 128-byte boundary (required of the shared
  // destination of cp.async.bulk.tensor).
  const uint32_t plane_bytes = (uint32_t)(W * (TY + 2) * sizeof(T));
  const int plane_elems = (int)(s7_stage_bytes(plane_bytes) / sizeof(T));

  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);
  T *ring = reinterpret_cast<T *>(smem + s7_bar_bytes(p.ns));

  const int tid = threadIdx.y * 32 + threadIdx.x;
  if (tid == 0) {
    prefetch_tmap(&tin);
    for (int s = 0; s < p.ns; ++s) mbar_init(&full[s], 1);
    fence_barrier_init();
  }
  __syncthreads();

  // Producer (thread 0) and consumer (all threads) positions in the ring.
  RingPos prod, cons;
  bool ok = true;
  for (int64_t item = blockIdx.x; item < p.items && ok; item += gridDim.x) {
    const int chunk = (int)(item / p.tiles);
    const int tile = (int)(item - (int64_t)chunk * p.tiles);
    const int zs = p.dmin2 + chunk * p.zlen;
    const int ze = min(zs + p.zlen, p.dmax2);
    ok = s7_item<T, K, RY>(&tin, p, full, ring, plane_elems, plane_bytes, TY, tile, zs, ze,
                           prod, cons);
  }
  if (!ok && tid == 0) {
    // Give copies still in flight a bounded chance to land before exit.
    for (int s = 0; s < p.ns; ++s) mbar_wait(&full[s], 0, nullptr, 1024);
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
