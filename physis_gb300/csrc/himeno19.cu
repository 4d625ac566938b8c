// Himeno 19-point variable-coefficient Jacobi sweep on GB300 (sm_103a),
// with the residual (gosa = sum of ss*ss) fused into the same pass.
//
// Semantics: the Physis Himeno kernel (examples/himeno/himenobmtxpa_physis.c:
// 331-361), i = x fastest, over the interior domain; cells outside the domain
// are never written.  The residual follows the original benchmark's loop
// (examples/himeno/himenobmtxpa_original.c:331-334), which the Physis port
// dropped; here it costs no extra HBM traffic.
//
// Design (persistent, like the 7-point kernel: (z-chunk, tile) work items in
// chunk-major order taken round-robin by SMs x occupancy CTAs, so resident
// CTAs march the same z-chunk of neighbouring tiles; a tile is 128 x warps
// cells in x,y):
// * p planes with a one-cell y halo and a 4-cell (16-byte) x halo arrive by
//   TMA into a ring of `ns` stages; the sweep at plane z reads planes z-1, z
//   and z+1 from the ring (the 19-point stencil needs xy neighbours on all
//   three planes, so a register queue alone does not suffice);
// * the 12 centre-only coefficient arrays (a0..a3, b0..b2, c0..c2, bnd,
//   wrk1) arrive as 12 TMA boxes of 128 x warps per plane into a second ring
//   of `ns2` stages, all signalled by one mbarrier per stage;
// * one thread per 4 consecutive x cells: 16-byte shared loads, x neighbours
//   by warp shuffles, one 16-byte store;
// * the arithmetic keeps the reference's expression order, round-to-nearest
//   without FMA contraction, so p matches the REF target bit for bit;
// * residual: FP32 per thread, FP32 warp-shuffle + block tree, one FP64
//   partial per CTA, and the last CTA to finish (atomic ticket) adds the
//   partials in FP64 in a fixed order (deterministic run to run).
#include "himeno_body.cuh"

namespace psg {
namespace {

struct HimenoMaps {
  CUtensorMap p;               // p0 with halo box {kHimW, TY+2, 1}
  CUtensorMap coef[kHimCoef];  // box {kHimTX, TY, 1}
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __fadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

template <bool GOSA>
__global__ void __launch_bounds__(256, 1)
himeno19_kernel(const __grid_constant__ HimenoMaps maps, const HParams p) {
  typedef RN<float> R;
  const int TY = blockDim.y;
  const int nsp = p.nsp, nsc = p.nsc;
  const uint32_t p_bytes = (uint32_t)(kHimW * (TY + 2) * 4);
  const int p_elems = (int)(h_align128(p_bytes) / 4);  // stage stride

  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  uint64_t *pfull = reinterpret_cast<uint64_t *>(smem);
  uint64_t *cfull = pfull + nsp;
  float *pring = reinterpret_cast<float *>(smem + h_bar_bytes(nsp + nsc));
  float *cring = pring + nsp * p_elems;
  __shared__ float red[32];
  __shared__ int last_cta;

  const int lane = threadIdx.x, row = threadIdx.y;
  const int tid = row * 32 + lane;
  if (tid == 0) {
    prefetch_tmap(&maps.p);
    for (int s = 0; s < nsp; ++s) mbar_init(&pfull[s], 1);
    for (int s = 0; s < nsc; ++s) mbar_init(&cfull[s], 1);
    fence_barrier_init();
  }
  __syncthreads();

  HRing pprod, pcons, cprod, ccons;
  bool ok = true;
  float acc = 0.0f;
  for (int64_t item = blockIdx.x; item < p.items && ok; item += gridDim.x) {
    const int chunk = (int)(item / p.tiles);
    const int tile = (int)(item - (int64_t)chunk * p.tiles);
    const int zs = p.dmin2 + chunk * p.zlen;
    const int ze = min(zs + p.zlen, p.dmax2);
    ok = himeno_item<GOSA>(&maps.p, maps.coef, p, pfull, cfull, pring, cring, tile, zs, ze,
                           pprod, pcons, cprod, ccons, acc);
  }
  if (!ok) {
    if (tid == 0) {
      // Give copies still in flight a bounded chance to land before exit.
      for (int s = 0; s < nsp; ++s) mbar_wait(&pfull[s], 0, nullptr, 1024);
      for (int s = 0; s < nsc; ++s) mbar_wait(&cfull[s], 0, nullptr, 1024);
    }
    return;
  }
  if (!GOSA) return;

  // Residual: FP32 block tree, FP64 partial per CTA, FP64 final combine.
  acc = warp_sum(acc);
  if (lane == 0) red[row] = acc;
  __syncthreads();
  if (tid == 0) {
    float bs = 0.0f;
    for (int w = 0; w < TY; ++w) bs = __fadd_rn(bs, red[w]);
    p.partials[blockIdx.x] = (double)bs;
    __threadfence();
    const unsigned prev = atomicAdd(p.ticket, 1u);
    last_cta = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (last_cta && row == 0) {
    __threadfence();
    double v = 0.0;
    for (unsigned i = lane; i < gridDim.x; i += 32) v = __dadd_rn(v, __ldcg(&p.partials[i]));
    v = warp_sum(v);
    if (lane == 0) {
      *p.result = v;
      *p.ticket = 0u;
    }
  }
}

}  // namespace

size_t himeno19_smem_bytes(const MarchConfig &cfg) {
  // 128 bytes of slack for aligning the dynamic shared-memory base
  return 128 + (size_t)h_bar_bytes(cfg.ns + cfg.ns2) +
         (size_t)cfg.ns * h_align128((uint32_t)(kHimW * (cfg.warps + 2) * 4)) +
         (size_t)cfg.ns2 * kHimCoef * kHimTX * cfg.warps * 4;
}

cudaError_t launch_himeno19(const Himeno19Args &a, const MarchConfig &cfg,
                            const CUtensorMap *tmaps, const ResidualSink &sink,
                            int *dev_err, int sm_count, cudaStream_t s) {
  HimenoMaps maps;
  maps.p = tmaps[0];
  for (int i = 0; i < kHimCoef; ++i) maps.coef[i] = tmaps[1 + i];
  HParams p;
  const GridView &out = a.g[1];
  p.out = static_cast<float *>(out.ptr);
  p.row = out.pitch / 4;
  p.plane = p.row * out.ny;
  p.dmin0 = a.dom.min[0];
  p.dmin1 = a.dom.min[1];
  p.dmin2 = a.dom.min[2];
  p.dmax0 = a.dom.max[0];
  p.dmax1 = a.dom.max[1];
  p.dmax2 = a.dom.max[2];
  p.xbase = (a.dom.min[0] / 4) * 4;
  p.nsp = cfg.ns;
  p.nsc = cfg.ns2;
  p.omega = a.omega;
  p.partials = sink.partials;
  p.ticket = sink.ticket;
  p.result = sink.result;
  p.err = dev_err;
  const int ex = a.dom.max[0] - p.xbase;
  const int ey = a.dom.max[1] - a.dom.min[1];
  const int ez = a.dom.max[2] - a.dom.min[2];
  if (ex <= 0 || ey <= 0 || ez <= 0) return cudaSuccess;
  if (cfg.warps < 1 || cfg.warps > 8 || cfg.ns < 3 || cfg.ns > 16 || cfg.ns2 < 1 ||
      cfg.ns2 > 8)
    return cudaErrorInvalidConfiguration;
  p.tiles_x = (ex + kHimTX - 1) / kHimTX;
  p.tiles = p.tiles_x * ((ey + cfg.warps - 1) / cfg.warps);
  const size_t smem = himeno19_smem_bytes(cfg);
  // Opt in to the dynamic shared memory this launch needs (the kernel also
  // has a little static shared memory, so the opt-in is the exact size).
  static size_t attr_set[2] = {0, 0};
  static int occ[2][9][17][9];  // [gosa][warps][ns][ns2] -> CTAs per SM
  auto kern = a.gosa ? himeno19_kernel<true> : himeno19_kernel<false>;
  size_t &have = attr_set[a.gosa ? 1 : 0];
  if (smem > have) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    have = smem;
  }
  // The round-robin schedule assumes every CTA is resident: never launch
  // more per SM than fit.
  int &oc = occ[a.gosa ? 1 : 0][cfg.warps][cfg.ns][cfg.ns2];
  if (oc == 0) {
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&oc, kern, 32 * cfg.warps,
                                                                  smem);
    if (e != cudaSuccess) return e;
    if (oc < 1) oc = 1;
  }
  const int per_sm = (cfg.ctas_per_sm > 0 && cfg.ctas_per_sm < oc) ? cfg.ctas_per_sm : oc;
  const int resident = sm_count * per_sm;
  p.zlen = choose_zchunk(p.tiles, ez, resident);
  p.items = (int64_t)p.tiles * ((ez + p.zlen - 1) / p.zlen);
  int64_t grid = resident;
  if (grid > p.items) grid = p.items;
  if (a.gosa && grid > sink.max_partials) grid = sink.max_partials;
  kern<<<(unsigned)grid, dim3(32, cfg.warps, 1), smem, s>>>(maps, p);
  return cudaGetLastError();
}

}  // namespace psg
