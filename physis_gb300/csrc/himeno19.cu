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
#include "ps_device.cuh"
#include "ps_internal.h"

namespace psg {
namespace {

constexpr int kTX = 128;      // tile width in cells (32 lanes x float4)
constexpr int kW = kTX + 8;   // shared p row width (4-cell halo each side)
constexpr int kNumCoef = 12;  // a0 a1 a2 a3 b0 b1 b2 c0 c1 c2 bnd wrk1

struct HimenoMaps {
  CUtensorMap p;               // p0 with halo box {kW, TY+2, 1}
  CUtensorMap coef[kNumCoef];  // box {kTX, TY, 1}
};

struct HParams {
  float *out;
  int64_t row, plane;  // out pitch / plane in elements
  int dmin0, dmin1, dmin2, dmax0, dmax1, dmax2;
  int xbase, tiles_x, tiles, zlen;
  int64_t items;
  int nsp, nsc;
  float omega;
  double *partials;
  unsigned *ticket;
  double *result;
  int *err;
};

__host__ __device__ constexpr int h_bar_bytes(int n) { return 128 * ((8 * n + 127) / 128); }
// Every TMA destination starts on a 128-byte boundary.
__host__ __device__ constexpr uint32_t h_align128(uint32_t b) { return (b + 127u) & ~127u; }

__device__ __forceinline__ void row6(const float *pl, int idx, int lane, float (&r)[6]) {
  float v[4];
  ld16_shared<float>(v, pl + idx);
  float l = shfl_up1(v[3]);
  float rr = shfl_down1(v[0]);
  if (lane == 0) l = pl[idx - 1];
  if (lane == 31) rr = pl[idx + 4];
  r[0] = l;
  r[1] = v[0];
  r[2] = v[1];
  r[3] = v[2];
  r[4] = v[3];
  r[5] = rr;
}

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

// Position in a ring of mbarrier-signalled stages used in issue order.
struct Ring {
  int stage = 0;
  uint32_t phase = 0;
  __device__ __forceinline__ void advance(int n) {
    if (++stage == n) {
      stage = 0;
      phase ^= 1u;
    }
  }
};

template <bool GOSA>
__global__ void __launch_bounds__(256, 1)
himeno19_kernel(const __grid_constant__ HimenoMaps maps, const HParams p) {
  typedef RN<float> R;
  const int TY = blockDim.y;
  const int nsp = p.nsp, nsc = p.nsc;
  const uint32_t p_bytes = (uint32_t)(kW * (TY + 2) * 4);
  const int p_elems = (int)(h_align128(p_bytes) / 4);  // stage stride
  const int c_tile = kTX * TY;                         // elements per coefficient tile
  const int c_elems = kNumCoef * c_tile;               // elements per coefficient stage
  const uint32_t c_bytes = (uint32_t)(c_elems * 4);

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

  Ring pprod, pcons, cprod, ccons;
  bool ok = true;
  float acc = 0.0f;
  const int cen = (row + 1) * kW + 4 + lane * 4;
  const int cidx = row * kTX + lane * 4;

  for (int64_t item = blockIdx.x; item < p.items && ok; item += gridDim.x) {
    const int chunk = (int)(item / p.tiles);
    const int tile = (int)(item - (int64_t)chunk * p.tiles);
    const int zs = p.dmin2 + chunk * p.zlen;
    const int ze = min(zs + p.zlen, p.dmax2);
    const int x0 = p.xbase + (tile % p.tiles_x) * kTX;
    const int y0 = p.dmin1 + (tile / p.tiles_x) * TY;
    const int nplanes = ze - zs + 2;  // p planes zs-1 .. ze
    const int ncoef = ze - zs;        // coefficient planes zs .. ze-1

    auto issue_p = [&](int q) {
      const int s = pprod.stage;
      mbar_arrive_expect_tx(&pfull[s], p_bytes);
      tma_load_3d(pring + s * p_elems, &maps.p, x0 - 4, y0 - 1, zs - 1 + q, &pfull[s]);
      pprod.advance(nsp);
    };
    auto issue_c = [&](int r) {
      const int s = cprod.stage;
      mbar_arrive_expect_tx(&cfull[s], c_bytes);
      float *dst = cring + s * c_elems;
#pragma unroll 1
      for (int a = 0; a < kNumCoef; ++a)
        tma_load_3d(dst + a * c_tile, &maps.coef[a], x0, y0, zs + r, &cfull[s]);
      cprod.advance(nsc);
    };
    auto wait_p = [&]() -> const float * {
      if (!mbar_wait(&pfull[pcons.stage], pcons.phase, p.err)) ok = false;
      const float *pl = pring + pcons.stage * p_elems;
      pcons.advance(nsp);
      return pl;
    };
    auto wait_c = [&]() -> const float * {
      if (!mbar_wait(&cfull[ccons.stage], ccons.phase, p.err)) ok = false;
      const float *pl = cring + ccons.stage * c_elems;
      ccons.advance(nsc);
      return pl;
    };

    if (tid == 0) {
      for (int q = 0; q < min(nsp, nplanes); ++q) issue_p(q);
      for (int r = 0; r < min(nsc, ncoef); ++r) issue_c(r);
    }
    const int y = y0 + row;
    const int x = x0 + lane * 4;
    const bool row_in = (y < p.dmax1);
    const bool vec_in = (x >= p.dmin0) && (x + 4 <= p.dmax0);

    const float *pm = wait_p();  // plane zs-1
    const float *pc = wait_p();  // plane zs
    for (int z = zs; z < ze; ++z) {
      const int r = z - zs;
      const float *pp = wait_p();  // plane z+1
      const float *cf = wait_c();  // coefficients of plane z

      float Zc[6], Zym[6], Zyp[6], Zpc[6], Zmc[6];
      float Zpyp[4], Zpym[4], Zmyp[4], Zmym[4];
      row6(pc, cen, lane, Zc);
      row6(pc, cen - kW, lane, Zym);
      row6(pc, cen + kW, lane, Zyp);
      row6(pp, cen, lane, Zpc);
      row6(pm, cen, lane, Zmc);
      ld16_shared<float>(Zpyp, pp + cen + kW);
      ld16_shared<float>(Zpym, pp + cen - kW);
      ld16_shared<float>(Zmyp, pm + cen + kW);
      ld16_shared<float>(Zmym, pm + cen - kW);
      float co[kNumCoef][4];
#pragma unroll
      for (int a = 0; a < kNumCoef; ++a) ld16_shared<float>(co[a], cf + a * c_tile + cidx);

      float o[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        // s0 = a0*p(k+1) + a1*p(j+1) + a2*p(i+1) + b0*(..) + b1*(..) + b2*(..)
        //    + c0*p(k-1) + c1*p(j-1) + c2*p(i-1) + wrk1   (left to right)
        float s0 = R::mul(co[0][i], Zpc[i + 1]);
        s0 = R::add(s0, R::mul(co[1][i], Zyp[i + 1]));
        s0 = R::add(s0, R::mul(co[2][i], Zc[i + 2]));
        float t0 = R::add(R::sub(R::sub(Zpyp[i], Zpym[i]), Zmyp[i]), Zmym[i]);
        s0 = R::add(s0, R::mul(co[4][i], t0));
        float t1 = R::add(R::sub(R::sub(Zyp[i + 2], Zym[i + 2]), Zyp[i]), Zym[i]);
        s0 = R::add(s0, R::mul(co[5][i], t1));
        float t2 = R::add(R::sub(R::sub(Zpc[i + 2], Zmc[i + 2]), Zpc[i]), Zmc[i]);
        s0 = R::add(s0, R::mul(co[6][i], t2));
        s0 = R::add(s0, R::mul(co[7][i], Zmc[i + 1]));
        s0 = R::add(s0, R::mul(co[8][i], Zym[i + 1]));
        s0 = R::add(s0, R::mul(co[9][i], Zc[i]));
        s0 = R::add(s0, co[11][i]);
        // ss = (s0*a3 - p) * bnd ; p1 = p + omega*ss
        const float ss = R::mul(R::sub(R::mul(s0, co[3][i]), Zc[i + 1]), co[10][i]);
        o[i] = R::add(Zc[i + 1], R::mul(p.omega, ss));
        if (GOSA) {
          const bool in = row_in && (x + i >= p.dmin0) && (x + i < p.dmax0);
          if (in) acc = R::add(acc, R::mul(ss, ss));
        }
      }
      if (ok && row_in) {
        float *dst = p.out + (int64_t)z * p.plane + (int64_t)y * p.row + x;
        if (vec_in) {
          st16_global<float>(dst, o);
        } else {
#pragma unroll
          for (int i = 0; i < 4; ++i)
            if (x + i >= p.dmin0 && x + i < p.dmax0) dst[i] = o[i];
        }
      }
      pm = pc;
      pc = pp;
      ok = __syncthreads_and(ok);
      if (!ok) break;
      // p plane r (z-1) and coefficient plane r are consumed by every thread.
      if (tid == 0) {
        if (r + nsp < nplanes) issue_p(r + nsp);
        if (r + nsc < ncoef) issue_c(r + nsc);
      }
    }
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
         (size_t)cfg.ns * h_align128((uint32_t)(kW * (cfg.warps + 2) * 4)) +
         (size_t)cfg.ns2 * kNumCoef * kTX * cfg.warps * 4;
}

cudaError_t launch_himeno19(const Himeno19Args &a, const MarchConfig &cfg,
                            const CUtensorMap *tmaps, const ResidualSink &sink,
                            int *dev_err, int sm_count, cudaStream_t s) {
  HimenoMaps maps;
  maps.p = tmaps[0];
  for (int i = 0; i < kNumCoef; ++i) maps.coef[i] = tmaps[1 + i];
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
  p.tiles_x = (ex + kTX - 1) / kTX;
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
