// Himeno 19-point variable-coefficient Jacobi sweep on GB300 (sm_103a),
// with the residual (gosa = sum of ss*ss) fused into the same pass.
//
// Semantics: the Physis Himeno kernel (examples/himeno/himenobmtxpa_physis.c:
// 331-361), i = x fastest, over the interior domain; cells outside the domain
// are never written.  The residual follows the original benchmark's loop
// (examples/himeno/himenobmtxpa_original.c:331-334), which the Physis port
// dropped; here it costs no extra HBM traffic.
//
// Design (one CTA = a 128 x TY tile in x,y marching over zchunk planes):
// * p planes with a one-cell y halo and a 4-cell (16-byte) x halo arrive by
//   TMA into a ring of `nsp` stages; the sweep at plane z reads planes z-1, z
//   and z+1 from the ring (the 19-point stencil needs xy neighbours on all
//   three planes, so a register queue alone does not suffice);
// * the 12 centre-only coefficient arrays (a0..a3, b0..b2, c0..c2, bnd,
//   wrk1) arrive as 12 TMA boxes of 128 x TY per plane into a second ring of
//   `nsc` stages, all signalled by one mbarrier per stage;
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

constexpr int kTX = 128;        // tile width in cells (32 lanes x float4)
constexpr int kW = kTX + 8;     // shared p row width (4-cell halo each side)
constexpr int kNumCoef = 12;    // a0 a1 a2 a3 b0 b1 b2 c0 c1 c2 bnd wrk1

struct HimenoMaps {
  CUtensorMap p;               // p0 with halo box {kW, TY+2, 1}
  CUtensorMap coef[kNumCoef];  // box {kTX, TY, 1}
};

struct HParams {
  float *out;
  int64_t row, plane;  // out pitch / plane in elements
  int dmin0, dmin1, dmin2, dmax0, dmax1, dmax2;
  int xbase, zchunk, nsp, nsc;
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

template <bool GOSA>
__global__ void __launch_bounds__(256, 1)
himeno19_kernel(const __grid_constant__ HimenoMaps maps, const HParams p) {
  typedef RN<float> R;
  const int TY = blockDim.y;
  const int nsp = p.nsp, nsc = p.nsc;
  const uint32_t p_bytes = (uint32_t)(kW * (TY + 2) * 4);
  const int p_elems = (int)(h_align128(p_bytes) / 4);  // stage stride
  const int c_tile = kTX * TY;             // elements per coefficient tile
  const int c_elems = kNumCoef * c_tile;   // elements per coefficient stage
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
  const int x0 = p.xbase + blockIdx.x * kTX;
  const int y0 = p.dmin1 + blockIdx.y * TY;
  const int zs = p.dmin2 + blockIdx.z * p.zchunk;
  const int ze = min(zs + p.zchunk, p.dmax2);
  const int nplanes = ze - zs + 2;  // p planes zs-1 .. ze
  const int ncoef = ze - zs;        // coefficient planes zs .. ze-1

  if (tid == 0) {
    prefetch_tmap(&maps.p);
    for (int s = 0; s < nsp; ++s) mbar_init(&pfull[s], 1);
    for (int s = 0; s < nsc; ++s) mbar_init(&cfull[s], 1);
    fence_barrier_init();
  }
  __syncthreads();

  auto issue_p = [&](int q) {
    const int s = q % nsp;
    mbar_arrive_expect_tx(&pfull[s], p_bytes);
    tma_load_3d(pring + s * p_elems, &maps.p, x0 - 4, y0 - 1, zs - 1 + q, &pfull[s]);
  };
  auto issue_c = [&](int r) {
    const int s = r % nsc;
    mbar_arrive_expect_tx(&cfull[s], c_bytes);
    float *dst = cring + s * c_elems;
#pragma unroll 1
    for (int a = 0; a < kNumCoef; ++a)
      tma_load_3d(dst + a * c_tile, &maps.coef[a], x0, y0, zs + r, &cfull[s]);
  };
  if (tid == 0) {
    for (int q = 0; q < min(nsp, nplanes); ++q) issue_p(q);
    for (int r = 0; r < min(nsc, ncoef); ++r) issue_c(r);
  }

  bool ok = true;
  auto wait_p = [&](int q) -> const float * {
    const int s = q % nsp;
    if (!mbar_wait(&pfull[s], (uint32_t)((q / nsp) & 1), p.err)) ok = false;
    return pring + s * p_elems;
  };
  auto wait_c = [&](int r) -> const float * {
    const int s = r % nsc;
    if (!mbar_wait(&cfull[s], (uint32_t)((r / nsc) & 1), p.err)) ok = false;
    return cring + s * c_elems;
  };

  const int cen = (row + 1) * kW + 4 + lane * 4;
  const int cidx = row * kTX + lane * 4;
  const int y = y0 + row;
  const int x = x0 + lane * 4;
  const bool row_in = (y < p.dmax1);
  const bool vec_in = (x >= p.dmin0) && (x + 4 <= p.dmax0);
  float acc = 0.0f;

  wait_p(0);
  wait_p(1);
  for (int z = zs; z < ze; ++z) {
    const int r = z - zs;
    const float *pm = pring + (r % nsp) * p_elems;        // plane z-1
    const float *pc = pring + ((r + 1) % nsp) * p_elems;  // plane z
    const float *pp = wait_p(r + 2);                      // plane z+1
    const float *cf = wait_c(r);

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
    ok = __syncthreads_and(ok);
    if (!ok) break;
    if (tid == 0) {
      if (r + nsp < nplanes) issue_p(r + nsp);
      if (r + nsc < ncoef) issue_c(r + nsc);
    }
  }
  if (!ok) {
    if (tid == 0) {
      for (int q = 0; q < nplanes; ++q)
        mbar_wait(&pfull[q % nsp], (uint32_t)((q / nsp) & 1), nullptr, 1024);
      for (int r = 0; r < ncoef; ++r)
        mbar_wait(&cfull[r % nsc], (uint32_t)((r / nsc) & 1), nullptr, 1024);
    }
    return;
  }
  if (!GOSA) return;

  // Residual: FP32 block tree, FP64 partial per CTA, FP64 final combine.
  const int nwarps = TY;
  acc = warp_sum(acc);
  if (lane == 0) red[row] = acc;
  __syncthreads();
  if (tid == 0) {
    float bs = 0.0f;
    for (int w = 0; w < nwarps; ++w) bs = __fadd_rn(bs, red[w]);
    const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
    const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    p.partials[bid] = (double)bs;
    __threadfence();
    const unsigned prev = atomicAdd(p.ticket, 1u);
    last_cta = (prev == nblocks - 1);
  }
  __syncthreads();
  if (last_cta && row == 0) {
    __threadfence();
    const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
    double v = 0.0;
    for (unsigned i = lane; i < nblocks; i += 32) v = __dadd_rn(v, __ldcg(&p.partials[i]));
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
         (size_t)cfg.ns * h_align128((uint32_t)(kW * (cfg.ty + 2) * 4)) +
         (size_t)cfg.ns2 * kNumCoef * kTX * cfg.ty * 4;
}

int himeno19_num_ctas(const Himeno19Args &a, const MarchConfig &cfg) {
  const int xbase = (a.dom.min[0] / 4) * 4;
  const int ex = a.dom.max[0] - xbase;
  const int ey = a.dom.max[1] - a.dom.min[1];
  const int ez = a.dom.max[2] - a.dom.min[2];
  if (ex <= 0 || ey <= 0 || ez <= 0) return 0;
  return ((ex + kTX - 1) / kTX) * ((ey + cfg.ty - 1) / cfg.ty) *
         ((ez + cfg.zchunk - 1) / cfg.zchunk);
}

cudaError_t launch_himeno19(const Himeno19Args &a, const MarchConfig &cfg,
                            const CUtensorMap *tmaps, const ResidualSink &sink,
                            int *dev_err, cudaStream_t s) {
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
  p.zchunk = cfg.zchunk;
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
  dim3 grid((ex + kTX - 1) / kTX, (ey + cfg.ty - 1) / cfg.ty,
            (ez + cfg.zchunk - 1) / cfg.zchunk);
  if (a.gosa && (int)(grid.x * grid.y * grid.z) > sink.max_partials)
    return cudaErrorInvalidConfiguration;
  if (grid.y > 65535 || grid.z > 65535 || cfg.ty < 1 || cfg.ty > 8 || cfg.ns < 3 ||
      cfg.ns2 < 1)
    return cudaErrorInvalidConfiguration;
  dim3 block(32, cfg.ty, 1);
  const size_t smem = himeno19_smem_bytes(cfg);
  // Opt in to the dynamic shared memory this launch needs (the kernel also
  // has a little static shared memory, so the opt-in is the exact size).
  static size_t attr_set[2] = {0, 0};
  size_t &have = attr_set[a.gosa ? 1 : 0];
  if (smem > have) {
    cudaError_t e = a.gosa
        ? cudaFuncSetAttribute(himeno19_kernel<true>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
        : cudaFuncSetAttribute(himeno19_kernel<false>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    have = smem;
  }
  if (a.gosa)
    himeno19_kernel<true><<<grid, block, smem, s>>>(maps, p);
  else
    himeno19_kernel<false><<<grid, block, smem, s>>>(maps, p);
  return cudaGetLastError();
}

}  // namespace psg
