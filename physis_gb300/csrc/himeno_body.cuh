// The per-item body of the Himeno 19-point sweep (himeno19.cu's kernel and
// the batched kernel in batch.cu both run it).  One item is one tile of one
// problem swept over planes [zs, ze).  See himeno19.cu for the design.
#pragma once

#include "ps_device.cuh"
#include "ps_internal.h"

namespace psg {

constexpr int kHimTX = 128;      // tile width in cells (32 lanes x float4)
constexpr int kHimW = kHimTX + 8;  // shared p row width (4-cell halo each side)
constexpr int kHimCoef = 12;     // a0 a1 a2 a3 b0 b1 b2 c0 c1 c2 bnd wrk1

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

__device__ __forceinline__ void him_row6(const float *pl, int idx, int lane, float (&r)[6]) {
  float v[4];
  ld16_shared<float>(v, pl + idx);
  float l = shfl_up1(v[3]);
  float rr = shfl_down1(v[0]);
  ld_shared_if(lane == 0, pl + idx - 1, l);
  ld_shared_if(lane == 31, pl + idx + 4, rr);
  r[0] = l;
  r[1] = v[0];
  r[2] = v[1];
  r[3] = v[2];
  r[4] = v[3];
  r[5] = rr;
}

// Position in a ring of mbarrier-signalled stages used in issue order.
struct HRing {
  int stage = 0;
  uint32_t phase = 0;
  __device__ __forceinline__ void advance(int n) {
    if (++stage == n) {
      stage = 0;
      phase ^= 1u;
    }
  }
};

// Sweeps tile `tile` of p over planes [zs, ze).  pmap is p0's halo map,
// cmaps the 12 coefficient maps in order; pfull/cfull and pring/cring the
// two rings' mbarriers and stages; acc accumulates ss*ss when GOSA.
// Returns false if a bounded wait gave up (the whole CTA agrees).
template <bool GOSA>
__device__ __forceinline__ bool himeno_item(const CUtensorMap *pmap, const CUtensorMap *cmaps,
                                            const HParams &p, uint64_t *pfull, uint64_t *cfull,
                                            float *pring, float *cring, int tile, int zs,
                                            int ze, HRing &pprod, HRing &pcons, HRing &cprod,
                                            HRing &ccons, float &acc) {
  typedef RN<float> R;
  constexpr int kTX = kHimTX, kW = kHimW, kNumCoef = kHimCoef;
  const int TY = blockDim.y;
  const int nsp = p.nsp, nsc = p.nsc;
  const uint32_t p_bytes = (uint32_t)(kW * (TY + 2) * 4);
  const int p_elems = (int)(h_align128(p_bytes) / 4);  // stage stride
  const int c_tile = kTX * TY;                         // elements per coefficient tile
  const int c_elems = kNumCoef * c_tile;               // elements per coefficient stage
  const uint32_t c_bytes = (uint32_t)(c_elems * 4);
  const int lane = threadIdx.x, row = threadIdx.y;
  const int tid = row * 32 + lane;
  const int cen = (row + 1) * kW + 4 + lane * 4;
  const int cidx = row * kTX + lane * 4;
  bool ok = true;

  const int x0 = p.xbase + (tile % p.tiles_x) * kTX;
  const int y0 = p.dmin1 + (tile / p.tiles_x) * TY;
  const int nplanes = ze - zs + 2;  // p planes zs-1 .. ze
  const int ncoef = ze - zs;        // coefficient planes zs .. ze-1

  auto issue_p = [&](int q) {
    const int s = pprod.stage;
    mbar_arrive_expect_tx(&pfull[s], p_bytes);
    tma_load_3d(pring + s * p_elems, pmap, x0 - 4, y0 - 1, zs - 1 + q, &pfull[s]);
    pprod.advance(nsp);
  };
  auto issue_c = [&](int r) {
    const int s = cprod.stage;
    mbar_arrive_expect_tx(&cfull[s], c_bytes);
    float *dst = cring + s * c_elems;
#pragma unroll 1
    for (int a = 0; a < kNumCoef; ++a)
      tma_load_3d(dst + a * c_tile, cmaps + a, x0, y0, zs + r, &cfull[s]);
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
    him_row6(pc, cen, lane, Zc);
    him_row6(pc, cen - kW, lane, Zym);
    him_row6(pc, cen + kW, lane, Zyp);
    him_row6(pp, cen, lane, Zpc);
    him_row6(pm, cen, lane, Zmc);
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
    if (!ok) return false;
    // p plane r (z-1) and coefficient plane r are consumed by every thread.
    if (tid == 0) {
      if (r + nsp < nplanes) issue_p(r + nsp);
      if (r + nsc < ncoef) issue_c(r + nsc);
    }
  }
  return true;
}

}  // namespace psg
