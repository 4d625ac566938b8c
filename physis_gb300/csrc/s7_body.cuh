// The per-item body of the 7-point z-march (stencil7.cu's kernel and the
// batched kernel in batch.cu both run it).  One item is one tile of one grid
// marched over planes [zs, ze).  See stencil7.cu for the design.
#pragma once

#include "ps_device.cuh"
#include "ps_internal.h"

namespace psg {

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

// Position in a ring of mbarrier-signalled stages used in issue order.
struct RingPos {
  int stage = 0;
  uint32_t phase = 0;
  __device__ __forceinline__ void advance(int n) {
    if (++stage == n) {
      stage = 0;
      phase ^= 1u;
    }
  }
};

// Marches tile `tile` of p over planes [zs, ze).  `full` are the ring's ns
// mbarriers, `ring` its stages (stride plane_elems elements), TY the tile
// height (blockDim.y * RY).  prod/cons persist across items.  Returns false
// if a bounded wait gave up (the whole CTA agrees).
template <typename T, int K, int RY>
__device__ __forceinline__ bool s7_item(const CUtensorMap *tin, const S7Params<T> &p,
                                        uint64_t *full, T *ring, int plane_elems,
                                        uint32_t plane_bytes, int TY, int tile, int zs,
                                        int ze, RingPos &prod, RingPos &cons) {
  constexpr int VEC = 16 / (int)sizeof(T);
  constexpr int TX = 32 * VEC;
  constexpr int W = TX + 2 * VEC;  // shared row width in elements
  constexpr bool kClamp = (K == kKernelDiffusion7);
  typedef RN<T> R;
  const int ns = p.ns;
  const int lane = threadIdx.x, warp = threadIdx.y;
  const int tid = warp * 32 + lane;
  const int rows0 = warp * RY;                          // first own row in the tile
  const int cen0 = (rows0 + 1) * W + VEC + lane * VEC;  // own first row, centre
  bool ok = true;

  const int x0 = p.xbase + (tile % p.tiles_x) * TX;
  const int y0 = p.dmin1 + (tile / p.tiles_x) * TY;
  const int nplanes = ze - zs + 2;  // planes zs-1 .. ze

  // Issues plane q (global plane zs-1+q) into the producer's next stage.
  auto issue = [&](int q) {
    mbar_arrive_expect_tx(&full[prod.stage], plane_bytes);
    tma_load_3d(ring + prod.stage * plane_elems, tin, x0 - VEC, y0 - 1, zs - 1 + q,
                &full[prod.stage]);
    prod.advance(ns);
  };
  // Waits for the next plane in issue order; returns its stage.
  auto wait_next = [&]() -> const T * {
    if (!mbar_wait(&full[cons.stage], cons.phase, p.err)) ok = false;
    const T *pl = ring + cons.stage * plane_elems;
    cons.advance(ns);
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
  if (!ok) return false;
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
    if (!ok) return false;
    // Plane q is consumed by every thread: refill its stage with q + ns.
    if (tid == 0 && q + ns < nplanes) issue(q + ns);
  }
  return true;
}

}  // namespace psg
