// The point-list stencil sweep, written once for two builds:
//  * points.cu compiles it with a run-time point table (PtsTableSpec): one
//    kernel serves every registered stencil;
//  * jit.cpp compiles it with NVRTC for one stencil at a time, with a
//    generated spec whose offsets, plane lags, weights and tile geometry are
//    compile-time constants (the point loop unrolls into shared-memory loads
//    at immediate offsets, and loads that two rows of a thread share are
//    issued once).
// No header dependencies beyond ps_arith.cuh, so NVRTC can compile it from
// memory.  See points.cu for the design.
#pragma once

#include "ps_arith.cuh"

namespace psg {

constexpr int kPtsTX = 128;       // tile width in cells
constexpr int kPtsVX = 4;         // columns per lane (lane + 32*j)
constexpr int kPtsPrefetch = 2;   // cp.async ring: planes in flight ahead of the newest needed one
constexpr int kPtsMaxPoints = 64;
// Shared memory: point table (run-time spec only: offsets, lags, weights),
// then the ring's mbarriers, then the ring (128-byte aligned stages).
constexpr int kPtsTableBytes = kPtsMaxPoints * (4 + 4 + 8);
constexpr int kPtsMaxStages = 16;
constexpr int kPtsRingOffset = kPtsTableBytes + 8 * kPtsMaxStages;
// Opaque TMA descriptor (the layout of CUtensorMap: 128 bytes, 64-aligned).
struct alignas(64) PtsTmap {
  unsigned long long opaque[16];
};
enum { kPtsNone = 0, kPtsPeriodic = 1, kPtsClamp = 2 };

template <typename T>
struct PtsParams {
  const T *in;
  T *out;            // may equal in (red/black)
  long long row;     // pitch in elements
  long long plane;   // elements per z-plane
  int nx, ny, nz;
  int dmin0, dmin1, dmin2, dmax0, dmax1, dmax2;
  int boundary;      // kPtsNone / kPtsPeriodic / kPtsClamp
  int color;         // -1 every cell, 0 red, 1 black
  int n;             // points
  int ryl, rzl, rzh;
  int lp, w, rows_h, nstage, plane_elems;
  int pstride;       // ring stage stride in elements (128-byte multiple)
  int use_tma;       // 1: the tmap parameter maps `in` with box {w, rows_h, 1}
  int xbase, tiles_x, tiles, zlen;
  long long items;
  int *err;          // device error word (bounded waits that give up)
  int off[kPtsMaxPoints];  // shared offset of point i relative to the cell
  int lag[kPtsMaxPoints];  // rzl + dz_i: the point's plane relative to z - rzl
  T wt[kPtsMaxPoints];
};

// Grid index of coordinate i on an axis of n cells.  Periodic: i mod n, which
// equals the reference's (i + n) % n for every i >= -n (the host admits only
// offsets with |d| <= n, so every read that is used has i >= -n; halo cells
// that are never read may lie further out and still land inside the grid).
// Clamp, and the never-read halo of boundary "none": the nearest face.
__device__ __forceinline__ int pts_map_axis(int i, int n, int boundary) {
  if (boundary == kPtsPeriodic) {
    const int m = i % n;
    return m < 0 ? m + n : m;
  }
  return min(max(i, 0), n - 1);
}

// Issues the copies of global plane zg (tile origin x0, y0) into `dst`:
// 16-byte copies for aligned chunks inside the grid, element copies through
// the boundary map for chunks that cross an edge.
template <typename T>
__device__ __forceinline__ void pts_load_plane(const PtsParams<T> &p, T *dst, int zg, int x0,
                                               int y0) {
  constexpr int VEC = 16 / (int)sizeof(T);
  const T *src_plane = p.in + (long long)pts_map_axis(zg, p.nz, p.boundary) * p.plane;
  const int nchunk = p.w / VEC;
  const int xs = x0 - p.lp;
  for (int r = threadIdx.y; r < p.rows_h; r += blockDim.y) {
    const T *src =
        src_plane + (long long)pts_map_axis(y0 - p.ryl + r, p.ny, p.boundary) * p.row;
    T *d = dst + r * p.w;
    for (int c = threadIdx.x; c < nchunk; c += 32) {
      const int x = xs + c * VEC;
      if (x >= 0 && x + VEC <= p.nx) {
        cp_async16(d + c * VEC, src + x);
      } else {
#pragma unroll
        for (int i = 0; i < VEC; ++i)
          cp_async_small<sizeof(T)>(d + c * VEC + i, src + pts_map_axis(x + i, p.nx, p.boundary));
      }
    }
  }
}

// After a TMA box load of plane zg (tile origin x0, y0; zero-filled outside
// the grid), rewrites the box cells that lie outside the grid with the
// values the boundary rule maps them to.  Only edge tiles of periodic and
// clamped stencils have such cells; all threads share the work.
template <typename T>
__device__ __forceinline__ void pts_fix_halo(const PtsParams<T> &p, T *dst, int zg, int x0,
                                             int y0, int W) {
  const int xs = x0 - p.lp, ys = y0 - p.ryl, H = p.rows_h;
  const T *plane = p.in + (long long)pts_map_axis(zg, p.nz, p.boundary) * p.plane;
  const int cl = min(max(0, -xs), W);
  const int cr = min(max(0, xs + W - p.nx), W - cl);
  const int rt = min(max(0, -ys), H);
  const int rb = min(max(0, ys + H - p.ny), H - rt);
  const int nfull = (rt + rb) * W;            // whole rows outside in y
  const int side = cl + cr;                   // cells per inner row outside in x
  const int total = nfull + (H - rt - rb) * side;
  const int nthr = blockDim.x * blockDim.y;
  for (int i = threadIdx.y * 32 + threadIdx.x; i < total; i += nthr) {
    int r, c;
    if (i < nfull) {
      const int rr = i / W;
      c = i - rr * W;
      r = rr < rt ? rr : H - rb + (rr - rt);
    } else {
      const int k = i - nfull;
      const int rr = k / side;
      const int cc = k - rr * side;
      r = rt + rr;
      c = cc < cl ? cc : W - cr + (cc - cl);
    }
    const int x = pts_map_axis(xs + c, p.nx, p.boundary);
    const int y = pts_map_axis(ys + r, p.ny, p.boundary);
    dst[r * W + c] = plane[(long long)y * p.row + x];
  }
}

// The run-time spec: the point table travels in the kernel parameters and is
// copied to shared memory; the tile geometry comes from the parameters.
struct PtsTableSpec {
  static constexpr bool kStatic = false;
  template <typename T>
  static __device__ __forceinline__ int w(const PtsParams<T> &p) { return p.w; }
  template <typename T>
  static __device__ __forceinline__ int nstage(const PtsParams<T> &p) { return p.nstage; }
  template <typename T>
  static __device__ __forceinline__ int pstride(const PtsParams<T> &p) { return p.pstride; }
};

// acc[r][j] (+)= w * src[r*W + 32*j]; `first` starts the sum.
template <typename T, int RY, bool UNIT>
__device__ __forceinline__ void pts_term(T (&acc)[RY][kPtsVX], const T *src, int W, T wk,
                                         bool first) {
  typedef RN<T> R;
#pragma unroll
  for (int r = 0; r < RY; ++r)
#pragma unroll
    for (int j = 0; j < kPtsVX; ++j) {
      const T v = src[r * W + 32 * j];
      const T t = UNIT ? v : R::mul(wk, v);
      acc[r][j] = first ? t : R::add(acc[r][j], t);
    }
}

// The sweep: persistent (z-chunk, tile) items, a ring of planes, the points
// summed in order, masked stores.  Each plane of a tile arrives by one TMA
// box load (mbarrier per stage); on the edge tiles of periodic and clamped
// stencils the out-of-grid cells of the box are then rewritten through the
// boundary map (with boundary "none" they are never read).  Without a TMA
// descriptor (p.use_tma == 0) planes are copied with cp.async through the
// boundary map instead (one commit group per plane).  `smem_raw` is the
// dynamic shared memory, `tmap` the TMA descriptor of `in`.
template <typename T, int RY, bool UNIT, class S>
__device__ __forceinline__ void pts_body(const PtsParams<T> &p, const void *tmap,
                                         unsigned char *smem_raw) {
  unsigned char *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  int *s_off = reinterpret_cast<int *>(smem);
  int *s_lag = s_off + kPtsMaxPoints;
  T *s_w = reinterpret_cast<T *>(smem + kPtsMaxPoints * 8);
  unsigned long long *bars = reinterpret_cast<unsigned long long *>(smem + kPtsTableBytes);
  T *ring = reinterpret_cast<T *>(smem + kPtsRingOffset);
  const int W = S::w(p), NST = S::nstage(p), PS = S::pstride(p);

  const int lane = threadIdx.x, warp = threadIdx.y;
  const int tid = warp * 32 + lane;
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) mbar_init(&bars[s], 1);
    fence_barrier_init();
  }
  if (!S::kStatic) {
    for (int i = tid; i < p.n; i += blockDim.x * blockDim.y) {
      s_off[i] = p.off[i];
      s_lag[i] = p.lag[i];
      s_w[i] = p.wt[i];
    }
  }
  __syncthreads();

  const int TY = blockDim.y * RY;
  const int pre = NST - 1;  // planes issued before the first compute step
  const int cell0 = warp * RY * W + lane;
  const unsigned tma_bytes = (unsigned)(p.plane_elems * (int)sizeof(T));
  unsigned phase = 0;  // bit s: parity of the next completion of stage s
  bool ok = true;

  for (long long item = blockIdx.x; item < p.items && ok; item += gridDim.x) {
    const int chunk = (int)(item / p.tiles);
    const int tile = (int)(item - (long long)chunk * p.tiles);
    const int zs = p.dmin2 + chunk * p.zlen;
    const int ze = min(zs + p.zlen, p.dmax2);
    const int x0 = p.xbase + (tile % p.tiles_x) * kPtsTX;
    const int y0 = p.dmin1 + (tile / p.tiles_x) * TY;
    const int nplanes = ze - zs + p.rzl + p.rzh;  // planes zs-rzl .. ze+rzh-1
    const bool tma = p.use_tma != 0;
    const bool fix = tma && p.boundary != kPtsNone &&
                     !(x0 - p.lp >= 0 && x0 - p.lp + W <= p.nx && y0 - p.ryl >= 0 &&
                       y0 - p.ryl + p.rows_h <= p.ny);
    // store masks: columns j in the domain, rows r in the domain
    unsigned colmask = 0, rowmask = 0;
#pragma unroll
    for (int j = 0; j < kPtsVX; ++j) {
      const int x = x0 + lane + 32 * j;
      if (x >= p.dmin0 && x < p.dmax0) colmask |= 1u << j;
    }
#pragma unroll
    for (int r = 0; r < RY; ++r)
      if (y0 + warp * RY + r < p.dmax1) rowmask |= 1u << r;
    const int xpar = (x0 + lane) & 1;  // parity of every column of this lane
    T *out0 = p.out + (long long)(y0 + warp * RY) * p.row + x0 + lane;

    int ld = 0, issued = 0, waited = 0, wslot = 0;
    auto issue = [&](int q) {
      if (tma) {
        if (tid == 0) {
          mbar_arrive_expect_tx(&bars[ld], tma_bytes);
          tma_load_3d(ring + ld * PS, tmap, x0 - p.lp, y0 - p.ryl,
                      pts_map_axis(zs - p.rzl + q, p.nz, p.boundary), &bars[ld]);
        }
        ++issued;
      } else {
        if (q < nplanes) pts_load_plane(p, ring + ld * PS, zs - p.rzl + q, x0, y0);
        cp_async_commit();
      }
      if (++ld == NST) ld = 0;
    };
    for (int q = 0; q < pre; ++q)
      if (q < nplanes || !tma) issue(q);
    int cs = 0;  // ring slot of plane z - rzl
    for (int z = zs; z < ze && ok; ++z) {
      const int q = z - zs + pre;
      if (q < nplanes || !tma) issue(q);
      if (tma) {
        const int need = z - zs + p.rzl + p.rzh;  // newest plane this step reads
        while (waited <= need) {
          if (!mbar_wait(&bars[wslot], (phase >> wslot) & 1u, p.err)) ok = false;
          if (fix && ok) pts_fix_halo(p, ring + wslot * PS, zs - p.rzl + waited, x0, y0, W);
          phase ^= 1u << wslot;
          ++waited;
          if (++wslot == NST) wslot = 0;
        }
      } else {
        cp_async_wait<kPtsPrefetch>();  // planes up to z + rzh have landed
      }
      ok = __syncthreads_and(ok);
      if (!ok) break;

      T acc[RY][kPtsVX];
      if constexpr (S::kStatic) {
#pragma unroll
        for (int k = 0; k < S::kN; ++k) {
          int s = cs + S::kLag[k];
          if (s >= NST) s -= NST;
          pts_term<T, RY, UNIT>(acc, ring + s * PS + cell0 + S::kOff[k], W, (T)S::kWt[k],
                                k == 0);
        }
      } else {
        for (int k = 0; k < p.n; ++k) {
          int s = cs + s_lag[k];
          if (s >= NST) s -= NST;
          pts_term<T, RY, UNIT>(acc, ring + s * PS + cell0 + s_off[k], W, s_w[k], k == 0);
        }
      }

      T *dst = out0 + (long long)z * p.plane;
#pragma unroll
      for (int r = 0; r < RY; ++r) {
        const int y = y0 + warp * RY + r;
        const bool row_on = ((rowmask >> r) & 1u) &&
                            (p.color < 0 || ((xpar + y + z + p.color) & 1) == 0);
        if (row_on) {
#pragma unroll
          for (int j = 0; j < kPtsVX; ++j)
            if ((colmask >> j) & 1u) dst[r * p.row + 32 * j] = acc[r][j];
        }
      }
      if (++cs == NST) cs = 0;
      __syncthreads();  // the slot of plane z - rzl is refilled next step
    }
    if (!tma) cp_async_wait<0>();  // only empty groups can remain
    if (!ok && tma && tid == 0) {
      // a wait gave up: let copies still in flight land (bounded) before exit
      for (; waited < issued; ++waited) {
        mbar_wait(&bars[wslot], (phase >> wslot) & 1u, nullptr, 1024);
        phase ^= 1u << wslot;
        if (++wslot == NST) wslot = 0;
      }
    }
  }
}

}  // namespace psg
