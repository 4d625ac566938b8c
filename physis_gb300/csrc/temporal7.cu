// Temporal blocking of the clamped 7-point diffusion on GB300 (sm_103a):
// one pass reads step t from HBM and writes step t+k.
//
// The reference runs one launch per map per time step
// (translator/cuda_runtime_builder.cc:1512-1583), so every step streams the
// grid through HBM twice.  Its hand-written benchmark variant blocks two
// steps per pass (examples/diffusion-benchmark/diffusion3d_cuda_temporal_
// blocking.cu).  Here the depth k is a launch parameter (2..VEC+1) and each
// cell's arithmetic is exactly the single-step kernel's, so k blocked steps
// are bit-identical to k plain steps.  When the runtime allows contraction
// (PSSetFusedMultiplyAdd), the FMA variant evaluates the same left-to-right
// sum as one multiply and six fused multiply-adds: 7 instead of 13 rounded
// operations, results within rounding of the REF target.
//
// Geometry.  A CTA computes an extended tile E of 32*VEC columns x TYE rows
// (TYE = warps*rows) and writes the output tile: E minus VEC columns on each
// side (the 16-byte x halo that TMA alignment makes us load anyway) and minus
// k-1 rows on each side.  Stage j (0-based) applies time step t+j+1; a
// stage's valid region shrinks by one cell per stage, so after k stages the
// output tile is exact.
// Pipeline along z.  At pipeline step s the TMA ring delivers input plane s;
// stage j computes plane s-1-j.  Every thread keeps, per stage, the previous
// and current plane of that stage's input at its own cells in registers (the
// z-neighbours); the x/y neighbours come from shared memory: the TMA plane
// for stage 0, and for stage j >= 1 a two-slot plane buffer in which stage
// j-1 wrote its previous output.  The new output of stage j goes to the
// buffer and, in registers, straight into stage j+1 as its next plane.  One
// __syncthreads per step separates a slot's writes from its next reads.
// Work items are (z-chunk, tile) pairs in chunk-major order taken
// round-robin by a persistent grid (as in stencil7.cu).
#include <type_traits>

#include "ps_device.cuh"
#include "ps_internal.h"

namespace psg {
namespace {

template <typename T>
struct TParams {
  T *out;
  int64_t row, plane;  // out pitch / plane in elements
  int nx, ny, nz;
  int k;               // steps per pass
  int tiles_x, tiles, zlen;
  int64_t items;
  int ns;
  T cc, cw, ce, cs, cn, cb, ct;
  int *err;
};

__host__ __device__ constexpr int t_bar_bytes(int ns) { return 128 * ((8 * ns + 127) / 128); }
__host__ __device__ constexpr uint32_t t_align128(uint32_t b) { return (b + 127u) & ~127u; }

// One diffusion update of a 16-byte vector of one row; with CLAMP, the
// neighbours across the grid's x faces are replaced by the centre.
template <typename T, int VEC, bool CLAMP, bool FMA>
__device__ __forceinline__ void diffuse_row(const T (&c)[VEC], const T (&n)[VEC],
                                            const T (&s)[VEC], const T (&b)[VEC],
                                            const T (&t)[VEC], T left, T right,
                                            bool west_face, int east_elem,
                                            const TParams<T> &p, T (&o)[VEC]) {
  typedef RN<T> R;
#pragma unroll
  for (int i = 0; i < VEC; ++i) {
    T w = (i == 0) ? left : c[i - 1];
    T e = (i == VEC - 1) ? right : c[i + 1];
    if (CLAMP) {
      if (i == 0 && west_face) w = c[0];
      if (i == east_elem) e = c[i];
    }
    T v = R::mul(p.cc, c[i]);
    if (FMA) {
      v = R::fma(p.cw, w, v);
      v = R::fma(p.ce, e, v);
      v = R::fma(p.cs, s[i], v);
      v = R::fma(p.cn, n[i], v);
      v = R::fma(p.cb, b[i], v);
      v = R::fma(p.ct, t[i], v);
    } else {
      v = R::add(v, R::mul(p.cw, w));
      v = R::add(v, R::mul(p.ce, e));
      v = R::add(v, R::mul(p.cs, s[i]));
      v = R::add(v, R::mul(p.cn, n[i]));
      v = R::add(v, R::mul(p.cb, b[i]));
      v = R::add(v, R::mul(p.ct, t[i]));
    }
    o[i] = v;
  }
}

// Per-item constants of a pass.
template <typename T>
struct T7Item {
  T *bufs;
  int plane_elems, cen0, lane, rows0, x, y, TYO, zs, ze;
  bool west_face, out_lane, vec_in;
  int east_elem;
};

// One pipeline step: the TMA plane `in_t` is input plane s.  Each stage's
// three register planes rotate roles with the step (ROT): b = slot ROT,
// c = slot ROT+1, t = slot ROT+2 (mod 3); a stage writes its output straight
// into the next stage's t slot, so no plane is ever copied between
// registers.  CL: the item's extended tile touches a grid face in x or y.
template <typename T, int RY, int K, int ROT, bool CL, bool FMA>
__device__ __forceinline__ void t7_step(T (&Q)[K][3][RY][16 / sizeof(T)], const T *in_t,
                                        const T *prev_in, int s, const TParams<T> &p,
                                        const T7Item<T> &it, bool ok) {
  constexpr int VEC = 16 / (int)sizeof(T);
  constexpr int W = 34 * VEC;
  constexpr int BS = ROT, CS = (ROT + 1) % 3, TS = (ROT + 2) % 3;
  const int cen0 = it.cen0, lane = it.lane;
#pragma unroll
  for (int r = 0; r < RY; ++r) ld16_shared<T>(Q[0][TS][r], in_t + cen0 + r * W);
#pragma unroll
  for (int j = 0; j < K; ++j) {
    const int pz = s - 1 - j;  // plane stage j computes
    const T *nb = (j == 0) ? prev_in : it.bufs + ((j - 1) * 2 + (pz & 1)) * it.plane_elems;
    if (pz == 0) {  // clamp below the first plane: b = c
#pragma unroll
      for (int r = 0; r < RY; ++r)
#pragma unroll
        for (int i = 0; i < VEC; ++i) Q[j][BS][r][i] = Q[j][CS][r][i];
    }
    if (pz == p.nz - 1) {  // clamp above the last plane: t = c
#pragma unroll
      for (int r = 0; r < RY; ++r)
#pragma unroll
        for (int i = 0; i < VEC; ++i) Q[j][TS][r][i] = Q[j][CS][r][i];
    }
    T nrow[VEC], srow[VEC];
    ld16_shared<T>(nrow, nb + cen0 - W);
    ld16_shared<T>(srow, nb + cen0 + RY * W);
#pragma unroll
    for (int r = 0; r < RY; ++r) {
      T nn[VEC], ss[VEC];
#pragma unroll
      for (int i = 0; i < VEC; ++i) {
        nn[i] = (r == 0) ? nrow[i] : Q[j][CS][r - 1][i];
        ss[i] = (r == RY - 1) ? srow[i] : Q[j][CS][r + 1][i];
      }
      if (CL) {
        if (it.y + r == 0) {
#pragma unroll
          for (int i = 0; i < VEC; ++i) nn[i] = Q[j][CS][r][i];
        }
        if (it.y + r == p.ny - 1) {
#pragma unroll
          for (int i = 0; i < VEC; ++i) ss[i] = Q[j][CS][r][i];
        }
      }
      T left = shfl_up1(Q[j][CS][r][VEC - 1]);
      T right = shfl_down1(Q[j][CS][r][0]);
      ld_shared_if(lane == 0, nb + cen0 + r * W - 1, left);
      ld_shared_if(lane == 31, nb + cen0 + r * W + VEC, right);
      if (j < K - 1) {
        diffuse_row<T, VEC, CL, FMA>(Q[j][CS][r], nn, ss, Q[j][BS][r], Q[j][TS][r], left,
                                     right, it.west_face, it.east_elem, p,
                                     Q[(j + 1) % K][TS][r]);
      } else {
        T o[VEC];
        diffuse_row<T, VEC, CL, FMA>(Q[j][CS][r], nn, ss, Q[j][BS][r], Q[j][TS][r], left,
                                     right, it.west_face, it.east_elem, p, o);
        const int er = it.rows0 + r;  // row within E
        const int gy = it.y + r;
        if (ok && pz >= it.zs && pz < it.ze && it.out_lane && er >= K - 1 &&
            er < K - 1 + it.TYO && gy < p.ny) {
          T *g = p.out + (int64_t)pz * p.plane + (int64_t)gy * p.row + it.x;
          if (it.vec_in) {
            st16_global<T>(g, o);
          } else {
#pragma unroll
            for (int i = 0; i < VEC; ++i)
              if (it.x + i < p.nx) g[i] = o[i];
          }
        }
      }
    }
    if (j < K - 1) {  // neighbours of this output for the next stage
      T *dst = it.bufs + (j * 2 + (pz & 1)) * it.plane_elems;
#pragma unroll
      for (int r = 0; r < RY; ++r)
        *reinterpret_cast<uint4 *>(dst + cen0 + r * W) =
            *reinterpret_cast<const uint4 *>(Q[(j + 1) % K][TS][r]);
    }
  }
}

template <typename T, int RY, int K, bool FMA>
__global__ void __launch_bounds__(256, 2)
t7_kernel(const __grid_constant__ CUtensorMap tin, const TParams<T> p) {
  constexpr int VEC = 16 / (int)sizeof(T);
  constexpr int W = 34 * VEC;   // shared row width (E plus a VEC apron each side)
  constexpr int TXO = 30 * VEC; // output columns per tile
  const int TYE = blockDim.y * RY;
  const int TYO = TYE - 2 * (K - 1);
  const uint32_t plane_bytes = (uint32_t)(W * (TYE + 2) * sizeof(T));
  const int plane_elems = (int)(t_align128(plane_bytes) / sizeof(T));
  const int ns = p.ns;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);
  T *ring = reinterpret_cast<T *>(smem + t_bar_bytes(ns));
  T *bufs = ring + ns * plane_elems;  // (K-1) stages x 2 slots

  const int lane = threadIdx.x, warp = threadIdx.y;
  const int tid = warp * 32 + lane;
  const int nthreads = 32 * blockDim.y;
  if (tid == 0) {
    prefetch_tmap(&tin);
    for (int s = 0; s < ns; ++s) mbar_init(&full[s], 1);
    fence_barrier_init();
  }
  // Zero the stage buffers once: their aprons are never written, and zeros
  // keep the (discarded) border cells finite.
  for (int i = tid; i < (K - 1) * 2 * plane_elems; i += nthreads) bufs[i] = T(0);
  __syncthreads();

  int pstage = 0, cstage = 0;
  uint32_t pphase = 0, cphase = 0;
  bool ok = true;
  T7Item<T> it;
  it.bufs = bufs;
  it.plane_elems = plane_elems;
  it.lane = lane;
  it.rows0 = warp * RY;
  it.cen0 = (it.rows0 + 1) * W + VEC + lane * VEC;
  it.TYO = TYO;
  it.out_lane = (lane >= 1 && lane <= 30);

  for (int64_t item = blockIdx.x; item < p.items && ok; item += gridDim.x) {
    const int chunk = (int)(item / p.tiles);
    const int tile = (int)(item - (int64_t)chunk * p.tiles);
    it.zs = chunk * p.zlen;
    it.ze = min(it.zs + p.zlen, p.nz);
    const int xo0 = (tile % p.tiles_x) * TXO;
    const int yo0 = (tile / p.tiles_x) * TYO;
    const int xe0 = xo0 - VEC;      // E's first column
    const int ye0 = yo0 - (K - 1);  // E's first row
    const int zin0 = it.zs - K;     // first input plane
    const int nplanes = it.ze - it.zs + 2 * K;

    auto issue = [&](int q) {
      mbar_arrive_expect_tx(&full[pstage], plane_bytes);
      tma_load_3d(ring + pstage * plane_elems, &tin, xe0 - VEC, ye0 - 1, zin0 + q,
                  &full[pstage]);
      if (++pstage == ns) {
        pstage = 0;
        pphase ^= 1u;
      }
    };
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
    it.x = xe0 + lane * VEC;
    it.y = ye0 + it.rows0;
    it.west_face = (it.x == 0);
    it.east_elem = p.nx - 1 - it.x;
    it.vec_in = it.out_lane && (it.x + VEC <= p.nx);

    T Q[K][3][RY][VEC];
    {
      const T *p0 = wait_next();  // input plane zs-K
      const T *p1 = wait_next();  // input plane zs-K+1
#pragma unroll
      for (int r = 0; r < RY; ++r) {
        ld16_shared<T>(Q[0][0][r], p0 + it.cen0 + r * W);
        ld16_shared<T>(Q[0][1][r], p1 + it.cen0 + r * W);
      }
#pragma unroll
      for (int j = 1; j < K; ++j)
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
          for (int r = 0; r < RY; ++r)
#pragma unroll
            for (int i = 0; i < VEC; ++i) Q[j][a][r][i] = T(0);
    }
    ok = __syncthreads_and(ok);
    if (!ok) break;
    if (tid == 0 && ns < nplanes) issue(ns);
    const T *prev_in = ring + ((cstage + ns - 1) % ns) * plane_elems;  // plane 1

    // One pipeline step for input plane q, with rotation R of the slots.
// One step body per slot rotation (three in all).  Every tile runs the
// clamp-aware body: a second, clamp-free copy for interior tiles doubled the
// code and cost more in instruction-cache misses than its selects saved.
#define PS_T7_STEP(R)                                                         \
  {                                                                           \
    const T *in_t = wait_next();                                              \
    t7_step<T, RY, K, R, true, FMA>(Q, in_t, prev_in, zin0 + q, p, it, ok);   \
    prev_in = in_t;                                                           \
    ok = __syncthreads_and(ok);                                               \
    if (!ok) break;                                                           \
    if (tid == 0 && q - 1 + ns < nplanes) issue(q - 1 + ns);                  \
    if (++q >= nplanes) break;                                                \
  }
    int q = 2;
    while (q < nplanes) {
      PS_T7_STEP(0)
      PS_T7_STEP(1)
      PS_T7_STEP(2)
    }
#undef PS_T7_STEP
  }
  if (!ok && tid == 0) {
    for (int s = 0; s < ns; ++s) mbar_wait(&full[s], 0, nullptr, 1024);
  }
}

template <typename T, int RY, int K, bool FMA>
cudaError_t launch_k(TParams<T> p, const MarchConfig &cfg, const CUtensorMap *tin,
                     int sm_count, cudaStream_t st) {
  constexpr int VEC = 16 / (int)sizeof(T);
  constexpr int TXO = 30 * VEC;
  const int tye = cfg.warps * cfg.rows;
  const int tyo = tye - 2 * (p.k - 1);
  if (tyo < 1) return cudaErrorInvalidConfiguration;
  const size_t smem = temporal7_smem_bytes((int)sizeof(T), cfg, p.k);
  auto kern = t7_kernel<T, RY, K, FMA>;
  static size_t attr_set = 0;
  if (smem > attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = smem;
  }
  int oc = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&oc, kern, 32 * cfg.warps, smem);
  if (e != cudaSuccess) return e;
  if (oc < 1) return cudaErrorInvalidConfiguration;  // does not fit on an SM
  const int per_sm = (cfg.ctas_per_sm > 0 && cfg.ctas_per_sm < oc) ? cfg.ctas_per_sm : oc;
  p.tiles_x = (p.nx + TXO - 1) / TXO;
  p.tiles = p.tiles_x * ((p.ny + tyo - 1) / tyo);
  const int resident = sm_count * per_sm;
  p.zlen = choose_zchunk_overhead(p.tiles, p.nz, resident, 2 * p.k - 1);
  p.items = (int64_t)p.tiles * ((p.nz + p.zlen - 1) / p.zlen);
  int64_t grid = resident;
  if (grid > p.items) grid = p.items;
  kern<<<(unsigned)grid, dim3(32, cfg.warps, 1), smem, st>>>(*tin, p);
  return cudaGetLastError();
}

template <typename T, int RY, bool FMA>
cudaError_t launch_rows(const TParams<T> &p, const MarchConfig &cfg, const CUtensorMap *tin,
                        int sm_count, cudaStream_t st) {
  constexpr int VEC = 16 / (int)sizeof(T);
  if (p.k <= 2) return launch_k<T, RY, 2, FMA>(p, cfg, tin, sm_count, st);
  if (p.k <= 3) return launch_k<T, RY, 3, FMA>(p, cfg, tin, sm_count, st);
  if constexpr (VEC >= 4) {
    if (p.k <= 4) return launch_k<T, RY, 4, FMA>(p, cfg, tin, sm_count, st);
    if (p.k <= 5) return launch_k<T, RY, 5, FMA>(p, cfg, tin, sm_count, st);
  }
  return cudaErrorInvalidValue;
}

template <typename T, bool FMA>
cudaError_t launch_shape(const TParams<T> &p, const MarchConfig &cfg, const CUtensorMap *tin,
                         int sm_count, cudaStream_t st) {
  switch (cfg.rows) {
    case 1: return launch_rows<T, 1, FMA>(p, cfg, tin, sm_count, st);
    case 2: return launch_rows<T, 2, FMA>(p, cfg, tin, sm_count, st);
    case 4: return launch_rows<T, 4, FMA>(p, cfg, tin, sm_count, st);
  }
  return cudaErrorInvalidConfiguration;
}

template <typename T>
cudaError_t launch_t(const Temporal7Args &a, const MarchConfig &cfg, const CUtensorMap *tin,
                     int *dev_err, int sm_count, cudaStream_t st) {
  TParams<T> p;
  p.out = static_cast<T *>(a.out.ptr);
  p.row = a.out.pitch / (int64_t)sizeof(T);
  p.plane = p.row * a.out.ny;
  p.nx = a.in.nx;
  p.ny = a.in.ny;
  p.nz = a.in.nz;
  p.k = a.k;
  p.ns = cfg.ns;
  p.ce = (T)a.coef[0];
  p.cw = (T)a.coef[1];
  p.cn = (T)a.coef[2];
  p.cs = (T)a.coef[3];
  p.ct = (T)a.coef[4];
  p.cb = (T)a.coef[5];
  p.cc = (T)a.coef[6];
  p.err = dev_err;
  if (cfg.warps < 1 || cfg.warps > 8 || cfg.ns < 2 || cfg.ns > 16)
    return cudaErrorInvalidConfiguration;
  return a.fma ? launch_shape<T, true>(p, cfg, tin, sm_count, st)
               : launch_shape<T, false>(p, cfg, tin, sm_count, st);
}

}  // namespace

int temporal7_max_k(int esz) { return 16 / esz + 1; }

size_t temporal7_smem_bytes(int esz, const MarchConfig &cfg, int k) {
  const int vec = 16 / esz;
  const int w = 34 * vec;
  const int tye = cfg.warps * cfg.rows;
  const size_t plane = t_align128((uint32_t)(w * (tye + 2) * esz));
  return 128 + (size_t)t_bar_bytes(cfg.ns) + (size_t)cfg.ns * plane +
         (size_t)(k - 1) * 2 * plane;
}

cudaError_t launch_temporal7(const Temporal7Args &a, const MarchConfig &cfg,
                             const CUtensorMap *tin, int *dev_err, int sm_count,
                             cudaStream_t s) {
  if (a.k < 2 || a.k > temporal7_max_k(a.in.esz)) return cudaErrorInvalidValue;
  switch (a.in.type) {
    case kFloat: return launch_t<float>(a, cfg, tin, dev_err, sm_count, s);
    case kDouble: return launch_t<double>(a, cfg, tin, dev_err, sm_count, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace psg
