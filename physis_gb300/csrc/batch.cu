// Batched execution of many independent stencil runs in one persistent
// launch per time step (GB300, sm_103a).  No counterpart in the reference,
// which runs every PSStencilRun by itself.
//
// Every problem (one run: a grid pair and its maps) is cut into (z-chunk,
// tile) work items exactly as its single-run kernel would cut it.  The items
// of all problems form one list, problem after problem and chunk-major within
// a problem; a persistent grid of SMs x occupancy CTAs takes items
// round-robin, so small problems fill the GPU together and large ones keep
// the chunk-major locality of the single-run kernels.  A CTA finds an item's
// problem by binary search over the problems' first item indices and runs
// the shared per-item body (s7_body.cuh / himeno_body.cuh) with that
// problem's parameters and tensor maps, both read from global memory.
// Problem kinds: the 7-point family (DIFFUSION7, SUM7, COPY; 1, 2 or 4 rows
// per thread) and the plain Himeno sweep, float grids.  The kernel is built
// per family (FAM = kBatch7, kBatchHimeno) so that each launch carries only
// its family's registers and shared memory; a batch holding both families
// launches one of each per step.
#include "batch.h"
#include "himeno_body.cuh"
#include "s7_body.cuh"

namespace psg {
namespace {

template <int K>
__device__ __forceinline__ bool s7_rows(const BatchProblem &bp, int parity,
                                        const CUtensorMap *tmaps, uint64_t *full, float *ring,
                                        int tile, int zs, int ze, RingPos &prod,
                                        RingPos &cons) {
  constexpr int W = 34 * 4;
  const S7Params<float> &p = bp.s7[parity];
  const CUtensorMap *tin = tmaps + bp.tmap[parity];
  const int TY = blockDim.y * bp.rows;
  const uint32_t plane_bytes = (uint32_t)(W * (TY + 2) * 4);
  const int plane_elems = (int)(s7_stage_bytes(plane_bytes) / 4);
  if (bp.rows == 1)
    return s7_item<float, K, 1>(tin, p, full, ring, plane_elems, plane_bytes, TY, tile, zs, ze,
                                prod, cons);
  if (bp.rows == 2)
    return s7_item<float, K, 2>(tin, p, full, ring, plane_elems, plane_bytes, TY, tile, zs, ze,
                                prod, cons);
  return s7_item<float, K, 4>(tin, p, full, ring, plane_elems, plane_bytes, TY, tile, zs, ze,
                              prod, cons);
}

template <int FAM>
__global__ void __launch_bounds__(256, 1)
batch_kernel(const BatchProblem *__restrict__ probs, int nprob, const CUtensorMap *tmaps,
             int64_t total_items, int parity, int ns7, int nsp, int nsc) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  uint64_t *full7 = reinterpret_cast<uint64_t *>(smem);
  uint64_t *pfull = full7 + ns7;
  uint64_t *cfull = pfull + nsp;
  unsigned char *data = smem + s7_bar_bytes(ns7 + nsp + nsc);
  // The 7-point ring and the Himeno rings share the data region: an item
  // consumes every plane it issues before the next item starts.
  float *ring7 = reinterpret_cast<float *>(data);
  const int TYh = blockDim.y;
  const int p_elems = (int)(h_align128((uint32_t)(kHimW * (TYh + 2) * 4)) / 4);
  float *pring = reinterpret_cast<float *>(data);
  float *cring = pring + nsp * p_elems;

  const int tid = threadIdx.y * 32 + threadIdx.x;
  if (tid == 0) {
    for (int s = 0; s < ns7 + nsp + nsc; ++s) mbar_init(&full7[s], 1);
    fence_barrier_init();
  }
  __syncthreads();

  RingPos prod7, cons7;
  HRing pprod, pcons, cprod, ccons;
  float acc = 0.0f;
  bool ok = true;
  for (int64_t item = blockIdx.x; item < total_items && ok; item += gridDim.x) {
    int lo = 0, hi = nprob - 1;  // last problem whose first item <= item
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (probs[mid].item_begin <= item) lo = mid;
      else hi = mid - 1;
    }
    const BatchProblem &bp = probs[lo];
    const int64_t local = item - bp.item_begin;
    const int chunk = (int)(local / bp.tiles);
    const int tile = (int)(local - (int64_t)chunk * bp.tiles);
    const int zs = bp.dmin2 + chunk * bp.zlen;
    const int ze = min(zs + bp.zlen, bp.dmax2);
    if constexpr (FAM == kBatch7) {
      switch (bp.kind) {
        case kKernelDiffusion7:
          ok = s7_rows<kKernelDiffusion7>(bp, parity, tmaps, full7, ring7, tile, zs, ze, prod7,
                                          cons7);
          break;
        case kKernelSum7:
          ok = s7_rows<kKernelSum7>(bp, parity, tmaps, full7, ring7, tile, zs, ze, prod7, cons7);
          break;
        default:
          ok = s7_rows<kKernelCopy>(bp, parity, tmaps, full7, ring7, tile, zs, ze, prod7, cons7);
          break;
      }
    } else {
      ok = himeno_item<false>(tmaps + bp.tmap[parity], tmaps + bp.cmap, bp.him[parity], pfull,
                              cfull, pring, cring, tile, zs, ze, pprod, pcons, cprod, ccons, acc);
    }
  }
  if (!ok && tid == 0) {
    for (int s = 0; s < ns7 + nsp + nsc; ++s) mbar_wait(&full7[s], 0, nullptr, 1024);
  }
}

}  // namespace

size_t batch_smem_bytes(const BatchShape &sh, int fam) {
  const size_t r7 = (size_t)sh.ns7 * s7_stage_bytes((uint32_t)(34 * 4 * (sh.warps * sh.max_rows + 2) * 4));
  const size_t rh = (size_t)sh.nsp * h_align128((uint32_t)(kHimW * (sh.warps + 2) * 4)) +
                    (size_t)sh.nsc * kHimCoef * kHimTX * sh.warps * 4;
  return 128 + (size_t)s7_bar_bytes(sh.ns7 + sh.nsp + sh.nsc) + (fam == kBatch7 ? r7 : rh);
}

namespace {
const void *batch_fn(int fam) {
  return fam == kBatch7 ? reinterpret_cast<const void *>(batch_kernel<kBatch7>)
                        : reinterpret_cast<const void *>(batch_kernel<kBatchHimeno>);
}
}  // namespace

int batch_occupancy(const BatchShape &sh, int fam) {
  int oc = 0;
  const size_t smem = batch_smem_bytes(sh, fam);
  if (cudaFuncSetAttribute(batch_fn(fam), cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&oc, batch_fn(fam), 32 * sh.warps, smem) !=
          cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return oc;
}

cudaError_t launch_batch(const BatchProblem *probs_dev, int nprob, const CUtensorMap *tmaps_dev,
                         int64_t total_items, int parity, const BatchShape &sh, int grid, int fam,
                         cudaStream_t s) {
  const size_t smem = batch_smem_bytes(sh, fam);
  if (fam == kBatch7)
    batch_kernel<kBatch7><<<grid, dim3(32, sh.warps, 1), smem, s>>>(
        probs_dev, nprob, tmaps_dev, total_items, parity, sh.ns7, sh.nsp, sh.nsc);
  else
    batch_kernel<kBatchHimeno><<<grid, dim3(32, sh.warps, 1), smem, s>>>(
        probs_dev, nprob, tmaps_dev, total_items, parity, sh.ns7, sh.nsp, sh.nsc);
  return cudaGetLastError();
}

}  // namespace psg
