// Host/device description of a batch of independent stencil runs
// (batch.cu).  Built by the runtime (runtime.cpp) and copied to the device.
#pragma once

#include "himeno_body.cuh"
#include "s7_body.cuh"

namespace psg {

struct BatchProblem {
  int kind;            // kKernelDiffusion7 / kKernelSum7 / kKernelCopy / kKernelHimeno19
  int rows;            // 7-point: rows per thread (1, 2 or 4)
  int64_t item_begin;  // index of this problem's first item in the batch
  int64_t items;
  int tiles, zlen, dmin2, dmax2;
  int tmap[2];         // input tensor map per parity (index into the batch's maps)
  int cmap;            // Himeno: first of the 12 coefficient maps
  S7Params<float> s7[2];
  HParams him[2];
};

struct BatchShape {
  int warps;     // CTA = 32 x warps threads
  int max_rows;  // largest 7-point rows per thread in the batch
  int ns7;       // 7-point ring stages
  int nsp, nsc;  // Himeno p ring and coefficient ring stages
};

// Kernel families: one launch runs the problems of one family.
constexpr int kBatch7 = 0;       // DIFFUSION7, SUM7, COPY
constexpr int kBatchHimeno = 1;  // HIMENO19

size_t batch_smem_bytes(const BatchShape &sh, int fam);
int batch_occupancy(const BatchShape &sh, int fam);  // CTAs per SM (0 on error)
// probs_dev[0 .. nprob) are the family's problems, item_begin counted from 0.
cudaError_t launch_batch(const BatchProblem *probs_dev, int nprob, const CUtensorMap *tmaps_dev,
                         int64_t total_items, int parity, const BatchShape &sh, int grid, int fam,
                         cudaStream_t s);

}  // namespace psg
