/*
 * physis_gb300.h -- additions to the Physis API exported by libphysis_gb300.so.
 *
 * 1. Non-variadic forms of the variadic Physis entry points, for foreign
 *    function interfaces (ctypes, cgo, JNI) that cannot build C varargs
 *    portably.  Each states the variadic call it is equivalent to.
 * 2. Error reporting (the reference aborts instead; physis_common.h:144-146,
 *    runtime_common_cuda.h:16-27).
 * 3. Device-resident access, timing on the runtime's stream and launch
 *    counting, used by benchmarks.
 * 4. Launch-shape control and the autotuner; batches of independent runs.
 * 5. A reduction for callers that cannot allocate.
 * 6. Test hooks that exercise failure handling without faulting a GPU.
 * 7. Point-list stencils and compiled stencil functions (the
 *    translator-free front ends) and the non-variadic red/black map.
 * 8. Building blocks of the learned warm start for the Jacobi solve.
 */
#ifndef PHYSIS_GB300_EXT_H_
#define PHYSIS_GB300_EXT_H_

#include "physis_gb300/physis.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Every declaration below is exported from the shared library even when it
 * is built with -fvisibility=hidden. */
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* ---- 1. Non-variadic entry points ------------------------------------- */

/* PSInit(NULL, NULL, 3) with an explicit trace switch. */
void PSInitV(int trace);

/* PSGrid{N}D{Type}New for any type (PS_FLOAT, ...) and rank 1..3; dims[i]
 * for i >= ndims are ignored.  Returns NULL on failure. */
void *PSGridNewV(int type, int ndims, const PSIndex *dims);

/* __PSGridSet(g, value, idx[0], ..., idx[rank-1]) with a status: value
 * points at one element of the grid's type.  Returns PS_OK or the error
 * code (an index outside the grid is PS_ERR_INVALID_ARGUMENT). */
int PSGridSetV(void *g, const PSIndex *idx, const void *value);

/* __PSStencilMap(kernel, *dom, grids[0..ngrids), scalars[0..nscalars)). */
PSStencil PSStencilMapV(int kernel, const PSDomain3D *dom, int ngrids,
                        void *const *grids, int nscalars,
                        const double *scalars);

/* PSStencilRun(stencils[0], ..., stencils[n-1], iter). */
void PSStencilRunV(int n, const PSStencil *stencils, int iter);

/* PSReduce(v, op, g). */
void PSReduceGridV(void *v, int op, void *g);

/* PSReduce(v, op, kernel, *dom, grids..., scalars...). */
void PSReduceKernelV(void *v, int op, int kernel, const PSDomain3D *dom,
                     int ngrids, void *const *grids, int nscalars,
                     const double *scalars);

/* Like PSReduceGridV but returns the FP64 combine of a float/double grid
 * before it is rounded to the element type. */
void PSReduceGridF64(double *v, int op, void *g);

/* ---- 2. Errors -------------------------------------------------------- */

enum PSErrorCode {
  PS_OK = 0,
  PS_ERR_NOT_INITIALIZED = 1,
  PS_ERR_INVALID_ARGUMENT = 2,
  PS_ERR_OUT_OF_MEMORY = 3,
  PS_ERR_CUDA = 4,
  PS_ERR_UNKNOWN_KERNEL = 5,
  PS_ERR_BAD_HANDLE = 6,
  PS_ERR_UNSUPPORTED = 7,
  PS_ERR_DEVICE_TIMEOUT = 8,
  PS_ERR_NO_DEVICE = 9,
  PS_ERR_IO = 10
};
/* First error recorded since the last PSClearError (sticky). */
int PSGetLastError(void);
const char *PSGetLastErrorString(void);
const char *PSGetErrorName(int code);
void PSClearError(void);

/* ---- 3. Device access, timing, counters ------------------------------- */

/* Device address, row pitch in bytes (a multiple of 128; nx * esz for grids
 * of a user-defined type) and element size of a grid.  Element (x,y,z) is at
 * ptr + (z*ny + y)*pitch + x*esz. */
void *PSGridDevicePtr(void *g);
size_t PSGridPitch(void *g);
int PSGridElemSize(void *g);
int PSGridType(void *g);
/* Copies a dense host buffer in/out without synchronising (the runtime's
 * stream orders it with kernels); host memory must stay valid until
 * PSSynchronize.  Pinned host memory gives DMA at full link speed. */
void PSGridCopyinAsync(void *g, const void *src);
void PSGridCopyoutAsync(void *g, void *dst);
/* Page-locked host allocation for the async copies. */
void *PSHostAlloc(size_t bytes);
void PSHostFree(void *p);
/* Waits for all work on the runtime's stream; checks the device error word
 * (a device-side bounded wait that gave up sets PS_ERR_DEVICE_TIMEOUT). */
void PSSynchronize(void);
/* The runtime's CUDA stream (a cudaStream_t). */
void *PSGetStream(void);
/* CUDA events on the runtime's stream: PSEventRecord(slot) records event
 * `slot` (0..63); PSEventElapsedMs(a, b) returns ms from a to b after
 * waiting for b. */
void PSEventRecord(int slot);
float PSEventElapsedMs(int a, int b);
/* Number of kernels this library launched since PSInit. */
long long PSGetLaunchCount(void);
/* Number of streaming multiprocessors of the runtime's device. */
int PSGetSMCount(void);

/* ---- 4. Launch shapes and the autotuner -------------------------------- */

/* Launch shape of a persistent z-marching sweep.  A CTA owns tiles 32
 * lanes x 16 bytes wide in x and warps*rows cells high in y and marches them
 * along z; each thread holds a column of `rows` rows in registers.  ns is
 * the number of shared-memory ring stages (planes in flight + 2), ns2 the
 * stages of Himeno's coefficient ring, ctas_per_sm the persistent grid size
 * per SM (0 = as many as fit).  A field <= 0 keeps the current value
 * (ctas_per_sm <= 0 selects "as many as fit").  Himeno kernels take
 * rows == 1 and at most 8 warps. */
typedef struct {
  int warps;
  int rows;
  int ns;
  int ns2;
  int ctas_per_sm;
} PSLaunchShape;
/* Sets the shape used for maps of `kernel` from now on (0 = every 7-point
 * kernel). */
void PSSetLaunchShape(int kernel, const PSLaunchShape *shape);
void PSGetLaunchShape(int kernel, PSLaunchShape *shape);

/* Temporal blocking: a PSStencilRun of the pair (g1 -> g2, g2 -> g1) of one
 * full-grid PS_KERNEL_DIFFUSION7 stencil runs k time steps per pass over
 * HBM (k = 1: off; at most 5 for float grids, 3 for double).  Results are
 * bit-identical to k plain steps and g1/g2 end holding the same steps as
 * with plain sweeps (their device storage may be exchanged).  `shape`
 * (warps <= 8, rows 1/2/4, ns; NULL keeps the current one) is the pass's own
 * launch shape; its tile height warps*rows must exceed 2*(k-1). */
void PSSetTemporalBlocking(int kernel, int k, const PSLaunchShape *shape);
void PSGetTemporalBlocking(int kernel, int *k, PSLaunchShape *shape);

/* Contraction (default 0: off).  With 1, temporal passes evaluate each
 * update's left-to-right sum as one multiply and six fused multiply-adds
 * instead of seven multiplies and six adds.  Results then differ from the
 * REF target, and from plain sweeps, by rounding only.  The difference grows
 * by about 1.3e-8 relative per step for the 7-point diffusion: under 1e-5 per
 * cell over 600 steps, about 1.2e-5 after 1000 (both measured at 512^3).
 * Plain sweeps stay bit-exact either way.  With contraction on, autotuner trials may mix the two
 * roundings. */
void PSSetFusedMultiplyAdd(int on);
int PSGetFusedMultiplyAdd(void);

/* Autotuner (replaces the reference's online trial of OPT_* variants and
 * block sizes, translator/reference_translator.cc:610-935).  When on
 * (PSSetAutotune(1) or PS_AUTOTUNE=1 at PSInit), the first iterations of a
 * PSStencilRun whose signature (kernels, grid size, type, domains, GPU) has
 * no tuned plan are spent trying launch shapes and, for full-grid diffusion
 * pairs, temporal depths; every candidate computes bit-identical results, so
 * the trials are ordinary iterations of the run.  Trials continue across
 * runs until all candidates are timed; the fastest becomes the signature's
 * plan.  With PS_TUNE_CACHE=<file> (or PSSetTuneCachePath) plans are
 * appended to that file as JSON lines and loaded at PSInit, so later
 * processes skip the trials.  A malformed cache line is ignored and
 * reported as PS_ERR_IO. */
void PSSetAutotune(int on);
void PSSetTuneCachePath(const char *path);
int PSLoadTuneCache(const char *path);  /* returns the number of plans loaded */
void PSClearTuning(void);               /* forgets all plans (not the file) */
/* The plan a stencil runs with: returns 1 if tuned, 0 if the defaults. */
int PSGetStencilPlan(PSStencil s, PSLaunchShape *shape, int *k, PSLaunchShape *tshape);

/* ---- 4b. Batches of independent runs ------------------------------------ */

/* No counterpart in the reference (Physis runs each PSStencilRun alone).
 * Many independent runs of uneven sizes advance together, one persistent
 * launch per time step over a (problem, z-chunk, tile) work list; runs of
 * more than 16 iterations replay a CUDA graph of 16.  maps holds nruns x
 * maps_per_run stencils (maps_per_run 1 or 2; the maps of one run share
 * kernel and domain, e.g. the g1->g2 / g2->g1 pair).  Float grids of
 * PS_KERNEL_DIFFUSION7, SUM7, COPY or HIMENO19.  A 7-point run uses the
 * rows per thread of its tuned plan (PSGetStencilPlan) if it has one.
 * Returns a batch id or -1. */
int PSBatchCreate(int nruns, int maps_per_run, const PSStencil *maps);
/* Runs `iter` iterations: every run executes its maps in order each time. */
void PSBatchRun(int batch, int iter);
void PSBatchFree(int batch);
/* Launch shape of batch kernels (default 4 warps, 4 rows, 4 / 4 / 2
 * stages): warps per CTA, rows per thread of untuned 7-point runs (1, 2, 4),
 * 7-point ring stages, Himeno p-ring and coefficient-ring stages. */
void PSSetBatchShape(int warps, int rows, int ns7, int nsp, int nsc);

/* ---- 5. Reduction for callers that cannot allocate --------------------- */

/* No counterpart in the reference.  PSReduce over a grid that the caller
 * holds in device memory, for callers that must not allocate GPU memory:
 * latency-bound loops that cannot afford the device-wide synchronisation a
 * cudaMalloc/cudaFree implies, and processes whose device memory is already
 * owned by another allocator (a framework's caching pool that has reserved
 * the free memory), where a further cudaMalloc fails or fragments it.  It
 * needs no PSInit and calls no cudaMalloc, cudaFree or allocating library
 * routine.
 *
 * data   : element (x,y,z) at data + (z*ny + y)*pitch + x*esz; 16-byte
 *          aligned, pitch a multiple of 16 bytes (grids of this library
 *          qualify: PSGridDevicePtr / PSGridPitch);
 * type   : PS_FLOAT, PS_DOUBLE, PS_INT or PS_LONG; op: a PSReduceOp;
 * result : 8 bytes of device memory receiving an FP64 value (float and
 *          double grids) or a 64-bit integer (int grids sign-extended from
 *          the 32-bit wrapped result, long grids as is);
 * stream : a cudaStream_t (NULL: the legacy default stream).  The call is
 *          asynchronous on that stream.
 * Scratch: a static device array of 2048 per-CTA partials plus a ticket
 * (16 KiB), held by every GPU that loads the library until exit.  A launch
 * that would need more partial slots than that is rejected
 * (PS_ERR_UNSUPPORTED; a 152-SM GB300 needs at most 608).  All calls share
 * the array and it keeps the last call's contents (the ticket is cleared on
 * the stream before each launch): calls whose work overlaps on the GPU race.
 * Set-up: the first call on a device (and the first after the device's
 * context was destroyed, e.g. by cudaDeviceReset) looks up the array's
 * device address with cudaGetSymbolAddress, which loads the module into the
 * current context and may synchronise with the device.  Set-up from
 * several host threads at once is serialised by a lock; after it, calls
 * take no lock.
 * Returns PS_OK or an error code (also recorded for PSGetLastError). */
int PSReduceNoAlloc(const void *data, size_t pitch, int nx, int ny, int nz, int type,
                    int op, void *result, void *stream);

/* ---- 6. Test hooks ------------------------------------------------------ */

/* The next `n` device allocations fail as if the GPU were out of memory. */
void PSTestFailNextAllocs(int n);
/* Launches one CTA that waits on an mbarrier nothing completes, with a
 * bounded wait of `limit` tries; afterwards PSSynchronize reports
 * PS_ERR_DEVICE_TIMEOUT and the context stays usable. */
void PSTestDeviceWaitTimeout(unsigned limit);

/* ---- 7. Point-list stencils --------------------------------------------- */

/* Boundary rules of a point stencil: none (the domain keeps every read inside
 * the grid), periodic ((i + n) % n per axis, include/physis/physis_ref.h:
 * 62-74, physis_cuda.h:247-269), clamp (the index is clamped to the grid; for
 * unit offsets this is the `if (x == 0) w = c;` face rule of
 * examples/diffusion-benchmark/diffusion3d_physis.c:40-54). */
enum PSBoundary { PS_BOUNDARY_NONE = 0, PS_BOUNDARY_PERIODIC = 1, PS_BOUNDARY_CLAMP = 2 };
#define PS_MAX_POINTS 64
#define PS_MAX_POINT_RADIUS 4

/* Registers the stencil
 *   out(x,y,z) = w[0]*in(x+o[0],y+o[1],z+o[2]) + w[1]*in(x+o[3],...) + ...
 * summed left to right in the given order, with `boundary` applied to each
 * read; weights == NULL means every term is the point value itself (the
 * plain neighbour sums of the reference's stencil functions, e.g.
 * tests/system_tests/test_cases/test_27-pt.c).  offsets holds 3*npoints
 * ints, each |offset| <= PS_MAX_POINT_RADIUS; 1 <= npoints <= PS_MAX_POINTS.
 * Returns a kernel id for PSStencilMap (grids: in, out; no scalars) and the
 * red/black maps (one grid, in place), or -1 with the error recorded.
 * Integer grids need integral weights and wrap on overflow.  Registering the
 * same stencil twice returns the same id.  No counterpart in the reference,
 * whose translator compiles the stencil function instead
 * (translator/reference_runtime_builder.cc:391-664). */
int PSPointStencilNew(int boundary, int npoints, const int *offsets, const double *weights);

/* Compiles a stencil function written in the reference's stencil language
 * and returns its kernel id, or -1 with the error recorded (the compiler log
 * for a source that does not compile; PS_ERR_UNSUPPORTED without NVRTC).
 * `source` holds the function `void name(const int x[, const int y[, const
 * int z]], <grids and scalars>)` -- index parameters first, then
 * PSGrid{1,2,3}D{Float,Double,Int,Long} grids and int/long/float/double
 * scalars in any order -- and whatever macros and helper functions it uses.
 * The body may use PSGridGet(g, ...), PSGridGetPeriodic(g, ...),
 * PSGridEmit(g, v) and PSGridDim(g, d) (include/physis/physis_user.h:75-81,
 * docs/programming.md).  PSStencilMap(id, dom, args...) then takes the
 * function's grids and scalars in its parameter order; the red/black maps
 * run it on one colour at a time (the function is then responsible for
 * reading only the other colour, as in the reference).  Float arithmetic
 * is compiled without FMA contraction, so results equal a REF build of the
 * same function (gcc -ffp-contract=off).  Compiling the same source and
 * name again returns the same id.  Replaces the translator's lowering of
 * stencil functions (translator/cuda_runtime_builder.cc:1099-1228). */
int PSStencilFunctionNew(const char *source, const char *name);

/* Parses and compiles a stencil function like PSStencilFunctionNew without
 * loading it (no device or PSInit needed).  Returns PS_OK, else
 * PS_ERR_INVALID_ARGUMENT (the reason and compiler log, truncated, in
 * log[0..logsize)) or PS_ERR_UNSUPPORTED without NVRTC.  On success log
 * names the grids the tiled entry stages in shared memory, one
 * "staged <grid> <rx> <ry> <rz> <clamp|periodic>;" each ("" if none). */
int PSStencilFunctionCheck(const char *source, const char *name, char *log, size_t logsize);

/* Map colours: every cell, red (x + y + z even), black (odd), red then black. */
enum PSMapColor {
  PS_COLOR_ALL = -1,
  PS_COLOR_RED = 0,
  PS_COLOR_BLACK = 1,
  PS_COLOR_REDBLACK = 2
};

/* __PSStencilMap / __PSStencilMapRed / Black / RedBlack(kernel, *dom,
 * grids..., scalars...) by colour (PS_COLOR_ALL is PSStencilMapV). */
PSStencil PSStencilMapColorV(int kernel, int color, const PSDomain3D *dom, int ngrids,
                             void *const *grids, int nscalars, const double *scalars);

/* ---- 8. Learned warm start for the 19-point Jacobi solve ----------------
 *
 * Building blocks of a small 3D convolutional network that predicts a warm
 * start for the Himeno Jacobi solve from its coefficient and source fields
 * (no counterpart in the reference).  Network tensors are channels-last
 * [batch][z][y][x][16] BF16 in device memory; weights are FP32 masters
 * [27 taps][16 in][16 out] (tap = (dz+1)*9 + (dy+1)*3 + (dx+1)) with BF16
 * copies for the kernels.  Every call takes device pointers and a stream
 * (NULL: the runtime's stream), allocates nothing, and returns PS_OK or an
 * error code (also recorded). */

/* y = epilogue(conv3x3x3(x, w_fwd) + bias) with zero padding; epilogue:
 * ReLU if relu != 0; times (mask > 0) if mask != NULL (the backward-data
 * pass: x = dY, w = w_bwd, mask = the layer's input).  y_ch0 (optional)
 * receives output channel 0 in FP32.  bias may be NULL. */
int PSWarmStartConv(const void *x, const void *w, const float *bias, const void *mask, int relu,
                    void *y, float *y_ch0, int batch, int nz, int ny, int nx, void *stream);

/* dw[27][16][16] = sum over voxels of x(v + tap) dy(v)^T, db[16] = sum of dy;
 * work holds nsplit * (27*256 + 16) floats of partial sums (reduced in a
 * fixed order: the result is deterministic). */
int PSWarmStartWeightGrad(const void *x, const void *dy, float *work, int nsplit, float *dw,
                          float *db, int batch, int nz, int ny, int nx, void *stream);

/* FP32 master w[27][16][16] -> BF16 w_fwd [27][out][in] and w_bwd (taps
 * reversed, [in][out]) for PSWarmStartConv. */
int PSWarmStartPrepareWeights(const float *w, void *w_fwd, void *w_bwd, void *stream);

/* One Adam step (Kingma & Ba 2015; step counts from 1) over n parameters. */
int PSWarmStartAdam(float *w, const float *g, float *m, float *v, long long n, float lr, float b1,
                    float b2, float eps, int step, void *stream);

/* dy (channel 0) = 2 (pred - target) / n, other channels 0; partials[i]
 * (one per 256 values) = sum of squared errors, in FP64. */
int PSWarmStartLoss(const float *pred, const float *target, long long n, void *dy,
                    double *partials, void *stream);

/* Instances of a Himeno batch laid out in stacked grids: instance b sits at
 * fine origin ((b % nsx) * inx, 0, (b / nsx) * inz) of float grids with row
 * pitch `pitch` bytes and ny rows per plane (PSGridDevicePtr / PSGridPitch
 * of grids made with PSGrid3DFloatNew). */
typedef struct PSWarmStartFields {
  const float *a0, *a1, *a2, *wrk1, *bnd, *p;
  long long pitch;
  int ny;
  int inx, iny, inz, nsx, factor, batch;
  float wscale, pscale;
  /* Mirror image the pooling calls read (0: the instance itself): bits 0, 1,
   * 2 mirror x, y, z; bit 3 swaps x and y together with a2 and a1, the x
   * and y coefficients (needs inx == iny).  With c_i = a_i and b = 0 the
   * mirrored fields' solution is the mirrored solution.  For the upsampling
   * calls, `coarse` is a prediction for this mirror image; they write the
   * stored instance. */
  int flip;
  /* Per-instance scale s[b] (NULL: 1): the pooling calls multiply the source
   * channels (and PoolTarget its target) by s[b], the upsampling calls
   * divide the prediction by it.  The equation is linear in the source, so
   * a residual source of any size can be brought to the network's input
   * range (PSWarmStartResidualSource computes such scales). */
  const float *inst_scale;
  /* PoolTarget only (NULL: none): the target is p - p_sub, the error of an
   * iterate p_sub against the solution p. */
  const float *p_sub;
} PSWarmStartFields;

/* Network input: per factor^3 block of each instance (of its mirror image),
 * channels: mean ln a0, mean ln a1, mean ln a2, mean wrk1 * wscale, mean bnd,
 * mean wrk1 * 3 / (a0 + a1 + a2) * wscale, -ln mean(1 / a0), -ln mean(1 / a1),
 * -ln mean(1 / a2), then zeros. */
int PSWarmStartPool(const PSWarmStartFields *f, void *out, void *stream);
/* Training target: p at each block's centre (c + 0.5) * factor - 0.5, the
 * mean of the fine cells nearest to it, times pscale (FP32). */
int PSWarmStartPoolTarget(const PSWarmStartFields *f, float *out, void *stream);
/* Warm start: p = bnd * cubic(coarse) / pscale at every fine cell:
 * Catmull-Rom interpolation per axis from coarse cell centres at
 * (c + 0.5) * factor - 0.5 (clamped). */
int PSWarmStartUpsample(const PSWarmStartFields *f, const float *coarse, float *p, void *stream);
/* The same added to p (p += ...): averaging the predictions for several
 * mirror images (pscale times their count) gives one warm start. */
int PSWarmStartUpsampleAdd(const PSWarmStartFields *f, const float *coarse, float *p,
                           void *stream);
/* Residual source of the iterate f->p for the correction problem.  The
 * 19-point residual (examples/himeno/himenobmtxpa_original.c:331-334) with
 * c_i = a_i, b = 0 is ss = (s0 a3 - p) bnd; r = ss / a3 is the source, in
 * wrk1's units, of the same equation for the error p* - p.  Writes r for
 * every cell of every instance into `r` (the fields' stacked layout; 0 on
 * the faces) and inst_scale[b] = target_rms / rms(r over instance b's
 * interior) (0 where r vanishes).  work: work_len doubles of caller scratch,
 * at least one per instance (64 per instance is used when given).  Pooling r
 * as wrk1 with these scales and upsampling the network's output with them
 * adds the network's prediction of the error: a learned restart. */
int PSWarmStartResidualSource(const PSWarmStartFields *f, float *r, float *inst_scale,
                              float target_rms, double *work, int work_len, void *stream);
/* p = p_scale * p + delta at every cell of every instance (the fields'
 * stacked layout; flip 0; delta may be NULL).  A restart sums the mirror
 * predictions into delta with PSWarmStartUpsample/UpsampleAdd and adds them
 * to the iterate with one rounding.  With delta NULL and p_scale = 1 - c
 * the iterate is pulled toward zero by a relative c: the last approach of
 * float32 Jacobi to its fixed point then runs along the solution, as a zero
 * start's does, instead of ending in a 2-cycle just above the tolerance
 * (which iterates brought very close by restarts often do). */
int PSWarmStartAddCorrection(const PSWarmStartFields *f, const float *delta, float p_scale,
                             float *p, void *stream);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif

#endif /* PHYSIS_GB300_EXT_H_ */
