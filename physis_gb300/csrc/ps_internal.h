// Internal interface between the host runtime (runtime.cpp) and the kernel
// translation units.  Nothing here is exported.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace psg {

// PSPrimitiveType values (include/physis/types.h:16-23 in the reference).
enum ElemType { kInt = 0, kLong = 1, kFloat = 2, kDouble = 3, kUser = 4 };
// PSReduceOp values (include/physis/reduce.h:16-21 in the reference).
enum ReduceOp { kMax = 0, kMin = 1, kSum = 2, kProd = 3 };

// Builtin stencil kernel ids (the values of PS_KERNEL_* in
// include/physis_gb300/physis.h).
enum BuiltinKernel {
  kKernelCopy = 1,
  kKernelDiffusion7 = 2,
  kKernelHimeno19 = 3,
  kKernelHimeno19Gosa = 4,
  kKernelSum7 = 5,
  kKernelSum7Periodic = 6,
};

// Device view of one pitched grid: element (x,y,z) lives at
// ptr + z*pitch*ny + y*pitch + x*esz.  pitch is a multiple of 128 bytes and
// ptr is 256-byte aligned.
struct GridView {
  void *ptr;
  int64_t pitch;  // bytes per x-row
  int nx, ny, nz;
  int type;       // ElemType
  int esz;        // element size in bytes
};

// Half-open box [min, max) per dimension (x, y, z).
struct Box {
  int min[3];
  int max[3];
};

// Launch shape of a persistent 2.5D z-marching stencil kernel.  A tile is
// 32 lanes x 16 bytes wide in x and warps*rows rows high; each thread owns a
// column of `rows` rows.  `ns` is the number of shared-memory ring stages
// for the marched field, `ns2` that of a second ring (Himeno's coefficient
// planes).  The grid is SMs x ctas_per_sm CTAs (0 = as many as fit).
struct MarchConfig {
  int warps;
  int rows;
  int ns;
  int ns2;
  int ctas_per_sm;
};

// Chunk length (planes) for a z-march over `tiles` tiles and `nz` planes by
// `resident` concurrently resident CTAs: maximises the fraction of CTA time
// spent on useful planes, counting whole rounds of `resident` items and one
// extra plane of pipeline start-up per item.  Shared by the marching kernels
// (march.cpp).
int choose_zchunk(int tiles, int nz, int resident);
// The same with `overhead` start-up planes per item (a k-step temporal pass
// reads 2k extra input planes per item).
int choose_zchunk_overhead(int tiles, int nz, int resident, int overhead);

// Builds a 3D tiled tensor map over g with box {box_w, box_h, 1} elements.
// Implemented in runtime.cpp (driver entry point looked up at run time).
bool make_tmap_3d(CUtensorMap *map, const GridView &g, int box_w, int box_h);

// ---- 7-point family (stencil7.cu) ---------------------------------------
struct Stencil7Args {
  int kernel;  // kKernelDiffusion7 / kKernelSum7 / kKernelCopy
  GridView in, out;
  Box dom;
  double coef[7];  // map argument order: ce cw cn cs ct cb cc
};
// Number of bytes of dynamic shared memory the launch will use.
size_t stencil7_smem_bytes(int esz, const MarchConfig &cfg);
cudaError_t launch_stencil7(const Stencil7Args &a, const MarchConfig &cfg,
                            const CUtensorMap *tin, int *dev_err, int sm_count,
                            cudaStream_t s);

// ---- Temporal blocking of DIFFUSION7 (temporal7.cu) -----------------------
// One pass: out = k clamped diffusion steps of in over the whole grid.
struct Temporal7Args {
  GridView in, out;
  double coef[7];  // map argument order: ce cw cn cs ct cb cc
  int k;
  bool fma;        // contract each multiply-add (else bit-exact to k plain steps)
};
int temporal7_max_k(int esz);
size_t temporal7_smem_bytes(int esz, const MarchConfig &cfg, int k);
cudaError_t launch_temporal7(const Temporal7Args &a, const MarchConfig &cfg,
                             const CUtensorMap *tin, int *dev_err, int sm_count,
                             cudaStream_t s);

// ---- Himeno 19-point Jacobi (himeno19.cu) --------------------------------
struct Himeno19Args {
  GridView g[14];  // p0 p1 a0 a1 a2 a3 b0 b1 b2 c0 c1 c2 bnd wrk1
  Box dom;
  float omega;
  bool gosa;       // fused residual sum of ss*ss
};
struct ResidualSink {
  double *partials;     // one FP64 partial per CTA
  int max_partials;
  unsigned *ticket;     // last-CTA-done counter (kept at 0 between launches)
  double *result;       // where the FP64 total goes
};
size_t himeno19_smem_bytes(const MarchConfig &cfg);
cudaError_t launch_himeno19(const Himeno19Args &a, const MarchConfig &cfg,
                            const CUtensorMap *tmaps /* 13: p0-halo, 12 coef */,
                            const ResidualSink &sink, int *dev_err, int sm_count,
                            cudaStream_t s);

// ---- Point-list stencils and red/black sweeps (points.cu) -----------------
constexpr int kMaxPoints = 64;      // points per stencil
constexpr int kMaxPointRadius = 4;  // |offset| per axis
enum Boundary { kBoundaryNone = 0, kBoundaryPeriodic = 1, kBoundaryClamp = 2 };
struct PointsArgs {
  GridView in, out;  // same type and size; out == in for red/black
  Box dom;
  int boundary;
  int color;         // -1 every cell, 0 red, 1 black
  int n;
  int d[kMaxPoints][3];
  double w[kMaxPoints];
  bool unit;         // every weight is 1: terms are the point values
  int *err;          // device error word
  bool has_tmap;     // tmap maps `in` with the box points_box() gives
  CUtensorMap tmap;
};
// cfg.warps x points_rows(cfg) (1, 2 or 4) rows per tile; the other fields
// are unused.
int points_rows(const MarchConfig &cfg);
// The TMA box of one ring plane: w cells by h rows.
void points_box(const PointsArgs &a, const MarchConfig &cfg, int *w, int *h);
size_t points_smem_bytes(const PointsArgs &a, const MarchConfig &cfg);
cudaError_t launch_points(const PointsArgs &a, const MarchConfig &cfg, int sm_count,
                          cudaStream_t s);

// ---- Stencil functions compiled at run time (jit.cpp) ---------------------
struct JitParam {
  bool grid;              // a PSGrid* parameter, else a scalar
  int type;               // ElemType
  int rank;               // grids: 1..3
  std::string decl_type;  // the type as declared ("PSGrid3DFloat", "float")
  std::string name;       // the parameter's name
  std::string utype;      // kUser grids: the element type (DeclareGrid's "struct Point")
  int esz = 0;            // kUser grids: its size in bytes (read from the module; 0 unknown)
};
// A grid the tiled entry stages in shared memory: planes of (64 + 2 rxw) x
// (16 + 2 ry) cells around the CTA's tile (rxw: rx rounded up to 16 bytes),
// a ring of 2 rz + 5 of them.
struct JitStage {
  int param;            // index into params
  int rx, ry, rz;       // halo widths the stencil's reads need
  int rxw;              // x halo of the staged window
  bool periodic;        // halo cells wrap (else clamp to the grid)
  int esz;              // element size
  size_t off, bytes;    // byte range in dynamic shared memory
};
struct JitKernel {
  std::string name, source;
  int nd = 0;                     // index parameters (x[, y[, z]])
  std::string idx[3];             // their names
  std::vector<JitParam> params;   // after the indices, in order
  int ngrids = 0, nscalars = 0;
  std::vector<JitStage> stages;   // grids the tiled entry stages (3D only)
  size_t stage_smem = 0;
  void *module = nullptr, *func = nullptr;
  void *func_tiled = nullptr;     // __ps_entry_t, when stages is not empty
  int tiled_occ = 0;              // its resident CTAs per SM
};
// Parses `void name(...)` in source and compiles source + entry for sm_103a
// into *image (no device needed).  false with *err on failure.
bool jit_build(const char *source, const char *name, JitKernel *k, std::vector<char> *image,
               std::string *err);
// jit_build, then loads the image into the current context.
bool jit_compile(const char *source, const char *name, JitKernel *k, std::string *err);
void jit_unload(JitKernel *k);
// Runs the compiled stencil over dom (color -1 every point, 0 red, 1 black):
// grids[] and scalars[] in parameter order.
cudaError_t jit_launch(const JitKernel &k, const Box &dom, int color, const GridView *grids,
                       const double *scalars, int sm_count, cudaStream_t s);

// Point stencils compiled per stencil (jit.cpp compiles points_body.cuh with
// the table below as constants).  The key is everything the generated code
// depends on; the kernel takes one PtsParams<T> by value.
struct PtsJitKey {
  int type;                  // ElemType
  int ry, warps, n;
  bool unit;
  int w, nstage, pstride;
  int off[kMaxPoints], lag[kMaxPoints];
  double wt[kMaxPoints];
};
// The compiled kernel (cached; nullptr if NVRTC is missing or compiling
// failed, after which the table kernel is used).
void *jit_points_function(const PtsJitKey &k);
// Sets the kernel's dynamic shared memory limit and returns its occupancy.
bool jit_prepare(void *fn, int threads, size_t smem, int *occ);
// Launches a compiled kernel; args[i] points at its i-th parameter.
cudaError_t jit_launch_raw(void *fn, int grid, dim3 block, size_t smem, cudaStream_t s,
                           void **args);

// ---- Learned warm start (nn.cu) -------------------------------------------
// Fine stacked grids of a batch of Himeno instances (float, row pitch
// `pitch` bytes, ny rows per plane): instance b at fine origin
// ((b % nsx) * inx, 0, (b / nsx) * inz), size inx x iny x inz; coarse cells
// are factor^3 blocks.
struct NNFields {
  const float *a0, *a1, *a2, *wrk1, *bnd, *p;
  long long pitch;
  int ny;
  int inx, iny, inz, nsx, factor, batch;
  float wscale, pscale;
  int flip;  // mirror image: bits 0-2 mirror x/y/z, bit 3 swaps x and y
  const float *inst_scale;  // per-instance scale of source and solution (NULL: 1)
  const float *p_sub;       // pool_target: p - p_sub (NULL: p)
};
// Each returns 0, -1 for invalid arguments, or the launch's cudaError_t.
// Device error word for the kernels' bounded waits (set at PSInit).
void nn_set_error_word(int *err);
// The convolution runs as a tcgen05 implicit GEMM unless PS_WARMSTART_TC=0
// selects the mma.sync kernel.
int nn_conv(const void *x, const void *w, const float *bias, const void *mask, int relu,
            void *y, float *yf, int B, int Z, int Y, int X, cudaStream_t s);
int nn_wgrad(const void *x, const void *dy, float *part, int S, float *dw, float *db, int B,
             int Z, int Y, int X, cudaStream_t s);
int nn_prep_weights(const float *w, void *wf, void *wb, cudaStream_t s);
int nn_adam(float *w, const float *g, float *m, float *v, long long n, float lr, float b1,
            float b2, float eps, int step, cudaStream_t s);
int nn_mse(const float *pred, const float *tgt, long long n, void *dy, double *part,
           cudaStream_t s);
int nn_pool_inputs(const NNFields &f, void *out, cudaStream_t s);
int nn_pool_target(const NNFields &f, float *out, cudaStream_t s);
int nn_upsample(const NNFields &f, const float *coarse, float *p, bool add, cudaStream_t s);
// Residual source r of f.p for the correction problem, in f's stacked
// layout, and inst_scale[b] = target_rms / rms(r of instance b); work holds
// work_len doubles (at least one per instance).
int nn_residual_source(const NNFields &f, float *r, float *inst_scale, float target_rms,
                       double *work, int work_len, cudaStream_t s);
// p = p_scale * p + delta over every cell of every instance (f's stacked
// layout; delta may be NULL).
int nn_add_correction(const NNFields &f, const float *delta, float p_scale, float *p,
                      cudaStream_t s);

// ---- Reductions (reduce.cu) ----------------------------------------------
// Reduces every element of g with op.  The 8-byte result is written to
// *result: FP64 for float and double grids, int64 for int (wrapped to 32
// bits) and long grids.  partials holds one 8-byte slot per CTA.
int reduce_num_ctas(const GridView &g, int sm_count);
cudaError_t launch_reduce(const GridView &g, int op, uint64_t *partials,
                          int num_ctas, unsigned *ticket, uint64_t *result,
                          int *dev_err, cudaStream_t s);

// The reduction above with its scratch in a static device array (no
// allocation).  Returns PS_OK or a PSErrorCode value; *why explains a failure.
int reduce_noalloc(const void *data, size_t pitch, int nx, int ny, int nz, int type,
                   int op, void *result, cudaStream_t stream, const char **why);

// ---- Test support (failure detection without a GPU fault) ----------------
// Runs one CTA that waits on an mbarrier that nothing completes, with a
// short iteration limit; the wait gives up and sets kDevErrWaitTimeout.
cudaError_t launch_wait_timeout_probe(int *dev_err, uint32_t limit,
                                      cudaStream_t s);

}  // namespace psg
