/*
 * physis.h -- drop-in C API of the GB300 stencil runtime (libphysis_gb300.so).
 *
 * Source-compatible with the user-level Physis API for the single-GPU CUDA
 * target: a program written against include/physis/physis.h of the reference
 * compiles against this header and links against libphysis_gb300.so.  The
 * one difference is PSStencilMap's first argument: the reference passes a
 * user stencil function that its source-to-source translator (physisc) turns
 * into a CUDA kernel; there is no translator here, so the first argument is a
 * builtin stencil id (PS_KERNEL_*) whose extra arguments follow the builtin's
 * documented signature.
 *
 * Every entry point below names the reference declaration it replaces.
 * Conventions kept from the reference:
 *  - grids are dense in host memory, x fastest ("column-major",
 *    docs/programming.md); PSGridCopyin/Copyout copy whole grids and return
 *    when the copy is complete;
 *  - float scalars pass through `...` promoted to double (C rules);
 *  - PSStencilRun runs `iter` times the listed maps in order, default 1
 *    (translator/reference_translator.cc:936-976);
 *  - PSReduce reduces every element of the grid (runtime/reduce_cuda.h:19-40).
 * Error handling: the reference aborts on CUDA errors
 * (runtime/runtime_common_cuda.h:16-27).  Here a failing call records a
 * sticky error readable with PSGetLastError()/PSGetLastErrorString() (see
 * physis_gb300.h) and returns; set PS_ABORT_ON_ERROR=1 in the environment to
 * abort instead.  The runtime is a process-global singleton on one GPU; calls
 * are not thread-safe (the reference is single-threaded too).
 */
#ifndef PHYSIS_GB300_PHYSIS_H_
#define PHYSIS_GB300_PHYSIS_H_

#include <limits.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Every declaration below is exported from the shared library even when it
 * is built with -fvisibility=hidden. */
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* include/physis/physis_common.h:27, 43-54: 32-bit index, at most 3 dims. */
#define PS_MAX_DIM (3)
typedef int32_t PSIndex;
typedef int PSVectorInt[PS_MAX_DIM];

/* include/physis/types.h:16-23 (PS_USER: grids of a user-defined struct) */
typedef int PSType;
enum PSPrimitiveType { PS_INT = 0, PS_LONG = 1, PS_FLOAT = 2, PS_DOUBLE = 3, PS_USER = 4 };

/* include/physis/reduce.h:16-21 */
enum PSReduceOp { PS_MAX, PS_MIN, PS_SUM, PS_PROD };

/* include/physis/physis_common.h:88-103: half-open box [min, max) per
 * dimension; local_* equals the global box on one GPU. */
typedef struct {
  PSIndex min[PS_MAX_DIM];
  PSIndex max[PS_MAX_DIM];
  PSIndex local_min[PS_MAX_DIM];
  PSIndex local_max[PS_MAX_DIM];
} __PSDomain;
typedef __PSDomain PSDomain1D;
typedef __PSDomain PSDomain2D;
typedef __PSDomain PSDomain3D;

/* Opaque grid handles (include/physis/physis_user.h:21-71 declares them as
 * pointers to per-type structs; user code never dereferences them). */
typedef struct __PSGrid1DFloat *PSGrid1DFloat;
typedef struct __PSGrid1DDouble *PSGrid1DDouble;
typedef struct __PSGrid1DInt *PSGrid1DInt;
typedef struct __PSGrid1DLong *PSGrid1DLong;
typedef struct __PSGrid2DFloat *PSGrid2DFloat;
typedef struct __PSGrid2DDouble *PSGrid2DDouble;
typedef struct __PSGrid2DInt *PSGrid2DInt;
typedef struct __PSGrid2DLong *PSGrid2DLong;
typedef struct __PSGrid3DFloat *PSGrid3DFloat;
typedef struct __PSGrid3DDouble *PSGrid3DDouble;
typedef struct __PSGrid3DInt *PSGrid3DInt;
typedef struct __PSGrid3DLong *PSGrid3DLong;

/* include/physis/physis_user.h:95 */
typedef int PSStencil;

/*
 * Builtin stencils (the PSStencilMap kernel argument).  After the domain,
 * each takes exactly the grids and scalars listed, in this order; scalars
 * are converted to the grid's element type as the reference's kernel
 * parameters would be.
 *
 * PS_KERNEL_COPY        (in, out): out = in over the domain.
 * PS_KERNEL_DIFFUSION7  (in, out, ce, cw, cn, cs, ct, cb, cc): clamped 7-point
 *     diffusion, out = cc*c + cw*w + ce*e + cs*s + cn*n + cb*b + ct*t with
 *     w/e = x-1/x+1, n/s = y-1/y+1, b/t = z-1/z+1 and a neighbour outside the
 *     grid replaced by the centre (examples/diffusion-benchmark/
 *     diffusion3d_physis.c:29-58).  Float and double grids.
 * PS_KERNEL_HIMENO19    (p0, p1, a0, a1, a2, a3, b0, b1, b2, c0, c1, c2, bnd,
 *     wrk1, omega): one 19-point Jacobi sweep p1 = jacobi(p0)
 *     (examples/himeno/himenobmtxpa_physis.c:331-361).  Float grids; the
 *     domain must stay one cell inside the grid.
 * PS_KERNEL_HIMENO19_GOSA (same arguments): the same sweep with the residual
 *     sum of ss*ss fused in; usable with PSReduce's kernel form (below).
 * PS_KERNEL_SUM7        (in, out): out = c + e + w + s + n + b + t, no clamp
 *     (tests/system_tests/test_cases/test_7-pt.c:12-20); the domain must
 *     stay one cell inside the grid.  All four element types.
 *
 * Further kernel ids come from PSPointStencilNew (physis_gb300.h): weighted
 * sums over a list of neighbour offsets with a boundary rule, taking
 * (in, out) and no scalars -- the 27-point, 9-point 2D, 3-point 1D,
 * periodic, asymmetric and red/black stencils of the reference's tests.
 */
enum PSBuiltinKernel {
  PS_KERNEL_COPY = 1,
  PS_KERNEL_DIFFUSION7 = 2,
  PS_KERNEL_HIMENO19 = 3,
  PS_KERNEL_HIMENO19_GOSA = 4,
  PS_KERNEL_SUM7 = 5
};

/* include/physis/physis_common.h:78 -- max dims after grid_num_dims are
 * accepted and ignored, as in the CUDA target (runtime/libphysis_rt_cuda.cc:
 * 25-36).  Removes "--physis-trace" from argv and, when present, prints
 * "Physis: Stencil started/finished" lines with times to stderr around each
 * PSStencilRun (runtime/runtime.h:20-30, reference_runtime_builder.cc:
 * 896-940).  argc/argv may be NULL. */
void PSInit(int *argc, char ***argv, int grid_num_dims, ...);
/* include/physis/physis_common.h:79 (libphysis_rt_cuda.cc:38-41).  Frees
 * every grid and the runtime's stream; unlike the reference it does not call
 * cudaDeviceReset, so other CUDA users in the process keep their context. */
void PSFinalize(void);
/* include/physis/physis_common.h:81: one line about the device and runtime. */
void PSPrintInternalInfo(FILE *out);

/* include/physis/physis_user.h:46-71 (DeclareGrid*D ... New).  Device
 * storage is zero-filled like the reference (libphysis_rt_cuda.cc:48-99).
 * Returns NULL on failure (out of memory, bad size, no runtime). */
PSGrid1DFloat PSGrid1DFloatNew(PSIndex nx, ...);
PSGrid1DDouble PSGrid1DDoubleNew(PSIndex nx, ...);
PSGrid1DInt PSGrid1DIntNew(PSIndex nx, ...);
PSGrid1DLong PSGrid1DLongNew(PSIndex nx, ...);
PSGrid2DFloat PSGrid2DFloatNew(PSIndex nx, PSIndex ny, ...);
PSGrid2DDouble PSGrid2DDoubleNew(PSIndex nx, PSIndex ny, ...);
PSGrid2DInt PSGrid2DIntNew(PSIndex nx, PSIndex ny, ...);
PSGrid2DLong PSGrid2DLongNew(PSIndex nx, PSIndex ny, ...);
PSGrid3DFloat PSGrid3DFloatNew(PSIndex nx, PSIndex ny, PSIndex nz, ...);
PSGrid3DDouble PSGrid3DDoubleNew(PSIndex nx, PSIndex ny, PSIndex nz, ...);
PSGrid3DInt PSGrid3DIntNew(PSIndex nx, PSIndex ny, PSIndex nz, ...);
PSGrid3DLong PSGrid3DLongNew(PSIndex nx, PSIndex ny, PSIndex nz, ...);

/* Grids of a user-defined element type (include/physis/physis_user.h:18-58,
 * DeclareGrid{1,2,3}D(name, type)).  `DeclareGrid3D(Point, struct Point);`
 * declares the handle type PSGrid3DPoint and PSGrid3DPointNew(nx, ny, nz),
 * which makes a zero-filled grid of sizeof(struct Point)-byte elements
 * (PSGridNewUtype).  Such grids are copied in and out like any other (dense
 * host arrays of the struct), written element by element with __PSGridSet,
 * and read and written by compiled stencil functions (PSStencilFunctionNew)
 * whose source holds the struct definition and the same DeclareGrid line;
 * PSGridGet(g, ...) there returns the struct and PSGridEmitUtype(g.member,
 * v) writes one member of the point being computed.  Builtin stencils,
 * point stencils and PSReduce take the primitive types only.  The elements
 * are stored densely (no row padding), in the host layout. */
void *PSGridNewUtype(size_t elem_size, int ndims, const PSIndex *dims);
#define DeclareGrid1D(name, type)                                              \
  typedef struct __PSGrid1D##name *PSGrid1D##name;                             \
  static inline PSGrid1D##name PSGrid1D##name##New(PSIndex nx, ...) {          \
    PSIndex d_[3] = {nx, 1, 1};                                                \
    return (PSGrid1D##name)PSGridNewUtype(sizeof(type), 1, d_);                \
  }                                                                            \
  typedef int PS__DeclaredGrid1D##name
#define DeclareGrid2D(name, type)                                              \
  typedef struct __PSGrid2D##name *PSGrid2D##name;                             \
  static inline PSGrid2D##name PSGrid2D##name##New(PSIndex nx, PSIndex ny, ...) { \
    PSIndex d_[3] = {nx, ny, 1};                                               \
    return (PSGrid2D##name)PSGridNewUtype(sizeof(type), 2, d_);                \
  }                                                                            \
  typedef int PS__DeclaredGrid2D##name
#define DeclareGrid3D(name, type)                                              \
  typedef struct __PSGrid3D##name *PSGrid3D##name;                             \
  static inline PSGrid3D##name PSGrid3D##name##New(PSIndex nx, PSIndex ny, PSIndex nz, \
                                                   ...) {                      \
    PSIndex d_[3] = {nx, ny, nz};                                              \
    return (PSGrid3D##name)PSGridNewUtype(sizeof(type), 3, d_);                \
  }                                                                            \
  typedef int PS__DeclaredGrid3D##name

/* include/physis/physis_common.h:83-86 (libphysis_rt_cuda.cc:101-137). */
void PSGridCopyin(void *g, const void *src_array);
void PSGridCopyout(void *g, void *dst_array);
void PSGridFree(void *g);
/* include/physis/physis_user.h:93 */
PSIndex PSGridDim(void *g, int d);

/* include/physis/physis_user.h:81 (PSGridSet(g, x[, y[, z]], v)) and the
 * target entry it becomes, __PSGridSet(g, &v, x, ...)
 * (include/physis/physis_cuda.h:137, runtime/libphysis_rt_cuda.cc:162-177):
 * writes one element from the host.  __PSGridSet takes as many PSIndex
 * arguments as the grid has dimensions and `buf` pointing at one element of
 * the grid's type.  The PSGridSet macro converts v to the grid's element
 * type as a C assignment would.  Indices are bounds-checked (the reference
 * does not check).  The element lands after every run already issued and
 * the call returns once it is on the GPU, like the reference's blocking
 * cudaMemcpy. */
void __PSGridSet(void *g, const void *buf, ...);
void __PSGridSetScalar(void *g, int nidx, PSIndex i, PSIndex j, PSIndex k, int is_float,
                       double vf, long long vi);
#define PS__NARG(...) PS__NARG_(__VA_ARGS__, 4, 3, 2, 1, 0)
#define PS__NARG_(a, b, c, d, n, ...) n
#define PS__CAT(a, b) PS__CAT_(a, b)
#define PS__CAT_(a, b) a##b
/* 1 when v has a floating type: (v*0 + 1)/2 is 0 in integer arithmetic and
 * 0.5 (NaN for an infinite or NaN v) in floating arithmetic. */
#define PS__IS_FLOAT(v) ((((v) * 0 + 1) / 2) != 0)
#define PS__SETV(v) PS__IS_FLOAT(v), (PS__IS_FLOAT(v) ? (double)(v) : 0.0), \
                    (PS__IS_FLOAT(v) ? 0LL : (long long)(v))
#define PS__GRIDSET2(g, i, v) __PSGridSetScalar((g), 1, (PSIndex)(i), 0, 0, PS__SETV(v))
#define PS__GRIDSET3(g, i, j, v) __PSGridSetScalar((g), 2, (PSIndex)(i), (PSIndex)(j), 0, \
                                                   PS__SETV(v))
#define PS__GRIDSET4(g, i, j, k, v) __PSGridSetScalar((g), 3, (PSIndex)(i), (PSIndex)(j), \
                                                      (PSIndex)(k), PS__SETV(v))
#define PSGridSet(g, ...) PS__CAT(PS__GRIDSET, PS__NARG(__VA_ARGS__))(g, __VA_ARGS__)

/* include/physis/physis_common.h:105-111 (libphysis_rt_ref.cc:91-109). */
PSDomain1D PSDomain1DNew(PSIndex minx, PSIndex maxx);
PSDomain2D PSDomain2DNew(PSIndex minx, PSIndex maxx, PSIndex miny, PSIndex maxy);
PSDomain3D PSDomain3DNew(PSIndex minx, PSIndex maxx, PSIndex miny,
                         PSIndex maxy, PSIndex minz, PSIndex maxz);

/* include/physis/physis_user.h:98-99: PSStencilMap(k, dom, args...).
 * k is a PS_KERNEL_* id; the domain is passed by value. */
PSStencil __PSStencilMap(void *kernel, ...);
#define PSStencilMap(k, ...) __PSStencilMap((void *)(intptr_t)(k), __VA_ARGS__)

/* include/physis/physis_user.h:100-105: red/black maps.  The kernel updates
 * its one grid in place, first the "red" cells (x + y + z even), then the
 * "black" ones (odd) for PSStencilMapRedBlack; PSStencilMapRed / Black run
 * one colour (translator/reference_runtime_builder.cc:585-600, 634-646,
 * 875-890).  k is a point stencil id (PSPointStencilNew), PS_KERNEL_SUM7 or
 * PS_KERNEL_DIFFUSION7; the arguments after the domain are the grid and
 * then the kernel's scalars.  Every non-centre point of the stencil must lie
 * at an odd distance (|dx|+|dy|+|dz|), so that a colour reads only cells of
 * the other colour and the parallel sweep equals the sequential one. */
PSStencil __PSStencilMapRedBlack(void *kernel, ...);
PSStencil __PSStencilMapRed(void *kernel, ...);
PSStencil __PSStencilMapBlack(void *kernel, ...);
#define PSStencilMapRedBlack(k, ...) __PSStencilMapRedBlack((void *)(intptr_t)(k), __VA_ARGS__)
#define PSStencilMapRed(k, ...) __PSStencilMapRed((void *)(intptr_t)(k), __VA_ARGS__)
#define PSStencilMapBlack(k, ...) __PSStencilMapBlack((void *)(intptr_t)(k), __VA_ARGS__)

/* include/physis/physis_user.h:106: PSStencilRun(s0, s1, ..., [iter]).
 * The macro appends PS_RUN_END so the runtime can find the end of the list;
 * an argument that is not a stencil id is the iteration count. */
#define PS_RUN_END INT_MIN
void PSStencilRun(PSStencil s, ...);
#define PSStencilRun(...) PSStencilRun(__VA_ARGS__, PS_RUN_END)

/* include/physis/physis_user.h:108, docs/programming.md:280-315.
 *   PSReduce(&v, op, grid)            reduce every element of grid; v has the
 *                                     grid's element type.
 *   PSReduce(&v, op, k, dom, args...) kernel form (documented in the
 *                                     reference, not implemented there): run
 *                                     builtin k over dom with args and reduce
 *                                     the value it yields per point.  Only
 *                                     PS_KERNEL_HIMENO19_GOSA has one (ss*ss,
 *                                     with the sweep's p1 emitted as well);
 *                                     v is a float.
 * Float sums are accumulated in FP32 per CTA and combined in FP64. */
void PSReduce(void *v, ...);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif

#endif /* PHYSIS_GB300_PHYSIS_H_ */
