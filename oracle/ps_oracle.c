/*
 * ps_oracle.c -- CPU oracle for the Physis stencil hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker, never the product:
 * only tests/, __graft_entry__.smoke() and the CPU-baseline legs of bench.py
 * load it.  The product library (libphysis_gb300.so) never links or calls it.
 *
 * It restates, in plain C, the semantics of Physis's REF (CPU) target for the
 * builtin stencils that the GPU library provides, plus an FP64 oracle of the
 * same arithmetic.  It is compiled with -ffp-contract=off so that every float
 * expression is evaluated exactly as written (no FMA contraction), which makes
 * its single-precision results bit-stable across x86-64 and aarch64 hosts.
 *
 * Layout: dense, x fastest: element (x,y,z) at x + y*nx + z*nx*ny
 *   (include/physis/physis_ref.h:50-74, include/physis/physis_cuda.h:237-244).
 * Domain: half-open box dom = {minx,maxx,miny,maxy,minz,maxz}
 *   (include/physis/physis_common.h:88-103; runtime/libphysis_rt_ref.cc:91-109).
 * Sweep: z -> y -> x nested loops over [min,max), stencil function applied at
 *   every point, emit = plain store at the same index
 *   (translator/reference_runtime_builder.cc:605-664, 142-177).
 * Run: for i < iter: for each map in order: sweep
 *   (translator/reference_runtime_builder.cc:837-894).
 * Reduce: sequential fold in the element type starting from d[0]
 *   (runtime/libphysis_rt_ref.cc:19-30, runtime/reduce.h:29-49).
 *
 * Parity pinning: tests/test_oracle_golden.py checks these functions against
 * the stdout of the reference's own hand-written REF oracles
 * (tests/system_tests/test_cases/test_*.manual.ref.c files), captured in tests/golden/.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* PSPrimitiveType (include/physis/types.h:16-23) */
enum { PSO_INT = 0, PSO_LONG = 1, PSO_FLOAT = 2, PSO_DOUBLE = 3 };
/* PSReduceOp (include/physis/reduce.h:16-21) */
enum { PSO_MAX = 0, PSO_MIN = 1, PSO_SUM = 2, PSO_PROD = 3 };
/* 7-point variants restated here (ids match physis_gb300 builtins). */
enum {
  PSO_V_DIFFUSION7 = 2, /* examples/diffusion-benchmark/diffusion3d_physis.c:29-58 */
  PSO_V_SUM7 = 5,       /* tests/system_tests/test_cases/test_7-pt.c:12-20 */
  PSO_V_SUM7_PERIODIC = 6 /* tests/system_tests/test_cases/test_7-pt-periodic.c:12-22 */
};

#define IDX(x, y, z) ((int64_t)(x) + (int64_t)(y) * nx + (int64_t)(z) * nx * ny)

static int pick_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads <= 0) return omp_get_max_threads();
  return nthreads;
#else
  (void)nthreads;
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* 7-point stencils                                                           */
/* ------------------------------------------------------------------------ */

/*
 * DIFFUSION7: clamped 7-point diffusion,
 *   c = g(x,y,z); w = x==0 ? c : g(x-1); e = x==nx-1 ? c : g(x+1);
 *   n = y==0 ? c : g(y-1); s = y==ny-1 ? c : g(y+1);
 *   b = z==0 ? c : g(z-1); t = z==nz-1 ? c : g(z+1);
 *   out = cc*c + cw*w + ce*e + cs*s + cn*n + cb*b + ct*t   (left to right)
 * (examples/diffusion-benchmark/diffusion3d_physis.c:29-58).
 * coef[] is in the map's argument order: ce, cw, cn, cs, ct, cb, cc
 * (diffusion3d_physis.c:31-33).
 *
 * SUM7: out = c + e + w + s + n + b + t, no clamp (the domain keeps every
 * neighbour inside the grid) (tests/system_tests/test_cases/test_7-pt.c:14-17).
 *
 * SUM7_PERIODIC: out = c + e + w + s + n + t + b with periodic wrap
 * (test_7-pt-periodic.c:14-21; periodic offsets include/physis/physis_ref.h:66-74).
 */
#define DEFINE_SWEEP7(NAME, T)                                                 \
  static void NAME(int variant, const T *g1, T *g2, int nx, int ny, int nz,   \
                   const int *dom, const double *coef, int nthreads) {         \
    const T ce = (T)coef[0], cw = (T)coef[1], cn = (T)coef[2],                 \
            cs = (T)coef[3], ct = (T)coef[4], cb = (T)coef[5],                 \
            cc = (T)coef[6];                                                   \
    int z;                                                                     \
    _Pragma("omp parallel for num_threads(nthreads) schedule(static)")         \
    for (z = dom[4]; z < dom[5]; ++z) {                                        \
      int y, x;                                                                \
      for (y = dom[2]; y < dom[3]; ++y) {                                      \
        for (x = dom[0]; x < dom[1]; ++x) {                                    \
          T c = g1[IDX(x, y, z)];                                              \
          T v;                                                                 \
          if (variant == PSO_V_DIFFUSION7) {                                   \
            T w = (x == 0) ? c : g1[IDX(x - 1, y, z)];                         \
            T e = (x == nx - 1) ? c : g1[IDX(x + 1, y, z)];                    \
            T n = (y == 0) ? c : g1[IDX(x, y - 1, z)];                         \
            T s = (y == ny - 1) ? c : g1[IDX(x, y + 1, z)];                    \
            T b = (z == 0) ? c : g1[IDX(x, y, z - 1)];                         \
            T t = (z == nz - 1) ? c : g1[IDX(x, y, z + 1)];                    \
            v = cc * c + cw * w + ce * e + cs * s + cn * n + cb * b + ct * t;  \
          } else if (variant == PSO_V_SUM7) {                                  \
            v = c + g1[IDX(x + 1, y, z)] + g1[IDX(x - 1, y, z)] +              \
                g1[IDX(x, y + 1, z)] + g1[IDX(x, y - 1, z)] +                  \
                g1[IDX(x, y, z - 1)] + g1[IDX(x, y, z + 1)];                   \
          } else {                                                             \
            int xp = (x + 1 + nx) % nx, xm = (x - 1 + nx) % nx;                \
            int yp = (y + 1 + ny) % ny, ym = (y - 1 + ny) % ny;                \
            int zp = (z + 1 + nz) % nz, zm = (z - 1 + nz) % nz;                \
            v = c + g1[IDX(xp, y, z)] + g1[IDX(xm, y, z)] +                    \
                g1[IDX(x, yp, z)] + g1[IDX(x, ym, z)] +                        \
                g1[IDX(x, y, zp)] + g1[IDX(x, y, zm)];                         \
          }                                                                    \
          g2[IDX(x, y, z)] = v;                                                \
        }                                                                      \
      }                                                                        \
    }                                                                          \
  }

DEFINE_SWEEP7(sweep7_f32, float)
DEFINE_SWEEP7(sweep7_f64, double)
DEFINE_SWEEP7(sweep7_i32, int32_t)
DEFINE_SWEEP7(sweep7_i64, int64_t)

/* One sweep of a 7-point variant: g2 = stencil(g1) over dom.  Returns 0 on
 * success, -1 on an unsupported (type, variant) pair. */
int pso_sweep7(int variant, int type, const void *g1, void *g2, int nx, int ny,
               int nz, const int *dom, const double *coef, int nthreads) {
  nthreads = pick_threads(nthreads);
  if (variant == PSO_V_DIFFUSION7 && (type == PSO_INT || type == PSO_LONG))
    return -1;
  switch (type) {
    case PSO_FLOAT:
      sweep7_f32(variant, (const float *)g1, (float *)g2, nx, ny, nz, dom, coef, nthreads);
      return 0;
    case PSO_DOUBLE:
      sweep7_f64(variant, (const double *)g1, (double *)g2, nx, ny, nz, dom, coef, nthreads);
      return 0;
    case PSO_INT:
      sweep7_i32(variant, (const int32_t *)g1, (int32_t *)g2, nx, ny, nz, dom, coef, nthreads);
      return 0;
    case PSO_LONG:
      sweep7_i64(variant, (const int64_t *)g1, (int64_t *)g2, nx, ny, nz, dom, coef, nthreads);
      return 0;
  }
  return -1;
}

/* PSStencilRun(PSStencilMap(k, dom, g1, g2, ...), PSStencilMap(k, dom, g2, g1, ...), iter)
 * in REF order (reference_runtime_builder.cc:837-894): each iteration runs
 * g1->g2 then g2->g1.  With pingpong == 0 only the first map is run. */
int pso_run7(int variant, int type, void *g1, void *g2, int nx, int ny, int nz,
             const int *dom, const double *coef, int iter, int pingpong,
             int nthreads) {
  int i, rc;
  for (i = 0; i < iter; ++i) {
    rc = pso_sweep7(variant, type, g1, g2, nx, ny, nz, dom, coef, nthreads);
    if (rc) return rc;
    if (pingpong) {
      rc = pso_sweep7(variant, type, g2, g1, nx, ny, nz, dom, coef, nthreads);
      if (rc) return rc;
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Point-list stencils and red/black sweeps                                  */
/* ------------------------------------------------------------------------ */

/*
 * out(x,y,z) = w0*in(p0) + w1*in(p1) + ... evaluated left to right, where
 * p_i = (x+dx_i, y+dy_i, z+dz_i) is mapped per axis by the boundary mode:
 *   0 none      every read is inside the grid (the caller's domain ensures it;
 *               e.g. test_27-pt.manual.ref.c, test_asymmetric.manual.ref.c);
 *   1 periodic  (i + n) % n (include/physis/physis_ref.h:62-74; the
 *               ((x - 1) + N) % N of test_27-pt-periodic.manual.ref.c);
 *   2 clamp     index clamped to [0, n-1] (for unit offsets this is the
 *               `if (x == 0) w = c; else w = g(x-1)` of
 *               test_7-pt-neumann-cond and test_16.manual.ref.c).
 * weights == NULL: every term is the point value itself (the plain sums of
 * the system tests; no multiply).  Integer grids wrap modulo 2^32 / 2^64.
 *
 * color -1: every cell of dom, out != in.  color 0 (red) / 1 (black): the
 * cells of dom with x starting at min + ((min & 1) ^ ((y + z + color) % 2)),
 * step 2 (translator/reference_runtime_builder.cc:585-600, 634-646), updated
 * in place (out may equal in) in z -> y -> x order, sequentially.
 * Returns 0, or -1 for an out-of-grid read in mode 0 or bad arguments.
 */
static inline int pso_map_axis(int i, int n, int boundary) {
  if (boundary == 1) return (i + n) % n;
  if (boundary == 2) return i < 0 ? 0 : (i >= n ? n - 1 : i);
  return i;
}

#define DEFINE_POINTS(NAME, T, U)                                              \
  static int NAME(int boundary, int npoints, const int *offs,                  \
                  const double *weights, const T *in, T *out, int nx, int ny,  \
                  int nz, const int *dom, int color, int nthreads) {           \
    T w[64];                                                                   \
    int i, z, bad = 0;                                                         \
    for (i = 0; i < npoints; ++i) w[i] = weights ? (T)weights[i] : (T)1;       \
    if (color < 0) {                                                           \
      _Pragma("omp parallel for num_threads(nthreads) schedule(static) reduction(|:bad)") \
      for (z = dom[4]; z < dom[5]; ++z) {                                      \
        int y, x, k;                                                           \
        for (y = dom[2]; y < dom[3]; ++y)                                      \
          for (x = dom[0]; x < dom[1]; ++x) {                                  \
            U v = 0;                                                           \
            for (k = 0; k < npoints; ++k) {                                    \
              int xx = pso_map_axis(x + offs[3 * k], nx, boundary);            \
              int yy = pso_map_axis(y + offs[3 * k + 1], ny, boundary);        \
              int zz = pso_map_axis(z + offs[3 * k + 2], nz, boundary);        \
              if (xx < 0 || xx >= nx || yy < 0 || yy >= ny || zz < 0 || zz >= nz) { \
                bad = 1;                                                       \
                continue;                                                      \
              }                                                                \
              U t = weights ? (U)((U)w[k] * (U)in[IDX(xx, yy, zz)])            \
                            : (U)in[IDX(xx, yy, zz)];                          \
              v = (k == 0) ? t : (U)(v + t);                                   \
            }                                                                  \
            out[IDX(x, y, z)] = (T)v;                                          \
          }                                                                    \
      }                                                                        \
      return bad ? -1 : 0;                                                     \
    }                                                                          \
    for (z = dom[4]; z < dom[5]; ++z) {                                        \
      int y, x, k;                                                             \
      for (y = dom[2]; y < dom[3]; ++y) {                                      \
        const int x0 = dom[0] + ((dom[0] & 1) ^ ((y + z + color) % 2));        \
        for (x = x0; x < dom[1]; x += 2) {                                     \
          U v = 0;                                                             \
          for (k = 0; k < npoints; ++k) {                                      \
            int xx = pso_map_axis(x + offs[3 * k], nx, boundary);              \
            int yy = pso_map_axis(y + offs[3 * k + 1], ny, boundary);          \
            int zz = pso_map_axis(z + offs[3 * k + 2], nz, boundary);          \
            if (xx < 0 || xx >= nx || yy < 0 || yy >= ny || zz < 0 || zz >= nz) \
              return -1;                                                       \
            U t = weights ? (U)((U)w[k] * (U)in[IDX(xx, yy, zz)])              \
                          : (U)in[IDX(xx, yy, zz)];                            \
            v = (k == 0) ? t : (U)(v + t);                                     \
          }                                                                    \
          out[IDX(x, y, z)] = (T)v;                                            \
        }                                                                      \
      }                                                                        \
    }                                                                          \
    return 0;                                                                  \
  }

DEFINE_POINTS(points_f32, float, float)
DEFINE_POINTS(points_f64, double, double)
DEFINE_POINTS(points_i32, int32_t, uint32_t)
DEFINE_POINTS(points_i64, int64_t, uint64_t)

int pso_points(int type, int boundary, int npoints, const int *offs,
               const double *weights, const void *in, void *out, int nx, int ny,
               int nz, const int *dom, int color, int nthreads) {
  if (npoints < 1 || npoints > 64 || boundary < 0 || boundary > 2 || color < -1 ||
      color > 1)
    return -1;
  nthreads = pick_threads(nthreads);
  switch (type) {
    case PSO_FLOAT:
      return points_f32(boundary, npoints, offs, weights, (const float *)in, (float *)out,
                        nx, ny, nz, dom, color, nthreads);
    case PSO_DOUBLE:
      return points_f64(boundary, npoints, offs, weights, (const double *)in,
                        (double *)out, nx, ny, nz, dom, color, nthreads);
    case PSO_INT:
      return points_i32(boundary, npoints, offs, weights, (const int32_t *)in,
                        (int32_t *)out, nx, ny, nz, dom, color, nthreads);
    case PSO_LONG:
      return points_i64(boundary, npoints, offs, weights, (const int64_t *)in,
                        (int64_t *)out, nx, ny, nz, dom, color, nthreads);
  }
  return -1;
}

/* ------------------------------------------------------------------------ */
/* Himeno 19-point Jacobi sweep                                              */
/* ------------------------------------------------------------------------ */

/*
 * One Jacobi sweep p1 = jacobi(p0) over dom, exactly as the Physis kernel
 * (examples/himeno/himenobmtxpa_physis.c:331-361), with i = x (fastest),
 * j = y, k = z:
 *   s0 = a0*p(i,j,k+1) + a1*p(i,j+1,k) + a2*p(i+1,j,k)
 *      + b0*(p(i,j+1,k+1) - p(i,j-1,k+1) - p(i,j+1,k-1) + p(i,j-1,k-1))
 *      + b1*(p(i+1,j+1,k) - p(i+1,j-1,k) - p(i-1,j+1,k) + p(i-1,j-1,k))
 *      + b2*(p(i+1,j,k+1) - p(i+1,j,k-1) - p(i-1,j,k+1) + p(i-1,j,k-1))
 *      + c0*p(i,j,k-1) + c1*p(i,j-1,k) + c2*p(i-1,j,k) + wrk1
 *   ss = (s0*a3 - p(i,j,k)) * bnd
 *   p1 = p(i,j,k) + omega*ss
 * The residual gosa = sum of ss*ss follows the original benchmark
 * (examples/himeno/himenobmtxpa_original.c:331-334).  Two residuals are
 * returned: *gosa_ref is the REF-style sequential float fold in z->y->x order
 * (only when nthreads == 1; NaN otherwise) and *gosa_fp64 is the FP64 sum of
 * the float ss*ss terms' exact squares (ss promoted to double).
 * arrays: p0,p1,a0,a1,a2,a3,b0,b1,b2,c0,c1,c2,bnd,wrk1 (the map's grid order,
 * himenobmtxpa_physis.c:381-383).
 */
#define DEFINE_HIMENO(NAME, T)                                                 \
  static void NAME(T *const *g, int nx, int ny, int nz, const int *dom,       \
                   double omega_d, int nthreads, float *gosa_ref,             \
                   double *gosa_fp64) {                                        \
    const T *p = g[0];                                                         \
    T *p1 = g[1];                                                              \
    const T *a0 = g[2], *a1 = g[3], *a2 = g[4], *a3 = g[5];                    \
    const T *b0 = g[6], *b1 = g[7], *b2 = g[8];                                \
    const T *c0 = g[9], *c1 = g[10], *c2 = g[11];                              \
    const T *bnd = g[12], *wrk1 = g[13];                                       \
    const T omega = (T)omega_d;                                                \
    double total = 0.0;                                                        \
    float fold = 0.0f;                                                         \
    int z;                                                                     \
    _Pragma("omp parallel for num_threads(nthreads) schedule(static) reduction(+:total)") \
    for (z = dom[4]; z < dom[5]; ++z) {                                        \
      int y, x;                                                                \
      for (y = dom[2]; y < dom[3]; ++y) {                                      \
        for (x = dom[0]; x < dom[1]; ++x) {                                    \
          int64_t c = IDX(x, y, z);                                            \
          T s0 = a0[c] * p[IDX(x, y, z + 1)] + a1[c] * p[IDX(x, y + 1, z)] +   \
                 a2[c] * p[IDX(x + 1, y, z)] +                                 \
                 b0[c] * (p[IDX(x, y + 1, z + 1)] - p[IDX(x, y - 1, z + 1)] -  \
                          p[IDX(x, y + 1, z - 1)] + p[IDX(x, y - 1, z - 1)]) + \
                 b1[c] * (p[IDX(x + 1, y + 1, z)] - p[IDX(x + 1, y - 1, z)] -  \
                          p[IDX(x - 1, y + 1, z)] + p[IDX(x - 1, y - 1, z)]) + \
                 b2[c] * (p[IDX(x + 1, y, z + 1)] - p[IDX(x + 1, y, z - 1)] -  \
                          p[IDX(x - 1, y, z + 1)] + p[IDX(x - 1, y, z - 1)]) + \
                 c0[c] * p[IDX(x, y, z - 1)] + c1[c] * p[IDX(x, y - 1, z)] +   \
                 c2[c] * p[IDX(x - 1, y, z)] + wrk1[c];                        \
          T ss = (s0 * a3[c] - p[c]) * bnd[c];                                 \
          p1[c] = p[c] + omega * ss;                                           \
          total += (double)ss * (double)ss;                                    \
          if (nthreads == 1) fold += (float)(ss * ss);                         \
        }                                                                      \
      }                                                                        \
    }                                                                          \
    if (gosa_fp64) *gosa_fp64 = total;                                         \
    if (gosa_ref) *gosa_ref = (nthreads == 1) ? fold : (float)NAN;             \
  }

DEFINE_HIMENO(himeno_f32, float)
DEFINE_HIMENO(himeno_f64, double)

int pso_himeno19(int type, void *const *grids, int nx, int ny, int nz,
                 const int *dom, double omega, int nthreads, float *gosa_ref,
                 double *gosa_fp64) {
  nthreads = pick_threads(nthreads);
  if (type == PSO_FLOAT) {
    himeno_f32((float *const *)grids, nx, ny, nz, dom, omega, nthreads, gosa_ref, gosa_fp64);
    return 0;
  }
  if (type == PSO_DOUBLE) {
    himeno_f64((double *const *)grids, nx, ny, nz, dom, omega, nthreads, gosa_ref, gosa_fp64);
    return 0;
  }
  return -1;
}

/* ------------------------------------------------------------------------ */
/* Reductions                                                                 */
/* ------------------------------------------------------------------------ */

/* REF PSReduce: v = d[0]; for i >= 1: v = op(v, d[i]) in the element type
 * (runtime/libphysis_rt_ref.cc:19-30; operators runtime/reduce.h:14-49:
 * max keeps x when x > y is false only if y is larger, i.e. (x > y) ? x : y). */
#define DEFINE_FOLD(NAME, T, ACC)                                              \
  static void NAME(const T *d, int64_t n, int op, void *out) {                 \
    ACC v = (ACC)d[0];                                                         \
    int64_t i;                                                                 \
    for (i = 1; i < n; ++i) {                                                  \
      ACC x = (ACC)d[i];                                                       \
      switch (op) {                                                            \
        case PSO_MAX: v = (v > x) ? v : x; break;                              \
        case PSO_MIN: v = (v < x) ? v : x; break;                              \
        case PSO_SUM: v = (ACC)(v + x); break;                                 \
        default: v = (ACC)(v * x); break;                                      \
      }                                                                        \
    }                                                                          \
    *(T *)out = (T)v;                                                          \
  }

DEFINE_FOLD(fold_f32, float, float)
DEFINE_FOLD(fold_f64, double, double)
/* int/long folds wrap modulo 2^32 / 2^64 (the REF fold overflows the same way
 * on every two's-complement host). */
DEFINE_FOLD(fold_i32_u, uint32_t, uint32_t)
DEFINE_FOLD(fold_i64_u, uint64_t, uint64_t)

static void fold_i32(const int32_t *d, int64_t n, int op, void *out) {
  if (op == PSO_SUM || op == PSO_PROD) {
    fold_i32_u((const uint32_t *)d, n, op, out);
    return;
  }
  int32_t v = d[0];
  for (int64_t i = 1; i < n; ++i) {
    if (op == PSO_MAX) v = (v > d[i]) ? v : d[i];
    else v = (v < d[i]) ? v : d[i];
  }
  *(int32_t *)out = v;
}

static void fold_i64(const int64_t *d, int64_t n, int op, void *out) {
  if (op == PSO_SUM || op == PSO_PROD) {
    fold_i64_u((const uint64_t *)d, n, op, out);
    return;
  }
  int64_t v = d[0];
  for (int64_t i = 1; i < n; ++i) {
    if (op == PSO_MAX) v = (v > d[i]) ? v : d[i];
    else v = (v < d[i]) ? v : d[i];
  }
  *(int64_t *)out = v;
}

int pso_reduce_ref(int type, int op, const void *data, int64_t n, void *out) {
  if (n <= 0 || op < 0 || op > 3) return -1;
  switch (type) {
    case PSO_FLOAT: fold_f32((const float *)data, n, op, out); return 0;
    case PSO_DOUBLE: fold_f64((const double *)data, n, op, out); return 0;
    case PSO_INT: fold_i32((const int32_t *)data, n, op, out); return 0;
    case PSO_LONG: fold_i64((const int64_t *)data, n, op, out); return 0;
  }
  return -1;
}

/* FP64 oracle of a reduction over float/double data: Neumaier-compensated
 * sum, product in double, exact min/max.  Elements are promoted exactly. */
int pso_reduce_fp64(int type, int op, const void *data, int64_t n, double *out) {
  if (n <= 0 || op < 0 || op > 3) return -1;
  if (type != PSO_FLOAT && type != PSO_DOUBLE) return -1;
  double v = 0.0, comp = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    double x = (type == PSO_FLOAT) ? (double)((const float *)data)[i]
                                   : ((const double *)data)[i];
    if (i == 0 && op != PSO_SUM) { v = x; continue; }
    switch (op) {
      case PSO_MAX: v = (v > x) ? v : x; break;
      case PSO_MIN: v = (v < x) ? v : x; break;
      case PSO_SUM: {
        double t = v + x;
        if (fabs(v) >= fabs(x)) comp += (v - t) + x;
        else comp += (x - t) + v;
        v = t;
        break;
      }
      default: v = v * x; break;
    }
  }
  *out = v + comp;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Input generation shared by the oracle, the tests and the benchmarks.      */
/* ------------------------------------------------------------------------ */

/* SplitMix64 (Steele, Lea, Flood 2014), counter-based so element i of a
 * stream with seed s is mix(s * 0x9E3779B97F4A7C15 + (i+1) * golden). */
static inline uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* out[i] = uniform[0,1) float with 24 random bits: (x >> 40) * 2^-24, where
 * x = splitmix64(seed * 2^32 + i).  Deterministic and parallel. */
void pso_fill_uniform_f32(float *out, int64_t n, uint64_t seed, int nthreads) {
  int64_t i;
  nthreads = pick_threads(nthreads);
  _Pragma("omp parallel for num_threads(nthreads) schedule(static)")
  for (i = 0; i < n; ++i) {
    uint64_t x = splitmix64((seed << 32) + (uint64_t)i);
    out[i] = (float)(x >> 40) * (1.0f / 16777216.0f);
  }
}

int pso_num_threads(void) { return pick_threads(0); }
