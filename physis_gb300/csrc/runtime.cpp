// Host runtime of libphysis_gb300.so: the PS* C ABI over device-resident
// pitched grids, builtin stencil maps and the launchers in stencil7.cu,
// himeno19.cu and reduce.cu.
//
// Replaces, for one GPU, the reference's CUDA runtime library
// (runtime/libphysis_rt_cuda.cc) and the per-program code its translator
// generates for PSStencilMap / PSStencilRun (translator/
// reference_runtime_builder.cc:391-541, 837-894; cuda_runtime_builder.cc:
// 1465-1583).  Differences by design:
//  * grids are pitched: every x-row starts on a 128-byte boundary (the
//    reference allocates dense rows, libphysis_rt_cuda.cc:48-99), so TMA boxes
//    and 16-byte vector accesses are always aligned;
//  * all work goes to one runtime-owned stream; PSGridCopyin/Copyout and
//    PSReduce wait for it, like the reference's blocking cudaMemcpy;
//  * errors are recorded (sticky) instead of exiting the process.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <unordered_set>
#include <vector>

#include "physis_gb300/physis_gb300.h"
#undef PSStencilRun
#include "ps_internal.h"
#include "batch.h"

using psg::GridView;
using psg::MarchConfig;

namespace {

constexpr uint32_t kGridMagic = 0x50534744u;  // "PSGD"
constexpr int kStencilTag = 0x5A000000;       // PSStencil = tag | map index
constexpr int kStencilTagMask = 0x7F000000;
constexpr int kMaxMaps = 1 << 24;
constexpr int kNumEvents = 64;
constexpr int kMaxPartials = 1 << 16;
constexpr int kNumKernels = 8;
constexpr int kSlotPoints = 7;     // launch-shape slot shared by all point stencils
constexpr int kPointsBase = 1024;  // kernel id of the first registered point stencil
constexpr int kMaxPointStencils = 1 << 16;
constexpr int kFuncBase = 1 << 20;     // kernel id of the first compiled stencil function
constexpr int kMaxFunctions = 1 << 16;

// Tensor maps are cached per (device view, box); an entry is dropped when
// its grid is freed.
struct TmapEntry {
  GridView v;
  int w, h;
  CUtensorMap map;
};

struct Grid {
  uint32_t magic;
  int type, esz, ndims;
  int dim[3];
  size_t pitch, bytes;
  void *dev;
};

// How a run executes: the sweep's launch shape and, for temporal-eligible
// pairs, the temporal depth and the passes' shape.
struct Plan {
  MarchConfig shape;
  int k;
  MarchConfig tshape;
};

// A registered point-list stencil (PSPointStencilNew).
struct PointStencil {
  int boundary = 0, n = 0;
  int d[psg::kMaxPoints][3];
  double w[psg::kMaxPoints];
  bool unit = true;
};

struct Map {
  int kernel;
  int color = -1;  // -1 every cell; 0 red, 1 black, 2 red then black (in place)
  __PSDomain dom;
  std::vector<Grid *> grids;  // red/black maps hold their one grid twice
  std::vector<double> scalars;
  bool has_plan = false;  // set by the autotuner (or its cache)
  Plan plan;
};

struct Runtime {
  int device = 0;
  cudaStream_t stream = nullptr;
  // a second stream for the Himeno launch of a batch step, forked from and
  // joined back into `stream` by the two events
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  int sm_count = 0;
  bool trace = false;
  int *dev_err = nullptr;
  uint64_t *partials = nullptr;
  unsigned *ticket = nullptr;
  uint64_t *results = nullptr;  // slot 0: reductions, slot 1: residuals
  cudaEvent_t events[kNumEvents] = {};
  long long launches = 0;
  std::deque<Map> maps;  // deque: references stay valid as maps are added
  std::unordered_set<Grid *> grids;
  MarchConfig shapes[kNumKernels];
  int tblock[kNumKernels] = {};            // temporal steps per pass (<= 1: off)
  MarchConfig tshapes[kNumKernels];        // launch shape of temporal passes
  std::vector<TmapEntry> tmaps;
  int fail_allocs = 0;
  bool fma = false;  // temporal passes may contract multiply-adds
  bool autotune = false;
  std::string tune_path;  // JSON-lines cache file ("" = in memory only)
  std::string gpu_name;
  std::vector<PointStencil> points;  // kernel id kPointsBase + index
  std::deque<psg::JitKernel> funcs;  // kernel id kFuncBase + index
};

Runtime *rt = nullptr;
int g_err = PS_OK;
std::string g_errmsg;

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t,
                                  void *, const cuuint64_t *, const cuuint64_t *,
                                  const cuuint32_t *, const cuuint32_t *,
                                  CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn g_encode = nullptr;

const char *err_name(int code) {
  switch (code) {
    case PS_OK: return "PS_OK";
    case PS_ERR_NOT_INITIALIZED: return "PS_ERR_NOT_INITIALIZED";
    case PS_ERR_INVALID_ARGUMENT: return "PS_ERR_INVALID_ARGUMENT";
    case PS_ERR_OUT_OF_MEMORY: return "PS_ERR_OUT_OF_MEMORY";
    case PS_ERR_CUDA: return "PS_ERR_CUDA";
    case PS_ERR_UNKNOWN_KERNEL: return "PS_ERR_UNKNOWN_KERNEL";
    case PS_ERR_BAD_HANDLE: return "PS_ERR_BAD_HANDLE";
    case PS_ERR_UNSUPPORTED: return "PS_ERR_UNSUPPORTED";
    case PS_ERR_DEVICE_TIMEOUT: return "PS_ERR_DEVICE_TIMEOUT";
    case PS_ERR_NO_DEVICE: return "PS_ERR_NO_DEVICE";
    case PS_ERR_IO: return "PS_ERR_IO";
  }
  return "PS_ERR_UNKNOWN";
}

bool abort_on_error() {
  const char *e = getenv("PS_ABORT_ON_ERROR");
  return e && e[0] == '1';
}

// Records the first error since the last PSClearError; always returns false
// so call sites can `return fail(...)`.
bool fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list vl;
  va_start(vl, fmt);
  vsnprintf(buf, sizeof(buf), fmt, vl);
  va_end(vl);
  if (g_err == PS_OK) {
    g_err = code;
    g_errmsg = std::string(err_name(code)) + ": " + buf;
  }
  if (abort_on_error()) {
    fprintf(stderr, "physis_gb300: %s: %s\n", err_name(code), buf);
    abort();
  }
  return false;
}

bool cuda_ok(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return true;
  if (e == cudaErrorMemoryAllocation)
    return fail(PS_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
  return fail(PS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

bool need_rt(const char *fn) {
  if (rt) return true;
  return fail(PS_ERR_NOT_INITIALIZED, "%s called before PSInit", fn);
}

Grid *as_grid(void *g, const char *fn) {
  Grid *p = static_cast<Grid *>(g);
  if (!rt) {
    fail(PS_ERR_NOT_INITIALIZED, "%s called before PSInit", fn);
    return nullptr;
  }
  if (!p || !rt->grids.count(p) || p->magic != kGridMagic) {
    fail(PS_ERR_BAD_HANDLE, "%s: %p is not a live grid", fn, g);
    return nullptr;
  }
  return p;
}

constexpr int kMaxUserElem = 4096;  // bytes per user-type element

int esize(int type) {
  switch (type) {
    case PS_INT: return 4;
    case PS_LONG: return 8;
    case PS_FLOAT: return 4;
    case PS_DOUBLE: return 8;
  }
  return 0;
}

GridView view(const Grid *g) {
  GridView v;
  v.ptr = g->dev;
  v.pitch = (int64_t)g->pitch;
  v.nx = g->dim[0];
  v.ny = g->dim[1];
  v.nz = g->dim[2];
  v.type = g->type;
  v.esz = g->esz;
  return v;
}

// Checks the device error word; a device-side wait that gave up leaves a
// non-zero value.  Also re-arms the reduction ticket, which an interrupted
// reduction may have left non-zero.
bool check_device_errors() {
  int h = 0;
  if (!cuda_ok(cudaMemcpyAsync(&h, rt->dev_err, sizeof(int), cudaMemcpyDeviceToHost,
                               rt->stream), "read device error word"))
    return false;
  if (!cuda_ok(cudaStreamSynchronize(rt->stream), "cudaStreamSynchronize")) return false;
  if (h != 0) {
    cudaMemsetAsync(rt->dev_err, 0, sizeof(int), rt->stream);
    cudaMemsetAsync(rt->ticket, 0, sizeof(unsigned), rt->stream);
    cudaStreamSynchronize(rt->stream);
    return fail(PS_ERR_DEVICE_TIMEOUT,
                "a device-side wait gave up (error bits 0x%x); results of the "
                "affected launch are invalid", h);
  }
  return true;
}

bool sync_rt() {
  cudaError_t e = cudaStreamSynchronize(rt->stream);
  if (!cuda_ok(e, "cudaStreamSynchronize")) return false;
  return check_device_errors();
}

bool same_view(const GridView &a, const GridView &b) {
  return a.ptr == b.ptr && a.pitch == b.pitch && a.nx == b.nx && a.ny == b.ny &&
         a.nz == b.nz && a.type == b.type;
}

// Returns a copy of the cached (or newly encoded) tensor map for view v
// with box {w, h, 1}; false on failure.
bool tmap_for(const GridView &v, int w, int h, CUtensorMap *out) {
  for (const auto &e : rt->tmaps)
    if (e.w == w && e.h == h && same_view(e.v, v)) {
      *out = e.map;
      return true;
    }
  TmapEntry e;
  e.v = v;
  e.w = w;
  e.h = h;
  if (!psg::make_tmap_3d(&e.map, v, w, h)) return false;
  rt->tmaps.push_back(e);
  *out = e.map;
  return true;
}

void drop_tmaps(const void *ptr) {
  auto &t = rt->tmaps;
  for (size_t i = 0; i < t.size();) {
    if (t[i].v.ptr == ptr) {
      t[i] = t.back();
      t.pop_back();
    } else {
      ++i;
    }
  }
}

struct KernelSig {
  int ngrids, nscalars;
  const char *name;
  const psg::JitKernel *fn = nullptr;  // compiled stencil functions: the signature
};

const PointStencil *point_stencil(int k) {
  if (!rt || k < kPointsBase || k - kPointsBase >= (int)rt->points.size()) return nullptr;
  return &rt->points[k - kPointsBase];
}

const psg::JitKernel *jit_kernel(int k) {
  if (!rt || k < kFuncBase || k - kFuncBase >= (int)rt->funcs.size()) return nullptr;
  return &rt->funcs[k - kFuncBase];
}

bool kernel_sig(int k, KernelSig *s) {
  if (const psg::JitKernel *f = jit_kernel(k)) {
    *s = {f->ngrids, f->nscalars, f->name.c_str(), f};
    return true;
  }
  switch (k) {
    case PS_KERNEL_COPY: *s = {2, 0, "PS_KERNEL_COPY"}; return true;
    case PS_KERNEL_DIFFUSION7: *s = {2, 7, "PS_KERNEL_DIFFUSION7"}; return true;
    case PS_KERNEL_HIMENO19: *s = {14, 1, "PS_KERNEL_HIMENO19"}; return true;
    case PS_KERNEL_HIMENO19_GOSA: *s = {14, 1, "PS_KERNEL_HIMENO19_GOSA"}; return true;
    case PS_KERNEL_SUM7: *s = {2, 0, "PS_KERNEL_SUM7"}; return true;
  }
  if (point_stencil(k)) {
    *s = {2, 0, "point stencil"};
    return true;
  }
  return false;
}

// Registers ps (or finds an identical registration); returns its kernel id
// or -1.
int register_points(const PointStencil &ps) {
  for (size_t i = 0; i < rt->points.size(); ++i) {
    const PointStencil &q = rt->points[i];
    if (q.boundary != ps.boundary || q.n != ps.n || q.unit != ps.unit) continue;
    bool same = true;
    for (int j = 0; j < ps.n && same; ++j)
      same = q.d[j][0] == ps.d[j][0] && q.d[j][1] == ps.d[j][1] && q.d[j][2] == ps.d[j][2] &&
             (ps.unit || q.w[j] == ps.w[j]);
    if (same) return kPointsBase + (int)i;
  }
  if ((int)rt->points.size() >= kMaxPointStencils) {
    fail(PS_ERR_OUT_OF_MEMORY, "more than %d point stencils", kMaxPointStencils);
    return -1;
  }
  rt->points.push_back(ps);
  return kPointsBase + (int)rt->points.size() - 1;
}

// The point-stencil equivalents of the 7-point builtins, for their red/black
// maps.  SUM7: c + e + w + s + n + b + t unclamped (test_7-pt.c:12-20, the
// same order as test_redblack.c).  DIFFUSION7: cc*c + cw*w + ce*e + cs*s +
// cn*n + cb*b + ct*t clamped; scalars in map order ce cw cn cs ct cb cc.
int builtin_as_points(int kernel, const std::vector<double> &sc) {
  PointStencil ps;
  ps.n = 7;
  if (kernel == PS_KERNEL_SUM7) {
    const int d[7][3] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0},
                         {0, -1, 0}, {0, 0, -1}, {0, 0, 1}};
    memcpy(ps.d, d, sizeof(d));
    ps.boundary = psg::kBoundaryNone;
    ps.unit = true;
    for (int i = 0; i < 7; ++i) ps.w[i] = 1.0;
  } else {
    const int d[7][3] = {{0, 0, 0}, {-1, 0, 0}, {1, 0, 0}, {0, 1, 0},
                         {0, -1, 0}, {0, 0, -1}, {0, 0, 1}};
    memcpy(ps.d, d, sizeof(d));
    ps.boundary = psg::kBoundaryClamp;
    ps.unit = false;
    const double w[7] = {sc[6], sc[1], sc[0], sc[3], sc[2], sc[5], sc[4]};
    memcpy(ps.w, w, sizeof(w));
  }
  return register_points(ps);
}

// Checks a point-stencil map: element type and weights, that every read of
// boundary "none" stays inside the grid, and the red/black conditions.
bool validate_points(const Map &m, const PointStencil &ps) {
  const Grid *g = m.grids[0];
  if ((g->type == PS_INT || g->type == PS_LONG) && !ps.unit) {
    const double lim = g->type == PS_INT ? 2147483648.0 : 9223372036854775808.0;
    for (int i = 0; i < ps.n; ++i)
      if (ps.w[i] != std::trunc(ps.w[i]) || ps.w[i] < -lim || ps.w[i] >= lim)
        return fail(PS_ERR_INVALID_ARGUMENT,
                    "point stencil: weight %g of point %d is not a value of the grid's "
                    "integer type", ps.w[i], i);
  }
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (int i = 0; i < ps.n; ++i)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], ps.d[i][d]);
      hi[d] = std::max(hi[d], ps.d[i][d]);
    }
  bool empty = false;
  for (int d = 0; d < 3; ++d) empty = empty || m.dom.min[d] >= m.dom.max[d];
  for (int d = 0; d < 3 && !empty; ++d) {
    const int n = g->dim[d];
    if (ps.boundary == psg::kBoundaryNone &&
        (m.dom.min[d] + lo[d] < 0 || m.dom.max[d] - 1 + hi[d] > n - 1))
      return fail(PS_ERR_INVALID_ARGUMENT,
                  "point stencil reads outside the grid: domain [%d,%d) with offsets "
                  "[%d,%d] in dim %d of size %d (boundary none)", m.dom.min[d],
                  m.dom.max[d], lo[d], hi[d], d, n);
    if (ps.boundary == psg::kBoundaryPeriodic && (-lo[d] > n || hi[d] > n))
      return fail(PS_ERR_INVALID_ARGUMENT,
                  "periodic point stencil: offsets [%d,%d] exceed the size %d of dim %d",
                  lo[d], hi[d], n, d);
  }
  if (m.color < 0) return true;
  for (int i = 0; i < ps.n; ++i) {
    const int ax = std::abs(ps.d[i][0]), ay = std::abs(ps.d[i][1]), az = std::abs(ps.d[i][2]);
    const int dist = ax + ay + az;
    if (dist != 0 && dist % 2 == 0)
      return fail(PS_ERR_UNSUPPORTED,
                  "red/black map: point %d (%d,%d,%d) has the colour of the cell it "
                  "updates", i, ps.d[i][0], ps.d[i][1], ps.d[i][2]);
    if (ps.boundary == psg::kBoundaryClamp && dist > 1)
      return fail(PS_ERR_UNSUPPORTED,
                  "red/black map with clamped faces needs unit axis offsets (point %d)", i);
  }
  if (ps.boundary == psg::kBoundaryPeriodic)
    for (int d = 0; d < 3; ++d)
      if ((lo[d] != 0 || hi[d] != 0) && g->dim[d] % 2 != 0)
        return fail(PS_ERR_UNSUPPORTED,
                    "periodic red/black map needs an even grid size in dim %d (got %d)", d,
                    g->dim[d]);
  return true;
}

// A compiled stencil function's map: each grid has the element type and rank
// its parameter declares, and every grid of the function's rank covers the
// domain (the point a map emits to).  Reads at other indices are the
// function's own business, as in the reference.
bool validate_function_map(const Map &m, const psg::JitKernel &f) {
  int gi = 0;
  for (const psg::JitParam &p : f.params) {
    if (!p.grid) continue;
    const Grid *g = m.grids[gi++];
    if (g->type != p.type || g->ndims != p.rank)
      return fail(PS_ERR_INVALID_ARGUMENT,
                  "%s: grid argument %d is a %dD grid of type %d, the parameter is %s",
                  f.name.c_str(), gi - 1, g->ndims, g->type, p.decl_type.c_str());
    if (p.type == PS_USER && p.esz > 0 && g->esz != p.esz)
      return fail(PS_ERR_INVALID_ARGUMENT,
                  "%s: grid argument %d has %d-byte elements, the parameter's type (%s) "
                  "has %d", f.name.c_str(), gi - 1, g->esz, p.utype.c_str(), p.esz);
    if (p.rank != f.nd) continue;
    for (int d = 0; d < 3; ++d)
      if (m.dom.min[d] < m.dom.max[d] &&
          (m.dom.min[d] < 0 || m.dom.max[d] > g->dim[d]))
        return fail(PS_ERR_INVALID_ARGUMENT,
                    "%s: domain [%d,%d) in dim %d outside grid argument %d of size %d",
                    f.name.c_str(), m.dom.min[d], m.dom.max[d], d, gi - 1, g->dim[d]);
  }
  for (int d = 0; d < 3; ++d)
    if (m.dom.min[d] > m.dom.max[d])
      return fail(PS_ERR_INVALID_ARGUMENT, "%s: empty-reversed domain in dim %d",
                  f.name.c_str(), d);
  return true;
}

// Validates a map's grids, scalars and domain against its builtin.
bool validate_map(const Map &m) {
  KernelSig sig;
  if (!kernel_sig(m.kernel, &sig))
    return fail(PS_ERR_UNKNOWN_KERNEL, "unknown builtin stencil id %d", m.kernel);
  if (sig.fn) return validate_function_map(m, *sig.fn);
  const Grid *g0 = m.grids[0];
  if (g0->type == PS_USER)
    return fail(PS_ERR_UNSUPPORTED,
                "%s: grids of a user-defined type run compiled stencil functions only",
                sig.name);
  for (const Grid *g : m.grids) {
    if (g->type != g0->type || g->dim[0] != g0->dim[0] || g->dim[1] != g0->dim[1] ||
        g->dim[2] != g0->dim[2])
      return fail(PS_ERR_INVALID_ARGUMENT,
                  "%s: all grids of a map must have the same type and size", sig.name);
  }
  if (m.color < 0 && m.grids[0] == m.grids[1])
    return fail(PS_ERR_INVALID_ARGUMENT, "%s: input and output grid are the same",
                sig.name);
  if (m.color >= 0 && m.grids[0] != m.grids[1])
    return fail(PS_ERR_INVALID_ARGUMENT, "%s: a red/black map updates one grid", sig.name);
  if (const PointStencil *ps = point_stencil(m.kernel)) {
    for (int d = 0; d < 3; ++d)
      if (m.dom.min[d] < 0 || m.dom.max[d] > g0->dim[d] || m.dom.min[d] > m.dom.max[d])
        return fail(PS_ERR_INVALID_ARGUMENT,
                    "%s: domain [%d,%d) in dim %d outside grid of size %d", sig.name,
                    m.dom.min[d], m.dom.max[d], d, g0->dim[d]);
    return validate_points(m, *ps);
  }
  const bool is_float = g0->type == PS_FLOAT, is_fp = is_float || g0->type == PS_DOUBLE;
  if ((m.kernel == PS_KERNEL_DIFFUSION7 && !is_fp) ||
      ((m.kernel == PS_KERNEL_HIMENO19 || m.kernel == PS_KERNEL_HIMENO19_GOSA) && !is_float))
    return fail(PS_ERR_UNSUPPORTED, "%s: unsupported element type %d", sig.name, g0->type);
  const bool interior = (m.kernel == PS_KERNEL_SUM7 || m.kernel == PS_KERNEL_HIMENO19 ||
                         m.kernel == PS_KERNEL_HIMENO19_GOSA);
  for (int d = 0; d < 3; ++d) {
    const int lo = m.dom.min[d], hi = m.dom.max[d], n = g0->dim[d];
    if (lo < 0 || hi > n || lo > hi)
      return fail(PS_ERR_INVALID_ARGUMENT,
                  "%s: domain [%d,%d) in dim %d outside grid of size %d", sig.name, lo,
                  hi, d, n);
    if (interior && lo < hi && (lo < 1 || hi > n - 1))
      return fail(PS_ERR_INVALID_ARGUMENT,
                  "%s reads neighbours without clamping: its domain [%d,%d) in dim %d "
                  "must stay inside [1,%d)", sig.name, lo, hi, d, n - 1);
  }
  return true;
}

int shape_slot(int kernel) {
  if (kernel >= kPointsBase) return kSlotPoints;
  return (kernel > 0 && kernel < kNumKernels) ? kernel : 0;
}

// One point-stencil map: one launch per colour it runs.
bool launch_points_map(const Map &m, const PointStencil &ps) {
  psg::PointsArgs a{};
  a.has_tmap = true;  // planes arrive by TMA (sizes the ring below)
  a.in = view(m.grids[0]);
  a.out = view(m.grids[1]);
  for (int d = 0; d < 3; ++d) {
    a.dom.min[d] = m.dom.min[d];
    a.dom.max[d] = m.dom.max[d];
  }
  if (a.dom.min[0] >= a.dom.max[0] || a.dom.min[1] >= a.dom.max[1] ||
      a.dom.min[2] >= a.dom.max[2])
    return true;
  a.boundary = ps.boundary;
  a.n = ps.n;
  memcpy(a.d, ps.d, sizeof(a.d));
  memcpy(a.w, ps.w, sizeof(a.w));
  a.unit = ps.unit;
  MarchConfig cfg = m.has_plan ? m.plan.shape : rt->shapes[kSlotPoints];
  // the widest stencils need a shorter tile to fit their plane ring
  while (psg::points_smem_bytes(a, cfg) > 220 * 1024 && (cfg.rows > 1 || cfg.warps > 1)) {
    if (cfg.rows > 1) cfg.rows /= 2;
    else cfg.warps /= 2;
  }
  a.err = rt->dev_err;
  int bw = 0, bh = 0;
  psg::points_box(a, cfg, &bw, &bh);
  a.has_tmap = tmap_for(a.in, bw, bh, &a.tmap);
  if (!a.has_tmap) return false;
  const int colors[2] = {m.color == 2 ? 0 : m.color, 1};
  const int ncol = m.color == 2 ? 2 : 1;
  for (int c = 0; c < ncol; ++c) {
    a.color = colors[c];
    cudaError_t e = psg::launch_points(a, cfg, rt->sm_count, rt->stream);
    if (!cuda_ok(e, "point stencil launch")) return false;
    ++rt->launches;
  }
  return true;
}

// One plain sweep of a 7-point-family map with explicit input/output views.
bool launch_s7(const Map &m, const GridView &in, const GridView &out) {
  psg::Stencil7Args a{};
  a.kernel = m.kernel;
  a.in = in;
  a.out = out;
  for (int d = 0; d < 3; ++d) {
    a.dom.min[d] = m.dom.min[d];
    a.dom.max[d] = m.dom.max[d];
  }
  if (a.dom.min[0] >= a.dom.max[0] || a.dom.min[1] >= a.dom.max[1] ||
      a.dom.min[2] >= a.dom.max[2])
    return true;
  for (int i = 0; i < 7; ++i) a.coef[i] = i < (int)m.scalars.size() ? m.scalars[i] : 0.0;
  const int vec = 16 / in.esz;
  const MarchConfig cfg = m.has_plan ? m.plan.shape : rt->shapes[shape_slot(m.kernel)];
  CUtensorMap t;
  if (!tmap_for(in, 34 * vec, cfg.warps * cfg.rows + 2, &t)) return false;
  cudaError_t e = psg::launch_stencil7(a, cfg, &t, rt->dev_err, rt->sm_count, rt->stream);
  if (!cuda_ok(e, "stencil7 launch")) return false;
  ++rt->launches;
  return true;
}

// One compiled-function map: one launch per colour it runs.
bool launch_function_map(const Map &m, const psg::JitKernel &f) {
  psg::Box box;
  for (int d = 0; d < 3; ++d) {
    box.min[d] = m.dom.min[d];
    box.max[d] = m.dom.max[d];
  }
  if (box.min[0] >= box.max[0] || box.min[1] >= box.max[1] || box.min[2] >= box.max[2])
    return true;
  GridView views[64];
  for (size_t i = 0; i < m.grids.size() && i < 64; ++i) views[i] = view(m.grids[i]);
  const int colors[2] = {m.color == 2 ? 0 : m.color, 1};
  const int ncol = m.color == 2 ? 2 : 1;
  for (int c = 0; c < ncol; ++c) {
    cudaError_t e = psg::jit_launch(f, box, colors[c], views, m.scalars.data(), rt->sm_count,
                                    rt->stream);
    if (!cuda_ok(e, "stencil function launch")) return false;
    ++rt->launches;
  }
  return true;
}

bool launch_map(const Map &m, bool want_gosa) {
  if (const PointStencil *ps = point_stencil(m.kernel)) return launch_points_map(m, *ps);
  if (const psg::JitKernel *f = jit_kernel(m.kernel)) return launch_function_map(m, *f);
  const Grid *g0 = m.grids[0];
  psg::Box box;
  for (int d = 0; d < 3; ++d) {
    box.min[d] = m.dom.min[d];
    box.max[d] = m.dom.max[d];
  }
  if (box.min[0] >= box.max[0] || box.min[1] >= box.max[1] || box.min[2] >= box.max[2])
    return true;  // empty domain: nothing to do, as in the REF loops
  cudaError_t e;
  if (m.kernel == PS_KERNEL_HIMENO19 || m.kernel == PS_KERNEL_HIMENO19_GOSA) {
    psg::Himeno19Args a{};
    for (int i = 0; i < 14; ++i) a.g[i] = view(m.grids[i]);
    a.dom = box;
    a.omega = (float)m.scalars[0];
    a.gosa = want_gosa;
    const MarchConfig cfg = m.has_plan ? m.plan.shape : rt->shapes[shape_slot(m.kernel)];
    CUtensorMap maps[13];
    if (!tmap_for(view(m.grids[0]), 136, cfg.warps + 2, &maps[0])) return false;
    for (int i = 0; i < 12; ++i)
      if (!tmap_for(view(m.grids[2 + i]), 128, cfg.warps, &maps[1 + i])) return false;
    psg::ResidualSink sink;
    sink.partials = reinterpret_cast<double *>(rt->partials);
    sink.max_partials = kMaxPartials;
    sink.ticket = rt->ticket;
    sink.result = reinterpret_cast<double *>(rt->results + 1);
    e = psg::launch_himeno19(a, cfg, maps, sink, rt->dev_err, rt->sm_count, rt->stream);
    if (!cuda_ok(e, "himeno19 launch")) return false;
    ++rt->launches;
    return true;
  }
  (void)g0;
  return launch_s7(m, view(m.grids[0]), view(m.grids[1]));
}

// One temporal pass: out = k steps of map m's stencil applied to in.
bool launch_t7(const Map &m, const GridView &in, const GridView &out, int k) {
  psg::Temporal7Args a{};
  a.in = in;
  a.out = out;
  a.k = k;
  a.fma = rt->fma;
  for (int i = 0; i < 7; ++i) a.coef[i] = m.scalars[i];
  const MarchConfig cfg = m.has_plan ? m.plan.tshape : rt->tshapes[shape_slot(m.kernel)];
  const int vec = 16 / in.esz;
  CUtensorMap t;
  if (!tmap_for(in, 34 * vec, cfg.warps * cfg.rows + 2, &t)) return false;
  cudaError_t e = psg::launch_temporal7(a, cfg, &t, rt->dev_err, rt->sm_count, rt->stream);
  if (!cuda_ok(e, "temporal7 launch")) return false;
  ++rt->launches;
  return true;
}

// A pair of maps (g1 -> g2, g2 -> g1) of the same full-grid DIFFUSION7
// stencil can run `iter` iterations as temporal passes.
int temporal_depth(const Map &a) {
  return a.has_plan ? a.plan.k : rt->tblock[shape_slot(a.kernel)];
}

// True if (a, b) is a ping-pong pair of one full-grid DIFFUSION7 stencil
// (the shape temporal blocking applies to), whatever the current depth.
bool pair_eligible(const Map &a, const Map &b) {
  if (a.kernel != PS_KERNEL_DIFFUSION7 || b.kernel != PS_KERNEL_DIFFUSION7) return false;
  const Grid *g1 = a.grids[0], *g2 = a.grids[1];
  if (b.grids[0] != g2 || b.grids[1] != g1) return false;
  if (g1->type != PS_FLOAT && g1->type != PS_DOUBLE) return false;
  for (int i = 0; i < 7; ++i)
    if (a.scalars[i] != b.scalars[i]) return false;
  for (int d = 0; d < 3; ++d)
    if (a.dom.min[d] != 0 || a.dom.max[d] != g1->dim[d] || b.dom.min[d] != 0 ||
        b.dom.max[d] != g1->dim[d])
      return false;
  return true;
}

bool temporal_pair(const Map &a, const Map &b) {
  const int k = temporal_depth(a);
  return k >= 2 && k <= psg::temporal7_max_k(a.grids[0]->esz) && pair_eligible(a, b);
}

// Runs (a, b) x iter as temporal passes.  Both maps cover the whole grid, so
// every step overwrites every cell and the two grids' storage may be
// exchanged freely; at the end g1 holds step 2*iter and g2 step 2*iter-1,
// exactly as the plain ping-pong leaves them.
bool run_temporal(const Map &a, int iter) {
  Grid *g1 = a.grids[0], *g2 = a.grids[1];
  const int total = 2 * iter;
  if (total <= 0) return true;
  const int k = temporal_depth(a);
  GridView cur = view(g1), oth = view(g2);
  int t = 0;
  // Temporal passes up to step total-1; the last step is a plain sweep so
  // the previous step also ends up in memory.
  while (total - 1 - t >= 2) {
    const int kk = std::min(k, total - 1 - t);
    if (!launch_t7(a, cur, oth, kk)) return false;
    std::swap(cur, oth);
    t += kk;
  }
  while (t < total) {
    if (!launch_s7(a, cur, oth)) return false;
    std::swap(cur, oth);
    ++t;
  }
  // cur holds step total, oth step total-1.
  g1->dev = cur.ptr;
  g2->dev = oth.ptr;
  return true;
}

// esz_user: element size of a PS_USER grid (ignored for the primitive types).
void *grid_new(int type, int ndims, const PSIndex *dims, size_t esz_user = 0) {
  if (!need_rt("PSGrid*New")) return nullptr;
  const int esz = type == PS_USER ? (int)esz_user : esize(type);
  if (type == PS_USER && (esz_user < 1 || esz_user > kMaxUserElem)) {
    fail(PS_ERR_INVALID_ARGUMENT, "user element size %zu not in 1..%d", esz_user,
         kMaxUserElem);
    return nullptr;
  }
  if (!esz) {
    fail(PS_ERR_INVALID_ARGUMENT, "unknown grid element type %d", type);
    return nullptr;
  }
  if (ndims < 1 || ndims > 3) {
    fail(PS_ERR_INVALID_ARGUMENT, "grid rank %d not in 1..3", ndims);
    return nullptr;
  }
  int dim[3] = {1, 1, 1};
  for (int d = 0; d < ndims; ++d) {
    if (dims[d] <= 0) {
      fail(PS_ERR_INVALID_ARGUMENT, "grid size %d in dim %d must be positive", dims[d], d);
      return nullptr;
    }
    dim[d] = dims[d];
  }
  // Rows of the primitive types start on 128-byte boundaries (TMA boxes,
  // 16-byte vectors); user-type rows are dense, so that an element index
  // times the element size addresses any element.
  const size_t pitch = type == PS_USER ? (size_t)dim[0] * esz
                                       : (((size_t)dim[0] * esz) + 127) / 128 * 128;
  const size_t bytes = pitch * (size_t)dim[1] * (size_t)dim[2];
  void *dev = nullptr;
  if (rt->fail_allocs > 0) {
    --rt->fail_allocs;
    fail(PS_ERR_OUT_OF_MEMORY, "device allocation of %zu bytes failed (test hook)", bytes);
    return nullptr;
  }
  if (!cuda_ok(cudaMalloc(&dev, bytes), "cudaMalloc")) {
    cudaGetLastError();
    return nullptr;
  }
  if (!cuda_ok(cudaMemsetAsync(dev, 0, bytes, rt->stream), "cudaMemsetAsync") ||
      !cuda_ok(cudaStreamSynchronize(rt->stream), "cudaStreamSynchronize")) {
    cudaFree(dev);
    return nullptr;
  }
  Grid *g = new Grid();
  g->magic = kGridMagic;
  g->type = type;
  g->esz = esz;
  g->ndims = ndims;
  for (int d = 0; d < 3; ++d) g->dim[d] = dim[d];
  g->pitch = pitch;
  g->bytes = bytes;
  g->dev = dev;
  rt->grids.insert(g);
  return g;
}

bool copy_grid(Grid *g, void *host, bool in, bool sync) {
  const size_t row = (size_t)g->dim[0] * g->esz;
  const size_t rows = (size_t)g->dim[1] * g->dim[2];
  cudaError_t e;
  if (row == g->pitch) {
    e = in ? cudaMemcpyAsync(g->dev, host, row * rows, cudaMemcpyHostToDevice, rt->stream)
           : cudaMemcpyAsync(host, g->dev, row * rows, cudaMemcpyDeviceToHost, rt->stream);
  } else {
    e = in ? cudaMemcpy2DAsync(g->dev, g->pitch, host, row, row, rows,
                               cudaMemcpyHostToDevice, rt->stream)
           : cudaMemcpy2DAsync(host, row, g->dev, g->pitch, row, rows,
                               cudaMemcpyDeviceToHost, rt->stream);
  }
  if (!cuda_ok(e, in ? "grid copy-in" : "grid copy-out")) return false;
  return sync ? sync_rt() : true;
}

PSStencil add_map(Map &&m) {
  if (!validate_map(m)) return -1;
  if ((int)rt->maps.size() >= kMaxMaps) {
    fail(PS_ERR_OUT_OF_MEMORY, "more than %d stencil maps", kMaxMaps);
    return -1;
  }
  rt->maps.push_back(std::move(m));
  return kStencilTag | (int)(rt->maps.size() - 1);
}

Map *lookup_map(PSStencil s) {
  if ((s & kStencilTagMask) != kStencilTag) return nullptr;
  const int idx = s & ~kStencilTagMask;
  if (idx < 0 || idx >= (int)rt->maps.size()) return nullptr;
  return &rt->maps[idx];
}

// Kernels a red/black map accepts: point stencils and the 7-point builtins
// (run as their point-stencil equivalents).
bool colorable(int kernel) {
  return point_stencil(kernel) || jit_kernel(kernel) || kernel == PS_KERNEL_SUM7 ||
         kernel == PS_KERNEL_DIFFUSION7;
}

// Grids a map of `kernel` with `color` takes: a red/black map updates its one
// grid in place.
int map_ngrids(const KernelSig &sig, int color) {
  return (color >= 0 && !sig.fn) ? 1 : sig.ngrids;
}

bool map_from(int kernel, const __PSDomain &dom, int ngrids, void *const *grids,
              int nscalars, const double *scalars, Map *out, int color = -1) {
  KernelSig sig;
  if (!kernel_sig(kernel, &sig))
    return fail(PS_ERR_UNKNOWN_KERNEL, "unknown builtin stencil id %d", kernel);
  if (color < -1 || color > 2)
    return fail(PS_ERR_INVALID_ARGUMENT, "unknown map colour %d", color);
  if (color >= 0 && !colorable(kernel))
    return fail(PS_ERR_UNSUPPORTED, "%s has no red/black form", sig.name);
  const int want = map_ngrids(sig, color);
  if (ngrids > 64 || nscalars > 64)
    return fail(PS_ERR_UNSUPPORTED, "%s: more than 64 grids or scalars", sig.name);
  if (ngrids != want || nscalars != sig.nscalars)
    return fail(PS_ERR_INVALID_ARGUMENT, "%s takes %d grids and %d scalars, got %d and %d",
                sig.name, want, sig.nscalars, ngrids, nscalars);
  out->kernel = kernel;
  out->color = color;
  out->dom = dom;
  out->grids.clear();
  for (int i = 0; i < ngrids; ++i) {
    Grid *g = as_grid(grids[i], sig.name);
    if (!g) return false;
    out->grids.push_back(g);
  }
  if (color >= 0 && !sig.fn) out->grids.push_back(out->grids[0]);
  out->scalars.assign(scalars, scalars + nscalars);
  if (color >= 0 && (kernel == PS_KERNEL_SUM7 || kernel == PS_KERNEL_DIFFUSION7)) {
    const int id = builtin_as_points(kernel, out->scalars);
    if (id < 0) return false;
    out->kernel = id;
    out->scalars.clear();
  }
  return true;
}

// ---- Autotuner ------------------------------------------------------------
//
// Replaces the reference's online trial (translator/reference_translator.cc:
// 610-935: each OPT_* / block-size variant times one iteration of the run
// during its first calls, nothing persists).  Here the candidates are launch
// shapes and temporal depths; because every candidate computes bit-identical
// results, the trials are simply the run's first iterations.  The winner is
// kept per run signature (kernels, grid size, type, domains, GPU) in memory
// and, when PS_TUNE_CACHE names a file, as one JSON object per line there.

struct TuneState {
  std::vector<Plan> cands;
  std::vector<double> ms;  // per-iteration time of each tried candidate
  size_t next = 0;
};

std::map<std::string, Plan> g_tuned;
std::map<std::string, TuneState> g_tuning;

std::string run_key(const std::vector<Map *> &ms) {
  std::string k;
  char buf[256];
  for (const Map *m : ms) {
    const Grid *g = m->grids[0];
    snprintf(buf, sizeof(buf), "k%d t%d g%dx%dx%d d%d:%d,%d:%d,%d:%d;", m->kernel, g->type,
             g->dim[0], g->dim[1], g->dim[2], m->dom.min[0], m->dom.max[0], m->dom.min[1],
             m->dom.max[1], m->dom.min[2], m->dom.max[2]);
    k += buf;
    if (const PointStencil *ps = point_stencil(m->kernel)) {
      // kernel ids are per process: name the stencil by its contents
      uint64_t h = 1469598103934665603ull;  // FNV-1a over boundary, colour, points
      auto mix = [&h](int v) {
        for (int b = 0; b < 4; ++b) {
          h ^= (uint64_t)((v >> (8 * b)) & 0xff);
          h *= 1099511628211ull;
        }
      };
      mix(ps->boundary);
      mix(m->color);
      mix(ps->unit ? 1 : 0);
      for (int i = 0; i < ps->n; ++i) mix(ps->d[i][0] * 81 + ps->d[i][1] * 9 + ps->d[i][2]);
      snprintf(buf, sizeof(buf), "pts%d:%016llx;", ps->n, (unsigned long long)h);
      k += buf;
    }
  }
  // temporal candidates time differently with contraction on
  if (ms.size() == 2 && pair_eligible(*ms[0], *ms[1])) k += rt->fma ? "pair-fma;" : "pair;";
  snprintf(buf, sizeof(buf), "%s/%dsm", rt->gpu_name.c_str(), rt->sm_count);
  return k + buf;
}

std::vector<Plan> candidates(const std::vector<Map *> &ms) {
  std::vector<Plan> out;
  const Map &m0 = *ms[0];
  const bool him = m0.kernel == PS_KERNEL_HIMENO19 || m0.kernel == PS_KERNEL_HIMENO19_GOSA;
  const MarchConfig tdef = rt->tshapes[shape_slot(m0.kernel)];
  bool all_points = true;
  for (const Map *m : ms) all_points = all_points && point_stencil(m->kernel);
  if (all_points) {  // {warps, rows} of the point-stencil tile
    const int sh[][2] = {{8, 2}, {8, 4}, {4, 2}, {4, 4}, {16, 2}, {8, 1}};
    for (auto &c : sh) out.push_back(Plan{MarchConfig{c[0], c[1], 4, 0, 0}, 1, tdef});
    return out;
  }
  if (him) {
    const int sh[][3] = {{4, 5, 2}, {2, 5, 2}, {8, 4, 2}, {4, 4, 3}, {4, 6, 2}, {2, 6, 3},
                         {8, 3, 2}, {4, 3, 1}};
    for (auto &c : sh) out.push_back(Plan{MarchConfig{c[0], 1, c[1], c[2], 0}, 1, tdef});
    return out;
  }
  const int sh[][3] = {{8, 2, 4}, {4, 2, 3}, {2, 2, 3}, {8, 4, 4}, {4, 4, 4},
                       {16, 4, 4}, {16, 2, 6}, {8, 8, 3}, {8, 1, 4}, {4, 1, 4}};
  for (auto &c : sh) out.push_back(Plan{MarchConfig{c[0], c[1], c[2], 0, 0}, 1, tdef});
  if (ms.size() == 2 && pair_eligible(*ms[0], *ms[1])) {
    const int maxk = psg::temporal7_max_k(m0.grids[0]->esz);
    // {k, warps, rows, stages}; 4 rows at k >= 3 spill registers
    const int tc[][4] = {{2, 8, 4, 3}, {2, 8, 2, 3}, {2, 4, 4, 3}, {3, 8, 2, 4},
                         {3, 4, 2, 4}, {4, 8, 2, 4}};
    for (auto &c : tc) {
      if (c[0] > maxk) continue;
      out.push_back(Plan{MarchConfig{8, 2, 4, 0, 0}, c[0], MarchConfig{c[1], c[2], c[3], 0, 0}});
    }
  }
  return out;
}

void apply_plan(const std::vector<Map *> &ms, const Plan &p) {
  for (Map *m : ms) {
    m->has_plan = true;
    m->plan = p;
  }
}

void save_tuned(const std::string &key, const Plan &p, double ms) {
  if (rt->tune_path.empty()) return;
  FILE *f = fopen(rt->tune_path.c_str(), "a");
  if (!f) {
    fail(PS_ERR_IO, "cannot append to the tune cache %s", rt->tune_path.c_str());
    return;
  }
  fprintf(f,
          "{\"key\": \"%s\", \"warps\": %d, \"rows\": %d, \"ns\": %d, \"ns2\": %d, "
          "\"ctas\": %d, \"k\": %d, \"twarps\": %d, \"trows\": %d, \"tns\": %d, "
          "\"ms\": %.6f}\n",
          key.c_str(), p.shape.warps, p.shape.rows, p.shape.ns, p.shape.ns2,
          p.shape.ctas_per_sm, p.k, p.tshape.warps, p.tshape.rows, p.tshape.ns, ms);
  fclose(f);
}

// Loads a JSON-lines tune cache written by save_tuned; malformed lines are
// skipped (and reported once as PS_ERR_IO).  Returns the entries loaded.
int load_tuned(const char *path) {
  FILE *f = fopen(path, "r");
  if (!f) return 0;
  char line[1024], key[512];
  int n = 0, bad = 0;
  while (fgets(line, sizeof(line), f)) {
    Plan p{};
    double ms = 0;
    const int got = sscanf(line,
                           "{\"key\": \"%511[^\"]\", \"warps\": %d, \"rows\": %d, \"ns\": %d, "
                           "\"ns2\": %d, \"ctas\": %d, \"k\": %d, \"twarps\": %d, \"trows\": %d, "
                           "\"tns\": %d, \"ms\": %lf}",
                           key, &p.shape.warps, &p.shape.rows, &p.shape.ns, &p.shape.ns2,
                           &p.shape.ctas_per_sm, &p.k, &p.tshape.warps, &p.tshape.rows,
                           &p.tshape.ns, &ms);
    const bool sane = got == 11 && p.shape.warps >= 1 && p.shape.warps <= 16 &&
                      p.shape.rows >= 1 && p.shape.rows <= 8 && p.shape.ns >= 2 &&
                      p.shape.ns <= 16 && p.k >= 1 && p.k <= 5 && p.tshape.warps >= 1 &&
                      p.tshape.warps <= 8 && p.tshape.ns >= 2 && p.tshape.ns <= 16;
    if (!sane) {
      ++bad;
      continue;
    }
    g_tuned[key] = p;
    ++n;
  }
  fclose(f);
  if (bad) fail(PS_ERR_IO, "tune cache %s: %d malformed line(s) ignored", path, bad);
  return n;
}

// Runs `iter` iterations of the maps, spending the first ones on tuning
// trials while the run's signature has no tuned plan.  Returns the number of
// iterations it ran (all of them unless an error occurs).
bool run_tuning(const std::vector<Map *> &ms, int &iter) {
  for (const Map *m : ms)
    if (jit_kernel(m->kernel)) return true;  // one launch shape: nothing to tune
  const std::string key = run_key(ms);
  auto hit = g_tuned.find(key);
  if (hit != g_tuned.end()) {
    apply_plan(ms, hit->second);
    return true;
  }
  if (!rt->autotune) return true;  // no plan: defaults
  TuneState &st = g_tuning[key];
  if (st.cands.empty()) st.cands = candidates(ms);
  const bool pair = ms.size() == 2 && pair_eligible(*ms[0], *ms[1]);
  while (iter > 0 && st.next < st.cands.size()) {
    const Plan &c = st.cands[st.next];
    apply_plan(ms, c);
    // temporal candidates need several iterations for the passes to dominate
    int reps = (pair && c.k > 1) ? 6 : 2;
    if (reps > iter) reps = iter;
    cudaEventRecord(rt->events[kNumEvents - 2], rt->stream);
    bool ok = true;
    if (pair && c.k > 1) {
      ok = run_temporal(*ms[0], reps);
    } else {
      for (int i = 0; i < reps && ok; ++i)
        for (Map *m : ms)
          if (!launch_map(*m, m->kernel == PS_KERNEL_HIMENO19_GOSA)) {
            ok = false;
            break;
          }
    }
    cudaEventRecord(rt->events[kNumEvents - 1], rt->stream);
    iter -= reps;
    float t = 0;
    if (!ok || cudaEventSynchronize(rt->events[kNumEvents - 1]) != cudaSuccess ||
        cudaEventElapsedTime(&t, rt->events[kNumEvents - 2], rt->events[kNumEvents - 1]) !=
            cudaSuccess) {
      // a candidate that cannot launch is skipped (the launch error is kept)
      cudaGetLastError();
      st.ms.push_back(1e30);
    } else {
      st.ms.push_back((double)t / reps);
    }
    ++st.next;
  }
  if (st.next < st.cands.size()) return true;  // continue in a later run
  size_t best = 0;
  for (size_t i = 1; i < st.ms.size(); ++i)
    if (st.ms[i] < st.ms[best]) best = i;
  const Plan p = st.cands[best];
  const double best_ms = st.ms[best];
  g_tuned[key] = p;
  g_tuning.erase(key);
  apply_plan(ms, p);
  save_tuned(key, p, best_ms);
  return true;
}

// ---- CUDA graphs for launch-bound runs -----------------------------------
//
// A plain (non-temporal) run re-launches the same kernels with the same
// arguments every iteration.  For small grids the launch overhead rivals the
// sweep itself, so after one ordinary iteration the runtime captures
// kGraphUnroll iterations into a CUDA graph and replays it; the remainder
// runs as ordinary launches.  Graphs are cached per map list and rebuilt
// when a grid's storage or a map's plan changes.  PS_GRAPH=0 disables them.

constexpr int kGraphUnroll = 16;

struct GraphEntry {
  std::vector<const Map *> maps;   // elements of rt->maps (a deque: stable)
  std::vector<const Grid *> grids; // every grid the maps touch
  std::vector<void *> ptrs;        // grid storage at capture
  std::vector<MarchConfig> cfgs;   // launch shapes at capture
  cudaGraphExec_t exec = nullptr;
};
std::vector<GraphEntry> g_graphs;

void graph_signature(const std::vector<Map *> &ms, std::vector<void *> *ptrs,
                     std::vector<MarchConfig> *cfgs) {
  for (const Map *m : ms) {
    for (const Grid *g : m->grids) ptrs->push_back(g->dev);
    cfgs->push_back(m->has_plan ? m->plan.shape : rt->shapes[shape_slot(m->kernel)]);
  }
}

bool same_cfg(const MarchConfig &a, const MarchConfig &b) {
  return a.warps == b.warps && a.rows == b.rows && a.ns == b.ns && a.ns2 == b.ns2 &&
         a.ctas_per_sm == b.ctas_per_sm;
}

void drop_graphs_for(const Grid *g) {
  for (size_t i = 0; i < g_graphs.size();) {
    bool uses = false;
    for (const Grid *x : g_graphs[i].grids) uses = uses || x == g;
    if (uses) {
      cudaGraphExecDestroy(g_graphs[i].exec);
      g_graphs[i] = g_graphs.back();
      g_graphs.pop_back();
    } else {
      ++i;
    }
  }
}

bool launch_iteration(const std::vector<Map *> &ms) {
  for (Map *m : ms)
    if (!launch_map(*m, m->kernel == PS_KERNEL_HIMENO19_GOSA)) return false;
  return true;
}

// Returns the cached or newly captured graph of kGraphUnroll iterations, or
// nullptr if capture is not possible (the caller then launches normally).
cudaGraphExec_t graph_for(const std::vector<Map *> &ms) {
  std::vector<void *> ptrs;
  std::vector<MarchConfig> cfgs;
  graph_signature(ms, &ptrs, &cfgs);
  for (size_t i = 0; i < g_graphs.size(); ++i) {
    GraphEntry &e = g_graphs[i];
    if (e.maps.size() != ms.size()) continue;
    bool same = true;
    for (size_t j = 0; j < ms.size(); ++j) same = same && e.maps[j] == ms[j];
    if (!same) continue;
    bool fresh = e.ptrs == ptrs && e.cfgs.size() == cfgs.size();
    for (size_t j = 0; fresh && j < cfgs.size(); ++j) fresh = same_cfg(e.cfgs[j], cfgs[j]);
    if (fresh) return e.exec;
    cudaGraphExecDestroy(e.exec);
    g_graphs[i] = g_graphs.back();
    g_graphs.pop_back();
    break;
  }
  const long long launches0 = rt->launches;
  cudaGraph_t graph = nullptr;
  if (cudaStreamBeginCapture(rt->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  bool ok = true;
  for (int u = 0; u < kGraphUnroll && ok; ++u) ok = launch_iteration(ms);
  const cudaError_t ee = cudaStreamEndCapture(rt->stream, &graph);
  rt->launches = launches0;  // captured launches run when the graph does
  if (!ok || ee != cudaSuccess || !graph) {
    cudaGetLastError();
    if (graph) cudaGraphDestroy(graph);
    return nullptr;
  }
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  GraphEntry e;
  e.maps.assign(ms.begin(), ms.end());
  for (const Map *m : ms) e.grids.insert(e.grids.end(), m->grids.begin(), m->grids.end());
  e.ptrs = ptrs;
  e.cfgs = cfgs;
  e.exec = exec;
  g_graphs.push_back(e);
  return exec;
}

bool graphs_enabled() {
  const char *e = getenv("PS_GRAPH");
  return !(e && e[0] == '0');
}

bool run_plain(const std::vector<Map *> &ms, int iter) {
  int i = 0;
  if (graphs_enabled() && iter > kGraphUnroll) {
    // one ordinary iteration first: sets kernel attributes and caches
    if (!launch_iteration(ms)) return false;
    ++i;
    cudaGraphExec_t g = graph_for(ms);
    if (g) {
      long long per = 0;
      for (const Map *m : ms) {
        const __PSDomain &d = m->dom;
        if (d.min[0] < d.max[0] && d.min[1] < d.max[1] && d.min[2] < d.max[2]) ++per;
      }
      for (; i + kGraphUnroll <= iter; i += kGraphUnroll) {
        if (!cuda_ok(cudaGraphLaunch(g, rt->stream), "cudaGraphLaunch")) return false;
        rt->launches += per * kGraphUnroll;
      }
    }
  }
  for (; i < iter; ++i)
    if (!launch_iteration(ms)) return false;
  return true;
}

// ---- Batches of independent runs (batch.cu) --------------------------------

struct Batch {
  bool live = false;
  int nruns = 0, maps_per_run = 0;
  std::vector<const Map *> maps;      // nruns x maps_per_run (deque elements: stable)
  std::vector<const Grid *> grids;    // every grid the batch touches
  std::vector<void *> ptrs;           // their storage when the device tables were built
  psg::BatchShape shape{};
  psg::BatchProblem *probs_dev = nullptr;  // the 7-point family's problems, then Himeno's
  CUtensorMap *tmaps_dev = nullptr;
  // per kernel family (psg::kBatch7, psg::kBatchHimeno): its problems
  // probs_dev[prob_off .. prob_off + nprob), their items, the launch's grid
  int nprob[2] = {0, 0}, prob_off[2] = {0, 0}, grid[2] = {0, 0};
  int64_t total_items[2] = {0, 0};
  cudaGraphExec_t graph = nullptr;    // maps_per_run x kGraphUnroll steps
  long long graph_launches = 0;       // kernels one replay of graph runs
};
std::vector<Batch> g_batches;
// {warps, max rows (computed per batch), 7-point stages, Himeno p / coef stages}
psg::BatchShape g_batch_shape{4, 4, 4, 4, 2};
int g_batch_rows = 4;  // rows per thread of untuned 7-point runs in a batch

void batch_release(Batch &b) {
  if (b.graph) cudaGraphExecDestroy(b.graph);
  if (b.probs_dev) cudaFree(b.probs_dev);
  if (b.tmaps_dev) cudaFree(b.tmaps_dev);
  b.graph = nullptr;
  b.probs_dev = nullptr;
  b.tmaps_dev = nullptr;
}

bool batch_kind_ok(int k) {
  return k == PS_KERNEL_DIFFUSION7 || k == PS_KERNEL_SUM7 || k == PS_KERNEL_COPY ||
         k == PS_KERNEL_HIMENO19;
}

// (Re)builds the device tables of a batch from its maps' current grids.
bool batch_build(Batch &b) {
  batch_release(b);
  b.ptrs.clear();
  for (const Grid *g : b.grids) b.ptrs.push_back(g->dev);
  const int M = b.maps_per_run;
  b.shape = g_batch_shape;
  b.shape.max_rows = 1;
  std::vector<int> rows(b.nruns, g_batch_rows);
  for (int r = 0; r < b.nruns; ++r) {
    const Map *m = b.maps[(size_t)r * M];
    if (m->kernel != PS_KERNEL_HIMENO19 && m->has_plan &&
        (m->plan.shape.rows == 1 || m->plan.shape.rows == 2 || m->plan.shape.rows == 4))
      rows[r] = m->plan.shape.rows;
    if (m->kernel != PS_KERNEL_HIMENO19 && rows[r] > b.shape.max_rows)
      b.shape.max_rows = rows[r];
  }
  // problems ordered by kernel family (each family is one launch), runs in
  // their given order inside a family
  auto family = [&](int r) {
    return b.maps[(size_t)r * M]->kernel == PS_KERNEL_HIMENO19 ? psg::kBatchHimeno
                                                               : psg::kBatch7;
  };
  std::vector<int> order;
  for (int f = 0; f < 2; ++f) {
    b.nprob[f] = 0;
    b.prob_off[f] = (int)order.size();
    b.total_items[f] = 0;
    for (int r = 0; r < b.nruns; ++r)
      if (family(r) == f) {
        order.push_back(r);
        ++b.nprob[f];
      }
  }
  int resident[2] = {0, 0};
  for (int f = 0; f < 2; ++f) {
    if (!b.nprob[f]) continue;
    const int occ = psg::batch_occupancy(b.shape, f);
    if (occ < 1) return fail(PS_ERR_CUDA, "batch kernel does not fit on an SM");
    resident[f] = rt->sm_count * occ;
  }
  std::vector<psg::BatchProblem> probs(b.nruns);
  std::vector<CUtensorMap> tmaps;
  for (int i = 0; i < b.nruns; ++i) {
    const int r = order[i];
    const int fam = family(r);
    psg::BatchProblem &bp = probs[i];
    memset(&bp, 0, sizeof(bp));
    const Map *m0 = b.maps[(size_t)r * M];
    const Grid *g = m0->grids[0];
    bp.kind = m0->kernel;
    bp.rows = rows[r];
    const int tyy = bp.kind == PS_KERNEL_HIMENO19 ? b.shape.warps : b.shape.warps * bp.rows;
    const int xbase = (m0->dom.min[0] / 4) * 4;
    const int tiles_x = (m0->dom.max[0] - xbase + 127) / 128;
    bp.tiles = tiles_x * ((m0->dom.max[1] - m0->dom.min[1] + tyy - 1) / tyy);
    const int nzd = m0->dom.max[2] - m0->dom.min[2];
    bp.zlen = psg::choose_zchunk(bp.tiles, nzd, resident[fam]);
    bp.items = (int64_t)bp.tiles * ((nzd + bp.zlen - 1) / bp.zlen);
    bp.item_begin = b.total_items[fam];
    b.total_items[fam] += bp.items;
    bp.dmin2 = m0->dom.min[2];
    bp.dmax2 = m0->dom.max[2];
    for (int par = 0; par < 2; ++par) {
      const Map *m = b.maps[(size_t)r * M + (par % M)];
      const GridView in = view(m->grids[0]), out = view(m->grids[1]);
      CUtensorMap t;
      const int box_h = (bp.kind == PS_KERNEL_HIMENO19 ? b.shape.warps : tyy) + 2;
      if (!tmap_for(in, 136, box_h, &t)) return false;
      bp.tmap[par] = (int)tmaps.size();
      tmaps.push_back(t);
      if (bp.kind == PS_KERNEL_HIMENO19) {
        psg::HParams &h = bp.him[par];
        h.out = static_cast<float *>(out.ptr);
        h.row = out.pitch / 4;
        h.plane = h.row * out.ny;
        h.dmin0 = m->dom.min[0];
        h.dmin1 = m->dom.min[1];
        h.dmin2 = m->dom.min[2];
        h.dmax0 = m->dom.max[0];
        h.dmax1 = m->dom.max[1];
        h.dmax2 = m->dom.max[2];
        h.xbase = xbase;
        h.tiles_x = tiles_x;
        h.tiles = bp.tiles;
        h.zlen = bp.zlen;
        h.items = bp.items;
        h.nsp = b.shape.nsp;
        h.nsc = b.shape.nsc;
        h.omega = (float)m->scalars[0];
        h.err = rt->dev_err;
        if (par == 0) {
          bp.cmap = (int)tmaps.size();
          for (int i = 0; i < 12; ++i) {
            if (!tmap_for(view(m->grids[2 + i]), 128, b.shape.warps, &t)) return false;
            tmaps.push_back(t);
          }
        }
      } else {
        psg::S7Params<float> &q = bp.s7[par];
        q.out = static_cast<float *>(out.ptr);
        q.row = out.pitch / 4;
        q.plane = q.row * out.ny;
        q.nx = g->dim[0];
        q.ny = g->dim[1];
        q.nz = g->dim[2];
        q.dmin0 = m->dom.min[0];
        q.dmin1 = m->dom.min[1];
        q.dmin2 = m->dom.min[2];
        q.dmax0 = m->dom.max[0];
        q.dmax1 = m->dom.max[1];
        q.dmax2 = m->dom.max[2];
        q.xbase = xbase;
        q.tiles_x = tiles_x;
        q.tiles = bp.tiles;
        q.zlen = bp.zlen;
        q.items = bp.items;
        q.ns = b.shape.ns7;
        const double *c = m->scalars.data();
        const bool has = m->scalars.size() >= 7;
        q.ce = has ? (float)c[0] : 0.f;
        q.cw = has ? (float)c[1] : 0.f;
        q.cn = has ? (float)c[2] : 0.f;
        q.cs = has ? (float)c[3] : 0.f;
        q.ct = has ? (float)c[4] : 0.f;
        q.cb = has ? (float)c[5] : 0.f;
        q.cc = has ? (float)c[6] : 0.f;
        q.err = rt->dev_err;
      }
    }
  }
  for (int f = 0; f < 2; ++f)
    b.grid[f] = (int)std::min<int64_t>(resident[f], std::max<int64_t>(b.total_items[f], 1));
  if (!cuda_ok(cudaMalloc(&b.probs_dev, sizeof(psg::BatchProblem) * probs.size()), "cudaMalloc") ||
      !cuda_ok(cudaMalloc(&b.tmaps_dev, sizeof(CUtensorMap) * tmaps.size()), "cudaMalloc") ||
      !cuda_ok(cudaMemcpyAsync(b.probs_dev, probs.data(), sizeof(psg::BatchProblem) * probs.size(),
                               cudaMemcpyHostToDevice, rt->stream), "batch table copy") ||
      !cuda_ok(cudaMemcpyAsync(b.tmaps_dev, tmaps.data(), sizeof(CUtensorMap) * tmaps.size(),
                               cudaMemcpyHostToDevice, rt->stream), "batch map copy") ||
      !cuda_ok(cudaStreamSynchronize(rt->stream), "cudaStreamSynchronize")) {
    batch_release(b);
    return false;
  }
  return true;
}

// One step of every run: one launch per kernel family present.  With both
// families the Himeno launch runs on the side stream, concurrently with the
// 7-point one, so each fills the SMs the other leaves idle at its tail.
bool batch_launch(Batch &b, int parity) {
  const bool both = b.nprob[0] && b.nprob[1];
  if (both && (!cuda_ok(cudaEventRecord(rt->fork, rt->stream), "cudaEventRecord") ||
               !cuda_ok(cudaStreamWaitEvent(rt->side, rt->fork, 0), "cudaStreamWaitEvent")))
    return false;
  for (int f = 0; f < 2; ++f) {
    if (!b.nprob[f]) continue;
    cudaStream_t s = (both && f == psg::kBatchHimeno) ? rt->side : rt->stream;
    cudaError_t e = psg::launch_batch(b.probs_dev + b.prob_off[f], b.nprob[f], b.tmaps_dev,
                                      b.total_items[f], parity, b.shape, b.grid[f], f, s);
    if (!cuda_ok(e, "batch launch")) return false;
    ++rt->launches;
  }
  if (both && (!cuda_ok(cudaEventRecord(rt->join, rt->side), "cudaEventRecord") ||
               !cuda_ok(cudaStreamWaitEvent(rt->stream, rt->join, 0), "cudaStreamWaitEvent")))
    return false;
  return true;
}

bool batch_stale(const Batch &b) {
  if (!b.probs_dev) return true;
  for (size_t i = 0; i < b.grids.size(); ++i)
    if (b.grids[i]->dev != b.ptrs[i]) return true;
  return false;
}

bool run_maps(const std::vector<Map *> &ms, int iter) {
  std::chrono::steady_clock::time_point t0;
  if (rt->trace) {
    fprintf(stderr, "Physis: Stencil started\n");
    t0 = std::chrono::steady_clock::now();
  }
  if ((rt->autotune || !g_tuned.empty()) && !run_tuning(ms, iter)) return false;
  if (iter <= 0) {
    // every iteration went into tuning trials
  } else if (ms.size() == 2 && temporal_pair(*ms[0], *ms[1])) {
    if (!run_temporal(*ms[0], iter)) return false;
  } else {
    if (!run_plain(ms, iter)) return false;
  }
  if (rt->trace) {
    if (!sync_rt()) return false;
    const double ms_ = std::chrono::duration<double, std::milli>(
                           std::chrono::steady_clock::now() - t0).count();
    fprintf(stderr, "Physis: Stencil finished (time: %f ms)\n", ms_);
  }
  return true;
}

bool read_result(int slot, uint64_t *bits) {
  if (!cuda_ok(cudaMemcpyAsync(bits, rt->results + slot, 8, cudaMemcpyDeviceToHost,
                               rt->stream), "read reduction result"))
    return false;
  return sync_rt();
}

bool reduce_grid(Grid *g, int op, uint64_t *bits) {
  if (op < PS_MAX || op > PS_PROD)
    return fail(PS_ERR_INVALID_ARGUMENT, "unknown reduction op %d", op);
  if (g->type == PS_USER)
    return fail(PS_ERR_UNSUPPORTED, "PSReduce: grids of a user-defined type are not reduced");
  const GridView v = view(g);
  const int n = psg::reduce_num_ctas(v, rt->sm_count);
  if (n > kMaxPartials) return fail(PS_ERR_UNSUPPORTED, "reduction grid too large");
  cudaError_t e = psg::launch_reduce(v, op, rt->partials, n, rt->ticket, rt->results,
                                     rt->dev_err, rt->stream);
  if (!cuda_ok(e, "reduce launch")) return false;
  ++rt->launches;
  return read_result(0, bits);
}

void store_reduced(void *v, int type, uint64_t bits) {
  switch (type) {
    case PS_FLOAT: {
      double d;
      memcpy(&d, &bits, 8);
      *static_cast<float *>(v) = (float)d;
      break;
    }
    case PS_DOUBLE: memcpy(v, &bits, 8); break;
    case PS_INT: {
      int32_t i = (int32_t)(uint32_t)bits;
      memcpy(v, &i, 4);
      break;
    }
    case PS_LONG: memcpy(v, &bits, 8); break;
  }
}

bool reduce_kernel_form(void *v, int op, int kernel, const __PSDomain &dom, int ngrids,
                        void *const *grids, int nscalars, const double *scalars,
                        double *out64) {
  if (kernel != PS_KERNEL_HIMENO19_GOSA)
    return fail(PS_ERR_UNSUPPORTED,
                "PSReduce kernel form: builtin %d yields no per-point value", kernel);
  if (op != PS_SUM)
    return fail(PS_ERR_UNSUPPORTED, "PSReduce kernel form supports PS_SUM only");
  Map m;
  if (!map_from(kernel, dom, ngrids, grids, nscalars, scalars, &m)) return false;
  if (!validate_map(m)) return false;
  if (!g_tuned.empty()) {  // a plan tuned for this sweep's PSStencilRun form
    auto hit = g_tuned.find(run_key({&m}));
    if (hit != g_tuned.end()) apply_plan({&m}, hit->second);
  }
  if (!launch_map(m, true)) return false;
  uint64_t bits = 0;
  if (!read_result(1, &bits)) return false;
  double d;
  memcpy(&d, &bits, 8);
  if (m.dom.min[0] >= m.dom.max[0] || m.dom.min[1] >= m.dom.max[1] ||
      m.dom.min[2] >= m.dom.max[2])
    d = 0.0;
  if (v) *static_cast<float *>(v) = (float)d;
  if (out64) *out64 = d;
  return true;
}

}  // namespace

namespace psg {

bool make_tmap_3d(CUtensorMap *map, const GridView &g, int box_w, int box_h) {
  if (!g_encode) return fail(PS_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  CUtensorMapDataType dt;
  switch (g.type) {
    case kFloat: dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT32; break;
    case kDouble: dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT64; break;
    case kInt: dt = CU_TENSOR_MAP_DATA_TYPE_INT32; break;
    default: dt = CU_TENSOR_MAP_DATA_TYPE_INT64; break;
  }
  cuuint64_t dims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
  cuuint64_t strides[2] = {(cuuint64_t)g.pitch, (cuuint64_t)g.pitch * (cuuint64_t)g.ny};
  cuuint32_t box[3] = {(cuuint32_t)box_w, (cuuint32_t)box_h, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = g_encode(map, dt, 3, g.ptr, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(PS_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d) for box %dx%d", (int)r,
                box_w, box_h);
  return true;
}

}  // namespace psg

extern "C" {

void PSInit(int *argc, char ***argv, int grid_num_dims, ...) {
  (void)grid_num_dims;
  bool trace = false;
  if (argc && argv && *argv) {
    int w = 0;
    for (int r = 0; r < *argc; ++r) {
      if ((*argv)[r] && strcmp((*argv)[r], "--physis-trace") == 0) {
        trace = true;
        continue;
      }
      (*argv)[w++] = (*argv)[r];
    }
    if (w < *argc) (*argv)[w] = nullptr;
    *argc = w;
  }
  const char *te = getenv("PS_TRACE");
  if (te && te[0] == '1') trace = true;
  PSInitV(trace ? 1 : 0);
}

void PSInitV(int trace) {
  if (rt) {
    rt->trace = rt->trace || trace;
    return;
  }
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    fail(PS_ERR_NO_DEVICE, "no CUDA device available (%s)",
         e != cudaSuccess ? cudaGetErrorString(e) : "count is 0");
    return;
  }
  Runtime *r = new Runtime();
  const char *de = getenv("PS_DEVICE");
  r->device = de ? atoi(de) : 0;
  if (!cuda_ok(cudaSetDevice(r->device), "cudaSetDevice")) {
    delete r;
    return;
  }
  cudaDeviceProp prop;
  if (!cuda_ok(cudaGetDeviceProperties(&prop, r->device), "cudaGetDeviceProperties")) {
    delete r;
    return;
  }
  if (prop.major < 10) {
    fail(PS_ERR_UNSUPPORTED, "device %s (sm_%d%d) is not a Blackwell GPU; this library "
         "is built for sm_103a only", prop.name, prop.major, prop.minor);
    delete r;
    return;
  }
  r->sm_count = prop.multiProcessorCount;
  r->gpu_name = prop.name;
  for (char &ch : r->gpu_name)
    if (ch == '"' || ch == ' ') ch = '_';
  r->trace = trace != 0;
  const char *at = getenv("PS_AUTOTUNE");
  r->autotune = at && at[0] == '1';
  const char *tc = getenv("PS_TUNE_CACHE");
  if (tc && tc[0]) r->tune_path = tc;
  if (!g_encode) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                         cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      fail(PS_ERR_CUDA, "cannot resolve cuTensorMapEncodeTiled");
      delete r;
      return;
    }
    g_encode = reinterpret_cast<EncodeTiledFn>(fn);
  }
  if (!cuda_ok(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking),
               "cudaStreamCreate") ||
      !cuda_ok(cudaStreamCreateWithFlags(&r->side, cudaStreamNonBlocking), "cudaStreamCreate") ||
      !cuda_ok(cudaEventCreateWithFlags(&r->fork, cudaEventDisableTiming), "cudaEventCreate") ||
      !cuda_ok(cudaEventCreateWithFlags(&r->join, cudaEventDisableTiming), "cudaEventCreate") ||
      !cuda_ok(cudaMalloc(&r->dev_err, sizeof(int)), "cudaMalloc") ||
      !cuda_ok(cudaMalloc(&r->partials, sizeof(uint64_t) * kMaxPartials), "cudaMalloc") ||
      !cuda_ok(cudaMalloc(&r->ticket, sizeof(unsigned)), "cudaMalloc") ||
      !cuda_ok(cudaMalloc(&r->results, sizeof(uint64_t) * 8), "cudaMalloc")) {
    delete r;
    return;
  }
  cudaMemset(r->dev_err, 0, sizeof(int));
  cudaMemset(r->ticket, 0, sizeof(unsigned));
  cudaMemset(r->results, 0, sizeof(uint64_t) * 8);
  for (int i = 0; i < kNumEvents; ++i) cudaEventCreate(&r->events[i]);
  // Default launch shapes (the autotuner may replace them):
  // {warps, rows per thread, ring stages, second-ring stages, CTAs per SM}.
  for (int k = 0; k < kNumKernels; ++k) r->shapes[k] = MarchConfig{8, 2, 4, 0, 0};
  for (int k = 0; k < kNumKernels; ++k) {
    r->tshapes[k] = MarchConfig{8, 4, 3, 0, 0};
    r->tblock[k] = 1;
  }
  // point stencils: 4 warps x 4 rows (a 128 x 16 tile; at 512^3 it equals 8 x 4 for the
  // 7-point stencil and is 6 % faster for the 27-point one: smaller rings, more CTAs)
  r->shapes[kSlotPoints] = MarchConfig{4, 4, 4, 0, 0};
  r->shapes[PS_KERNEL_HIMENO19] = MarchConfig{4, 1, 5, 2, 0};
  r->shapes[PS_KERNEL_HIMENO19_GOSA] = MarchConfig{4, 1, 5, 2, 0};
  cudaDeviceSynchronize();
  psg::nn_set_error_word(r->dev_err);
  rt = r;
  if (!rt->tune_path.empty()) load_tuned(rt->tune_path.c_str());
}

void PSFinalize(void) {
  if (!rt) return;
  cudaStreamSynchronize(rt->stream);
  for (Grid *g : rt->grids) {
    cudaFree(g->dev);
    g->magic = 0;
    delete g;
  }
  rt->grids.clear();
  for (GraphEntry &e : g_graphs) cudaGraphExecDestroy(e.exec);
  g_graphs.clear();
  for (Batch &b : g_batches) batch_release(b);
  g_batches.clear();
  for (psg::JitKernel &k : rt->funcs) psg::jit_unload(&k);
  cudaFree(rt->dev_err);
  cudaFree(rt->partials);
  cudaFree(rt->ticket);
  cudaFree(rt->results);
  for (int i = 0; i < kNumEvents; ++i) cudaEventDestroy(rt->events[i]);
  cudaEventDestroy(rt->fork);
  cudaEventDestroy(rt->join);
  cudaStreamDestroy(rt->side);
  cudaStreamDestroy(rt->stream);
  delete rt;
  rt = nullptr;
}

void PSPrintInternalInfo(FILE *out) {
  if (!out) out = stderr;
  if (!rt) {
    fprintf(out, "physis_gb300: not initialized\n");
    return;
  }
  cudaDeviceProp p;
  cudaGetDeviceProperties(&p, rt->device);
  fprintf(out, "physis_gb300: device %d %s sm_%d%d, %d SMs, %zu grids, %zu maps\n",
          rt->device, p.name, p.major, p.minor, rt->sm_count, rt->grids.size(),
          rt->maps.size());
}

void *PSGridNewV(int type, int ndims, const PSIndex *dims) {
  if (type == PS_USER) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSGridNewV: user-type grids come from PSGridNewUtype");
    return nullptr;
  }
  return grid_new(type, ndims, dims);
}

void *PSGridNewUtype(size_t elem_size, int ndims, const PSIndex *dims) {
  if (!dims) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSGridNewUtype: NULL dims");
    return nullptr;
  }
  return grid_new(PS_USER, ndims, dims, elem_size);
}

#define PS_DEFINE_NEW(RANK, NAME, TYPE, ...)                 \
  PS##NAME PS##NAME##New(__VA_ARGS__, ...) {                 \
    PSIndex d[3] = {PS_NEW_DIMS_##RANK};                     \
    return static_cast<PS##NAME>(grid_new(TYPE, RANK, d));   \
  }
#define PS_NEW_DIMS_1 nx, 1, 1
#define PS_NEW_DIMS_2 nx, ny, 1
#define PS_NEW_DIMS_3 nx, ny, nz
PS_DEFINE_NEW(1, Grid1DFloat, PS_FLOAT, PSIndex nx)
PS_DEFINE_NEW(1, Grid1DDouble, PS_DOUBLE, PSIndex nx)
PS_DEFINE_NEW(1, Grid1DInt, PS_INT, PSIndex nx)
PS_DEFINE_NEW(1, Grid1DLong, PS_LONG, PSIndex nx)
PS_DEFINE_NEW(2, Grid2DFloat, PS_FLOAT, PSIndex nx, PSIndex ny)
PS_DEFINE_NEW(2, Grid2DDouble, PS_DOUBLE, PSIndex nx, PSIndex ny)
PS_DEFINE_NEW(2, Grid2DInt, PS_INT, PSIndex nx, PSIndex ny)
PS_DEFINE_NEW(2, Grid2DLong, PS_LONG, PSIndex nx, PSIndex ny)
PS_DEFINE_NEW(3, Grid3DFloat, PS_FLOAT, PSIndex nx, PSIndex ny, PSIndex nz)
PS_DEFINE_NEW(3, Grid3DDouble, PS_DOUBLE, PSIndex nx, PSIndex ny, PSIndex nz)
PS_DEFINE_NEW(3, Grid3DInt, PS_INT, PSIndex nx, PSIndex ny, PSIndex nz)
PS_DEFINE_NEW(3, Grid3DLong, PS_LONG, PSIndex nx, PSIndex ny, PSIndex nz)

void PSGridCopyin(void *g, const void *src_array) {
  Grid *p = as_grid(g, "PSGridCopyin");
  if (!p) return;
  if (!src_array) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSGridCopyin: NULL source");
    return;
  }
  copy_grid(p, const_cast<void *>(src_array), true, true);
}

void PSGridCopyout(void *g, void *dst_array) {
  Grid *p = as_grid(g, "PSGridCopyout");
  if (!p) return;
  if (!dst_array) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSGridCopyout: NULL destination");
    return;
  }
  copy_grid(p, dst_array, false, true);
}

void PSGridCopyinAsync(void *g, const void *src) {
  Grid *p = as_grid(g, "PSGridCopyinAsync");
  if (p && src) copy_grid(p, const_cast<void *>(src), true, false);
}

void PSGridCopyoutAsync(void *g, void *dst) {
  Grid *p = as_grid(g, "PSGridCopyoutAsync");
  if (p && dst) copy_grid(p, dst, false, false);
}

void PSGridFree(void *g) {
  Grid *p = as_grid(g, "PSGridFree");
  if (!p) return;
  cudaStreamSynchronize(rt->stream);
  drop_tmaps(p->dev);
  drop_graphs_for(p);
  cudaFree(p->dev);
  rt->grids.erase(p);
  p->magic = 0;
  delete p;
}

// One element of a grid from the host: the grid's rank of indices (x first),
// bounds-checked, then a stream-ordered copy of the element, so it lands
// after every stencil run already issued and before any later one.
static int grid_set(void *g, const PSIndex *idx, const void *buf, const char *fn) {
  Grid *p = as_grid(g, fn);
  if (!p) return g_err;
  if (!idx || !buf) {
    fail(PS_ERR_INVALID_ARGUMENT, "%s: NULL index or value", fn);
    return PS_ERR_INVALID_ARGUMENT;
  }
  PSIndex c[3] = {0, 0, 0};
  for (int d = 0; d < p->ndims; ++d) {
    if (idx[d] < 0 || idx[d] >= p->dim[d]) {
      fail(PS_ERR_INVALID_ARGUMENT, "%s: index %d of dimension %d outside [0, %d)", fn,
           (int)idx[d], d, (int)p->dim[d]);
      return PS_ERR_INVALID_ARGUMENT;
    }
    c[d] = idx[d];
  }
  char *dst = static_cast<char *>(p->dev) +
              ((size_t)c[2] * p->dim[1] + c[1]) * p->pitch + (size_t)c[0] * p->esz;
  if (!cuda_ok(cudaMemcpyAsync(dst, buf, p->esz, cudaMemcpyHostToDevice, rt->stream), fn) ||
      !cuda_ok(cudaStreamSynchronize(rt->stream), fn))
    return g_err;
  return PS_OK;
}

int PSGridSetV(void *g, const PSIndex *idx, const void *value) {
  return grid_set(g, idx, value, "PSGridSetV");
}

void __PSGridSet(void *g, const void *buf, ...) {
  Grid *p = as_grid(g, "__PSGridSet");
  if (!p) return;
  PSIndex idx[3] = {0, 0, 0};
  va_list vl;
  va_start(vl, buf);
  for (int d = 0; d < p->ndims; ++d) idx[d] = va_arg(vl, PSIndex);
  va_end(vl);
  grid_set(g, idx, buf, "__PSGridSet");
}

void __PSGridSetScalar(void *g, int nidx, PSIndex i, PSIndex j, PSIndex k, int is_float,
                       double vf, long long vi) {
  Grid *p = as_grid(g, "PSGridSet");
  if (!p) return;
  if (p->type == PS_USER) {
    fail(PS_ERR_INVALID_ARGUMENT,
         "PSGridSet: a user-type grid takes __PSGridSet(g, &value, indices...)");
    return;
  }
  if (nidx != p->ndims) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSGridSet: %d indices for a %d-dimensional grid", nidx,
         p->ndims);
    return;
  }
  // The value converted to the element type as a C assignment would.
  union {
    float f;
    double d;
    int32_t i;
    int64_t l;
  } v;
  switch (p->type) {
    case PS_FLOAT: v.f = is_float ? (float)vf : (float)vi; break;
    case PS_DOUBLE: v.d = is_float ? vf : (double)vi; break;
    case PS_INT: v.i = is_float ? (int32_t)vf : (int32_t)vi; break;
    default: v.l = is_float ? (int64_t)vf : (int64_t)vi; break;
  }
  const PSIndex idx[3] = {i, j, k};
  grid_set(g, idx, &v, "PSGridSet");
}

PSIndex PSGridDim(void *g, int d) {
  Grid *p = as_grid(g, "PSGridDim");
  if (!p) return 0;
  if (d < 0 || d >= 3) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSGridDim: dimension %d", d);
    return 0;
  }
  return p->dim[d];
}

void *PSGridDevicePtr(void *g) {
  Grid *p = as_grid(g, "PSGridDevicePtr");
  return p ? p->dev : nullptr;
}
size_t PSGridPitch(void *g) {
  Grid *p = as_grid(g, "PSGridPitch");
  return p ? p->pitch : 0;
}
int PSGridElemSize(void *g) {
  Grid *p = as_grid(g, "PSGridElemSize");
  return p ? p->esz : 0;
}
int PSGridType(void *g) {
  Grid *p = as_grid(g, "PSGridType");
  return p ? p->type : -1;
}

PSDomain1D PSDomain1DNew(PSIndex minx, PSIndex maxx) {
  PSDomain1D d = {{minx, 0, 0}, {maxx, 1, 1}, {minx, 0, 0}, {maxx, 1, 1}};
  return d;
}
PSDomain2D PSDomain2DNew(PSIndex minx, PSIndex maxx, PSIndex miny, PSIndex maxy) {
  PSDomain2D d = {{minx, miny, 0}, {maxx, maxy, 1}, {minx, miny, 0}, {maxx, maxy, 1}};
  return d;
}
PSDomain3D PSDomain3DNew(PSIndex minx, PSIndex maxx, PSIndex miny, PSIndex maxy,
                         PSIndex minz, PSIndex maxz) {
  PSDomain3D d = {{minx, miny, minz}, {maxx, maxy, maxz},
                  {minx, miny, minz}, {maxx, maxy, maxz}};
  return d;
}

static PSStencil map_varargs(const char *fn, void *kernel, int color, va_list vl);

PSStencil __PSStencilMap(void *kernel, ...) {
  va_list vl;
  va_start(vl, kernel);
  const PSStencil s = map_varargs("PSStencilMap", kernel, -1, vl);
  va_end(vl);
  return s;
}

PSStencil PSStencilMapV(int kernel, const PSDomain3D *dom, int ngrids, void *const *grids,
                        int nscalars, const double *scalars) {
  if (!need_rt("PSStencilMapV")) return -1;
  if (!dom || (ngrids && !grids) || (nscalars && !scalars)) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSStencilMapV: NULL argument");
    return -1;
  }
  Map m;
  if (!map_from(kernel, *dom, ngrids, grids, nscalars, scalars, &m)) return -1;
  return add_map(std::move(m));
}

// Reads a map's grid handles and scalars from C varargs.  Builtins take their
// grids, then float scalars (promoted to double).  A compiled stencil
// function takes them in its parameter order, each scalar with its declared
// type's promotion (int, long, double).
static void read_map_args(const KernelSig &sig, int ng, va_list vl, void **grids, double *sc) {
  if (!sig.fn) {
    for (int i = 0; i < ng; ++i) grids[i] = va_arg(vl, void *);
    for (int i = 0; i < sig.nscalars; ++i) sc[i] = va_arg(vl, double);
    return;
  }
  int gi = 0, si = 0;
  for (const psg::JitParam &p : sig.fn->params) {
    if (p.grid) {
      grids[gi++] = va_arg(vl, void *);
    } else if (p.type == psg::kInt) {
      sc[si++] = (double)va_arg(vl, int);
    } else if (p.type == psg::kLong) {
      sc[si++] = (double)va_arg(vl, long);
    } else {
      sc[si++] = va_arg(vl, double);
    }
  }
}

// __PSStencilMap and its red/black forms: kernel, domain, grids, scalars.
static PSStencil map_varargs(const char *fn, void *kernel, int color, va_list vl) {
  if (!need_rt(fn)) return -1;
  const int k = (int)(intptr_t)kernel;
  KernelSig sig;
  if (!kernel_sig(k, &sig)) {
    fail(PS_ERR_UNKNOWN_KERNEL, "%s: unknown stencil id %d", fn, k);
    return -1;
  }
  __PSDomain dom = va_arg(vl, __PSDomain);
  void *grids[64];
  double sc[64];
  const int ng = map_ngrids(sig, color);
  if (ng > 64 || sig.nscalars > 64) {
    fail(PS_ERR_UNSUPPORTED, "%s: more than 64 grids or scalars", fn);
    return -1;
  }
  read_map_args(sig, ng, vl, grids, sc);
  Map m;
  if (!map_from(k, dom, ng, grids, sig.nscalars, sc, &m, color)) return -1;
  return add_map(std::move(m));
}

PSStencil __PSStencilMapRedBlack(void *kernel, ...) {
  va_list vl;
  va_start(vl, kernel);
  const PSStencil s = map_varargs("PSStencilMapRedBlack", kernel, 2, vl);
  va_end(vl);
  return s;
}

PSStencil __PSStencilMapRed(void *kernel, ...) {
  va_list vl;
  va_start(vl, kernel);
  const PSStencil s = map_varargs("PSStencilMapRed", kernel, 0, vl);
  va_end(vl);
  return s;
}

PSStencil __PSStencilMapBlack(void *kernel, ...) {
  va_list vl;
  va_start(vl, kernel);
  const PSStencil s = map_varargs("PSStencilMapBlack", kernel, 1, vl);
  va_end(vl);
  return s;
}

PSStencil PSStencilMapColorV(int kernel, int color, const PSDomain3D *dom, int ngrids,
                             void *const *grids, int nscalars, const double *scalars) {
  if (!need_rt("PSStencilMapColorV")) return -1;
  if (!dom || (ngrids && !grids) || (nscalars && !scalars)) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSStencilMapColorV: NULL argument");
    return -1;
  }
  Map m;
  if (!map_from(kernel, *dom, ngrids, grids, nscalars, scalars, &m, color)) return -1;
  return add_map(std::move(m));
}

int PSStencilFunctionCheck(const char *source, const char *name, char *log, size_t logsize) {
  if (log && logsize) log[0] = '\0';
  if (!source || !name || !name[0]) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSStencilFunctionCheck: NULL source or name");
    return PS_ERR_INVALID_ARGUMENT;
  }
  psg::JitKernel k;
  std::vector<char> image;
  std::string why;
  if (psg::jit_build(source, name, &k, &image, &why)) {
    std::string rep;
    for (const psg::JitStage &st : k.stages)
      rep += "staged " + k.params[st.param].name + " " + std::to_string(st.rx) + " " +
             std::to_string(st.ry) + " " + std::to_string(st.rz) +
             (st.periodic ? " periodic;" : " clamp;");
    if (log && logsize) snprintf(log, logsize, "%s", rep.c_str());
    return PS_OK;
  }
  if (log && logsize) snprintf(log, logsize, "%s", why.c_str());
  const bool missing = why.find("not available") != std::string::npos ||
                       why.find("lacks") != std::string::npos;
  return missing ? PS_ERR_UNSUPPORTED : PS_ERR_INVALID_ARGUMENT;
}

int PSStencilFunctionNew(const char *source, const char *name) {
  if (!need_rt("PSStencilFunctionNew")) return -1;
  if (!source || !name || !name[0]) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSStencilFunctionNew: NULL source or name");
    return -1;
  }
  for (size_t i = 0; i < rt->funcs.size(); ++i)
    if (rt->funcs[i].name == name && rt->funcs[i].source == source)
      return kFuncBase + (int)i;
  if ((int)rt->funcs.size() >= kMaxFunctions) {
    fail(PS_ERR_OUT_OF_MEMORY, "more than %d stencil functions", kMaxFunctions);
    return -1;
  }
  psg::JitKernel k;
  std::string why;
  if (!psg::jit_compile(source, name, &k, &why)) {
    const bool missing = why.find("not available") != std::string::npos ||
                         why.find("unavailable") != std::string::npos ||
                         why.find("lacks") != std::string::npos;
    fail(missing ? PS_ERR_UNSUPPORTED : PS_ERR_INVALID_ARGUMENT, "PSStencilFunctionNew: %s",
         why.c_str());
    return -1;
  }
  rt->funcs.push_back(std::move(k));
  return kFuncBase + (int)rt->funcs.size() - 1;
}

int PSPointStencilNew(int boundary, int npoints, const int *offsets, const double *weights) {
  if (!need_rt("PSPointStencilNew")) return -1;
  if (boundary < PS_BOUNDARY_NONE || boundary > PS_BOUNDARY_CLAMP) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSPointStencilNew: unknown boundary rule %d", boundary);
    return -1;
  }
  if (npoints < 1 || npoints > PS_MAX_POINTS || !offsets) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSPointStencilNew: %d points (1..%d, offsets non-NULL)",
         npoints, PS_MAX_POINTS);
    return -1;
  }
  PointStencil ps;
  ps.boundary = boundary;
  ps.n = npoints;
  ps.unit = true;
  for (int i = 0; i < npoints; ++i) {
    for (int d = 0; d < 3; ++d) {
      const int o = offsets[3 * i + d];
      if (o < -PS_MAX_POINT_RADIUS || o > PS_MAX_POINT_RADIUS) {
        fail(PS_ERR_INVALID_ARGUMENT, "PSPointStencilNew: offset %d of point %d beyond +-%d",
             o, i, PS_MAX_POINT_RADIUS);
        return -1;
      }
      ps.d[i][d] = o;
    }
    ps.w[i] = weights ? weights[i] : 1.0;
    if (weights && !std::isfinite(weights[i])) {
      fail(PS_ERR_INVALID_ARGUMENT, "PSPointStencilNew: weight %d is not finite", i);
      return -1;
    }
    if (ps.w[i] != 1.0) ps.unit = false;
  }
  return register_points(ps);
}

void PSStencilRunV(int n, const PSStencil *stencils, int iter) {
  if (!need_rt("PSStencilRun")) return;
  if (n <= 0 || !stencils || iter < 0) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSStencilRun: %d stencils, iter %d", n, iter);
    return;
  }
  std::vector<Map *> ms;
  for (int i = 0; i < n; ++i) {
    Map *m = lookup_map(stencils[i]);
    if (!m) {
      fail(PS_ERR_BAD_HANDLE, "PSStencilRun: %d is not a stencil", stencils[i]);
      return;
    }
    for (const Grid *g : m->grids)
      if (!rt->grids.count(const_cast<Grid *>(g))) {
        fail(PS_ERR_BAD_HANDLE, "PSStencilRun: stencil %d uses a freed grid", stencils[i]);
        return;
      }
    ms.push_back(m);
  }
  run_maps(ms, iter);
}

void PSStencilRun(PSStencil s, ...) {
  if (!need_rt("PSStencilRun")) return;
  std::vector<PSStencil> list;
  int iter = 1;
  list.push_back(s);
  va_list vl;
  va_start(vl, s);
  for (int guard = 0; guard < 4096; ++guard) {
    const int a = va_arg(vl, int);
    if (a == PS_RUN_END) break;
    if ((a & kStencilTagMask) == kStencilTag) {
      list.push_back(a);
    } else {
      iter = a;
      const int end = va_arg(vl, int);
      if (end != PS_RUN_END) {
        va_end(vl);
        fail(PS_ERR_INVALID_ARGUMENT,
             "PSStencilRun: the iteration count must be the last argument");
        return;
      }
      break;
    }
  }
  va_end(vl);
  PSStencilRunV((int)list.size(), list.data(), iter);
}

void PSReduceGridV(void *v, int op, void *g) {
  Grid *p = as_grid(g, "PSReduce");
  if (!p) return;
  if (!v) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSReduce: NULL result pointer");
    return;
  }
  uint64_t bits;
  if (reduce_grid(p, op, &bits)) store_reduced(v, p->type, bits);
}

void PSReduceGridF64(double *v, int op, void *g) {
  Grid *p = as_grid(g, "PSReduceGridF64");
  if (!p) return;
  if (p->type != PS_FLOAT && p->type != PS_DOUBLE) {
    fail(PS_ERR_UNSUPPORTED, "PSReduceGridF64 needs a float or double grid");
    return;
  }
  uint64_t bits;
  if (v && reduce_grid(p, op, &bits)) memcpy(v, &bits, 8);
}

void PSReduceKernelV(void *v, int op, int kernel, const PSDomain3D *dom, int ngrids,
                     void *const *grids, int nscalars, const double *scalars) {
  if (!need_rt("PSReduce")) return;
  if (!dom) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSReduceKernelV: NULL domain");
    return;
  }
  reduce_kernel_form(v, op, kernel, *dom, ngrids, grids, nscalars, scalars, nullptr);
}

void PSReduce(void *v, ...) {
  if (!need_rt("PSReduce")) return;
  va_list vl;
  va_start(vl, v);
  const int op = va_arg(vl, int);
  void *third = va_arg(vl, void *);
  Grid *g = static_cast<Grid *>(third);
  if (g && rt->grids.count(g)) {
    va_end(vl);
    PSReduceGridV(v, op, g);
    return;
  }
  const int k = (int)(intptr_t)third;
  KernelSig sig;
  if (!kernel_sig(k, &sig)) {
    va_end(vl);
    fail(PS_ERR_BAD_HANDLE, "PSReduce: third argument is neither a grid nor a builtin");
    return;
  }
  __PSDomain dom = va_arg(vl, __PSDomain);
  void *grids[16];
  double sc[16];
  for (int i = 0; i < sig.ngrids; ++i) grids[i] = va_arg(vl, void *);
  for (int i = 0; i < sig.nscalars; ++i) sc[i] = va_arg(vl, double);
  va_end(vl);
  if (!v) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSReduce: NULL result pointer");
    return;
  }
  reduce_kernel_form(v, op, k, dom, sig.ngrids, grids, sig.nscalars, sc, nullptr);
}

int PSGetLastError(void) { return g_err; }
const char *PSGetLastErrorString(void) { return g_errmsg.c_str(); }
const char *PSGetErrorName(int code) { return err_name(code); }
void PSClearError(void) {
  g_err = PS_OK;
  g_errmsg.clear();
}

void *PSHostAlloc(size_t bytes) {
  void *p = nullptr;
  if (!cuda_ok(cudaMallocHost(&p, bytes), "cudaMallocHost")) return nullptr;
  return p;
}
void PSHostFree(void *p) {
  if (p) cudaFreeHost(p);
}

void PSSynchronize(void) {
  if (!need_rt("PSSynchronize")) return;
  sync_rt();
}

void *PSGetStream(void) { return rt ? (void *)rt->stream : nullptr; }

void PSEventRecord(int slot) {
  if (!need_rt("PSEventRecord")) return;
  if (slot < 0 || slot >= kNumEvents) {
    fail(PS_ERR_INVALID_ARGUMENT, "event slot %d", slot);
    return;
  }
  cuda_ok(cudaEventRecord(rt->events[slot], rt->stream), "cudaEventRecord");
}

float PSEventElapsedMs(int a, int b) {
  if (!need_rt("PSEventElapsedMs")) return -1.0f;
  if (a < 0 || a >= kNumEvents || b < 0 || b >= kNumEvents) {
    fail(PS_ERR_INVALID_ARGUMENT, "event slots %d %d", a, b);
    return -1.0f;
  }
  if (!cuda_ok(cudaEventSynchronize(rt->events[b]), "cudaEventSynchronize")) return -1.0f;
  float ms = 0.0f;
  if (!cuda_ok(cudaEventElapsedTime(&ms, rt->events[a], rt->events[b]),
               "cudaEventElapsedTime"))
    return -1.0f;
  return ms;
}

long long PSGetLaunchCount(void) { return rt ? rt->launches : 0; }
int PSGetSMCount(void) { return rt ? rt->sm_count : 0; }

void PSSetLaunchShape(int kernel, const PSLaunchShape *shape) {
  if (!need_rt("PSSetLaunchShape")) return;
  if (!shape) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSSetLaunchShape: NULL shape");
    return;
  }
  for (int k = 0; k < kNumKernels; ++k) {
    if (kernel != 0 && k != shape_slot(kernel)) continue;
    const bool kh = (k == PS_KERNEL_HIMENO19 || k == PS_KERNEL_HIMENO19_GOSA);
    if (kernel == 0 && kh) continue;  // a global shape does not touch Himeno's
    MarchConfig c = rt->shapes[k];
    if (shape->warps > 0) c.warps = shape->warps;
    if (shape->rows > 0) c.rows = shape->rows;
    if (shape->ns > 0) c.ns = shape->ns;
    if (shape->ns2 > 0) c.ns2 = shape->ns2;
    c.ctas_per_sm = shape->ctas_per_sm > 0 ? shape->ctas_per_sm : 0;
    const bool rows_ok = kh ? c.rows == 1
                            : (c.rows == 1 || c.rows == 2 || c.rows == 4 || c.rows == 8);
    const int max_warps = kh ? 8 : 16;
    if (c.warps < 1 || c.warps > max_warps || !rows_ok || c.ns < (kh ? 3 : 2) ||
        c.ns > 16 || (kh && (c.ns2 < 1 || c.ns2 > 8)) || c.ctas_per_sm > 32) {
      fail(PS_ERR_INVALID_ARGUMENT,
           "PSSetLaunchShape: warps %d rows %d ns %d ns2 %d ctas/SM %d out of range",
           c.warps, c.rows, c.ns, c.ns2, c.ctas_per_sm);
      return;
    }
    const size_t smem = kh ? psg::himeno19_smem_bytes(c) : psg::stencil7_smem_bytes(8, c);
    if (smem > 200 * 1024) {
      fail(PS_ERR_INVALID_ARGUMENT, "PSSetLaunchShape: %zu bytes of shared memory", smem);
      return;
    }
    rt->shapes[k] = c;
  }
}

void PSSetTemporalBlocking(int kernel, int k, const PSLaunchShape *shape) {
  if (!need_rt("PSSetTemporalBlocking")) return;
  if (kernel != PS_KERNEL_DIFFUSION7) {
    fail(PS_ERR_UNSUPPORTED, "temporal blocking is implemented for PS_KERNEL_DIFFUSION7 only");
    return;
  }
  if (k < 1 || k > psg::temporal7_max_k(4)) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSSetTemporalBlocking: k %d not in 1..%d", k,
         psg::temporal7_max_k(4));
    return;
  }
  MarchConfig c = rt->tshapes[kernel];
  if (shape) {
    if (shape->warps > 0) c.warps = shape->warps;
    if (shape->rows > 0) c.rows = shape->rows;
    if (shape->ns > 0) c.ns = shape->ns;
    c.ctas_per_sm = shape->ctas_per_sm > 0 ? shape->ctas_per_sm : 0;
  }
  if (c.warps < 1 || c.warps > 8 || !(c.rows == 1 || c.rows == 2 || c.rows == 4) ||
      c.ns < 2 || c.ns > 16 || c.warps * c.rows - 2 * (k - 1) < 1 ||
      psg::temporal7_smem_bytes(8, c, k) > 227 * 1024) {
    fail(PS_ERR_INVALID_ARGUMENT,
         "PSSetTemporalBlocking: shape warps %d rows %d ns %d does not fit k %d", c.warps,
         c.rows, c.ns, k);
    return;
  }
  rt->tshapes[kernel] = c;
  rt->tblock[kernel] = k;
}

void PSSetFusedMultiplyAdd(int on) {
  if (!need_rt("PSSetFusedMultiplyAdd")) return;
  rt->fma = on != 0;
}

int PSGetFusedMultiplyAdd(void) {
  if (!need_rt("PSGetFusedMultiplyAdd")) return 0;
  return rt->fma ? 1 : 0;
}

void PSGetTemporalBlocking(int kernel, int *k, PSLaunchShape *shape) {
  if (!need_rt("PSGetTemporalBlocking")) return;
  const int slot = shape_slot(kernel);
  if (k) *k = rt->tblock[slot];
  if (shape) {
    const MarchConfig &c = rt->tshapes[slot];
    shape->warps = c.warps;
    shape->rows = c.rows;
    shape->ns = c.ns;
    shape->ns2 = c.ns2;
    shape->ctas_per_sm = c.ctas_per_sm;
  }
}

void PSGetLaunchShape(int kernel, PSLaunchShape *shape) {
  if (!need_rt("PSGetLaunchShape") || !shape) return;
  const MarchConfig &c = rt->shapes[shape_slot(kernel)];
  shape->warps = c.warps;
  shape->rows = c.rows;
  shape->ns = c.ns;
  shape->ns2 = c.ns2;
  shape->ctas_per_sm = c.ctas_per_sm;
}

static cudaStream_t ws_stream(void *stream) {
  if (stream) return static_cast<cudaStream_t>(stream);
  return rt ? rt->stream : nullptr;
}

// rc: 0, -1 (invalid arguments) or a cudaError_t from the launch.
static int ws_status(int rc, const char *what) {
  if (rc == 0) return PS_OK;
  if (rc > 0) {
    fail(PS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(static_cast<cudaError_t>(rc)));
    return PS_ERR_CUDA;
  }
  fail(PS_ERR_INVALID_ARGUMENT, "%s: invalid arguments", what);
  return PS_ERR_INVALID_ARGUMENT;
}

static psg::NNFields ws_fields(const PSWarmStartFields *f) {
  psg::NNFields n{};
  n.a0 = f->a0;
  n.a1 = f->a1;
  n.a2 = f->a2;
  n.wrk1 = f->wrk1;
  n.bnd = f->bnd;
  n.p = f->p;
  n.pitch = f->pitch;
  n.ny = f->ny;
  n.inx = f->inx;
  n.iny = f->iny;
  n.inz = f->inz;
  n.nsx = f->nsx;
  n.factor = f->factor;
  n.batch = f->batch;
  n.wscale = f->wscale;
  n.pscale = f->pscale;
  n.flip = f->flip;
  n.inst_scale = f->inst_scale;
  n.p_sub = f->p_sub;
  return n;
}

static bool ws_fields_ok(const PSWarmStartFields *f, const char *what, bool need_p) {
  if (!f || !f->a0 || !f->a1 || !f->a2 || !f->wrk1 || !f->bnd || (need_p && !f->p) ||
      f->pitch <= 0 || f->pitch % 4 || f->inx < 1 || f->iny < 1 || f->inz < 1 || f->nsx < 1 ||
      f->factor < 1 || f->batch < 1 || f->ny < f->iny || f->pitch / 4 < (long long)f->inx ||
      f->flip < 0 || f->flip > 15 || ((f->flip & 8) && f->inx != f->iny)) {
    fail(PS_ERR_INVALID_ARGUMENT, "%s: bad field description", what);
    return false;
  }
  return true;
}

int PSWarmStartConv(const void *x, const void *w, const float *bias, const void *mask, int relu,
                    void *y, float *y_ch0, int batch, int nz, int ny, int nx, void *stream) {
  if (!x || !w || !y || batch < 1 || nz < 1 || ny < 1 || nx < 1)
    return ws_status(-1, "PSWarmStartConv");
  return ws_status(psg::nn_conv(x, w, bias, mask, relu, y, y_ch0, batch, nz, ny, nx,
                                ws_stream(stream)),
                   "PSWarmStartConv");
}

int PSWarmStartWeightGrad(const void *x, const void *dy, float *work, int nsplit, float *dw,
                          float *db, int batch, int nz, int ny, int nx, void *stream) {
  if (!x || !dy || !work || !dw || nsplit < 1 || nsplit > 65535 || batch < 1 || nz < 1 ||
      ny < 1 || nx < 1)
    return ws_status(-1, "PSWarmStartWeightGrad");
  return ws_status(psg::nn_wgrad(x, dy, work, nsplit, dw, db, batch, nz, ny, nx,
                                 ws_stream(stream)),
                   "PSWarmStartWeightGrad");
}

int PSWarmStartPrepareWeights(const float *w, void *w_fwd, void *w_bwd, void *stream) {
  if (!w || !w_fwd || !w_bwd) return ws_status(-1, "PSWarmStartPrepareWeights");
  return ws_status(psg::nn_prep_weights(w, w_fwd, w_bwd, ws_stream(stream)),
                   "PSWarmStartPrepareWeights");
}

int PSWarmStartAdam(float *w, const float *g, float *m, float *v, long long n, float lr, float b1,
                    float b2, float eps, int step, void *stream) {
  if (!w || !g || !m || !v) return ws_status(-1, "PSWarmStartAdam");
  return ws_status(psg::nn_adam(w, g, m, v, n, lr, b1, b2, eps, step, ws_stream(stream)),
                   "PSWarmStartAdam");
}

int PSWarmStartLoss(const float *pred, const float *target, long long n, void *dy,
                    double *partials, void *stream) {
  if (!pred || !target || !dy || !partials) return ws_status(-1, "PSWarmStartLoss");
  return ws_status(psg::nn_mse(pred, target, n, dy, partials, ws_stream(stream)),
                   "PSWarmStartLoss");
}

int PSWarmStartPool(const PSWarmStartFields *f, void *out, void *stream) {
  if (!ws_fields_ok(f, "PSWarmStartPool", false) || !out) return PS_ERR_INVALID_ARGUMENT;
  return ws_status(psg::nn_pool_inputs(ws_fields(f), out, ws_stream(stream)), "PSWarmStartPool");
}

int PSWarmStartResidualSource(const PSWarmStartFields *f, float *r, float *inst_scale,
                              float target_rms, double *work, int work_len, void *stream) {
  if (!ws_fields_ok(f, "PSWarmStartResidualSource", true) || !r || !inst_scale || !work ||
      work_len < f->batch || f->flip != 0)
    return ws_status(-1, "PSWarmStartResidualSource");
  return ws_status(psg::nn_residual_source(ws_fields(f), r, inst_scale, target_rms, work,
                                           work_len, ws_stream(stream)),
                   "PSWarmStartResidualSource");
}

int PSWarmStartAddCorrection(const PSWarmStartFields *f, const float *delta, float p_scale,
                             float *p, void *stream) {
  if (!ws_fields_ok(f, "PSWarmStartAddCorrection", false) || !p || f->flip != 0)
    return ws_status(-1, "PSWarmStartAddCorrection");
  return ws_status(psg::nn_add_correction(ws_fields(f), delta, p_scale, p, ws_stream(stream)),
                   "PSWarmStartAddCorrection");
}

int PSWarmStartPoolTarget(const PSWarmStartFields *f, float *out, void *stream) {
  if (!ws_fields_ok(f, "PSWarmStartPoolTarget", true) || !out) return PS_ERR_INVALID_ARGUMENT;
  return ws_status(psg::nn_pool_target(ws_fields(f), out, ws_stream(stream)),
                   "PSWarmStartPoolTarget");
}

int PSWarmStartUpsample(const PSWarmStartFields *f, const float *coarse, float *p, void *stream) {
  if (!ws_fields_ok(f, "PSWarmStartUpsample", false) || !coarse || !p)
    return PS_ERR_INVALID_ARGUMENT;
  return ws_status(psg::nn_upsample(ws_fields(f), coarse, p, false, ws_stream(stream)),
                   "PSWarmStartUpsample");
}

int PSWarmStartUpsampleAdd(const PSWarmStartFields *f, const float *coarse, float *p,
                           void *stream) {
  if (!ws_fields_ok(f, "PSWarmStartUpsampleAdd", false) || !coarse || !p)
    return PS_ERR_INVALID_ARGUMENT;
  return ws_status(psg::nn_upsample(ws_fields(f), coarse, p, true, ws_stream(stream)),
                   "PSWarmStartUpsampleAdd");
}

int PSReduceNoAlloc(const void *data, size_t pitch, int nx, int ny, int nz, int type,
                    int op, void *result, void *stream) {
  const char *why = "";
  const int code = psg::reduce_noalloc(data, pitch, nx, ny, nz, type, op, result,
                                       static_cast<cudaStream_t>(stream), &why);
  if (code != PS_OK) fail(code, "PSReduceNoAlloc: %s", why);
  return code;
}

int PSBatchCreate(int nruns, int maps_per_run, const PSStencil *maps) {
  if (!need_rt("PSBatchCreate")) return -1;
  if (nruns < 1 || maps_per_run < 1 || maps_per_run > 2 || !maps) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSBatchCreate: %d runs of %d maps", nruns, maps_per_run);
    return -1;
  }
  Batch b;
  b.nruns = nruns;
  b.maps_per_run = maps_per_run;
  for (int r = 0; r < nruns; ++r) {
    const Map *first = nullptr;
    for (int j = 0; j < maps_per_run; ++j) {
      const Map *m = lookup_map(maps[r * maps_per_run + j]);
      if (!m) {
        fail(PS_ERR_BAD_HANDLE, "PSBatchCreate: %d is not a stencil", maps[r * maps_per_run + j]);
        return -1;
      }
      if (!batch_kind_ok(m->kernel) || m->grids[0]->type != PS_FLOAT) {
        fail(PS_ERR_UNSUPPORTED,
             "PSBatchCreate: batches take float maps of DIFFUSION7, SUM7, COPY or HIMENO19");
        return -1;
      }
      const __PSDomain &d = m->dom;
      if (d.min[0] >= d.max[0] || d.min[1] >= d.max[1] || d.min[2] >= d.max[2]) {
        fail(PS_ERR_INVALID_ARGUMENT, "PSBatchCreate: empty domain");
        return -1;
      }
      if (first) {
        bool same = first->kernel == m->kernel;
        for (int k = 0; k < 3; ++k)
          same = same && first->dom.min[k] == d.min[k] && first->dom.max[k] == d.max[k];
        if (!same) {
          fail(PS_ERR_INVALID_ARGUMENT,
               "PSBatchCreate: the maps of one run must share kernel and domain");
          return -1;
        }
      }
      first = first ? first : m;
      b.maps.push_back(m);
      for (const Grid *g : m->grids) b.grids.push_back(g);
    }
  }
  if (!batch_build(b)) return -1;
  b.live = true;
  g_batches.push_back(b);
  return (int)g_batches.size() - 1;
}

void PSBatchRun(int batch, int iter) {
  if (!need_rt("PSBatchRun")) return;
  if (batch < 0 || batch >= (int)g_batches.size() || !g_batches[batch].live) {
    fail(PS_ERR_BAD_HANDLE, "PSBatchRun: %d is not a batch", batch);
    return;
  }
  Batch &b = g_batches[batch];
  for (const Grid *g : b.grids)
    if (!rt->grids.count(const_cast<Grid *>(g))) {
      fail(PS_ERR_BAD_HANDLE, "PSBatchRun: the batch uses a freed grid");
      return;
    }
  if (batch_stale(b) && !batch_build(b)) return;
  const int M = b.maps_per_run;
  int i = 0;
  if (graphs_enabled() && iter > kGraphUnroll) {
    for (int p = 0; p < M; ++p)
      if (!batch_launch(b, p)) return;
    ++i;
    if (!b.graph) {
      cudaGraph_t graph = nullptr;
      const long long l0 = rt->launches;
      if (cudaStreamBeginCapture(rt->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        bool ok = true;
        for (int u = 0; u < kGraphUnroll && ok; ++u)
          for (int p = 0; p < M && ok; ++p) ok = batch_launch(b, p);
        if (cudaStreamEndCapture(rt->stream, &graph) == cudaSuccess && ok && graph &&
            cudaGraphInstantiate(&b.graph, graph, 0) != cudaSuccess)
          b.graph = nullptr;
        if (graph) cudaGraphDestroy(graph);
      }
      cudaGetLastError();
      b.graph_launches = rt->launches - l0;  // kernels in one replay
      rt->launches = l0;
    }
    if (b.graph) {
      for (; i + kGraphUnroll <= iter; i += kGraphUnroll) {
        if (!cuda_ok(cudaGraphLaunch(b.graph, rt->stream), "cudaGraphLaunch")) return;
        rt->launches += b.graph_launches;
      }
    }
  }
  for (; i < iter; ++i)
    for (int p = 0; p < M; ++p)
      if (!batch_launch(b, p)) return;
}

void PSSetBatchShape(int warps, int rows, int ns7, int nsp, int nsc) {
  if (!need_rt("PSSetBatchShape")) return;
  psg::BatchShape sh{warps, 4, ns7, nsp, nsc};
  if (warps < 1 || warps > 8 || !(rows == 1 || rows == 2 || rows == 4) || ns7 < 2 ||
      ns7 > 8 || nsp < 3 || nsp > 8 || nsc < 1 || nsc > 4 ||
      psg::batch_smem_bytes(sh, psg::kBatch7) > 227 * 1024 ||
      psg::batch_smem_bytes(sh, psg::kBatchHimeno) > 227 * 1024) {
    fail(PS_ERR_INVALID_ARGUMENT, "PSSetBatchShape: warps %d ns7 %d nsp %d nsc %d", warps,
         ns7, nsp, nsc);
    return;
  }
  g_batch_shape = sh;
  g_batch_rows = rows;
  for (Batch &b : g_batches) batch_release(b);  // rebuilt on the next run
}

void PSBatchFree(int batch) {
  if (!need_rt("PSBatchFree")) return;
  if (batch < 0 || batch >= (int)g_batches.size() || !g_batches[batch].live) {
    fail(PS_ERR_BAD_HANDLE, "PSBatchFree: %d is not a batch", batch);
    return;
  }
  cudaStreamSynchronize(rt->stream);
  batch_release(g_batches[batch]);
  g_batches[batch].live = false;
}

void PSSetAutotune(int on) {
  if (need_rt("PSSetAutotune")) rt->autotune = on != 0;
}

int PSLoadTuneCache(const char *path) {
  if (!need_rt("PSLoadTuneCache") || !path) return 0;
  return load_tuned(path);
}

void PSSetTuneCachePath(const char *path) {
  if (need_rt("PSSetTuneCachePath")) rt->tune_path = path ? path : "";
}

void PSClearTuning(void) {
  g_tuned.clear();
  g_tuning.clear();
  if (!rt) return;
  for (Map &m : rt->maps) m.has_plan = false;
}

int PSGetStencilPlan(PSStencil s, PSLaunchShape *shape, int *k, PSLaunchShape *tshape) {
  if (!need_rt("PSGetStencilPlan")) return 0;
  Map *m = lookup_map(s);
  if (!m) {
    fail(PS_ERR_BAD_HANDLE, "PSGetStencilPlan: %d is not a stencil", s);
    return 0;
  }
  const MarchConfig c = m->has_plan ? m->plan.shape : rt->shapes[shape_slot(m->kernel)];
  const MarchConfig t = m->has_plan ? m->plan.tshape : rt->tshapes[shape_slot(m->kernel)];
  if (shape) *shape = PSLaunchShape{c.warps, c.rows, c.ns, c.ns2, c.ctas_per_sm};
  if (tshape) *tshape = PSLaunchShape{t.warps, t.rows, t.ns, t.ns2, t.ctas_per_sm};
  if (k) *k = temporal_depth(*m);
  return m->has_plan ? 1 : 0;
}

void PSTestFailNextAllocs(int n) {
  if (need_rt("PSTestFailNextAllocs")) rt->fail_allocs = n;
}

void PSTestDeviceWaitTimeout(unsigned limit) {
  if (!need_rt("PSTestDeviceWaitTimeout")) return;
  if (cuda_ok(psg::launch_wait_timeout_probe(rt->dev_err, limit, rt->stream),
              "wait-timeout probe launch"))
    ++rt->launches;
}

}  // extern "C"
