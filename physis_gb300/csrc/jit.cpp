// Stencil functions compiled at run time (NVRTC) -- the translator-free
// front end.
//
// The reference turns a user stencil function such as
//     void kernel(const int x, const int y, const int z,
//                 PSGrid3DFloat g1, PSGrid3DFloat g2, float c) {
//       float v = PSGridGet(g1, x, y, z) + ... ;
//       PSGridEmit(g2, v * c);
//     }
// into a CUDA kernel with its source-to-source translator (physisc;
// translator/cuda_runtime_builder.cc:1099-1228 generates the run kernel, one
// thread per (x, y) and a loop over z; include/physis/physis_cuda.h:237-269
// the index arithmetic).  Here the function's own source text is compiled at
// run time: a short device prelude gives PSGridGet / PSGridGetPeriodic /
// PSGridEmit / PSGridDim and the PSGrid* types their device meaning, every
// unannotated function is a device function (-default-device), and a
// generated __global__ entry walks the domain and calls the function at each
// point.  Options --fmad=false and IEEE division/square root keep every
// float expression exactly as the C source writes it, so results match the
// REF target (the same source built by gcc with -ffp-contract=off) bit for
// bit.  NVRTC is loaded with dlopen; without it the entry points report
// PS_ERR_UNSUPPORTED.  The compiled image is loaded with the driver API into
// the runtime's context and never inspected.
#include <cuda.h>
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <regex>
#include <string>
#include <vector>

#include "ps_internal.h"
// kEmbedArith, kEmbedPointsBody: ps_arith.cuh and points_body.cuh as text
// (written into the build directory by buildlib.py).
#include "embedded_headers.inc"

#include <map>

namespace psg {
namespace {

// ---- NVRTC, resolved at run time -----------------------------------------
typedef int nvrtcResult_t;
typedef struct _nvrtcProgram *nvrtcProgram_t;
struct Nvrtc {
  bool tried = false, ok = false;
  nvrtcResult_t (*create)(nvrtcProgram_t *, const char *, const char *, int,
                          const char *const *, const char *const *) = nullptr;
  nvrtcResult_t (*compile)(nvrtcProgram_t, int, const char *const *) = nullptr;
  nvrtcResult_t (*log_size)(nvrtcProgram_t, size_t *) = nullptr;
  nvrtcResult_t (*log)(nvrtcProgram_t, char *) = nullptr;
  nvrtcResult_t (*cubin_size)(nvrtcProgram_t, size_t *) = nullptr;
  nvrtcResult_t (*cubin)(nvrtcProgram_t, char *) = nullptr;
  nvrtcResult_t (*destroy)(nvrtcProgram_t *) = nullptr;
};
Nvrtc g_nvrtc;

bool load_nvrtc(std::string *err) {
  if (g_nvrtc.tried) {
    if (!g_nvrtc.ok) *err = "NVRTC (libnvrtc.so) is not available";
    return g_nvrtc.ok;
  }
  g_nvrtc.tried = true;
  const char *names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                         "/usr/local/cuda/lib64/libnvrtc.so"};
  void *h = nullptr;
  for (const char *n : names)
    if ((h = dlopen(n, RTLD_NOW | RTLD_LOCAL))) break;
  if (!h) {
    *err = "NVRTC (libnvrtc.so) is not available";
    return false;
  }
#define PS_NVRTC_SYM(field, sym) \
  g_nvrtc.field = reinterpret_cast<decltype(g_nvrtc.field)>(dlsym(h, sym))
  PS_NVRTC_SYM(create, "nvrtcCreateProgram");
  PS_NVRTC_SYM(compile, "nvrtcCompileProgram");
  PS_NVRTC_SYM(log_size, "nvrtcGetProgramLogSize");
  PS_NVRTC_SYM(log, "nvrtcGetProgramLog");
  PS_NVRTC_SYM(cubin_size, "nvrtcGetCUBINSize");
  PS_NVRTC_SYM(cubin, "nvrtcGetCUBIN");
  PS_NVRTC_SYM(destroy, "nvrtcDestroyProgram");
#undef PS_NVRTC_SYM
  g_nvrtc.ok = g_nvrtc.create && g_nvrtc.compile && g_nvrtc.log_size && g_nvrtc.log &&
               g_nvrtc.cubin_size && g_nvrtc.cubin && g_nvrtc.destroy;
  if (!g_nvrtc.ok) *err = "libnvrtc.so lacks the expected entry points";
  return g_nvrtc.ok;
}

// ---- driver API, resolved through the runtime ------------------------------
struct Driver {
  bool tried = false, ok = false;
  CUresult (*load)(CUmodule *, const void *) = nullptr;
  CUresult (*get)(CUfunction *, CUmodule, const char *) = nullptr;
  CUresult (*launch)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                     unsigned, CUstream, void **, void **) = nullptr;
  CUresult (*unload)(CUmodule) = nullptr;
  CUresult (*set_attr)(CUfunction, CUfunction_attribute, int) = nullptr;
  CUresult (*occupancy)(int *, CUfunction, int, size_t) = nullptr;
  CUresult (*global)(CUdeviceptr *, size_t *, CUmodule, const char *) = nullptr;
};
Driver g_drv;

bool load_driver(std::string *err) {
  if (g_drv.tried) {
    if (!g_drv.ok) *err = "driver entry points for module loading are unavailable";
    return g_drv.ok;
  }
  g_drv.tried = true;
  auto sym = [](const char *name) -> void * {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    return fn;
  };
  g_drv.load = reinterpret_cast<decltype(g_drv.load)>(sym("cuModuleLoadData"));
  g_drv.get = reinterpret_cast<decltype(g_drv.get)>(sym("cuModuleGetFunction"));
  g_drv.launch = reinterpret_cast<decltype(g_drv.launch)>(sym("cuLaunchKernel"));
  g_drv.unload = reinterpret_cast<decltype(g_drv.unload)>(sym("cuModuleUnload"));
  g_drv.set_attr = reinterpret_cast<decltype(g_drv.set_attr)>(sym("cuFuncSetAttribute"));
  g_drv.occupancy = reinterpret_cast<decltype(g_drv.occupancy)>(
      sym("cuOccupancyMaxActiveBlocksPerMultiprocessor"));
  g_drv.global = reinterpret_cast<decltype(g_drv.global)>(sym("cuModuleGetGlobal"));
  g_drv.ok = g_drv.load && g_drv.get && g_drv.launch && g_drv.unload && g_drv.set_attr &&
             g_drv.occupancy && g_drv.global;
  if (!g_drv.ok) {
    cudaGetLastError();
    *err = "driver entry points for module loading are unavailable";
  }
  return g_drv.ok;
}

// ---- the device prelude -----------------------------------------------------
// PSGrid{1,2,3}D{Float,Double,Int,Long} are one device struct per element
// type; `cur` is the element the map's current point emits to.  Index
// arithmetic as the reference's (physis_cuda.h:237-269): x fastest, periodic
// reads wrap with (i + n) % n.
const char *kPrelude = R"PSJIT(
#include "ps_arith.cuh"
typedef int PSIndex;
// Kernel parameter (host layout: GridArg in jit.cpp).
template <typename T> struct __PSGridArg {
  T *p; long long row; long long plane; int nx; int ny; int nz; int rank; long long cur;
};
// What the stencil function sees.  For a grid the tiled entry staged in
// shared memory (staged == 1) the entry also records the cell being computed
// (cx, cy, cz) and, for each plane offset d within rz, a pointer c[d + 4] to
// that cell's position in the staged plane z + d; a read at (cx + dx, cy +
// dy, cz + dz) with |dx| <= rx, |dy| <= ry, |dz| <= rz is then
// c[dz + 4][dy * sw + dx].  With the function inlined, reads written as x +
// const make every test and index a constant; any other read is tested at
// run time and falls back to global memory outside the window.
template <typename T> struct __PSGridDev {
  T *p; long long row; long long plane; int nx; int ny; int nz; int rank; long long cur;
  int staged, rx, ry, rz, sw, cx, cy, cz;
  const T *c[9];
};
template <typename T> __device__ __forceinline__ __PSGridDev<T> __ps_dev(const __PSGridArg<T> &a) {
  __PSGridDev<T> g;
  g.p = a.p; g.row = a.row; g.plane = a.plane; g.nx = a.nx; g.ny = a.ny; g.nz = a.nz;
  g.rank = a.rank; g.cur = 0; g.staged = 0;
  return g;
}
#define __PS_GRID_TYPES(N, T) \
  typedef __PSGridDev<T> PSGrid1D##N; typedef __PSGridDev<T> PSGrid2D##N; \
  typedef __PSGridDev<T> PSGrid3D##N;
__PS_GRID_TYPES(Float, float)
__PS_GRID_TYPES(Double, double)
__PS_GRID_TYPES(Int, int)
__PS_GRID_TYPES(Long, long long)
template <typename T>
__device__ __forceinline__ bool __ps_in_stage(const __PSGridDev<T> &g, int x, int y, int z) {
  const int dx = x - g.cx, dy = y - g.cy, dz = z - g.cz;
  return g.staged && dx >= -g.rx && dx <= g.rx && dy >= -g.ry && dy <= g.ry && dz >= -g.rz &&
         dz <= g.rz;
}
template <typename T>
__device__ __forceinline__ T __ps_staged(const __PSGridDev<T> &g, int x, int y, int z) {
  return g.c[z - g.cz + 4][(y - g.cy) * g.sw + (x - g.cx)];
}
template <typename T> __device__ __forceinline__ T __ps_get(const __PSGridDev<T> &g, int x) {
  return g.p[x];
}
template <typename T> __device__ __forceinline__ T __ps_get(const __PSGridDev<T> &g, int x, int y) {
  return g.p[(long long)y * g.row + x];
}
template <typename T>
__device__ __forceinline__ T __ps_get(const __PSGridDev<T> &g, int x, int y, int z) {
  if (__ps_in_stage(g, x, y, z)) return __ps_staged(g, x, y, z);
  return g.p[(long long)z * g.plane + (long long)y * g.row + x];
}
template <typename T> __device__ __forceinline__ T __ps_getp(const __PSGridDev<T> &g, int x) {
  return g.p[(x + g.nx) % g.nx];
}
template <typename T>
__device__ __forceinline__ T __ps_getp(const __PSGridDev<T> &g, int x, int y) {
  return g.p[(long long)((y + g.ny) % g.ny) * g.row + (x + g.nx) % g.nx];
}
// Staged windows of periodic grids hold the wrapped values at the unwrapped
// coordinates, so the window is looked up before wrapping.
template <typename T>
__device__ __forceinline__ T __ps_getp(const __PSGridDev<T> &g, int x, int y, int z) {
  if (__ps_in_stage(g, x, y, z)) return __ps_staged(g, x, y, z);
  return g.p[(long long)((z + g.nz) % g.nz) * g.plane + (long long)((y + g.ny) % g.ny) * g.row +
             (x + g.nx) % g.nx];
}
template <typename T> __device__ __forceinline__ int __ps_dim(const __PSGridDev<T> &g, int d) {
  return d == 0 ? g.nx : (d == 1 ? g.ny : g.nz);
}
// Grids of a user-defined element type: the source's own struct definition
// and DeclareGrid line; PSGridEmitUtype(g.m, v) reaches __PS_EMITU as
// __PS_EMITU((g).p[(g).cur].m, v) (the front end rewrites the call), i.e. a
// store to member m of the point being computed.
#define DeclareGrid1D(N, T) typedef __PSGridDev<T> PSGrid1D##N
#define DeclareGrid2D(N, T) typedef __PSGridDev<T> PSGrid2D##N
#define DeclareGrid3D(N, T) typedef __PSGridDev<T> PSGrid3D##N
#define __PS_EMITU(lhs, v) ((void)((lhs) = (v)))
#define PSGridGet(g, ...) __ps_get((g), __VA_ARGS__)
#define PSGridGetPeriodic(g, ...) __ps_getp((g), __VA_ARGS__)
#define PSGridEmit(g, v) ((void)((g).p[(g).cur] = (v)))
#define PSGridDim(g, d) __ps_dim((g), (d))

// ---- staging for the tiled entry ----
template <int S> __device__ __forceinline__ int __ps_slot(int z) { return ((z % S) + S) % S; }
template <bool PER> __device__ __forceinline__ int __ps_fit(int v, int n) {
  if (PER) {
    if ((unsigned)v >= (unsigned)n) {
      v %= n;
      if (v < 0) v += n;
    }
    return v;
  }
  return min(max(v, 0), n - 1);
}
// Plane zp (unwrapped) of the W x H window at (x0 - RX, y0 - RY) into its
// ring slot.  vec (the CTA's window lies inside the grid in x and every
// window row starts on a 16-byte boundary): 16-byte cp.async chunks, rows
// clamped or wrapped in y.  Otherwise one cp.async per cell, warp w copying
// rows w, w + 8, ..., cells outside the grid wrapped (PER) or clamped.
template <typename T, int W, int H, int S, int RX, int RY, bool PER>
__device__ __forceinline__ void __ps_stage(T *ring, const __PSGridArg<T> &a, int x0, int y0,
                                           bool vec, int zp) {
  T *dst = ring + __ps_slot<S>(zp) * (W * H);
  const T *src = a.p + (long long)__ps_fit<PER>(zp, a.nz) * a.plane;
  if (vec) {
    constexpr int V = 16 / (int)sizeof(T), NV = W / V;
    for (int e = threadIdx.x; e < NV * H; e += 256) {
      const int r = e / NV, c = e - r * NV;
      const T *srow = src + (long long)__ps_fit<PER>(y0 - RY + r, a.ny) * a.row + (x0 - RX);
      psg::cp_async16(dst + r * W + c * V, srow + c * V);
    }
    return;
  }
  const int lane = threadIdx.x & 31;
  for (int r = threadIdx.x >> 5; r < H; r += 8) {
    const T *srow = src + (long long)__ps_fit<PER>(y0 - RY + r, a.ny) * a.row;
    T *drow = dst + r * W;
#pragma unroll
    for (int c = lane; c < W; c += 32)
      psg::cp_async_small<(int)sizeof(T)>(drow + c, srow + __ps_fit<PER>(x0 - RX + c, a.nx));
  }
}
// Whether a window of width W at x0 - RX can be staged in 16-byte chunks.
template <typename T, int W, int RX>
__device__ __forceinline__ bool __ps_vec_ok(const __PSGridArg<T> &a, int x0) {
  const T *row0 = a.p + (x0 - RX);
  return x0 - RX >= 0 && x0 - RX + W <= a.nx &&
         ((unsigned long long)row0 & 15) == 0 && ((a.row * (long long)sizeof(T)) & 15) == 0;
}
)PSJIT";

// Host mirror of __PSGridDev<T> (same layout for every T: one pointer).
struct GridArg {
  void *p;
  long long row, plane;
  int nx, ny, nz, rank;
  long long cur;
};

std::string trim(const std::string &s) {
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// User grid types the source declares: "PSGrid3DPoint" -> (3, "struct Point").
typedef std::map<std::string, std::pair<int, std::string>> UserGrids;

UserGrids declared_grids(const std::string &src) {
  UserGrids out;
  static const std::regex re("\\bDeclareGrid([123])D\\s*\\(\\s*(\\w+)\\s*,\\s*([^)]*?)\\s*\\)");
  for (auto it = std::sregex_iterator(src.begin(), src.end(), re); it != std::sregex_iterator();
       ++it) {
    const int rank = (*it)[1].str()[0] - '0';
    out["PSGrid" + (*it)[1].str() + "D" + (*it)[2].str()] = {rank, trim((*it)[3].str())};
  }
  return out;
}

// Parses one parameter declaration ("const int x", "PSGrid3DFloat g1",
// "float c") into p; false if its type is not one the front end knows.
bool parse_param(const std::string &decl, JitParam *p, std::string *err,
                 const UserGrids &user = UserGrids()) {
  static const std::regex grid_re("^PSGrid([123])D(Float|Double|Int|Long)$");
  std::string d = " " + trim(decl) + " ";
  for (const char *q : {" const ", " register ", " volatile "}) {
    size_t at;
    while ((at = d.find(q)) != std::string::npos) d.replace(at, strlen(q) - 1, "");
  }
  d = trim(d);
  const size_t cut = d.find_last_of(" \t*&");
  if (cut == std::string::npos) {
    *err = "parameter '" + trim(decl) + "' has no name";
    return false;
  }
  std::string type = trim(d.substr(0, cut));
  std::string t;  // type with single spaces
  for (char c : type)
    if (!(c == ' ' && (t.empty() || t.back() == ' '))) t += (c == '\t' ? ' ' : c);
  type = trim(t);
  p->decl_type = type;
  p->name = trim(d.substr(cut + 1));
  std::smatch m;
  const auto u = user.find(type);
  if (u != user.end()) {
    p->grid = true;
    p->rank = u->second.first;
    p->type = kUser;
    p->utype = u->second.second;
    return true;
  }
  if (std::regex_match(type, m, grid_re)) {
    p->grid = true;
    p->rank = m[1].str()[0] - '0';
    const std::string e = m[2].str();
    p->type = e == "Float" ? kFloat : e == "Double" ? kDouble : e == "Int" ? kInt : kLong;
    return true;
  }
  p->grid = false;
  p->rank = 0;
  if (type == "int" || type == "PSIndex" || type == "signed int") p->type = kInt;
  else if (type == "long" || type == "long int" || type == "long long" ||
           type == "long long int")
    p->type = kLong;
  else if (type == "float") p->type = kFloat;
  else if (type == "double") p->type = kDouble;
  else {
    *err = "parameter type '" + type + "' is not supported (grids PSGrid{1,2,3}D{Float,"
           "Double,Int,Long}, scalars int/long/float/double)";
    return false;
  }
  return true;
}

// Finds `void name(...)` in src and parses its parameters.
bool parse_signature(const std::string &src, const std::string &name, JitKernel *k,
                     std::string *err) {
  const std::regex head("\\bvoid\\s+" + name + "\\s*\\(");
  std::smatch m;
  if (!std::regex_search(src, m, head)) {
    *err = "no definition 'void " + name + "(...)' in the stencil source";
    return false;
  }
  size_t i = m.position(0) + m.length(0);
  int depth = 1;
  std::string cur;
  std::vector<std::string> decls;
  for (; i < src.size() && depth > 0; ++i) {
    const char c = src[i];
    if (c == '(') ++depth;
    if (c == ')' && --depth == 0) break;
    if (c == ',' && depth == 1) {
      decls.push_back(cur);
      cur.clear();
    } else {
      cur += c;
    }
  }
  if (depth != 0) {
    *err = "unbalanced parameter list of " + name;
    return false;
  }
  if (!trim(cur).empty()) decls.push_back(cur);
  k->params.clear();
  k->nd = 0;
  bool seen_grid = false;
  const UserGrids user = declared_grids(src);
  for (const std::string &d : decls) {
    JitParam p;
    if (!parse_param(d, &p, err, user)) return false;
    if (!p.grid && !seen_grid && p.type == kInt && k->params.empty() && k->nd < 3) {
      k->idx[k->nd++] = p.name;  // a leading index parameter
      continue;
    }
    if (p.grid) seen_grid = true;
    if (!p.grid && !seen_grid) {
      *err = "stencil " + name + ": index parameters must come first, then the grids";
      return false;
    }
    k->params.push_back(p);
  }
  if (k->nd < 1) {
    *err = "stencil " + name + " has no index parameters (const int x[, y[, z]])";
    return false;
  }
  k->ngrids = k->nscalars = 0;
  for (const JitParam &p : k->params) (p.grid ? k->ngrids : k->nscalars)++;
  if (k->ngrids < 1) {
    *err = "stencil " + name + " takes no grid";
    return false;
  }
  return true;
}

std::string scalar_ctype(int type) {
  switch (type) {
    case kInt: return "int";
    case kLong: return "long long";
    case kFloat: return "float";
    default: return "double";
  }
}

// A grid parameter's element type in generated code.
std::string elem_ctype(const JitParam &p) {
  return p.type == kUser ? p.utype : scalar_ctype(p.type);
}

// Source expression of the grid argument arg in an entry: the device view
// g<i> the entry built from kernel parameter a<i>.
std::string cur_expr(const JitParam &p, const std::string &g) {
  return p.rank == 1 ? std::string("x")
         : p.rank == 2 ? "(long long)y * " + g + ".row + x"
                       : "(long long)z * " + g + ".plane + (long long)y * " + g + ".row + x";
}

std::string entry_params(const JitKernel &k) {
  std::string s;
  for (size_t i = 0; i < k.params.size(); ++i) {
    const JitParam &p = k.params[i];
    s += ", " + (p.grid ? "__PSGridArg<" + elem_ctype(p) + ">" : scalar_ctype(p.type)) +
         " a" + std::to_string(i);
  }
  return s;
}

std::string call_source(const JitKernel &k) {
  std::string s = k.name + "(x";
  if (k.nd >= 2) s += ", y";
  if (k.nd >= 3) s += ", z";
  for (size_t i = 0; i < k.params.size(); ++i)
    s += (k.params[i].grid ? ", g" : ", a") + std::to_string(i);
  return s + ");\n";
}

// The generated entry: one thread per (x, y), a z-chunk per block row in z;
// red/black maps visit every other x from the REF start
// min + ((min & 1) ^ ((y + z + color) % 2))
// (translator/reference_runtime_builder.cc:585-600).
std::string entry_source(const JitKernel &k) {
  std::string s =
      "\nextern \"C\" __global__ void __launch_bounds__(256) __ps_entry(int dmin0, int dmax0, "
      "int dmin1, int dmax1, int dmin2, int dmax2, int color, int zlen" +
      entry_params(k) + ") {\n";
  for (size_t i = 0; i < k.params.size(); ++i)
    if (k.params[i].grid)
      s += "  auto g" + std::to_string(i) + " = __ps_dev(a" + std::to_string(i) + ");\n";
  s += "  const int tx = blockIdx.x * blockDim.x + threadIdx.x;\n"
       "  const int y = dmin1 + blockIdx.y * blockDim.y + threadIdx.y;\n"
       "  if (y >= dmax1) return;\n"
       "  const int zs = dmin2 + blockIdx.z * zlen;\n"
       "  const int ze = min(zs + zlen, dmax2);\n"
       "  for (int z = zs; z < ze; ++z) {\n"
       "    const int x = color < 0 ? dmin0 + tx\n"
       "        : dmin0 + ((dmin0 & 1) ^ ((y + z + color) % 2)) + 2 * tx;\n"
       "    if (x >= dmax0) continue;\n";
  for (size_t i = 0; i < k.params.size(); ++i) {
    if (!k.params[i].grid) continue;
    const std::string g = "g" + std::to_string(i);
    s += "    " + g + ".cur = " + cur_expr(k.params[i], g) + ";\n";
  }
  s += "    " + call_source(k) + "  }\n}\n";
  return s;
}

// ---- the tiled entry ---------------------------------------------------------
// A CTA of 256 threads owns a 64 x 16 (x, y) tile and a chunk of z.  Grids
// the stencil reads at neighbour offsets (and never emits to) are staged:
// each z step copies one plane of the tile plus halo into a ring of
// shared-memory planes with cp.async, kAhead planes ahead of the compute, and
// the function's reads inside the window come from there.  The reads themselves
// are unchanged, so every result is bit-identical to the plain entry's.
constexpr int kTileX = 64, kTileY = 16;
constexpr int kAhead = 3;                   // planes in flight ahead of the compute
constexpr size_t kStageBudget = 96 * 1024;  // two or more CTAs per SM

// Ring planes of a grid staged with z halo rz: the 2 rz + 1 planes a step
// reads, kAhead in flight, and one more so that a plane is never refilled
// while a thread still one step behind reads it.
int ring_planes(int rz) { return 2 * rz + 2 + kAhead; }

// Splits the argument list of the call whose '(' is at src[open] into its
// top-level arguments; npos-safe (returns false if unbalanced).
bool call_args(const std::string &src, size_t open, std::vector<std::string> *args,
               size_t *close) {
  int depth = 0;
  std::string cur;
  for (size_t i = open; i < src.size(); ++i) {
    const char c = src[i];
    if (c == '(' || c == '[' || c == '{') {
      if (depth++ > 0) cur += c;
      continue;
    }
    if (c == ')' || c == ']' || c == '}') {
      if (--depth == 0) {
        args->push_back(cur);
        *close = i;
        return true;
      }
      cur += c;
      continue;
    }
    if (c == ',' && depth == 1) {
      args->push_back(cur);
      cur.clear();
      continue;
    }
    cur += c;
  }
  return false;
}

// Chooses the staged grids of a 3D stencil from its source text.  A grid is
// staged when some PSGridGet / PSGridGetPeriodic of it reads off the centre
// and no PSGridEmit anywhere in the source names it.  A coordinate written
// as `x`, `x + c` or `x - c` (x the index parameter of that axis, c a
// literal) widens the halo to c; any other coordinate expression widens it to
// at least 1.  Halos are capped at 4: the window test in the accessors sends
// any read outside the staged window to global memory, so the choice affects
// speed only, never results.
void choose_stages(JitKernel *k) {
  k->stages.clear();
  k->stage_smem = 0;
  if (k->nd != 3) return;
  const std::string &src = k->source;
  std::vector<std::string> emitted;
  {
    const std::regex emit_re("\\bPSGridEmit(?:Utype)?\\s*\\(\\s*(\\w+)");
    for (auto it = std::sregex_iterator(src.begin(), src.end(), emit_re);
         it != std::sregex_iterator(); ++it)
      emitted.push_back((*it)[1].str());
  }
  const std::regex get_re("\\bPSGridGet(Periodic)?\\s*\\(");
  for (size_t pi = 0; pi < k->params.size(); ++pi) {
    const JitParam &p = k->params[pi];
    if (!p.grid || p.rank != 3 || p.type == kUser) continue;
    bool is_emitted = false;
    for (const std::string &e : emitted) is_emitted |= (e == p.name);
    if (is_emitted) continue;
    int r[3] = {0, 0, 0};
    bool off_centre = false, periodic = false;
    for (auto it = std::sregex_iterator(src.begin(), src.end(), get_re);
         it != std::sregex_iterator(); ++it) {
      const size_t open = it->position(0) + it->length(0) - 1;
      std::vector<std::string> args;
      size_t close = 0;
      if (!call_args(src, open, &args, &close) || args.size() != 4 || trim(args[0]) != p.name)
        continue;
      if ((*it)[1].matched) periodic = true;
      for (int d = 0; d < 3; ++d) {
        std::smatch m;
        const std::string a = trim(args[d + 1]);
        static const std::regex lit_re("^(\\w+)\\s*(?:([+-])\\s*([0-9]+))?$");
        if (std::regex_match(a, m, lit_re) && m[1].str() == k->idx[d]) {
          const int c = m[3].matched ? std::atoi(m[3].str().c_str()) : 0;
          if (c) off_centre = true;
          r[d] = std::max(r[d], std::min(c, 4));
        } else {
          off_centre = true;
          r[d] = std::max(r[d], 1);
        }
      }
    }
    if (!off_centre) continue;
    JitStage st;
    st.param = (int)pi;
    st.rx = r[0];
    st.ry = r[1];
    st.rz = r[2];
    st.periodic = periodic;
    st.esz = (p.type == kFloat || p.type == kInt) ? 4 : 8;
    const int v = 16 / st.esz;  // the window's x halo: rx rounded up to 16 bytes
    st.rxw = (st.rx + v - 1) / v * v;
    st.bytes = (size_t)ring_planes(st.rz) * (kTileX + 2 * st.rxw) * (kTileY + 2 * st.ry) * st.esz;
    st.bytes = (st.bytes + 15) / 16 * 16;
    if (k->stage_smem + st.bytes > kStageBudget) continue;
    st.off = k->stage_smem;
    k->stage_smem += st.bytes;
    k->stages.push_back(st);
  }
}

std::string tiled_entry_source(const JitKernel &k) {
  std::string s =
      "\nextern \"C\" __global__ void __launch_bounds__(256) __ps_entry_t(int dmin0, int dmax0, "
      "int dmin1, int dmax1, int dmin2, int dmax2, int ntx, int zlen" +
      entry_params(k) + ") {\n"
      "  extern __shared__ __align__(16) unsigned char __ps_sm[];\n"
      "  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;\n"
      "  const int x0 = dmin0 + (int)(blockIdx.x % (unsigned)ntx) * " + std::to_string(kTileX) +
      ";\n"
      "  const int y0 = dmin1 + (int)(blockIdx.x / (unsigned)ntx) * " + std::to_string(kTileY) +
      ";\n"
      "  const int zs = dmin2 + (int)blockIdx.y * zlen;\n"
      "  const int ze = min(zs + zlen, dmax2);\n"
      "  if (zs >= ze) return;\n";
  for (size_t i = 0; i < k.params.size(); ++i)
    if (k.params[i].grid)
      s += "  auto g" + std::to_string(i) + " = __ps_dev(a" + std::to_string(i) + ");\n";
  // prologue: the planes step zs reads (one commit group), then the planes
  // ahead of it one group each; step z adds plane z + rz + kAhead and waits
  // until at most kAhead groups are pending, i.e. plane z + rz has landed.
  std::string first, ahead, next;
  for (size_t j = 0; j < k.stages.size(); ++j) {
    const JitStage &st = k.stages[j];
    const std::string i = std::to_string(st.param), sj = std::to_string(j);
    const std::string T = scalar_ctype(k.params[st.param].type);
    const int W = kTileX + 2 * st.rxw, H = kTileY + 2 * st.ry, S = ring_planes(st.rz);
    const std::string rz = std::to_string(st.rz), vj = "v" + sj;
    const std::string stage = "__ps_stage<" + T + ", " + std::to_string(W) + ", " +
                              std::to_string(H) + ", " + std::to_string(S) + ", " +
                              std::to_string(st.rxw) + ", " + std::to_string(st.ry) + ", " +
                              (st.periodic ? "true" : "false") + ">(s" + sj + ", a" + i +
                              ", x0, y0, " + vj + ", ";
    s += "  " + T + " *s" + sj + " = reinterpret_cast<" + T + " *>(__ps_sm + " +
         std::to_string(st.off) + ");\n";
    s += "  const bool " + vj + " = __ps_vec_ok<" + T + ", " + std::to_string(W) + ", " +
         std::to_string(st.rxw) + ">(a" + i + ", x0);\n";
    s += "  g" + i + ".staged = 1; g" + i + ".rx = " + std::to_string(st.rxw) + "; g" + i +
         ".ry = " + std::to_string(st.ry) + "; g" + i + ".rz = " + rz + "; g" + i + ".sw = " +
         std::to_string(W) + ";\n";
    first += "  for (int d = -" + rz + "; d <= " + rz + "; ++d) " + stage + "zs + d);\n";
    ahead += "    if (zs + a < ze) " + stage + "zs + " + rz + " + a);\n";
    next += "      " + stage + "z + " + rz + " + " + std::to_string(kAhead) + ");\n";
  }
  s += first + "  psg::cp_async_commit();\n";
  s += "  for (int a = 1; a < " + std::to_string(kAhead) + "; ++a) {\n" + ahead +
       "    psg::cp_async_commit();\n  }\n";
  s += "  for (int z = zs; z < ze; ++z) {\n"
       "    if (z + " + std::to_string(kAhead) + " < ze) {\n" + next + "    }\n"
       "    psg::cp_async_commit();\n"
       "    psg::cp_async_wait<" + std::to_string(kAhead) + ">();\n"
       "    __syncthreads();\n";
  // per step: each staged grid's plane pointers; per cell: the cell's
  // coordinates and its position in those planes
  std::string cell;
  for (size_t j = 0; j < k.stages.size(); ++j) {
    const JitStage &st = k.stages[j];
    const std::string g = "g" + std::to_string(st.param), sj = std::to_string(j);
    const int W = kTileX + 2 * st.rxw, S = ring_planes(st.rz);
    const std::string rz = std::to_string(st.rz);
    s += "    const " + scalar_ctype(k.params[st.param].type) + " *pl" + sj + "[9];\n";
    s += "    for (int d = -" + rz + "; d <= " + rz + "; ++d) pl" + sj + "[d + 4] = s" + sj +
         " + __ps_slot<" + std::to_string(S) + ">(z + d) * " +
         std::to_string(W * (kTileY + 2 * st.ry)) + ";\n";
    cell += "          " + g + ".cx = x; " + g + ".cy = y; " + g + ".cz = z;\n";
    cell += "          for (int d = -" + rz + "; d <= " + rz + "; ++d) " + g + ".c[d + 4] = pl" +
            sj + "[d + 4] + (y - y0 + " + std::to_string(st.ry) + ") * " + std::to_string(W) +
            " + (x - x0 + " + std::to_string(st.rxw) + ");\n";
  }
  s += "#pragma unroll\n"
       "    for (int jy = 0; jy < " + std::to_string(kTileY / 8) + "; ++jy) {\n"
       "      const int y = y0 + warp + 8 * jy;\n"
       "#pragma unroll\n"
       "      for (int jx = 0; jx < " + std::to_string(kTileX / 32) + "; ++jx) {\n"
       "        const int x = x0 + lane + 32 * jx;\n"
       "        if (x < dmax0 && y < dmax1) {\n" + cell;
  for (size_t i = 0; i < k.params.size(); ++i) {
    if (!k.params[i].grid) continue;
    const std::string g = "g" + std::to_string(i);
    s += "          " + g + ".cur = " + cur_expr(k.params[i], g) + ";\n";
  }
  s += "          " + call_source(k) + "        }\n      }\n    }\n  }\n"
       "  psg::cp_async_wait<0>();\n}\n";
  return s;
}

}  // namespace

namespace {

// PSGridEmitUtype(g.member, v) -> __PS_EMITU((g).p[(g).cur].member, v): the
// member expression is applied to the point being computed.
std::string rewrite_emit_utype(const std::string &src) {
  static const std::regex re("\\bPSGridEmitUtype\\s*\\(\\s*([A-Za-z_]\\w*)");
  return std::regex_replace(src, re, "__PS_EMITU(($1).p[($1).cur]");
}

// One device global per user-type grid parameter holding its element size,
// read back after loading to check the grids a map passes.
std::string utype_sizes_source(const JitKernel &k) {
  std::string s;
  for (size_t i = 0; i < k.params.size(); ++i)
    if (k.params[i].grid && k.params[i].type == kUser)
      s += "extern \"C\" __device__ const int __ps_esz" + std::to_string(i) +
           " = (int)sizeof(" + k.params[i].utype + ");\n";
  return s;
}

// Compiles one program text for sm_103a (headers: ps_arith.cuh).
bool nvrtc_compile(const std::string &program, std::vector<char> *image, std::string *log) {
  nvrtcProgram_t prog = nullptr;
  const char *hdr_src[] = {kEmbedArith};
  const char *hdr_name[] = {"ps_arith.cuh"};
  if (g_nvrtc.create(&prog, program.c_str(), "stencil.cu", 1, hdr_src, hdr_name) != 0) {
    *log = "nvrtcCreateProgram failed";
    return false;
  }
  const char *opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "--fmad=false",
                        "--prec-div=true", "--prec-sqrt=true", "--ftz=false",
                        "--device-as-default-execution-space", "-DPS_JIT=1"};
  const int rc = g_nvrtc.compile(prog, (int)(sizeof(opts) / sizeof(opts[0])), opts);
  if (rc != 0) {
    size_t n = 0;
    g_nvrtc.log_size(prog, &n);
    log->assign(n, '\0');
    if (n) g_nvrtc.log(prog, &(*log)[0]);
    g_nvrtc.destroy(&prog);
    return false;
  }
  size_t n = 0;
  g_nvrtc.cubin_size(prog, &n);
  image->resize(n);
  g_nvrtc.cubin(prog, image->data());
  g_nvrtc.destroy(&prog);
  return true;
}

}  // namespace

bool jit_build(const char *source, const char *name, JitKernel *k, std::vector<char> *image,
               std::string *err) {
  if (!load_nvrtc(err)) return false;
  k->name = name;
  k->source = source;
  if (!parse_signature(k->source, k->name, k, err)) return false;
  choose_stages(k);
  const std::string base = std::string(kPrelude) + "#line 1 \"stencil\"\n" +
                           rewrite_emit_utype(k->source) + "\n" + entry_source(*k) +
                           utype_sizes_source(*k);
  std::string log;
  // PS_JIT_DUMP=<dir> writes the generated program to <dir>/<name>.cu (for
  // building it offline with nvcc to read its resource usage).
  if (const char *dir = getenv("PS_JIT_DUMP")) {
    const std::string path = std::string(dir) + "/" + k->name + ".cu";
    if (FILE *f = fopen(path.c_str(), "w")) {
      const std::string text = base + (k->stages.empty() ? "" : tiled_entry_source(*k));
      fwrite(text.data(), 1, text.size(), f);
      fclose(f);
    }
  }
  // Both entries in one program; should the tiled one not compile, the plain
  // entry alone (the stencil then runs untiled).
  if (!k->stages.empty() && nvrtc_compile(base + tiled_entry_source(*k), image, &log))
    return true;
  k->stages.clear();
  k->stage_smem = 0;
  if (nvrtc_compile(base, image, &log)) return true;
  *err = "stencil " + k->name + " does not compile: " + log.substr(0, 600);
  return false;
}

bool jit_compile(const char *source, const char *name, JitKernel *k, std::string *err) {
  std::vector<char> image;
  if (!jit_build(source, name, k, &image, err) || !load_driver(err)) return false;
  CUmodule mod = nullptr;
  CUfunction fn = nullptr, fn_t = nullptr;
  if (g_drv.load(&mod, image.data()) != CUDA_SUCCESS) {
    *err = "loading the compiled stencil failed";
    return false;
  }
  if (g_drv.get(&fn, mod, "__ps_entry") != CUDA_SUCCESS) {
    g_drv.unload(mod);
    *err = "compiled stencil has no entry";
    return false;
  }
  if (!k->stages.empty()) {
    if (g_drv.get(&fn_t, mod, "__ps_entry_t") != CUDA_SUCCESS ||
        g_drv.set_attr(fn_t, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES,
                       (int)k->stage_smem) != CUDA_SUCCESS) {
      fn_t = nullptr;
      k->stages.clear();
      k->stage_smem = 0;
    }
  }
  k->tiled_occ = 0;
  if (fn_t && (g_drv.occupancy(&k->tiled_occ, fn_t, 256, k->stage_smem) != CUDA_SUCCESS ||
               k->tiled_occ < 1)) {
    k->tiled_occ = 0;
    fn_t = nullptr;
  }
  // element sizes of the user-type grid parameters, as the compiler laid
  // the structs out
  for (size_t i = 0; i < k->params.size(); ++i) {
    JitParam &p = k->params[i];
    if (!p.grid || p.type != kUser) continue;
    CUdeviceptr dptr = 0;
    size_t bytes = 0;
    int esz = 0;
    const std::string sym = "__ps_esz" + std::to_string(i);
    if (g_drv.global(&dptr, &bytes, mod, sym.c_str()) != CUDA_SUCCESS || bytes != sizeof(int) ||
        cudaMemcpy(&esz, reinterpret_cast<void *>(dptr), sizeof(int), cudaMemcpyDeviceToHost) !=
            cudaSuccess) {
      cudaGetLastError();
      g_drv.unload(mod);
      *err = "cannot read the element size of " + p.utype;
      return false;
    }
    p.esz = esz;
  }
  k->module = mod;
  k->func = fn;
  k->func_tiled = fn_t;
  return true;
}

void jit_unload(JitKernel *k) {
  if (k->module && g_drv.unload) g_drv.unload(static_cast<CUmodule>(k->module));
  k->module = k->func = k->func_tiled = nullptr;
}

namespace {

// PS_FUNCTION_TILED=0 runs every map on the plain entry (read per launch).
bool tiled_enabled() {
  const char *e = getenv("PS_FUNCTION_TILED");
  return !(e && e[0] == '0');
}

}  // namespace

// The tiled entry runs every-point maps of stencils with staged grids when
// no staged grid shares its memory with another grid argument (a staged copy
// of a grid that the same launch writes would be stale); red/black maps and
// everything else run the plain entry.
cudaError_t jit_launch(const JitKernel &k, const Box &dom, int color, const GridView *grids,
                       const double *scalars, int sm_count, cudaStream_t s) {
  const int nxd = dom.max[0] - dom.min[0], nyd = dom.max[1] - dom.min[1],
            nzd = dom.max[2] - dom.min[2];
  if (nxd <= 0 || nyd <= 0 || nzd <= 0) return cudaSuccess;
  bool tiled = k.func_tiled && color < 0 && tiled_enabled() && k.tiled_occ > 0;
  for (const JitStage &st : k.stages) {
    int gi = 0, sgi = -1;
    for (size_t i = 0; i < k.params.size(); ++i)
      if (k.params[i].grid) {
        if ((int)i == st.param) sgi = gi;
        ++gi;
      }
    for (int j = 0; j < gi && tiled; ++j)
      if (j != sgi && grids[j].ptr == grids[sgi].ptr) tiled = false;
  }
  unsigned gx, gy, gz, bx, by;
  int head[8];
  if (tiled) {
    const long long ntx = (nxd + kTileX - 1) / kTileX, nty = (nyd + kTileY - 1) / kTileY;
    const long long tiles = ntx * nty;
    // z chunks: the count whose waves of resident CTAs finish with the least
    // idle time, counting each chunk's warm-up planes (2 rz + kAhead) as work
    const long long want = std::max(1LL, (long long)k.tiled_occ * sm_count);
    int ovh = kAhead;
    for (const JitStage &st : k.stages) ovh = std::max(ovh, 2 * st.rz + kAhead);
    const long long c0 = std::max(1LL, (want + tiles - 1) / tiles);
    const long long cmax = std::max(1LL, std::min(16 * c0, (long long)(nzd + 7) / 8));
    long long chunks = 1;
    int zlen = nzd;
    double best = -1.0;
    for (long long c = std::min(c0, cmax); c <= cmax; ++c) {
      const int zl = (int)((nzd + c - 1) / c);
      const long long cc = (nzd + zl - 1) / zl;
      const long long waves = (tiles * cc + want - 1) / want;
      const double eff = (double)tiles * nzd / ((double)want * waves * (zl + ovh));
      if (eff > best + 1e-9) {
        best = eff;
        chunks = cc;
        zlen = zl;
      }
    }
    if (tiles > 0x7fffffffLL || chunks > 65535) return cudaErrorInvalidConfiguration;
    gx = (unsigned)tiles;
    gy = (unsigned)chunks;
    gz = 1;
    bx = 256;
    by = 1;
    const int h[8] = {dom.min[0], dom.max[0], dom.min[1], dom.max[1],
                      dom.min[2], dom.max[2], (int)ntx, zlen};
    memcpy(head, h, sizeof(h));
  } else {
    bx = 64;
    by = 4;
    const int xs = color < 0 ? nxd : (nxd + 1) / 2;
    gx = (unsigned)((xs + bx - 1) / bx);
    gy = (unsigned)((nyd + by - 1) / by);
    long long want = 8LL * sm_count;  // blocks in flight: a few per SM
    long long nz = (want + (long long)gx * gy - 1) / ((long long)gx * gy);
    if (nz < 1) nz = 1;
    if (nz > nzd) nz = nzd;
    const int zlen = (int)((nzd + nz - 1) / nz);
    nz = (nzd + zlen - 1) / zlen;
    if (gy > 65535 || nz > 65535) return cudaErrorInvalidConfiguration;
    gz = (unsigned)nz;
    const int h[8] = {dom.min[0], dom.max[0], dom.min[1], dom.max[1],
                      dom.min[2], dom.max[2], color, zlen};
    memcpy(head, h, sizeof(h));
  }

  // argument storage: 8 ints, then each parameter at its alignment
  std::vector<unsigned char> buf(64 + 64 * k.params.size());
  std::vector<void *> args;
  size_t off = 0;
  auto put = [&](const void *v, size_t n, size_t align) {
    off = (off + align - 1) / align * align;
    memcpy(buf.data() + off, v, n);
    args.push_back(buf.data() + off);
    off += n;
  };
  for (int v : head) put(&v, 4, 4);
  int gi = 0, si = 0;
  for (const JitParam &p : k.params) {
    if (p.grid) {
      const GridView &g = grids[gi++];
      GridArg a;
      a.p = g.ptr;
      a.row = g.pitch / g.esz;
      a.plane = a.row * g.ny;
      a.nx = g.nx;
      a.ny = g.ny;
      a.nz = g.nz;
      a.rank = p.rank;
      a.cur = 0;
      put(&a, sizeof(a), 8);
    } else {
      const double v = scalars[si++];
      switch (p.type) {
        case kInt: { const int t = (int)v; put(&t, 4, 4); break; }
        case kLong: { const long long t = (long long)v; put(&t, 8, 8); break; }
        case kFloat: { const float t = (float)v; put(&t, 4, 4); break; }
        default: put(&v, 8, 8); break;
      }
    }
  }
  const CUresult r = g_drv.launch(static_cast<CUfunction>(tiled ? k.func_tiled : k.func), gx,
                                  gy, gz, bx, by, 1, tiled ? (unsigned)k.stage_smem : 0,
                                  static_cast<CUstream>(s), args.data(), nullptr);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorLaunchFailure;
}

namespace {

const char *type_name(int type) {
  switch (type) {
    case kFloat: return "float";
    case kDouble: return "double";
    case kInt: return "int";
    default: return "long long";
  }
}

std::string key_string(const PtsJitKey &k) {
  std::string s;
  char buf[64];
  snprintf(buf, sizeof(buf), "%d,%d,%d,%d,%d,%d,%d,%d;", k.type, k.ry, k.warps, k.n,
           k.unit ? 1 : 0, k.w, k.nstage, k.pstride);
  s += buf;
  for (int i = 0; i < k.n; ++i) {
    snprintf(buf, sizeof(buf), "%d:%d:%a;", k.off[i], k.lag[i], k.wt[i]);
    s += buf;
  }
  return s;
}

std::string points_source(const PtsJitKey &k) {
  std::string s = "#include \"points_body.cuh\"\nstruct GenSpec {\n"
                  "  static constexpr bool kStatic = true;\n";
  char buf[96];
  snprintf(buf, sizeof(buf), "  static constexpr int kN = %d;\n", k.n);
  s += buf;
  s += "  static constexpr int kOff[kN] = {";
  for (int i = 0; i < k.n; ++i) s += (i ? ", " : "") + std::to_string(k.off[i]);
  s += "};\n  static constexpr int kLag[kN] = {";
  for (int i = 0; i < k.n; ++i) s += (i ? ", " : "") + std::to_string(k.lag[i]);
  s += "};\n  static constexpr double kWt[kN] = {";
  for (int i = 0; i < k.n; ++i) {
    snprintf(buf, sizeof(buf), "%s%a", i ? ", " : "", k.wt[i]);
    s += buf;
  }
  s += "};\n";
  snprintf(buf, sizeof(buf), "%d", k.w);
  s += "  template <typename T> static __device__ __forceinline__ int w(const psg::PtsParams<T> &)"
       " { return " + std::string(buf) + "; }\n";
  s += "  template <typename T> static __device__ __forceinline__ int nstage("
       "const psg::PtsParams<T> &) { return " + std::to_string(k.nstage) + "; }\n";
  s += "  template <typename T> static __device__ __forceinline__ int pstride("
       "const psg::PtsParams<T> &) { return " + std::to_string(k.pstride) + "; }\n};\n";
  const std::string T = type_name(k.type);
  s += "extern \"C\" __global__ void __launch_bounds__(" + std::to_string(32 * k.warps) +
       ", 1) __ps_points(const __grid_constant__ psg::PtsParams<" + T + "> p, "
       "const __grid_constant__ psg::PtsTmap tm) {\n"
       "  extern __shared__ __align__(128) unsigned char smem[];\n"
       "  psg::pts_body<" + T + ", " + std::to_string(k.ry) + ", " +
       (k.unit ? "true" : "false") + ", GenSpec>(p, &tm, smem);\n}\n";
  return s;
}

std::map<std::string, void *> g_points_jit;  // key -> CUfunction (nullptr: failed)

}  // namespace

void *jit_points_function(const PtsJitKey &k) {
  const std::string key = key_string(k);
  auto hit = g_points_jit.find(key);
  if (hit != g_points_jit.end()) return hit->second;
  std::string err;
  void *fn = nullptr;
  if (load_nvrtc(&err) && load_driver(&err)) {
    const std::string program = points_source(k);
    const char *hdr_src[] = {kEmbedArith, kEmbedPointsBody};
    const char *hdr_name[] = {"ps_arith.cuh", "points_body.cuh"};
    nvrtcProgram_t prog = nullptr;
    if (g_nvrtc.create(&prog, program.c_str(), "points.cu", 2, hdr_src, hdr_name) == 0) {
      const char *opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "--fmad=false"};
      if (g_nvrtc.compile(prog, 3, opts) == 0) {
        size_t n = 0;
        g_nvrtc.cubin_size(prog, &n);
        std::vector<char> image(n);
        g_nvrtc.cubin(prog, image.data());
        CUmodule mod = nullptr;
        CUfunction f = nullptr;
        if (g_drv.load(&mod, image.data()) == CUDA_SUCCESS) {
          if (g_drv.get(&f, mod, "__ps_points") == CUDA_SUCCESS) fn = f;
          else g_drv.unload(mod);
        }
      }
      g_nvrtc.destroy(&prog);
    }
  }
  g_points_jit[key] = fn;
  return fn;
}

bool jit_prepare(void *fn, int threads, size_t smem, int *occ) {
  CUfunction f = static_cast<CUfunction>(fn);
  if (g_drv.set_attr(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem) !=
      CUDA_SUCCESS)
    return false;
  return g_drv.occupancy(occ, f, threads, smem) == CUDA_SUCCESS;
}

cudaError_t jit_launch_raw(void *fn, int grid, dim3 block, size_t smem, cudaStream_t s,
                           void **args) {
  const CUresult r = g_drv.launch(static_cast<CUfunction>(fn), (unsigned)grid, 1, 1, block.x,
                                  block.y, block.z, (unsigned)smem, static_cast<CUstream>(s),
                                  args, nullptr);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorLaunchFailure;
}

}  // namespace psg
