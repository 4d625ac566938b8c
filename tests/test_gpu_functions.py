"""Stencil functions compiled at run time (PSStencilFunctionNew) on the GPU.

The stencil functions below are written in the reference's stencil language
(PSGridGet / PSGridGetPeriodic / PSGridEmit over PSGrid* parameters) and do
what the named reference system test's stencil does, in the same expression
order; the bar is the exact stdout of that test's REF program
(tests/golden/).  Beyond the goldens: scalars of every type through the
variadic C entry, red/black maps of a function, a random-weight function
against the oracle, and the compiler's error reporting.
"""
import subprocess

import numpy as np
import pytest

import golden_io as gio
import physis_gb300 as ps
import system_cases as sc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rt():
    ps.build()
    ps.init()
    yield ps
    ps.clear_error()


@pytest.fixture(autouse=True, params=["tiled", "plain"])
def entry(request, monkeypatch):
    # Every test runs on both generated entries: the tiled one (grids read
    # at neighbour offsets staged in shared memory) and the plain one
    # (PS_FUNCTION_TILED=0).  Both must give the same bits.
    monkeypatch.setenv("PS_FUNCTION_TILED", "1" if request.param == "tiled" else "0")
    return request.param


def _bits(a):
    return a.view({4: np.uint32, 8: np.uint64}[a.dtype.itemsize])


def _grid(arr):
    g = ps.Grid(arr.shape, arr.dtype)
    g.copyin(arr)
    return g


def _iota(shape, dtype):
    n = int(np.prod(shape))
    return np.arange(n, dtype=np.int64).astype(dtype).reshape(shape)


BRANCHY = r"""
#define EDGE 32
void branchy(const int x, const int y, const int z, PSGrid3DFloat in,
             PSGrid3DFloat out) {
  float c = PSGridGet(in, x, y, z);
  float l = 0.0f;
  if (x > 0) l = PSGridGet(in, x - 1, y, z);
  if (x > 0) l += PSGridGet(in, x - 1, y, z); else l += PSGridGet(in, x, y, z);
  if (x > 0) l += PSGridGet(in, x - 1, y, z); else l += c;
  if (x > 0 && x < EDGE - 1)
    l += PSGridGet(in, x - 1, y, z) + PSGridGet(in, x + 1, y, z);
  else
    l += PSGridGet(in, x, y, z);
  if (x % 2 == 0) l += PSGridGet(in, x, y, z);
  PSGridEmit(out, c + l);
}
"""

CLAMPED_SUM = r"""
static float at(PSGrid3DFloat g, int x, int y, int z, float c, int edge) {
  return edge ? c : PSGridGet(g, x, y, z);
}
void clamped(const int x, const int y, const int z, PSGrid3DFloat g,
             PSGrid3DFloat out) {
  const int nx = PSGridDim(g, 0), ny = PSGridDim(g, 1), nz = PSGridDim(g, 2);
  float c = PSGridGet(g, x, y, z);
  float w = at(g, x - 1, y, z, c, x == 0);
  float e = at(g, x + 1, y, z, c, x == nx - 1);
  float n = at(g, x, y - 1, z, c, y == 0);
  float s = at(g, x, y + 1, z, c, y == ny - 1);
  float b = at(g, x, y, z - 1, c, z == 0);
  float t = at(g, x, y, z + 1, c, z == nz - 1);
  PSGridEmit(out, c + w + e + s + n + b + t);
}
"""

TYPE_MIX = r"""
void mix7(const int x, const int y, const int z, PSGrid3DFloat src,
          PSGrid3DDouble dst, PSGrid3DInt scale) {
  double acc = (double)PSGridGet(src, x, y, z) + (double)PSGridGet(src, x + 1, y, z)
      + (double)PSGridGet(src, x - 1, y, z) + (double)PSGridGet(src, x, y + 1, z)
      + (double)PSGridGet(src, x, y - 1, z) + (double)PSGridGet(src, x, y, z - 1)
      + (double)PSGridGet(src, x, y, z + 1);
  PSGridEmit(dst, acc * PSGridGet(scale, x, y, z));
}
"""

MIXED1 = r"""
void line3(const int x, const int y, const int z, PSGrid3DFloat a,
           PSGrid3DFloat b, PSGrid1DFloat k) {
  PSGridEmit(b, PSGridGet(a, x, y, z) * PSGridGet(k, x)
                + PSGridGet(a, x - 1, y, z) * PSGridGet(k, x - 1)
                + PSGridGet(a, x + 1, y, z) * PSGridGet(k, x + 1));
}
"""

MIXED2 = r"""
void axes(const int x, const int y, const int z, PSGrid3DFloat a, PSGrid3DFloat b,
          PSGrid1DFloat ci, PSGrid1DFloat cj, PSGrid1DFloat ck) {
  float v = PSGridGet(a, x, y, z)
      + PSGridGet(a, x - 1, y, z) * PSGridGet(ci, x - 1)
      + PSGridGet(a, x + 1, y, z) * PSGridGet(ci, x + 1)
      + PSGridGet(a, x, y - 1, z) * PSGridGet(cj, y - 1)
      + PSGridGet(a, x, y + 1, z) * PSGridGet(cj, y + 1)
      + PSGridGet(a, x, y, z - 1) * PSGridGet(ck, z - 1)
      + PSGridGet(a, x, y, z + 1) * PSGridGet(ck, z + 1);
  PSGridEmit(b, v);
}
"""

MIXED3 = r"""
void planes(const int x, const int y, const int z, PSGrid3DFloat a, PSGrid3DFloat b,
            PSGrid1DFloat ci, PSGrid2DFloat cyz) {
  float v = PSGridGet(a, x, y, z)
      + PSGridGet(a, x - 1, y, z) * PSGridGet(ci, x - 1)
      + PSGridGet(a, x + 1, y, z) * PSGridGet(ci, x + 1)
      + PSGridGet(a, x, y - 1, z) * PSGridGet(cyz, y - 1, z)
      + PSGridGet(a, x, y + 1, z) * PSGridGet(cyz, y + 1, z)
      + PSGridGet(a, x, y, z - 1) * PSGridGet(cyz, y, z - 1)
      + PSGridGet(a, x, y, z + 1) * PSGridGet(cyz, y, z + 1);
  PSGridEmit(b, v);
}
"""

PERIODIC27 = r"""
void wrap27(const int x, const int y, const int z, PSGrid3DFloat a, PSGrid3DFloat b) {
  float v = 0.0f;
  int first = 1;
  for (int dz = -1; dz <= 1; ++dz) {
    const int dxs[9] = {0, 1, -1, 0, 1, -1, 0, 1, -1};
    const int dys[9] = {0, 0, 0, 1, 1, 1, -1, -1, -1};
    for (int i = 0; i < 9; ++i) {
      float t = PSGridGetPeriodic(a, x + dxs[i], y + dys[i], z + dz);
      v = first ? t : v + t;
      first = 0;
    }
  }
  PSGridEmit(b, v);
}
"""

REDBLACK = r"""
void rb7(const int x, const int y, const int z, PSGrid3DFloat g) {
  float v = PSGridGet(g, x, y, z) + PSGridGet(g, x + 1, y, z) + PSGridGet(g, x - 1, y, z)
      + PSGridGet(g, x, y + 1, z) + PSGridGet(g, x, y - 1, z)
      + PSGridGet(g, x, y, z - 1) + PSGridGet(g, x, y, z + 1);
  PSGridEmit(g, v);
}
"""

LINE1D = r"""
void three(const int x, PSGrid1DFloat a, PSGrid1DFloat b) {
  PSGridEmit(b, PSGridGet(a, x - 1) + PSGridGet(a, x) + PSGridGet(a, x + 1));
}
"""

NINE2D_INT = r"""
void nine(const int x, const int y, PSGrid2DInt a, PSGrid2DInt b) {
  float v = PSGridGet(a, x, y) + PSGridGet(a, x - 1, y) + PSGridGet(a, x + 1, y)
      + PSGridGet(a, x, y - 1) + PSGridGet(a, x, y + 1) + PSGridGet(a, x - 1, y - 1)
      + PSGridGet(a, x + 1, y - 1) + PSGridGet(a, x - 1, y + 1) + PSGridGet(a, x + 1, y + 1);
  PSGridEmit(b, v);
}
"""


def _run(kernel, dom, grids, scalars=()):
    ps.stencil_run([ps.stencil_map(kernel, dom, grids, scalars)])


def test_branchy_function_test_15(rt):
    n = 32
    k = ps.stencil_function(BRANCHY, "branchy")
    a, b = _grid(_iota((n, n, n), np.float32)), _grid(_iota((n, n, n), np.float32))
    _run(k, ps.full_domain((n, n, n)), [a, b])
    assert gio.dump_text(b.copyout()) == gio.stdout_text("test_15")
    a.free()
    b.free()


def test_clamped_function_with_helper_test_16(rt):
    n = 32
    k = ps.stencil_function(CLAMPED_SUM, "clamped")
    a, b = _grid(_iota((n, n, n), np.float32)), _grid(_iota((n, n, n), np.float32))
    _run(k, ps.full_domain((n, n, n)), [a, b])
    assert gio.dump_text(b.copyout()) == gio.stdout_text("test_16")
    a.free()
    b.free()


def test_type_mix(rt):
    n = 32
    k = ps.stencil_function(TYPE_MIX, "mix7")
    a = _grid(_iota((n, n, n), np.float32))
    b = _grid(np.zeros((n, n, n), np.float64))
    c = _grid((np.arange(n ** 3) % 10).astype(np.int32).reshape(n, n, n))
    _run(k, ps.domain(1, n - 1, 1, n - 1, 1, n - 1), [a, b, c])
    assert gio.dump_text(b.copyout()) == gio.stdout_text("test_7-pt-type-mix")
    for g in (a, b, c):
        g.free()


def test_mixed_dimensions(rt):
    n = 32
    coef = (1 + np.arange(n) % 2).astype(np.float32)
    k1 = ps.stencil_function(MIXED1, "line3")
    a, b = _grid(_iota((n, n, n), np.float32)), _grid(_iota((n, n, n), np.float32))
    kg = _grid(coef)
    _run(k1, ps.domain(1, n - 1, 0, n, 0, n), [a, b, kg])
    assert gio.dump_text(b.copyout()) == gio.stdout_text("test_mixed-dim")
    b.copyin(_iota((n, n, n), np.float32))
    k2 = ps.stencil_function(MIXED2, "axes")
    _run(k2, ps.domain(1, n - 1, 1, n - 1, 1, n - 1), [a, b, kg, kg, kg])
    assert gio.dump_text(b.copyout()) == gio.stdout_text("test_mixed-dim2")
    for g in (a, b, kg):
        g.free()
    m = n + 2
    k3 = ps.stencil_function(MIXED3, "planes")
    a, b = _grid(_iota((n, m, n), np.float32)), _grid(_iota((n, m, n), np.float32))
    ci = _grid(coef)
    cyz = _grid((1 + np.arange(m * n) % 2).astype(np.float32).reshape(n, m))
    _run(k3, ps.domain(1, n - 1, 1, m - 1, 1, n - 1), [a, b, ci, cyz])
    assert gio.dump_text(b.copyout()) == gio.stdout_text("test_mixed-dim3")
    for g in (a, b, ci, cyz):
        g.free()


def test_periodic_function_test_27_pt_periodic(rt):
    n = 32
    k = ps.stencil_function(PERIODIC27, "wrap27")
    a, b = _grid(_iota((n, n, n), np.float32)), _grid(_iota((n, n, n), np.float32))
    _run(k, ps.full_domain((n, n, n)), [a, b])
    assert gio.dump_text(b.copyout()) == gio.stdout_text("test_27-pt-periodic")
    a.free()
    b.free()


def test_red_black_function_test_redblack(rt):
    n = 32
    k = ps.stencil_function(REDBLACK, "rb7")
    g = _grid(_iota((n, n, n), np.float32))
    dom = ps.domain(1, n - 1, 1, n - 1, 1, n - 1)
    ps.stencil_run([ps.stencil_map_color(k, ps.COLOR_REDBLACK, dom, [g])])
    assert gio.dump_text(g.copyout()) == gio.stdout_text("test_redblack")
    g.free()


def test_1d_and_2d_functions(rt):
    k = ps.stencil_function(LINE1D, "three")
    a, b = _grid(_iota((1024,), np.float32)), _grid(_iota((1024,), np.float32))
    _run(k, ps.domain(1, 1023, 0, 1, 0, 1), [a, b])
    assert gio.dump_text(b.copyout()) == gio.stdout_text("test_3-pt-1d")
    a.free()
    b.free()
    n = 32
    k = ps.stencil_function(NINE2D_INT, "nine")
    a, b = _grid(_iota((n, n), np.int32)), _grid(_iota((n, n), np.int32))
    dom = ps.domain(1, n - 1, 1, n - 1, 0, 1)
    ps.stencil_run([ps.stencil_map(k, dom, [a, b]), ps.stencil_map(k, dom, [b, a])])
    assert "%d\n" % int(ps.reduce(a, ps.PS_SUM)) == gio.stdout_text("test_9-pt-reduction")
    a.free()
    b.free()


WEIGHTED = r"""
void weighted(const int x, const int y, const int z, PSGrid3DDouble a, double c0,
              PSGrid3DDouble b, float c1, int c2, long c3) {
  double v = c0 * PSGridGet(a, x, y, z) + c1 * PSGridGet(a, x - 1, y, z)
      + (double)c2 * PSGridGet(a, x, y + 1, z) + (double)c3 * PSGridGet(a, x, y, z - 2);
  PSGridEmit(b, v);
}
"""


def test_scalars_of_every_type_against_oracle(rt, oracle):
    # Grids and scalars interleaved in the parameter list; the map takes
    # them in that order.  Oracle: the same weighted sum as a point stencil.
    rng = np.random.default_rng(5)
    shape = (11, 23, 150)
    src = rng.uniform(-1, 1, size=shape)
    w = [0.3, float(np.float32(-1.7)), 3.0, -2.0]
    pts = [(0, 0, 0), (-1, 0, 0), (0, 1, 0), (0, 0, -2)]
    nz, ny, nx = shape
    dom = (1, nx, 0, ny - 1, 2, nz)
    ref = np.zeros(shape)
    oracle.points(src, ref, dom, pts, weights=w)
    k = ps.stencil_function(WEIGHTED, "weighted")
    a, b = _grid(src), _grid(np.zeros(shape))
    ps.stencil_run([ps.stencil_map(k, ps.domain(*dom), [a, b], w)])
    assert np.array_equal(_bits(b.copyout()), _bits(ref))
    a.free()
    b.free()


def _weighted_source(name, offsets, periodic, dtype="Float", ctype="float"):
    get = "PSGridGetPeriodic" if periodic else "PSGridGet"
    params = ", ".join("%s w%d" % (ctype, i) for i in range(len(offsets)))
    terms = []
    for i, (dx, dy, dz) in enumerate(offsets):
        co = ["x", "y", "z"]
        for j, d in enumerate((dx, dy, dz)):
            if d:
                co[j] += (" + %d" % d) if d > 0 else (" - %d" % -d)
        terms.append("w%d * %s(a, %s)" % (i, get, ", ".join(co)))
    return ("void %s(const int x, const int y, const int z, PSGrid3D%s a, PSGrid3D%s b, %s) {\n"
            "  PSGridEmit(b, %s);\n}\n" % (name, dtype, dtype, params, " + ".join(terms)))


FAR = [(0, 0, 0), (6, 0, 0), (-4, 0, 0), (0, 2, 0), (0, -3, 0), (0, 0, 4), (0, 0, -1),
       (1, 1, 1), (-1, 2, -1), (3, -1, 0)]


@pytest.mark.parametrize("periodic", [False, True], ids=["clamp-free", "periodic"])
def test_staged_reads_with_wide_and_capped_halos(rt, oracle, periodic):
    # Offsets up to 6 in x (past the halo cap of 4: those reads come from
    # global memory), partial 64 x 16 tiles, an odd domain origin, z chunks;
    # periodic reads wrap at every face.  Oracle: the same left-to-right
    # weighted sum as a point stencil.
    rng = np.random.default_rng(21)
    shape = (37, 45, 150)
    nz, ny, nx = shape
    src = rng.uniform(-1, 1, size=shape).astype(np.float32)
    w = [float(v) for v in rng.uniform(-1, 1, size=len(FAR)).astype(np.float32)]
    if periodic:
        dom = (0, nx, 0, ny, 0, nz)
    else:
        dom = (5, nx - 6, 3, ny - 2, 1, nz - 4)
    ref = np.zeros(shape, np.float32)
    oracle.points(src, ref, dom, FAR, weights=w, boundary=1 if periodic else 0)
    code, log = ps.stencil_function_check(_weighted_source("far", FAR, periodic), "far")
    assert code == ps.PS_OK
    assert log == "staged a 4 3 4 %s;" % ("periodic" if periodic else "clamp")
    k = ps.stencil_function(_weighted_source("far", FAR, periodic), "far")
    a, b = _grid(src), _grid(np.zeros(shape, np.float32))
    ps.stencil_run([ps.stencil_map(k, ps.domain(*dom), [a, b], w)])
    assert np.array_equal(_bits(b.copyout()), _bits(ref))
    a.free()
    b.free()


def test_staged_double_grid_beside_an_unstaged_one(rt, oracle):
    # two input grids: the one read at offsets is staged (double), the one
    # read at the centre only is not; the emitted grid never is
    rng = np.random.default_rng(22)
    shape = (20, 33, 70)
    nz, ny, nx = shape
    src = rng.uniform(-1, 1, size=shape)
    scale = rng.uniform(0.5, 2.0, size=shape)
    pts = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
    dom = (1, nx - 1, 1, ny - 1, 1, nz - 1)
    sums = np.zeros(shape)
    oracle.points(src, sums, dom, pts, weights=[1.0] * 7)
    ref = np.zeros(shape)
    sl = (slice(1, nz - 1), slice(1, ny - 1), slice(1, nx - 1))
    ref[sl] = sums[sl] * scale[sl]
    code = r"""
void s7(const int x, const int y, const int z, PSGrid3DDouble a, PSGrid3DDouble s,
        PSGrid3DDouble out) {
  double v = PSGridGet(a, x, y, z) + PSGridGet(a, x + 1, y, z) + PSGridGet(a, x - 1, y, z)
      + PSGridGet(a, x, y + 1, z) + PSGridGet(a, x, y - 1, z) + PSGridGet(a, x, y, z + 1)
      + PSGridGet(a, x, y, z - 1);
  PSGridEmit(out, v * PSGridGet(s, x, y, z));
}
"""
    assert ps.stencil_function_check(code, "s7") == (ps.PS_OK, "staged a 1 1 1 clamp;")
    k = ps.stencil_function(code, "s7")
    a, sg, out = _grid(src), _grid(scale), _grid(np.zeros(shape))
    ps.stencil_run([ps.stencil_map(k, ps.domain(*dom), [a, sg, out])])
    assert np.array_equal(_bits(out.copyout()), _bits(ref))
    for g in (a, sg, out):
        g.free()


def test_function_ids_are_cached_and_errors_reported(rt):
    k1 = ps.stencil_function(REDBLACK, "rb7")
    assert ps.stencil_function(REDBLACK, "rb7") == k1
    bad = [
        ("void f(const int x, PSGrid1DFloat a, PSGrid1DFloat b) { PSGridEmit(b, nope); }", "f"),
        ("void f(const int x, struct thing *t) { }", "f"),
        ("void g(const int x, PSGrid1DFloat a) { }", "f"),
        ("void f(PSGrid1DFloat a, PSGrid1DFloat b) { }", "f"),
    ]
    for src, name in bad:
        ps.clear_error()
        with pytest.raises(ps.PSError) as e:
            ps.stencil_function(src, name)
        assert e.value.code == ps.PS_ERR_INVALID_ARGUMENT
    # a map whose grid does not match the parameter type or rank
    k = ps.stencil_function(LINE1D, "three")
    g3 = ps.Grid((4, 4, 4))
    g1 = ps.Grid((8,))
    with pytest.raises(ps.PSError) as e:
        ps.stencil_map(k, ps.domain(1, 3, 0, 1, 0, 1), [g3, g1])
    assert e.value.code == ps.PS_ERR_INVALID_ARGUMENT
    g3.free()
    g1.free()


C_FUNCTION_PROGRAM = r"""
#include <stdio.h>
#include <stdlib.h>
#include "physis_gb300/physis_gb300.h"

static const char *src =
  "void scaled(const int x, const int y, const int z, PSGrid3DFloat a,\n"
  "            PSGrid3DFloat b, float s, int k) {\n"
  "  PSGridEmit(b, s * PSGridGet(a, x, y, z) + (float)k * PSGridGet(a, x + 1, y, z));\n"
  "}\n";

int main(int argc, char **argv) {
  PSInit(&argc, &argv, 3, 8, 8, 8);
  int id = PSStencilFunctionNew(src, "scaled");
  PSGrid3DFloat a = PSGrid3DFloatNew(8, 8, 8), b = PSGrid3DFloatNew(8, 8, 8);
  float in[512], out[512];
  for (int i = 0; i < 512; ++i) { in[i] = (float)i; out[i] = 0.0f; }
  PSGridCopyin(a, in);
  PSGridCopyin(b, out);
  PSDomain3D d = PSDomain3DNew(0, 7, 0, 8, 0, 8);
  PSStencilRun(PSStencilMap(id, d, a, b, 0.5f, 3));
  PSGridCopyout(b, out);
  for (int i = 0; i < 512; ++i) printf("%f\n", out[i]);
  int err = PSGetLastError();
  PSFinalize();
  return err;
}
"""


def test_c_program_calls_a_function_through_varargs(rt, tmp_path):
    # float and int scalars through C varargs (double and int promotions).
    from test_abi import compile_c_program
    exe = compile_c_program(tmp_path, C_FUNCTION_PROGRAM, "fn")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr + r.stdout
    a = np.arange(512, dtype=np.float32).reshape(8, 8, 8)
    want = np.zeros_like(a)
    want[:, :, :7] = np.float32(0.5) * a[:, :, :7] + np.float32(3) * a[:, :, 1:]
    assert r.stdout == gio.dump_text(want)


def test_benchmark_functions_match_oracle_and_builtin(rt, oracle):
    # The stencil functions bench.py times: the 27-point sum against the
    # oracle's point-stencil restatement, the clamped diffusion function
    # against the DIFFUSION7 builtin, bit for bit.
    import bench
    rng = np.random.default_rng(9)
    shape = (20, 30, 140)
    nz, ny, nx = shape
    src = rng.uniform(0, 1, size=shape).astype(np.float32)
    inner = (1, nx - 1, 1, ny - 1, 1, nz - 1)
    ref = np.zeros(shape, np.float32)
    oracle.points(src, ref, inner, sc.P27)
    a, b = _grid(src), _grid(np.zeros(shape, np.float32))
    _run(ps.stencil_function(bench.FN27, "sum27"), ps.domain(*inner), [a, b])
    assert np.array_equal(_bits(b.copyout()), _bits(ref))
    coef = (0.1, 0.1, 0.1, 0.1, 0.1, 0.1, 0.4)
    full = ps.full_domain(shape)
    c = _grid(np.zeros(shape, np.float32))
    _run(ps.stencil_function(bench.FN_DIFFUSION, "diffusion"), full, [a, b], coef)
    _run(ps.PS_KERNEL_DIFFUSION7, full, [a, c], coef)
    assert np.array_equal(_bits(b.copyout()), _bits(c.copyout()))
    for g in (a, b, c):
        g.free()
