"""Grids of user-defined struct types (DeclareGrid3D(name, struct ...)).

Each case restates, in the reference's stencil language, what the named
reference system test's stencil function does over a struct-typed grid
(member reads through PSGridGet(...).m, whole-struct PSGridEmit, member
writes through PSGridEmitUtype(g.m, v)), in the same expression order, runs
it through PSStencilFunctionNew on the GPU and compares the dump with the
exact stdout of that test's REF program
(tests/system_tests/test_cases/<test>.manual.ref.c, tests/golden/).  Grids
here are numpy structured arrays of the same layout as the C structs.
"""
import subprocess

import numpy as np
import pytest

import golden_io as gio
import physis_gb300 as ps

pytestmark = pytest.mark.gpu

N = 32


@pytest.fixture(scope="module")
def rt():
    ps.build()
    ps.init()
    yield ps
    ps.clear_error()


def _dump(arr, fields):
    """printf("%f %f ...\\n", e.f1, e.f2, ...) per element, x fastest."""
    cols = [np.asarray(arr[f] if isinstance(f, str) else f(arr), np.float64).reshape(-1)
            for f in fields]
    return "".join(" ".join("%f" % c[i] for c in cols) + "\n" for i in range(cols[0].size))


def _iota():
    return np.arange(N ** 3, dtype=np.float64).reshape(N, N, N)


def _run(src, name, dom, grids, iters=1, more=()):
    maps = [ps.stencil_map(ps.stencil_function(src, name), dom, grids)]
    for s2, n2, g2 in more:
        maps.append(ps.stencil_map(ps.stencil_function(src, n2), dom, g2))
    ps.stencil_run(maps, iters)


INNER = (1, N - 1, 1, N - 1, 1, N - 1)
FULL = (0, N, 0, N, 0, N)

PQ = np.dtype([("p", "<f4"), ("q", "<f4")])

SEVEN_PT = r"""
struct Point { float p; float q; };
DeclareGrid3D(Point, struct Point);
void seven(const int x, const int y, const int z, PSGrid3DPoint g) {
  float v = PSGridGet(g, x, y, z).p + PSGridGet(g, x + 1, y, z).p +
      PSGridGet(g, x - 1, y, z).p + PSGridGet(g, x, y + 1, z).p +
      PSGridGet(g, x, y - 1, z).p + PSGridGet(g, x, y, z + 1).p +
      PSGridGet(g, x, y, z - 1).p;
  PSGridEmitUtype(g.q, v);
}
"""


@pytest.mark.parametrize("periodic", [False, True])
def test_seven_point_member_emit(rt, periodic):
    test = "test_user-defined-type-7-pt" + ("-periodic" if periodic else "")
    src = SEVEN_PT.replace("PSGridGet(", "PSGridGetPeriodic(") if periodic else SEVEN_PT
    a = np.zeros((N, N, N), PQ)
    a["p"] = _iota()
    g = ps.Grid(a.shape, PQ)
    g.copyin(a)
    _run(src, "seven", ps.domain(*(FULL if periodic else INNER)), [g])
    assert _dump(g.copyout(), ["p", "q"]) == gio.stdout_text(test)
    g.free()


COMPLEX = r"""
struct Complex { float r; float i; };
DeclareGrid3D(Complex, struct Complex);
void csum(const int x, const int y, const int z, PSGrid3DComplex g1, PSGrid3DComplex g2) {
  struct Complex t = PSGridGetPeriodic(g1, x, y, z);
  struct Complex t1 = PSGridGetPeriodic(g1, x + 1, y, z);
  struct Complex t2 = PSGridGetPeriodic(g1, x - 1, y, z);
  struct Complex t3 = PSGridGetPeriodic(g1, x, y + 1, z);
  struct Complex t4 = PSGridGetPeriodic(g1, x, y - 1, z);
  struct Complex t5 = PSGridGetPeriodic(g1, x, y, z + 1);
  struct Complex t6 = PSGridGetPeriodic(g1, x, y, z - 1);
  float r = t.r + t1.r + t2.r + t3.r + t4.r + t5.r + t6.r;
  float i = t.i + t1.i + t2.i + t3.i + t4.i + t5.i + t6.i;
  struct Complex v = {r, i};
  PSGridEmit(g2, v);
}
"""


def test_periodic_complex_whole_struct(rt):
    dt = np.dtype([("r", "<f4"), ("i", "<f4")])
    a = np.zeros((N, N, N), dt)
    a["r"] = _iota()
    a["i"] = _iota() + 1
    g1, g2 = ps.Grid(a.shape, dt), ps.Grid(a.shape, dt)
    g1.copyin(a)
    _run(COMPLEX, "csum", ps.domain(*FULL), [g1, g2])
    assert _dump(g2.copyout(), ["r", "i"]) == gio.stdout_text(
        "test_user-defined-type-7-pt-periodic-complex")
    g1.free()
    g2.free()


def _seven(member):
    """The seven reads of one member in the order c, x-1, x+1, y-1, y+1,
    z-1, z+1."""
    pts = ["x, y, z", "x - 1, y, z", "x + 1, y, z", "x, y - 1, z", "x, y + 1, z",
           "x, y, z - 1", "x, y, z + 1"]
    return " +\n      ".join(f"PSGridGet(g, {p}){member}" for p in pts)


ARRAY_MEMBER = r"""
struct Point { float p[2]; };
DeclareGrid3D(Point, struct Point);
void am(const int x, const int y, const int z, PSGrid3DPoint g) {
  float v = %s;
  PSGridEmitUtype(g.p[1], v);
}
""" % _seven(".p[0]")

MULTI_DIM = r"""
struct Point { float p[3][2]; };
DeclareGrid3D(Point, struct Point);
static void md(const int x, const int y, const int z, PSGrid3DPoint g) {
  float v1 = %s;
  float v2 = %s;
  PSGridEmitUtype(g.p[1][0], v1 + v2);
}
""" % (_seven(".p[0][0]"), _seven(".p[2][1]"))

MULTI_MEMBERS = r"""
struct Point { float p[2]; float q; float r; };
DeclareGrid3D(Point, struct Point);
static void mm(const int x, const int y, const int z, PSGrid3DPoint g) {
  float v1 = %s;
  float v2 = %s;
  float v3 = %s;
  PSGridEmitUtype(g.r, v1 + v2 + v3);
}
""" % (_seven(".p[0]"), _seven(".p[1]"), _seven(".q"))


def test_array_member(rt):
    dt = np.dtype([("p", "<f4", (2,))])
    a = np.zeros((N, N, N), dt)
    a["p"][..., 0] = _iota()
    g = ps.Grid(a.shape, dt)
    g.copyin(a)
    _run(ARRAY_MEMBER, "am", ps.domain(*INNER), [g])
    out = g.copyout()
    assert _dump(out, [lambda o: o["p"][..., 1]]) == gio.stdout_text("test_user-defined-type5")
    g.free()


def test_multi_dimensional_member(rt):
    dt = np.dtype([("p", "<f4", (3, 2))])
    a = np.zeros((N, N, N), dt)
    i = _iota()
    for j in range(3):
        for k in range(2):
            a["p"][..., j, k] = i + j + k
    g = ps.Grid(a.shape, dt)
    g.copyin(a)
    _run(MULTI_DIM, "md", ps.domain(*INNER), [g])
    out = g.copyout()
    assert _dump(out, [lambda o: o["p"][..., 1, 0]]) == gio.stdout_text(
        "test_user-defined-type-multi-dim-member")
    g.free()


def test_multiple_members(rt):
    dt = np.dtype([("p", "<f4", (2,)), ("q", "<f4"), ("r", "<f4")])
    a = np.zeros((N, N, N), dt)
    i = _iota()
    a["p"][..., 0] = i
    a["p"][..., 1] = i + 1
    a["q"] = i + 2
    g = ps.Grid(a.shape, dt)
    g.copyin(a)
    _run(MULTI_MEMBERS, "mm", ps.domain(*INNER), [g])
    assert _dump(g.copyout(), ["r"]) == gio.stdout_text("test_user-defined-type-multi-members")
    g.free()


XYZ = r"""
struct Point { float x; float y; float z; };
DeclareGrid3D(Point, struct Point);
void xyz(const int x, const int y, const int z, PSGrid3DPoint g1, PSGrid3DPoint g2) {
  float p = (PSGridGet(g1, x, y, z).x + PSGridGet(g1, x + 1, y, z).x +
             PSGridGet(g1, x - 1, y, z).x) / 3.3f;
  float q = (PSGridGet(g1, x, y, z).y + PSGridGet(g1, x, y + 1, z).y +
             PSGridGet(g1, x, y - 1, z).y + PSGridGet(g1, x, y, z + 1).y +
             PSGridGet(g1, x, y, z - 1).y) / 5.5f;
  float r = (PSGridGet(g1, x, y, z).z + PSGridGet(g1, x, y, z + 1).z +
             PSGridGet(g1, x, y, z - 1).z) / 3.3f;
  struct Point v = {p, q, r};
  PSGridEmit(g2, v);
}
"""


def test_struct_pingpong_ten_steps(rt):
    dt = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4")])
    a = np.zeros((N, N, N), dt)
    i = _iota()
    a["x"], a["y"], a["z"] = i, i + 1, i + 2
    g1, g2 = ps.Grid(a.shape, dt), ps.Grid(a.shape, dt)
    g1.copyin(a)
    g2.copyin(a)
    k = ps.stencil_function(XYZ, "xyz")
    dom = ps.domain(*INNER)
    ps.stencil_run([ps.stencil_map(k, dom, [g1, g2]), ps.stencil_map(k, dom, [g2, g1])], 5)
    assert _dump(g1.copyout(), ["x", "y", "z"]) == gio.stdout_text("test_user-defined-type1")
    g1.free()
    g2.free()


PQR = r"""
struct Point { float p; float q; float r; };
DeclareGrid3D(Point, struct Point);
void k1(const int x, const int y, const int z, PSGrid3DPoint g) {
  float v = (PSGridGet(g, x, y, z).p + PSGridGet(g, x + 1, y, z).p +
             PSGridGet(g, x - 1, y, z).p + PSGridGet(g, x, y + 1, z).p +
             PSGridGet(g, x, y - 1, z).p + PSGridGet(g, x, y, z + 1).p +
             PSGridGet(g, x, y, z - 1).p + PSGridGet(g, x, y, z).q +
             PSGridGet(g, x + 1, y, z).q + PSGridGet(g, x - 1, y, z).q +
             PSGridGet(g, x, y + 1, z).q + PSGridGet(g, x, y - 1, z).q +
             PSGridGet(g, x, y, z + 1).q + PSGridGet(g, x, y, z - 1).q) / 14.3;
  PSGridEmitUtype(g.r, v);
}
void k2(const int x, const int y, const int z, PSGrid3DPoint g) {
  PSGridEmitUtype(g.p, (PSGridGet(g, x, y, z).p + PSGridGet(g, x, y, z).r) * 0.5);
  PSGridEmitUtype(g.q, (PSGridGet(g, x, y, z).q + PSGridGet(g, x, y, z).r) * 0.5);
}
"""


def test_two_functions_alternating_in_place(rt):
    dt = np.dtype([("p", "<f4"), ("q", "<f4"), ("r", "<f4")])
    a = np.zeros((N, N, N), dt)
    a["p"] = _iota()
    a["q"] = _iota() + 1
    g = ps.Grid(a.shape, dt)
    g.copyin(a)
    dom = ps.domain(*INNER)
    ps.stencil_run([ps.stencil_map(ps.stencil_function(PQR, "k1"), dom, [g]),
                    ps.stencil_map(ps.stencil_function(PQR, "k2"), dom, [g])], 10)
    assert _dump(g.copyout(), ["p", "q", "r"]) == gio.stdout_text("test_user-defined-type3")
    g.free()


def test_user_grid_checks(rt):
    # element size must match the function's struct; builtins, point
    # stencils and reductions reject user-type grids; __PSGridSet writes a
    # whole element
    import ctypes
    wrong = ps.Grid((4, 4, 4), np.dtype([("a", "<f4"), ("b", "<f4"), ("c", "<f4")]))
    k = ps.stencil_function(SEVEN_PT, "seven")
    with pytest.raises(ps.PSError):
        ps.stencil_map(k, ps.domain(1, 3, 1, 3, 1, 3), [wrong])
    ps.clear_error()
    g = ps.Grid((4, 4, 4), PQ)
    h = ps.Grid((4, 4, 4), PQ)
    with pytest.raises(ps.PSError):
        ps.stencil_map(ps.PS_KERNEL_COPY, ps.full_domain((4, 4, 4)), [g, h])
    ps.clear_error()
    out = np.zeros(1, np.float64)
    ps.lib().PSReduceGridV(out.ctypes.data_as(ctypes.c_void_p), ps.PS_SUM, g.handle)
    assert ps.last_error()[0] == ps.PS_ERR_UNSUPPORTED
    ps.clear_error()
    v = np.zeros(1, PQ)
    v["p"], v["q"] = 1.5, -2.0
    idx = (ctypes.c_int32 * 3)(1, 2, 3)
    assert ps.lib().PSGridSetV(g.handle, idx, v.ctypes.data_as(ctypes.c_void_p)) == ps.PS_OK
    got = g.copyout()
    assert got[3, 2, 1]["p"] == 1.5 and got[3, 2, 1]["q"] == -2.0
    assert got["p"].sum() == 1.5
    for x in (wrong, g, h):
        x.free()


# A C program written like the reference's test_user-defined-type-7-pt.c:
# DeclareGrid3D of a struct, PSGrid3DPointNew, copy-in/out of struct arrays;
# the stencil function is handed to PSStencilFunctionNew as text.
C_UTYPE_PROGRAM = r"""
#include <stdio.h>
#include <stdlib.h>
#include "physis_gb300/physis.h"
#include "physis_gb300/physis_gb300.h"
#define N 32
struct Point {
  float p;
  float q;
};
DeclareGrid3D(Point, struct Point);
static const char *kernel_src =
    "struct Point { float p; float q; };\n"
    "DeclareGrid3D(Point, struct Point);\n"
    "void kernel1(const int x, const int y, const int z, PSGrid3DPoint g) {\n"
    "  float v = PSGridGet(g, x, y, z).p + PSGridGet(g, x+1, y, z).p +\n"
    "      PSGridGet(g, x-1, y, z).p + PSGridGet(g, x, y+1, z).p +\n"
    "      PSGridGet(g, x, y-1, z).p + PSGridGet(g, x, y, z+1).p +\n"
    "      PSGridGet(g, x, y, z-1).p;\n"
    "  PSGridEmitUtype(g.q, v);\n"
    "}\n";
int main(int argc, char *argv[]) {
  int i;
  size_t nelms = N * N * N;
  struct Point *indata, *outdata;
  PSInit(&argc, &argv, 3, N, N, N);
  PSGrid3DPoint g = PSGrid3DPointNew(N, N, N);
  PSDomain3D d = PSDomain3DNew(1, N - 1, 1, N - 1, 1, N - 1);
  int kernel1 = PSStencilFunctionNew(kernel_src, "kernel1");
  indata = (struct Point *)malloc(sizeof(struct Point) * nelms);
  outdata = (struct Point *)malloc(sizeof(struct Point) * nelms);
  for (i = 0; i < (int)nelms; i++) {
    indata[i].p = i;
    indata[i].q = 0;
  }
  PSGridCopyin(g, indata);
  PSStencilRun(PSStencilMap(kernel1, d, g));
  PSGridCopyout(g, outdata);
  for (i = 0; i < (int)nelms; ++i) printf("%f %f\n", outdata[i].p, outdata[i].q);
  PSGridFree(g);
  PSFinalize();
  free(indata);
  free(outdata);
  return PSGetLastError();
}
"""


def test_c_program_with_a_user_type(rt, tmp_path):
    from test_abi import compile_c_program
    exe = compile_c_program(tmp_path, C_UTYPE_PROGRAM, "utype")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout == gio.stdout_text("test_user-defined-type-7-pt")
