"""The stencil-function front end without a GPU: parsing the signature and
compiling with NVRTC for sm_103a (PSStencilFunctionCheck).  Every function
the GPU tests run must compile here; malformed ones must be rejected with
PS_ERR_INVALID_ARGUMENT and a reason."""
import pytest

import physis_gb300 as ps
import test_gpu_functions as fns


@pytest.fixture(scope="module")
def built():
    ps.build()
    return ps.lib()


GOOD = [(fns.BRANCHY, "branchy"), (fns.CLAMPED_SUM, "clamped"), (fns.TYPE_MIX, "mix7"),
        (fns.MIXED1, "line3"), (fns.MIXED2, "axes"), (fns.MIXED3, "planes"),
        (fns.PERIODIC27, "wrap27"), (fns.REDBLACK, "rb7"), (fns.LINE1D, "three"),
        (fns.NINE2D_INT, "nine"), (fns.WEIGHTED, "weighted")]


@pytest.mark.parametrize("src,name", GOOD, ids=[g[1] for g in GOOD])
def test_stencil_functions_compile(built, src, name):
    code, log = ps.stencil_function_check(src, name)
    if code == ps.PS_ERR_UNSUPPORTED:
        pytest.skip("NVRTC not available: " + log)
    assert code == ps.PS_OK, log


# The grids the tiled entry stages: read off the centre and never emitted;
# literal offsets set the halo, other coordinate expressions widen it to 1.
STAGES = {"branchy": "staged in 1 0 0 clamp;", "clamped": "",
          "mix7": "staged src 1 1 1 clamp;", "line3": "staged a 1 0 0 clamp;",
          "axes": "staged a 1 1 1 clamp;", "planes": "staged a 1 1 1 clamp;",
          "wrap27": "staged a 1 1 1 periodic;", "rb7": "", "three": "", "nine": "",
          "weighted": "staged a 1 1 2 clamp;"}


@pytest.mark.parametrize("src,name", GOOD, ids=[g[1] for g in GOOD])
def test_staged_grids(built, src, name):
    code, log = ps.stencil_function_check(src, name)
    if code == ps.PS_ERR_UNSUPPORTED:
        pytest.skip("NVRTC not available: " + log)
    assert code == ps.PS_OK
    assert log == STAGES[name]


def test_staging_caps_and_budget(built):
    # halos are capped at 4 (reads beyond come from global memory); grids
    # are staged in parameter order while the 96 KB budget lasts
    src = r"""
void far(const int x, const int y, const int z, PSGrid3DDouble a, PSGrid3DDouble b,
         PSGrid3DDouble c, PSGrid3DDouble out) {
  PSGridEmit(out, PSGridGet(a, x + 6, y, z - 4) + PSGridGet(b, x, y + 2, z + 3)
                  + PSGridGet(c, x - 1, y, z));
}
"""
    code, log = ps.stencil_function_check(src, "far")
    if code == ps.PS_ERR_UNSUPPORTED:
        pytest.skip("NVRTC not available: " + log)
    assert code == ps.PS_OK, log
    # rings of 2 rz + 5 planes: a (13 planes x 72 x 16 x 8 B = 117 KB) and b
    # (11 x 64 x 20 x 8 B = 110 KB) are over the budget; c (5 x 66 x 16 x 8 B
    # = 41 KB) fits
    assert log == "staged c 1 0 0 clamp;"


@pytest.mark.parametrize("src,name,why", [
    ("void f(const int x, PSGrid1DFloat a, PSGrid1DFloat b) { PSGridEmit(b, nope); }", "f",
     "does not compile"),
    ("void f(const int x, struct thing *t) { }", "f", "not supported"),
    ("void g(const int x, PSGrid1DFloat a) { }", "f", "no definition"),
    ("void f(PSGrid1DFloat a, PSGrid1DFloat b) { }", "f", "no index parameters"),
    ("void f(const int x, float s, PSGrid1DFloat a) { }", "f", "index parameters must"),
    ("void f(const int x, const int y) { }", "f", "takes no grid"),
])
def test_malformed_stencil_functions_are_rejected(built, src, name, why):
    code, log = ps.stencil_function_check(src, name)
    if code == ps.PS_ERR_UNSUPPORTED:
        pytest.skip("NVRTC not available: " + log)
    assert code == ps.PS_ERR_INVALID_ARGUMENT
    assert why in log, log


@pytest.mark.parametrize("src,name,staged", [
    # int and long grids, offsets up to 2
    ("void i5(const int x, const int y, const int z, PSGrid3DInt a, PSGrid3DInt b) {\n"
     "  PSGridEmit(b, PSGridGet(a, x + 2, y, z) + PSGridGet(a, x, y - 2, z) * 3);\n}\n",
     "i5", "staged a 2 2 0 clamp;"),
    ("void l3(const int x, const int y, const int z, PSGrid3DLong a, PSGrid3DLong b) {\n"
     "  PSGridEmit(b, PSGridGet(a, x, y, z + 1) - PSGridGet(a, x, y, z - 1));\n}\n",
     "l3", "staged a 0 0 1 clamp;"),
    # reads through a macro: not literal in the function body, halo 1
    ("#define NB(g, dx) PSGridGet(g, x + dx, y, z)\n"
     "void m3(const int x, const int y, const int z, PSGrid3DFloat a, PSGrid3DFloat b) {\n"
     "  PSGridEmit(b, NB(a, -1) + NB(a, 0) + NB(a, 1));\n}\n",
     "m3", ""),
    # different index names
    ("void ijk(const int i, const int j, const int k, PSGrid3DDouble u, PSGrid3DDouble v,\n"
     "         double c) {\n"
     "  PSGridEmit(v, c * (PSGridGet(u, i + 1, j, k) + PSGridGet(u, i, j, k - 3)));\n}\n",
     "ijk", "staged u 1 0 3 clamp;"),
    # a grid read only at the centre is not staged; an emitted one never is
    ("void c1(const int x, const int y, const int z, PSGrid3DFloat a, PSGrid3DFloat s,\n"
     "        PSGrid3DFloat b) {\n"
     "  PSGridEmit(b, PSGridGet(a, x - 1, y, z) * PSGridGet(s, x, y, z));\n}\n",
     "c1", "staged a 1 0 0 clamp;"),
])
def test_staging_decisions_and_compiles(built, src, name, staged):
    code, log = ps.stencil_function_check(src, name)
    if code == ps.PS_ERR_UNSUPPORTED:
        pytest.skip("NVRTC not available: " + log)
    assert code == ps.PS_OK, log
    assert log == staged


# Stencil functions over grids of user-defined struct types: they compile
# for sm_103a, and no user-type grid is staged (PSGridEmitUtype counts as an
# emit, and struct elements are not staged at all).
import test_gpu_user_types as ut  # noqa: E402

USER = [(ut.SEVEN_PT, "seven"), (ut.COMPLEX, "csum"), (ut.ARRAY_MEMBER, "am"),
        (ut.MULTI_DIM, "md"), (ut.MULTI_MEMBERS, "mm"), (ut.XYZ, "xyz"), (ut.PQR, "k1"),
        (ut.PQR, "k2")]


@pytest.mark.parametrize("src,name", USER, ids=[u[1] for u in USER])
def test_user_type_functions_compile_unstaged(built, src, name):
    code, log = ps.stencil_function_check(src, name)
    if code == ps.PS_ERR_UNSUPPORTED:
        pytest.skip("NVRTC not available: " + log)
    assert code == ps.PS_OK, log
    assert "staged" not in log, log


def test_user_type_c_program_compiles_and_links(built, tmp_path):
    from test_abi import compile_c_program
    assert compile_c_program(tmp_path, ut.C_UTYPE_PROGRAM, "utype").exists()
