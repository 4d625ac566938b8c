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
