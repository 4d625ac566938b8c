"""C-ABI boundary checks that need no GPU.

* the library builds, loads and exports every function that
  include/physis_gb300/*.h declares;
* a C program written like the reference's own test programs compiles
  against the headers and links against the library unchanged;
* host-side argument checking and error reporting work without a device.
"""
import ctypes
import os
import re
import subprocess

import pytest

import physis_gb300 as ps

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


def _declared_functions():
    names = set()
    for h in ("physis.h", "physis_gb300.h"):
        src = open(os.path.join(INC, "physis_gb300", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = src.replace("\\\n", " ")  # macro continuation lines
        src = re.sub(r"^\s*#.*$", "", src, flags=re.M)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{}]*)\)\s*;", src):
            name = m.group(1)
            if name not in ("if", "while", "for", "sizeof"):
                names.add(name)
    return names


@pytest.fixture(scope="module")
def built_lib():
    ps.build()
    return ps.lib()


def test_every_declared_symbol_is_exported(built_lib):
    declared = _declared_functions()
    assert declared, "no declarations parsed"
    assert declared == set(ps.EXPORTED), declared ^ set(ps.EXPORTED)
    out = subprocess.run(["nm", "-D", "--defined-only", ps.LIB_PATH],
                         capture_output=True, text=True, check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    missing = declared - exported
    assert not missing, missing
    for name in declared:
        assert hasattr(built_lib, name)


def test_library_is_sm103a_only(built_lib):
    # The one -gencode in the build recipe is sm_103a; cuobjdump is not
    # used (the build's own flags are the evidence).
    from physis_gb300 import buildlib as b
    assert b.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_calls_before_init_record_errors(built_lib):
    ps.clear_error()
    built_lib.PSGridDim(None, 0)
    code, msg = ps.last_error()
    assert code == ps.PS_ERR_NOT_INITIALIZED
    assert "before PSInit" in msg
    ps.clear_error()
    assert ps.last_error()[0] == ps.PS_OK


def test_domain_struct_layout(built_lib):
    d = ps.domain(1, 9, 2, 8, 3, 7)
    assert list(d.min) == [1, 2, 3] and list(d.max) == [9, 8, 7]
    assert list(d.local_min) == [1, 2, 3] and list(d.local_max) == [9, 8, 7]
    assert ctypes.sizeof(ps.PSDomain) == 48


def test_error_names(built_lib):
    for code, name in ps.ERROR_NAMES.items():
        assert built_lib.PSGetErrorName(code).decode() == name


def test_abort_on_error_env(tmp_path, built_lib):
    # PS_ABORT_ON_ERROR=1 turns a recorded error into abort(), like the
    # reference's PSAbort/exit on error.
    code = ("import ctypes,sys; L=ctypes.CDLL(sys.argv[1]); "
            "L.PSGridDim.argtypes=[ctypes.c_void_p, ctypes.c_int]; "
            "L.PSGridDim(None, 0)")
    r = subprocess.run(["python", "-c", code, ps.LIB_PATH],
                       env=dict(os.environ, PS_ABORT_ON_ERROR="1"),
                       capture_output=True, text=True)
    assert r.returncode != 0
    assert "PS_ERR_NOT_INITIALIZED" in r.stderr


C_PROGRAM = r"""
#include <stdio.h>
#include <stdlib.h>
#include "physis_gb300/physis.h"
#include "physis_gb300/physis_gb300.h"

#define N 8
int main(int argc, char *argv[]) {
  PSInit(&argc, &argv, 3, N, N, N);
  if (PSGetLastError()) {
    printf("init: %s\n", PSGetErrorName(PSGetLastError()));
    return 3;
  }
  PSGrid3DFloat g1 = PSGrid3DFloatNew(N, N, N);
  PSGrid3DFloat g2 = PSGrid3DFloatNew(N, N, N);
  PSDomain3D d = PSDomain3DNew(0, N, 0, N, 0, N);
  float *in = (float *)malloc(sizeof(float) * N * N * N);
  float *out = (float *)malloc(sizeof(float) * N * N * N);
  int i;
  for (i = 0; i < N * N * N; i++) in[i] = i;
  PSGridCopyin(g1, in);
  float one = 1.0f;
  PSStencilRun(PSStencilMap(PS_KERNEL_DIFFUSION7, d, g1, g2,
                            one, one, one, one, one, one, one));
  PSGridCopyout(g2, out);
  for (i = 0; i < N * N * N; ++i) printf("%f\n", out[i]);
  float v;
  PSReduce(&v, PS_SUM, g2);
  fprintf(stderr, "sum %f\n", v);
  PSGridFree(g1);
  PSGridFree(g2);
  PSFinalize();
  return PSGetLastError() ? 4 : 0;
}
"""


def compile_c_program(tmp_path, src=C_PROGRAM, name="neumann"):
    c = tmp_path / f"{name}.c"
    c.write_text(src)
    exe = tmp_path / name
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", INC, str(c),
                    "-o", str(exe), "-L", os.path.dirname(ps.LIB_PATH),
                    "-lphysis_gb300",
                    "-Wl,-rpath," + os.path.dirname(ps.LIB_PATH)], check=True)
    return exe


def test_reference_style_c_program_compiles_and_links(tmp_path, built_lib):
    exe = compile_c_program(tmp_path)
    assert exe.exists()
