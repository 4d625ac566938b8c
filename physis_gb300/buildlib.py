"""Build recipe for libphysis_gb300.so (sm_103a only).

Compiles each translation unit under physis_gb300/csrc/ with nvcc in
parallel, then links one shared library in-tree at
physis_gb300/libphysis_gb300.so.  Object files go to physis_gb300/_build/.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libphysis_gb300.so")
SOURCES = ["runtime.cpp", "march.cpp", "stencil7.cu", "temporal7.cu", "himeno19.cu",
           "reduce.cu", "batch.cu", "points.cu", "jit.cpp", "nn.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Translation units whose kernels may contract multiply-adds (the warm-start
# network's FP32 epilogues and elementwise kernels); every other unit is
# compiled with contraction off.
CONTRACTING = {"nn.cu"}


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"),
              "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def common_flags():
    return ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
            "-Xcompiler", "-fvisibility=hidden", "-I", os.path.join(ROOT, "include"),
            "-I", CSRC, "-I", BUILD] + ARCH


EMBEDDED = ["ps_arith.cuh", "points_body.cuh"]  # headers NVRTC compiles from memory


def _write_embedded():
    """BUILD/embedded_headers.inc: the headers jit.cpp hands to NVRTC, as
    raw string literals (rewritten only when their text changes)."""
    names = {"ps_arith.cuh": "kEmbedArith", "points_body.cuh": "kEmbedPointsBody"}
    out = ["// Generated by buildlib.py from physis_gb300/csrc; do not edit.\n"]
    for h in EMBEDDED:
        text = open(os.path.join(CSRC, h)).read()
        assert ")PSEMBED" not in text
        out.append(f'static const char *{names[h]} = R"PSEMBED({text})PSEMBED";\n')
    data = "".join(out)
    path = os.path.join(BUILD, "embedded_headers.inc")
    if not os.path.exists(path) or open(path).read() != data:
        with open(path, "w") as f:
            f.write(data)


def _compile(src):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC)
                     if h.endswith((".h", ".cuh"))]
    deps += [os.path.join(BUILD, "embedded_headers.inc")]
    deps += [os.path.join(ROOT, "include", "physis_gb300", h)
             for h in os.listdir(os.path.join(ROOT, "include", "physis_gb300"))]
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d)
                                   for d in deps):
        return obj
    cmd = [nvcc()] + common_flags() + ["-c", path, "-o", obj]
    if src not in CONTRACTING:
        # Bit-exact sweeps: no multiply-add contraction anywhere in these
        # units (their arithmetic is explicit round-to-nearest already; this
        # keeps any plain expression from being fused too).
        cmd += ["-Xptxas", "--fmad=false"]
    if src.endswith(".cpp"):
        cmd += ["-x", "cu"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    _write_embedded()
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(o)
                                   for o in objs):
        return LIB
    cmd = [nvcc(), "-shared"] + ARCH + ["-o", LIB] + objs + ["-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
