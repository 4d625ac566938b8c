"""ctypes binding of the CPU oracle (oracle/ps_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py, and only there as the checker or the timed CPU
baseline.  The product (physis_gb300) never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libps_oracle.so")

# PSPrimitiveType (include/physis/types.h:16-23)
PS_INT, PS_LONG, PS_FLOAT, PS_DOUBLE = 0, 1, 2, 3
# PSReduceOp (include/physis/reduce.h:16-21)
PS_MAX, PS_MIN, PS_SUM, PS_PROD = 0, 1, 2, 3
# 7-point variants (same ids as the library's builtin stencils)
V_DIFFUSION7, V_SUM7, V_SUM7_PERIODIC = 2, 5, 6

NP_OF_TYPE = {PS_INT: np.int32, PS_LONG: np.int64, PS_FLOAT: np.float32,
              PS_DOUBLE: np.float64}
TYPE_OF_NP = {np.dtype(v): k for k, v in NP_OF_TYPE.items()}

_lib = None


def build():
    """Compile libps_oracle.so with the committed recipe (oracle/Makefile)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "libps_oracle.so"])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or (
                os.path.getmtime(LIB_PATH) <
                os.path.getmtime(os.path.join(HERE, "ps_oracle.c"))):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, i, i64, d = (ctypes.c_void_p, ctypes.c_int, ctypes.c_int64,
                         ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        dp = ctypes.POINTER(ctypes.c_double)
        L.pso_sweep7.argtypes = [i, i, vp, vp, i, i, i, ip, dp, i]
        L.pso_run7.argtypes = [i, i, vp, vp, i, i, i, ip, dp, i, i, i]
        L.pso_himeno19.argtypes = [i, ctypes.POINTER(vp), i, i, i, ip, d, i,
                                   ctypes.POINTER(ctypes.c_float), dp]
        L.pso_points.argtypes = [i, i, i, ip, dp, vp, vp, i, i, i, ip, i, i]
        L.pso_reduce_ref.argtypes = [i, i, vp, i64, vp]
        L.pso_reduce_fp64.argtypes = [i, i, vp, i64, dp]
        L.pso_fill_uniform_f32.argtypes = [vp, i64, ctypes.c_uint64, i]
        L.pso_fill_uniform_f32.restype = None
        L.pso_num_threads.restype = i
        _lib = L
    return _lib


def _dom(dom):
    return (ctypes.c_int * 6)(*[int(v) for v in dom])


def _coef(coef):
    c = list(coef) + [0.0] * (7 - len(coef))
    return (ctypes.c_double * 7)(*[float(v) for v in c])


def _ptr(a):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


def num_threads():
    return lib().pso_num_threads()


def sweep7(variant, g1, g2, dom, coef=(), nthreads=1):
    """One REF sweep g2 = stencil(g1) over dom; arrays shaped (nz, ny, nx)."""
    nz, ny, nx = g1.shape
    assert g1.dtype == g2.dtype and g1.shape == g2.shape
    rc = lib().pso_sweep7(variant, TYPE_OF_NP[g1.dtype], _ptr(g1), _ptr(g2),
                          nx, ny, nz, _dom(dom), _coef(coef), nthreads)
    if rc:
        raise ValueError("unsupported variant/type for the oracle")


def run7(variant, g1, g2, dom, coef=(), iter=1, pingpong=True, nthreads=1):
    """REF PSStencilRun of (g1->g2, g2->g1) x iter (or g1->g2 x iter)."""
    nz, ny, nx = g1.shape
    rc = lib().pso_run7(variant, TYPE_OF_NP[g1.dtype], _ptr(g1), _ptr(g2),
                        nx, ny, nz, _dom(dom), _coef(coef), iter,
                        1 if pingpong else 0, nthreads)
    if rc:
        raise ValueError("unsupported variant/type for the oracle")


def points(g_in, g_out, dom, offsets, weights=None, boundary=0, color=-1,
           nthreads=1):
    """REF sweep of a point-list stencil: g_out = sum_i w_i * g_in(p + d_i).

    offsets: sequence of (dx, dy, dz); weights None = plain sum.  boundary:
    0 none, 1 periodic, 2 clamp.  color -1 = every cell (g_out != g_in);
    0 red / 1 black = in-place REF red/black order (pass the same array
    twice).  Arrays are shaped (nz, ny, nx).
    """
    nz, ny, nx = g_in.shape
    assert g_in.dtype == g_out.dtype and g_in.shape == g_out.shape
    n = len(offsets)
    offs = (ctypes.c_int * (3 * n))(*[int(v) for o in offsets for v in o])
    w = None if weights is None else (ctypes.c_double * n)(
        *[float(v) for v in weights])
    rc = lib().pso_points(TYPE_OF_NP[g_in.dtype], boundary, n, offs, w,
                          _ptr(g_in), _ptr(g_out), nx, ny, nz, _dom(dom),
                          color, nthreads)
    if rc:
        raise ValueError("point stencil reads outside the grid, or bad args")


def himeno19(grids, dom, omega, nthreads=1):
    """One REF Himeno sweep; grids = [p0,p1,a0,a1,a2,a3,b0,b1,b2,c0,c1,c2,bnd,wrk1].

    Returns (gosa_ref_float32, gosa_fp64).
    """
    assert len(grids) == 14
    nz, ny, nx = grids[0].shape
    t = TYPE_OF_NP[grids[0].dtype]
    arr = (ctypes.c_void_p * 14)(*[_ptr(g) for g in grids])
    gr = ctypes.c_float(0.0)
    g64 = ctypes.c_double(0.0)
    rc = lib().pso_himeno19(t, arr, nx, ny, nz, _dom(dom), float(omega),
                            nthreads, ctypes.byref(gr), ctypes.byref(g64))
    if rc:
        raise ValueError("unsupported type for the oracle")
    return np.float32(gr.value), g64.value


def reduce_ref(data, op):
    """REF PSReduce: sequential fold in the element type from d[0]."""
    data = np.ascontiguousarray(data)
    out = np.zeros(1, dtype=data.dtype)
    rc = lib().pso_reduce_ref(TYPE_OF_NP[data.dtype], op, _ptr(data),
                              data.size, _ptr(out))
    if rc:
        raise ValueError("bad reduction")
    return out[0]


def reduce_fp64(data, op):
    """FP64 oracle of a float/double reduction."""
    data = np.ascontiguousarray(data)
    out = ctypes.c_double(0.0)
    rc = lib().pso_reduce_fp64(TYPE_OF_NP[data.dtype], op, _ptr(data),
                               data.size, ctypes.byref(out))
    if rc:
        raise ValueError("bad reduction")
    return out.value


def fill_uniform(shape, seed, nthreads=0):
    """uniform[0,1) float32 field from the counter-based SplitMix64 stream."""
    a = np.empty(shape, dtype=np.float32)
    lib().pso_fill_uniform_f32(_ptr(a), a.size, seed, nthreads)
    return a
