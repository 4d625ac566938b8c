"""physis_gb300: GB300-native Physis stencil runtime (single GPU, sm_103a).

The product is the C library libphysis_gb300.so (C ABI in
include/physis_gb300/physis.h and physis_gb300.h).  This module loads it
with ctypes and offers thin Python wrappers of the same calls for tests and
benchmarks.  There is no CPU fallback: if the library is missing, every call
raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libphysis_gb300.so")

# enums of include/physis_gb300/physis.h
PS_INT, PS_LONG, PS_FLOAT, PS_DOUBLE, PS_USER = 0, 1, 2, 3, 4
PS_MAX, PS_MIN, PS_SUM, PS_PROD = 0, 1, 2, 3
PS_KERNEL_COPY = 1
PS_KERNEL_DIFFUSION7 = 2
PS_KERNEL_HIMENO19 = 3
PS_KERNEL_HIMENO19_GOSA = 4
PS_KERNEL_SUM7 = 5
PS_RUN_END = -(2 ** 31)
# enums of include/physis_gb300/physis_gb300.h (point stencils, map colours)
BOUNDARY_NONE, BOUNDARY_PERIODIC, BOUNDARY_CLAMP = 0, 1, 2
COLOR_ALL, COLOR_RED, COLOR_BLACK, COLOR_REDBLACK = -1, 0, 1, 2

PS_OK = 0
ERROR_NAMES = {
    0: "PS_OK", 1: "PS_ERR_NOT_INITIALIZED", 2: "PS_ERR_INVALID_ARGUMENT",
    3: "PS_ERR_OUT_OF_MEMORY", 4: "PS_ERR_CUDA", 5: "PS_ERR_UNKNOWN_KERNEL",
    6: "PS_ERR_BAD_HANDLE", 7: "PS_ERR_UNSUPPORTED", 8: "PS_ERR_DEVICE_TIMEOUT",
    9: "PS_ERR_NO_DEVICE", 10: "PS_ERR_IO"}
for _c, _n in ERROR_NAMES.items():
    globals()[_n] = _c

DTYPE_OF = {PS_INT: np.int32, PS_LONG: np.int64, PS_FLOAT: np.float32,
            PS_DOUBLE: np.float64}
TYPE_OF = {np.dtype(v): k for k, v in DTYPE_OF.items()}

# Every symbol the C headers declare (checked by the CPU test suite).
EXPORTED = """PSInit PSFinalize PSPrintInternalInfo
PSGrid1DFloatNew PSGrid1DDoubleNew PSGrid1DIntNew PSGrid1DLongNew
PSGrid2DFloatNew PSGrid2DDoubleNew PSGrid2DIntNew PSGrid2DLongNew
PSGrid3DFloatNew PSGrid3DDoubleNew PSGrid3DIntNew PSGrid3DLongNew
PSGridNewUtype PSGridCopyin PSGridCopyout PSGridFree PSGridDim __PSGridSet __PSGridSetScalar PSGridSetV
PSDomain1DNew PSDomain2DNew PSDomain3DNew __PSStencilMap PSStencilRun PSReduce
PSInitV PSGridNewV PSStencilMapV PSStencilRunV PSReduceGridV PSReduceKernelV
PSReduceGridF64 PSGetLastError PSGetLastErrorString PSGetErrorName PSClearError
PSGridDevicePtr PSGridPitch PSGridElemSize PSGridType PSGridCopyinAsync
PSGridCopyoutAsync PSHostAlloc PSHostFree PSSynchronize PSGetStream
PSEventRecord PSEventElapsedMs PSGetLaunchCount PSGetSMCount PSSetLaunchShape
PSGetLaunchShape PSTestFailNextAllocs PSTestDeviceWaitTimeout PSReduceNoAlloc
PSSetTemporalBlocking PSGetTemporalBlocking PSSetFusedMultiplyAdd PSGetFusedMultiplyAdd
PSSetAutotune PSSetTuneCachePath
PSLoadTuneCache PSClearTuning PSGetStencilPlan PSBatchCreate PSBatchRun PSBatchFree
PSSetBatchShape __PSStencilMapRedBlack __PSStencilMapRed __PSStencilMapBlack
PSStencilMapColorV PSPointStencilNew PSStencilFunctionNew
PSStencilFunctionCheck PSWarmStartConv PSWarmStartWeightGrad PSWarmStartPrepareWeights
PSWarmStartAdam PSWarmStartLoss PSWarmStartPool PSWarmStartPoolTarget
PSWarmStartUpsample PSWarmStartUpsampleAdd PSWarmStartResidualSource
PSWarmStartAddCorrection""".split()


class PSDomain(ctypes.Structure):
    """__PSDomain (include/physis/physis_common.h:88-103)."""
    _fields_ = [("min", ctypes.c_int32 * 3), ("max", ctypes.c_int32 * 3),
                ("local_min", ctypes.c_int32 * 3),
                ("local_max", ctypes.c_int32 * 3)]


class PSLaunchShape(ctypes.Structure):
    _fields_ = [("warps", ctypes.c_int), ("rows", ctypes.c_int),
                ("ns", ctypes.c_int), ("ns2", ctypes.c_int),
                ("ctas_per_sm", ctypes.c_int)]


class PSWarmStartFields(ctypes.Structure):
    """PSWarmStartFields (include/physis_gb300/physis_gb300.h)."""
    _fields_ = [("a0", ctypes.c_void_p), ("a1", ctypes.c_void_p), ("a2", ctypes.c_void_p),
                ("wrk1", ctypes.c_void_p), ("bnd", ctypes.c_void_p), ("p", ctypes.c_void_p),
                ("pitch", ctypes.c_longlong), ("ny", ctypes.c_int), ("inx", ctypes.c_int),
                ("iny", ctypes.c_int), ("inz", ctypes.c_int), ("nsx", ctypes.c_int),
                ("factor", ctypes.c_int), ("batch", ctypes.c_int), ("wscale", ctypes.c_float),
                ("pscale", ctypes.c_float), ("flip", ctypes.c_int),
                ("inst_scale", ctypes.c_void_p), ("p_sub", ctypes.c_void_p)]


class PSError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


_lib = None


def build():
    from physis_gb300 import buildlib
    return buildlib.build()


def lib():
    """The loaded C library.  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(LIB_PATH)
    vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    L.PSInitV.argtypes = [i]
    L.PSInitV.restype = None
    L.PSFinalize.argtypes = []
    L.PSGridNewV.argtypes = [i, i, ctypes.POINTER(ctypes.c_int32)]
    L.PSGridNewV.restype = vp
    L.PSGridNewUtype.argtypes = [ctypes.c_size_t, i, ctypes.POINTER(ctypes.c_int32)]
    L.PSGridNewUtype.restype = vp
    L.PSGridCopyin.argtypes = [vp, vp]
    L.PSGridCopyout.argtypes = [vp, vp]
    L.PSGridCopyinAsync.argtypes = [vp, vp]
    L.PSGridCopyoutAsync.argtypes = [vp, vp]
    L.PSGridFree.argtypes = [vp]
    L.PSGridDim.argtypes = [vp, i]
    L.PSGridDim.restype = ctypes.c_int32
    L.PSGridSetV.argtypes = [vp, ctypes.POINTER(ctypes.c_int32), vp]
    L.PSGridSetV.restype = i
    L.PSDomain3DNew.argtypes = [ctypes.c_int32] * 6
    L.PSDomain3DNew.restype = PSDomain
    L.PSStencilMapV.argtypes = [i, ctypes.POINTER(PSDomain), i,
                                ctypes.POINTER(vp), i, ctypes.POINTER(d)]
    L.PSStencilMapV.restype = i
    L.PSStencilRunV.argtypes = [i, ctypes.POINTER(i), i]
    L.PSReduceGridV.argtypes = [vp, i, vp]
    L.PSReduceGridF64.argtypes = [ctypes.POINTER(d), i, vp]
    L.PSReduceKernelV.argtypes = [vp, i, i, ctypes.POINTER(PSDomain), i,
                                  ctypes.POINTER(vp), i, ctypes.POINTER(d)]
    L.PSGetLastError.restype = i
    L.PSGetLastErrorString.restype = ctypes.c_char_p
    L.PSGetErrorName.argtypes = [i]
    L.PSGetErrorName.restype = ctypes.c_char_p
    L.PSGridDevicePtr.argtypes = [vp]
    L.PSGridDevicePtr.restype = vp
    L.PSGridPitch.argtypes = [vp]
    L.PSGridPitch.restype = ctypes.c_size_t
    L.PSGridElemSize.argtypes = [vp]
    L.PSGridType.argtypes = [vp]
    L.PSHostAlloc.argtypes = [ctypes.c_size_t]
    L.PSHostAlloc.restype = vp
    L.PSHostFree.argtypes = [vp]
    L.PSGetStream.restype = vp
    L.PSEventRecord.argtypes = [i]
    L.PSEventElapsedMs.argtypes = [i, i]
    L.PSEventElapsedMs.restype = ctypes.c_float
    L.PSGetLaunchCount.restype = ctypes.c_longlong
    L.PSGetSMCount.restype = i
    L.PSSetLaunchShape.argtypes = [i, ctypes.POINTER(PSLaunchShape)]
    L.PSGetLaunchShape.argtypes = [i, ctypes.POINTER(PSLaunchShape)]
    L.PSTestFailNextAllocs.argtypes = [i]
    L.PSTestDeviceWaitTimeout.argtypes = [ctypes.c_uint]
    L.PSSetTemporalBlocking.argtypes = [i, i, ctypes.POINTER(PSLaunchShape)]
    L.PSGetTemporalBlocking.argtypes = [i, ctypes.POINTER(i), ctypes.POINTER(PSLaunchShape)]
    L.PSSetAutotune.argtypes = [i]
    L.PSSetTuneCachePath.argtypes = [ctypes.c_char_p]
    L.PSLoadTuneCache.argtypes = [ctypes.c_char_p]
    L.PSLoadTuneCache.restype = i
    L.PSGetStencilPlan.argtypes = [i, ctypes.POINTER(PSLaunchShape), ctypes.POINTER(i),
                                   ctypes.POINTER(PSLaunchShape)]
    L.PSGetStencilPlan.restype = i
    L.PSBatchCreate.argtypes = [i, i, ctypes.POINTER(i)]
    L.PSBatchCreate.restype = i
    L.PSBatchRun.argtypes = [i, i]
    L.PSBatchFree.argtypes = [i]
    L.PSSetBatchShape.argtypes = [i, i, i, i, i]
    L.PSReduceNoAlloc.argtypes = [vp, ctypes.c_size_t, i, i, i, i, i, vp, vp]
    L.PSReduceNoAlloc.restype = i
    L.PSPointStencilNew.argtypes = [i, i, ctypes.POINTER(i), ctypes.POINTER(d)]
    L.PSPointStencilNew.restype = i
    L.PSStencilMapColorV.argtypes = [i, i, ctypes.POINTER(PSDomain), i,
                                     ctypes.POINTER(vp), i, ctypes.POINTER(d)]
    L.PSStencilMapColorV.restype = i
    L.PSStencilFunctionNew.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    L.PSStencilFunctionNew.restype = i
    L.PSStencilFunctionCheck.argtypes = [ctypes.c_char_p, ctypes.c_char_p,
                                         ctypes.c_char_p, ctypes.c_size_t]
    L.PSStencilFunctionCheck.restype = i
    L.PSWarmStartConv.argtypes = [vp, vp, vp, vp, i, vp, vp, i, i, i, i, vp]
    L.PSWarmStartWeightGrad.argtypes = [vp, vp, vp, i, vp, vp, i, i, i, i, vp]
    L.PSWarmStartPrepareWeights.argtypes = [vp, vp, vp, vp]
    L.PSWarmStartAdam.argtypes = [vp, vp, vp, vp, ctypes.c_longlong, ctypes.c_float,
                                  ctypes.c_float, ctypes.c_float, ctypes.c_float, i, vp]
    L.PSWarmStartLoss.argtypes = [vp, vp, ctypes.c_longlong, vp, vp, vp]
    fp = ctypes.POINTER(PSWarmStartFields)
    L.PSWarmStartPool.argtypes = [fp, vp, vp]
    L.PSWarmStartPoolTarget.argtypes = [fp, vp, vp]
    L.PSWarmStartUpsample.argtypes = [fp, vp, vp, vp]
    L.PSWarmStartUpsampleAdd.argtypes = [fp, vp, vp, vp]
    L.PSWarmStartResidualSource.argtypes = [fp, vp, vp, ctypes.c_float, vp, i, vp]
    L.PSWarmStartAddCorrection.argtypes = [fp, vp, ctypes.c_float, vp, vp]
    for name in ("PSWarmStartConv", "PSWarmStartWeightGrad", "PSWarmStartPrepareWeights",
                 "PSWarmStartAdam", "PSWarmStartLoss", "PSWarmStartPool",
                 "PSWarmStartPoolTarget", "PSWarmStartUpsample", "PSWarmStartUpsampleAdd",
                 "PSWarmStartResidualSource", "PSWarmStartAddCorrection"):
        getattr(L, name).restype = i
    _lib = L
    return L


# ---- thin wrappers --------------------------------------------------------

def last_error():
    L = lib()
    return L.PSGetLastError(), (L.PSGetLastErrorString() or b"").decode()


def clear_error():
    lib().PSClearError()


def check():
    """Raise PSError if the library recorded an error (and clear it)."""
    code, msg = last_error()
    if code != PS_OK:
        clear_error()
        raise PSError(code, msg)


def init(trace=False):
    lib().PSInitV(1 if trace else 0)
    check()


def finalize():
    lib().PSFinalize()


def domain(minx, maxx, miny, maxy, minz, maxz):
    return lib().PSDomain3DNew(minx, maxx, miny, maxy, minz, maxz)


def full_domain(shape):
    nz, ny, nx = shape
    return domain(0, nx, 0, ny, 0, nz)


class Grid:
    """A device grid; shape is (nz, ny, nx) like the numpy arrays it mirrors."""

    def __init__(self, shape, dtype=np.float32):
        self.dtype = np.dtype(dtype)
        shape = tuple(int(s) for s in shape)
        self.shape = shape
        dims = list(reversed(shape)) + [1] * (3 - len(shape))
        arr = (ctypes.c_int32 * 3)(*dims)
        if self.dtype.fields is not None:  # a struct: a user-defined element type
            self.handle = lib().PSGridNewUtype(self.dtype.itemsize, len(shape), arr)
        else:
            self.handle = lib().PSGridNewV(TYPE_OF[self.dtype], len(shape), arr)
        if not self.handle:
            check()
            raise PSError(PS_ERR_OUT_OF_MEMORY, "grid allocation failed")

    @property
    def nbytes(self):
        return int(np.prod(self.shape)) * self.dtype.itemsize

    def copyin(self, arr):
        a = np.ascontiguousarray(arr, dtype=self.dtype)
        assert a.shape == self.shape, (a.shape, self.shape)
        lib().PSGridCopyin(self.handle, a.ctypes.data_as(ctypes.c_void_p))
        check()

    def copyout(self, out=None):
        if out is None:
            out = np.empty(self.shape, dtype=self.dtype)
        assert out.flags["C_CONTIGUOUS"] and out.dtype == self.dtype
        lib().PSGridCopyout(self.handle, out.ctypes.data_as(ctypes.c_void_p))
        check()
        return out

    def set(self, index, value):
        """PSGridSet: one element; index is (x, y, z) truncated to the
        grid's rank (x first, as the reference's PSGridSet takes it)."""
        idx = (ctypes.c_int32 * 3)(*(list(index) + [0] * (3 - len(index))))
        v = np.array([value], dtype=self.dtype)
        rc = lib().PSGridSetV(self.handle, idx, v.ctypes.data_as(ctypes.c_void_p))
        if rc != PS_OK:
            check()
            raise PSError(rc, "PSGridSetV failed")

    def free(self):
        if self.handle:
            lib().PSGridFree(self.handle)
            self.handle = None

    @property
    def dev_ptr(self):
        return lib().PSGridDevicePtr(self.handle)

    @property
    def pitch(self):
        return lib().PSGridPitch(self.handle)


def stencil_map(kernel, dom, grids, scalars=()):
    n = len(grids)
    garr = (ctypes.c_void_p * max(n, 1))(*[g.handle for g in grids])
    sarr = (ctypes.c_double * max(len(scalars), 1))(*[float(s) for s in scalars])
    s = lib().PSStencilMapV(kernel, ctypes.byref(dom), n, garr, len(scalars),
                            sarr)
    check()
    return s


def point_stencil(points, weights=None, boundary=BOUNDARY_NONE):
    """Registers a point-list stencil; returns its kernel id.

    points: sequence of (dx, dy, dz) in summation order; weights: None for a
    plain sum, else one weight per point.
    """
    n = len(points)
    offs = (ctypes.c_int * (3 * n))(*[int(v) for p in points for v in p])
    w = None if weights is None else (ctypes.c_double * n)(
        *[float(v) for v in weights])
    k = lib().PSPointStencilNew(boundary, n, offs, w)
    check()
    return k


def stencil_function(source, name):
    """Compiles a stencil function (the reference's stencil language) with
    NVRTC; returns its kernel id."""
    k = lib().PSStencilFunctionNew(source.encode(), name.encode())
    check()
    return k


def stencil_function_check(source, name):
    """(code, log) of compiling a stencil function without a device."""
    buf = ctypes.create_string_buffer(4096)
    code = lib().PSStencilFunctionCheck(source.encode(), name.encode(), buf, len(buf))
    return code, buf.value.decode(errors="replace")


def stencil_map_color(kernel, color, dom, grids, scalars=()):
    """A red (0) / black (1) / red-then-black (2) map, or -1 = PSStencilMapV."""
    n = len(grids)
    garr = (ctypes.c_void_p * max(n, 1))(*[g.handle for g in grids])
    sarr = (ctypes.c_double * max(len(scalars), 1))(*[float(s) for s in scalars])
    s = lib().PSStencilMapColorV(kernel, color, ctypes.byref(dom), n, garr,
                                 len(scalars), sarr)
    check()
    return s


def stencil_run(stencils, iter=1):
    arr = (ctypes.c_int * len(stencils))(*stencils)
    lib().PSStencilRunV(len(stencils), arr, iter)
    check()


def reduce(grid, op):
    out = np.zeros(1, dtype=grid.dtype)
    lib().PSReduceGridV(out.ctypes.data_as(ctypes.c_void_p), op, grid.handle)
    check()
    return out[0]


def reduce_f64(grid, op):
    out = ctypes.c_double(0.0)
    lib().PSReduceGridF64(ctypes.byref(out), op, grid.handle)
    check()
    return out.value


def reduce_kernel(op, kernel, dom, grids, scalars=()):
    out = np.zeros(1, dtype=np.float32)
    n = len(grids)
    garr = (ctypes.c_void_p * n)(*[g.handle for g in grids])
    sarr = (ctypes.c_double * max(len(scalars), 1))(*[float(s) for s in scalars])
    lib().PSReduceKernelV(out.ctypes.data_as(ctypes.c_void_p), op, kernel,
                          ctypes.byref(dom), n, garr, len(scalars), sarr)
    check()
    return out[0]


def synchronize():
    lib().PSSynchronize()
    check()


def set_launch_shape(kernel, warps=0, rows=0, ns=0, ns2=0, ctas_per_sm=0):
    sh = PSLaunchShape(warps, rows, ns, ns2, ctas_per_sm)
    lib().PSSetLaunchShape(kernel, ctypes.byref(sh))
    check()


def get_launch_shape(kernel):
    """(warps, rows, ns, ns2, ctas_per_sm) of a kernel's launch shape."""
    sh = PSLaunchShape()
    lib().PSGetLaunchShape(kernel, ctypes.byref(sh))
    return sh.warps, sh.rows, sh.ns, sh.ns2, sh.ctas_per_sm


def set_temporal(kernel, k, warps=0, rows=0, ns=0, ctas_per_sm=0):
    """Temporal blocking depth k (1 = off) and the passes' launch shape."""
    sh = PSLaunchShape(warps, rows, ns, 0, ctas_per_sm)
    lib().PSSetTemporalBlocking(kernel, k, ctypes.byref(sh))
    check()


def set_fma(on):
    """Allow temporal passes to contract multiply-adds (PSSetFusedMultiplyAdd)."""
    lib().PSSetFusedMultiplyAdd(1 if on else 0)
    check()


def get_temporal(kernel):
    """(k, (warps, rows, ns, ctas_per_sm)) of a kernel's temporal blocking."""
    k = ctypes.c_int(0)
    sh = PSLaunchShape()
    lib().PSGetTemporalBlocking(kernel, ctypes.byref(k), ctypes.byref(sh))
    return k.value, (sh.warps, sh.rows, sh.ns, sh.ctas_per_sm)


def set_autotune(on=True, cache_path=None):
    L = lib()
    if cache_path is not None:
        L.PSSetTuneCachePath(cache_path.encode())
    L.PSSetAutotune(1 if on else 0)
    check()


def stencil_plan(s):
    """(tuned?, (warps, rows, ns, ns2, ctas), k, temporal shape) of a stencil."""
    sh, tsh, k = PSLaunchShape(), PSLaunchShape(), ctypes.c_int(0)
    tuned = lib().PSGetStencilPlan(s, ctypes.byref(sh), ctypes.byref(k),
                                   ctypes.byref(tsh))
    check()
    return (bool(tuned), (sh.warps, sh.rows, sh.ns, sh.ns2, sh.ctas_per_sm), k.value,
            (tsh.warps, tsh.rows, tsh.ns))


def batch_create(runs):
    """runs: list of stencil lists (all of the same length, 1 or 2)."""
    m = len(runs[0])
    flat = [s for r in runs for s in r]
    arr = (ctypes.c_int * len(flat))(*flat)
    b = lib().PSBatchCreate(len(runs), m, arr)
    check()
    return b


def batch_run(b, iter):
    lib().PSBatchRun(b, iter)
    check()


def batch_free(b):
    lib().PSBatchFree(b)
    check()


def launch_count():
    return lib().PSGetLaunchCount()
