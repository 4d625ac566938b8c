"""Parity of the GB300 kernels with the oracle and the reference's outputs.

All tests here run on a GB300 through the C ABI (ctypes).  The bar:
* stencil sweeps: bit-identical to the REF restatement (same expression
  order, round-to-nearest, no FMA contraction on either side);
* system-test programs: exact stdout text of the reference's own oracles;
* float reductions: within 1e-6 relative of the FP64 oracle (the REF fold's
  own error is reported beside it, it is not the criterion); integer reductions
  exact (modulo 2^32 / 2^64 like the REF fold).
"""
import numpy as np
import pytest

import golden_io as gio
import physis_gb300 as ps
from physis_gb300 import synth

pytestmark = pytest.mark.gpu

DIFF_COEF = (0.1, 0.1, 0.1, 0.1, 0.1, 0.1, 0.4)  # ce cw cn cs ct cb cc


@pytest.fixture(scope="module")
def rt():
    ps.build()
    ps.init()
    yield ps
    ps.clear_error()


def _iota(n, dtype):
    return np.arange(n ** 3, dtype=np.int64).astype(dtype).reshape(n, n, n)


def _bits(a):
    return a.view(np.uint32 if a.dtype.itemsize == 4 else np.uint64)


def run_pingpong(kernel, init, dom, scalars, iters, dtype=np.float32, out0=None):
    g1, g2 = ps.Grid(init.shape, dtype), ps.Grid(init.shape, dtype)
    g1.copyin(init)
    g2.copyin(init if out0 is None else out0)
    m1 = ps.stencil_map(kernel, dom, [g1, g2], scalars)
    m2 = ps.stencil_map(kernel, dom, [g2, g1], scalars)
    ps.stencil_run([m1, m2], iters)
    a, b = g1.copyout(), g2.copyout()
    g1.free()
    g2.free()
    return a, b


# ---- the reference's system tests (exact stdout) ---------------------------

@pytest.mark.parametrize("test,dtype,fmt", [
    ("test_7-pt", np.float32, "%f"),
    ("test_7-pt-double-type", np.float64, "%f"),
    ("test_7-pt-int-type", np.int32, "%d"),
])
def test_system_sum7(rt, test, dtype, fmt):
    n = 32
    g1, g2 = ps.Grid((n, n, n), dtype), ps.Grid((n, n, n), dtype)
    g1.copyin(_iota(n, dtype))
    g2.copyin(_iota(n, dtype))
    s = ps.stencil_map(ps.PS_KERNEL_SUM7, ps.domain(1, n - 1, 1, n - 1, 1, n - 1),
                       [g1, g2])
    ps.stencil_run([s])
    assert gio.dump_text(g2.copyout(), fmt) == gio.stdout_text(test)
    g1.free()
    g2.free()


def test_system_multi_iterations(rt):
    n = 32
    a, _ = run_pingpong(ps.PS_KERNEL_SUM7, _iota(n, np.float32),
                        ps.domain(1, n - 1, 1, n - 1, 1, n - 1), (), 5)
    assert gio.dump_text(a) == gio.stdout_text("test_7-pt-multi-iterations")


def test_system_neumann(rt):
    n = 8
    g1, g2 = ps.Grid((n, n, n)), ps.Grid((n, n, n))
    g1.copyin(_iota(n, np.float32))
    s = ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, ps.full_domain((n, n, n)),
                       [g1, g2], [1.0] * 7)
    ps.stencil_run([s])
    assert gio.dump_text(g2.copyout()) == gio.stdout_text("test_7-pt-neumann-cond")


def test_system_reduction_sum(rt):
    g = ps.Grid((16, 16, 16))
    g.copyin(np.arange(16 ** 3, dtype=np.float32).reshape(16, 16, 16))
    v = ps.reduce(g, ps.PS_SUM)
    assert "%f\n" % float(v) == gio.stdout_text("test_reduction-3d-sum")
    g.free()


# ---- the reference's benchmark programs (bit-exact) ------------------------

def test_diffusion_matches_reference_baseline(rt):
    n = 21
    init = gio.f32("diffusion_ref_n21_c6.init.f32.gz", (n, n, n))
    final = gio.f32("diffusion_ref_n21_c6.final.f32.gz", (n, n, n))
    coef = gio.hexfloats("diffusion_ref_n21_c6.coef.txt")
    a, _ = run_pingpong(ps.PS_KERNEL_DIFFUSION7, init, ps.full_domain(init.shape),
                        coef, 3)
    assert np.array_equal(_bits(a), _bits(final))


def himeno_grids(shape, arrays):
    gs = [ps.Grid(shape) for _ in range(14)]
    for g, a in zip(gs, arrays):
        g.copyin(a)
    return gs


def test_himeno_matches_original(rt):
    from test_oracle_golden import himeno_inputs
    nz, ny, nx = 33, 17, 19
    arrays = himeno_inputs(nx, ny, nz)
    gs = himeno_grids((nz, ny, nx), arrays)
    dom = ps.domain(1, nx - 1, 1, ny - 1, 1, nz - 1)
    p0, p1 = gs[0], gs[1]
    gosa = None
    for s in range(3):
        args = [p0, p1] + gs[2:]
        gosa = ps.reduce_kernel(ps.PS_SUM, ps.PS_KERNEL_HIMENO19_GOSA, dom, args,
                                [np.float32(0.8)])
        p0, p1 = p1, p0
    ref_p = gio.f32("himeno_ref_33x17x19_nn3.p.f32.gz", (nz, ny, nx))
    assert np.array_equal(_bits(p0.copyout()), _bits(ref_p))
    # gosa: FP64-combined sum vs the oracle's FP64 sum of the same ss terms
    g = [a.copy() for a in arrays]
    for s in range(3):
        _, g64 = pytest.importorskip("oracle.pyoracle").himeno19(
            g, (1, nx - 1, 1, ny - 1, 1, nz - 1), np.float32(0.8))
        g[0], g[1] = g[1], g[0]
    assert abs(float(gosa) - g64) <= 1e-6 * abs(g64)
    ref_gosa = gio.hexfloats("himeno_ref_33x17x19_nn3.gosa.txt")[0]
    assert abs(float(gosa) - ref_gosa) <= 1e-4 * abs(ref_gosa)
    for x in gs:
        x.free()


# ---- seeded configurations vs the oracle -----------------------------------

def test_diffusion_64cubed_100_steps_then_reduce(rt, oracle):
    # 64^3 uniform[0,1) seed 0, cc=0.4 others 0.1, clamped, 100 steps
    # (50 x 2 maps), then PSReduce sum: cell-by-cell bit-exact vs REF.
    shape = (64, 64, 64)
    init = synth.uniform(shape, 0)
    a, b = run_pingpong(ps.PS_KERNEL_DIFFUSION7, init, ps.full_domain(shape),
                        DIFF_COEF, 50)
    r1, r2 = init.copy(), np.zeros_like(init)
    oracle.run7(oracle.V_DIFFUSION7, r1, r2, (0, 64, 0, 64, 0, 64), DIFF_COEF,
                iter=50, nthreads=0)
    assert np.array_equal(_bits(a), _bits(r1))
    assert np.array_equal(_bits(b), _bits(r2))
    g = ps.Grid(shape)
    g.copyin(a)
    v = ps.reduce(g, ps.PS_SUM)
    v64 = ps.reduce_f64(g, ps.PS_SUM)
    exact = oracle.reduce_fp64(r1, oracle.PS_SUM)
    assert abs(v64 - exact) <= 1e-6 * abs(exact)
    assert abs(float(v) - exact) <= 1e-6 * abs(exact)
    g.free()


SHAPES = [(9, 17, 33), (5, 3, 130), (1, 1, 7), (40, 67, 45), (2, 130, 4),
          (16, 16, 256)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_diffusion_ragged_shapes(rt, oracle, shape, dtype):
    init = synth.uniform(shape, 3).astype(dtype)
    a, b = run_pingpong(ps.PS_KERNEL_DIFFUSION7, init, ps.full_domain(shape),
                        DIFF_COEF, 2, dtype)
    r1, r2 = init.copy(), np.zeros_like(init)
    nz, ny, nx = shape
    oracle.run7(oracle.V_DIFFUSION7, r1, r2, (0, nx, 0, ny, 0, nz), DIFF_COEF,
                iter=2)
    assert np.array_equal(_bits(a), _bits(r1))
    assert np.array_equal(_bits(b), _bits(r2))


@pytest.mark.parametrize("dom", [(1, 40, 2, 30, 3, 20), (5, 6, 0, 31, 0, 1),
                                 (0, 0, 0, 31, 0, 21), (7, 41, 13, 14, 2, 19)])
def test_diffusion_subdomains_leave_outside_untouched(rt, oracle, dom):
    shape = (21, 31, 41)
    init = synth.uniform(shape, 4)
    other = synth.uniform(shape, 5)
    a, b = run_pingpong(ps.PS_KERNEL_DIFFUSION7, init, ps.domain(*dom),
                        DIFF_COEF, 3, out0=other)
    r1, r2 = init.copy(), other.copy()
    oracle.run7(oracle.V_DIFFUSION7, r1, r2, dom, DIFF_COEF, iter=3)
    assert np.array_equal(_bits(a), _bits(r1))
    assert np.array_equal(_bits(b), _bits(r2))


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32, np.int64])
def test_sum7_types_interior(rt, oracle, dtype):
    shape = (12, 19, 37)
    rng = np.random.default_rng(7)
    if np.issubdtype(dtype, np.integer):
        init = rng.integers(-1000, 1000, shape).astype(dtype)
    else:
        init = rng.random(shape).astype(dtype)
    dom = (1, 36, 1, 18, 1, 11)
    a, b = run_pingpong(ps.PS_KERNEL_SUM7, init, ps.domain(*dom), (), 3, dtype)
    r1, r2 = init.copy(), init.copy()
    oracle.run7(oracle.V_SUM7, r1, r2, dom, iter=3)
    assert np.array_equal(a, r1) and np.array_equal(b, r2)


@pytest.mark.parametrize("warps,rows,ns,ctas", [
    (1, 1, 2, 0), (2, 2, 3, 1), (4, 4, 4, 0), (8, 2, 6, 2), (16, 1, 3, 0),
    (4, 8, 5, 0), (1, 8, 2, 3), (16, 4, 3, 1)])
def test_launch_shapes_do_not_change_results(rt, oracle, warps, rows, ns, ctas):
    shape = (23, 45, 150)
    init = synth.uniform(shape, 6)
    before = ps.get_launch_shape(ps.PS_KERNEL_DIFFUSION7)
    ps.set_launch_shape(ps.PS_KERNEL_DIFFUSION7, warps=warps, rows=rows, ns=ns,
                        ctas_per_sm=ctas)
    try:
        a, _ = run_pingpong(ps.PS_KERNEL_DIFFUSION7, init, ps.full_domain(shape),
                            DIFF_COEF, 2)
    finally:
        ps.set_launch_shape(ps.PS_KERNEL_DIFFUSION7, *before)
    r1, r2 = init.copy(), np.zeros_like(init)
    nz, ny, nx = shape
    oracle.run7(oracle.V_DIFFUSION7, r1, r2, (0, nx, 0, ny, 0, nz), DIFF_COEF, 2)
    assert np.array_equal(_bits(a), _bits(r1))


def _himeno_random(shape, seed):
    rng = np.random.default_rng(seed)
    arrs = [rng.random(shape, dtype=np.float32) for _ in range(14)]
    arrs[1] = arrs[0].copy()
    for i in range(6, 9):  # b0..b2 non-zero so every term is exercised
        arrs[i] = (arrs[i] - 0.5).astype(np.float32)
    arrs[13] = (arrs[13] * 0.01).astype(np.float32)
    return arrs


HIMENO_SHAPES = [(4, 1, 5, 2, 0), (1, 1, 3, 1, 1), (8, 1, 4, 3, 0), (2, 1, 6, 1, 2)]


@pytest.mark.parametrize("shape", [(9, 11, 13), (20, 33, 130), (6, 70, 257)])
@pytest.mark.parametrize("launch", HIMENO_SHAPES)
def test_himeno_random_coefficients_bit_exact(rt, oracle, shape, launch):
    for k in (ps.PS_KERNEL_HIMENO19, ps.PS_KERNEL_HIMENO19_GOSA):
        ps.set_launch_shape(k, *launch)
    try:
        _himeno_random_case(oracle, shape)
    finally:
        for k in (ps.PS_KERNEL_HIMENO19, ps.PS_KERNEL_HIMENO19_GOSA):
            ps.set_launch_shape(k, *HIMENO_SHAPES[0])


def _himeno_random_case(oracle, shape):
    arrays = _himeno_random(shape, 11)
    gs = himeno_grids(shape, arrays)
    nz, ny, nx = shape
    domt = (1, nx - 1, 1, ny - 1, 1, nz - 1)
    dom = ps.domain(*domt)
    g = [a.copy() for a in arrays]
    p0, p1 = gs[0], gs[1]
    for s in range(2):
        gosa = ps.reduce_kernel(ps.PS_SUM, ps.PS_KERNEL_HIMENO19_GOSA, dom,
                                [p0, p1] + gs[2:], [0.8])
        _, g64 = oracle.himeno19(g, domt, np.float32(0.8))
        assert abs(float(gosa) - g64) <= 1e-6 * abs(g64)
        p0, p1 = p1, p0
        g[0], g[1] = g[1], g[0]
    assert np.array_equal(_bits(p0.copyout()), _bits(g[0]))
    assert np.array_equal(_bits(p1.copyout()), _bits(g[1]))
    # the plain sweep (no residual) via PSStencilRun gives the same p
    m1 = ps.stencil_map(ps.PS_KERNEL_HIMENO19, dom, [p0, p1] + gs[2:], [0.8])
    ps.stencil_run([m1])
    oracle.himeno19(g, domt, np.float32(0.8))
    assert np.array_equal(_bits(p1.copyout()), _bits(g[1]))
    for x in gs:
        x.free()


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32, np.int64])
@pytest.mark.parametrize("op", [ps.PS_MAX, ps.PS_MIN, ps.PS_SUM, ps.PS_PROD])
@pytest.mark.parametrize("shape", [(1, 1, 1), (3, 5, 7), (17, 33, 129), (2, 2, 4099)])
def test_reduce_all_ops_and_types(rt, oracle, dtype, op, shape):
    rng = np.random.default_rng(13)
    if np.issubdtype(dtype, np.integer):
        data = rng.integers(-50, 50, shape).astype(dtype)
        if op == ps.PS_PROD:
            data = rng.choice(np.array([-1, 1, 1, 3], dtype=dtype), shape)
    else:
        data = (rng.random(shape) + 0.5).astype(dtype)
        if op == ps.PS_PROD:
            data = (1.0 + (rng.random(shape) - 0.5) * 1e-3).astype(dtype)
    g = ps.Grid(shape, dtype)
    g.copyin(data)
    v = ps.reduce(g, op)
    if np.issubdtype(dtype, np.integer) or op in (ps.PS_MAX, ps.PS_MIN):
        assert v == oracle.reduce_ref(data, op)
    else:
        exact = oracle.reduce_fp64(data, op)
        assert abs(float(v) - exact) <= 1e-6 * abs(exact)
    g.free()


def test_reduce_int_sum_wraps_like_ref(rt, oracle):
    data = np.full((4, 4, 4), 2 ** 30, dtype=np.int32)
    g = ps.Grid(data.shape, np.int32)
    g.copyin(data)
    assert ps.reduce(g, ps.PS_SUM) == oracle.reduce_ref(data, oracle.PS_SUM)
    g.free()


def test_reduce_is_deterministic(rt):
    shape = (64, 128, 256)
    data = synth.uniform(shape, 9)
    g = ps.Grid(shape)
    g.copyin(data)
    vals = {ps.reduce_f64(g, ps.PS_SUM) for _ in range(5)}
    assert len(vals) == 1
    g.free()


# ---- failure handling without a GPU fault -----------------------------------

def test_device_wait_timeout_is_reported_and_context_survives(rt):
    ps.clear_error()
    ps.lib().PSTestDeviceWaitTimeout(2000)
    ps.lib().PSSynchronize()
    code, msg = ps.last_error()
    assert code == ps.PS_ERR_DEVICE_TIMEOUT, msg
    ps.clear_error()
    g = ps.Grid((4, 4, 4))
    g.copyin(np.ones((4, 4, 4), np.float32))
    assert ps.reduce(g, ps.PS_SUM) == 64.0
    g.free()


def test_alloc_failure_hook(rt):
    ps.lib().PSTestFailNextAllocs(1)
    with pytest.raises(ps.PSError) as e:
        ps.Grid((8, 8, 8))
    assert e.value.code == ps.PS_ERR_OUT_OF_MEMORY
    g = ps.Grid((8, 8, 8))
    g.free()


def test_invalid_arguments_are_rejected(rt):
    g1, g2 = ps.Grid((8, 8, 8)), ps.Grid((8, 8, 8))
    g3 = ps.Grid((8, 8, 9))
    with pytest.raises(ps.PSError) as e:
        ps.stencil_map(ps.PS_KERNEL_SUM7, ps.full_domain((8, 8, 8)), [g1, g2])
    assert e.value.code == ps.PS_ERR_INVALID_ARGUMENT
    with pytest.raises(ps.PSError) as e:
        ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, ps.full_domain((8, 8, 8)),
                       [g1, g3], DIFF_COEF)
    assert e.value.code == ps.PS_ERR_INVALID_ARGUMENT
    with pytest.raises(ps.PSError) as e:
        ps.stencil_map(99, ps.full_domain((8, 8, 8)), [g1, g2])
    assert e.value.code == ps.PS_ERR_UNKNOWN_KERNEL
    with pytest.raises(ps.PSError) as e:
        ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, ps.domain(0, 9, 0, 8, 0, 8),
                       [g1, g2], DIFF_COEF)
    assert e.value.code == ps.PS_ERR_INVALID_ARGUMENT
    with pytest.raises(ps.PSError) as e:
        ps.stencil_run([12345])
    assert e.value.code == ps.PS_ERR_BAD_HANDLE
    gi = ps.Grid((8, 8, 8), np.int32)
    with pytest.raises(ps.PSError) as e:
        ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, ps.full_domain((8, 8, 8)),
                       [gi, ps.Grid((8, 8, 8), np.int32)], DIFF_COEF)
    assert e.value.code == ps.PS_ERR_UNSUPPORTED
    for g in (g1, g2, g3, gi):
        g.free()
    ps.lib().PSGridCopyin(g1.handle or 1234, None)
    assert ps.last_error()[0] == ps.PS_ERR_BAD_HANDLE
    ps.clear_error()


def test_reference_style_c_program_runs(rt, tmp_path):
    # The same C source a Physis user would write (variadic PSStencilMap,
    # PSStencilRun, PSReduce), compiled by gcc and linked to the library:
    # stdout must equal the reference's test_7-pt-neumann-cond oracle.
    import subprocess
    from test_abi import compile_c_program
    exe = compile_c_program(tmp_path)
    r = subprocess.run([str(exe), "--physis-trace"], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr + r.stdout
    assert r.stdout == gio.stdout_text("test_7-pt-neumann-cond")
    assert "Physis: Stencil started" in r.stderr
    total = float(np.arange(512, dtype=np.float64).sum())
    assert "sum %f" % (7 * total) in r.stderr


# The reference's examples/test_set.c, written against this library's
# header: PSGridSet(g, i, j, k, v) over a 2x2x2 float grid, then a copy-out
# check (i is x, the fastest index), plus the same for int and 1D/2D grids
# with values of other types converted on assignment.
GRIDSET_PROGRAM = r"""
#include <stdio.h>
#include <stdlib.h>
#include "physis_gb300/physis.h"
#include "physis_gb300/physis_gb300.h"
#define N 2
#define IDX3(x, y, z) ((x) + (y) * N + (z) * N * N)
int main(int argc, char *argv[]) {
  int i, j, k, bad = 0;
  float v = 0;
  PSInit(&argc, &argv, 3, N, N, N);
  PSGrid3DFloat g = PSGrid3DFloatNew(N, N, N);
  float *out = (float *)malloc(sizeof(float) * N * N * N);
  for (i = 0; i < N; ++i)
    for (j = 0; j < N; ++j)
      for (k = 0; k < N; ++k) {
        PSGridSet(g, i, j, k, v);
        ++v;
      }
  PSGridCopyout(g, out);
  v = 0;
  for (i = 0; i < N; ++i)
    for (j = 0; j < N; ++j)
      for (k = 0; k < N; ++k) {
        if (out[IDX3(i, j, k)] != v) ++bad;
        ++v;
      }
  {
    PSGrid2DInt h = PSGrid2DIntNew(3, 2);
    PSGrid1DDouble d = PSGrid1DDoubleNew(4);
    int ho[6];
    double dd[4];
    long big = 1234567L;
    PSGridSet(h, 2, 1, 7.9);   /* converted like an int assignment: 7 */
    PSGridSet(h, 0, 0, big);
    PSGridSet(d, 3, 0.1f);     /* a float value, widened */
    PSGridCopyout(h, ho);
    PSGridCopyout(d, dd);
    if (ho[5] != 7 || ho[0] != 1234567 || ho[1] != 0) ++bad;
    if (dd[3] != (double)0.1f || dd[0] != 0.0) ++bad;
    PSGridSet(h, 3, 0, 1);     /* x outside [0, 3): rejected, recorded */
    if (PSGetLastError() != PS_ERR_INVALID_ARGUMENT) ++bad;
    PSClearError();
  }
  printf("%s %d\n", bad ? "FAIL" : "OK", bad);
  PSFinalize();
  return bad != 0;
}
"""


def test_grid_set_reference_example(rt, tmp_path):
    import subprocess
    from test_abi import compile_c_program
    exe = compile_c_program(tmp_path, GRIDSET_PROGRAM, "gridset")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr + r.stdout
    assert r.stdout.strip() == "OK 0"


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32, np.int64])
def test_grid_set_orders_with_stencil_runs(rt, oracle, dtype):
    # A PSGridSet issued between runs lands after the first and before the
    # second: the result equals the oracle run with the same edit between.
    shape = (12, 9, 20)
    init = _iota(20, dtype)[:12, :9, :20].copy() if dtype in (np.int32, np.int64) else \
        synth.uniform(shape, 4).astype(dtype)
    g1, g2 = ps.Grid(shape, dtype), ps.Grid(shape, dtype)
    g1.copyin(init)
    g2.copyin(np.zeros(shape, dtype))
    dom = ps.domain(1, 19, 1, 8, 1, 11)
    m1 = ps.stencil_map(ps.PS_KERNEL_SUM7, dom, [g1, g2])
    m2 = ps.stencil_map(ps.PS_KERNEL_SUM7, dom, [g2, g1])
    ps.stencil_run([m1, m2], 1)
    g1.set((5, 4, 6), 77)
    ps.stencil_run([m1], 1)
    r1, r2 = init.copy(), np.zeros(shape, dtype)
    lim = (1, 19, 1, 8, 1, 11)
    oracle.run7(oracle.V_SUM7, r1, r2, lim, (), iter=1)
    r1[6, 4, 5] = 77
    oracle.sweep7(oracle.V_SUM7, r1, r2, lim)
    assert np.array_equal(_bits(g1.copyout()), _bits(r1))
    assert np.array_equal(_bits(g2.copyout()), _bits(r2))
    g1.free()
    g2.free()


# ---- temporal blocking -------------------------------------------------------

TEMPORAL = [  # (k, warps, rows, ns)
    (2, 8, 4, 3), (3, 8, 2, 3), (4, 8, 4, 2), (5, 4, 4, 3), (2, 1, 4, 2), (3, 2, 4, 4)]


@pytest.mark.parametrize("k,warps,rows,ns", TEMPORAL)
@pytest.mark.parametrize("shape,iters", [((37, 45, 70), 5), ((9, 17, 250), 3),
                                         ((64, 64, 64), 2), ((1, 3, 9), 4),
                                         ((20, 130, 121), 1)])
def test_temporal_blocking_bit_exact(rt, oracle, k, warps, rows, ns, shape, iters):
    init = synth.uniform(shape, 8)
    ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, k, warps=warps, rows=rows, ns=ns)
    try:
        a, b = run_pingpong(ps.PS_KERNEL_DIFFUSION7, init, ps.full_domain(shape),
                            DIFF_COEF, iters)
    finally:
        ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, 1)
    r1, r2 = init.copy(), np.zeros_like(init)
    nz, ny, nx = shape
    oracle.run7(oracle.V_DIFFUSION7, r1, r2, (0, nx, 0, ny, 0, nz), DIFF_COEF,
                iter=iters)
    assert np.array_equal(_bits(a), _bits(r1))
    assert np.array_equal(_bits(b), _bits(r2))


@pytest.mark.parametrize("k,warps,rows,ns", [(2, 8, 4, 3), (3, 8, 2, 3), (5, 4, 4, 3)])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_temporal_blocking_with_fma_within_tolerance(rt, oracle, k, warps, rows, ns, dtype):
    # Contracted temporal passes: within 1e-5 relative per cell of the REF
    # target and of an FP64 evaluation; not bit-identical to it (the fused
    # kernel really ran); plain sweeps stay bit-exact with contraction on.
    if dtype == np.float64 and k > 3:
        pytest.skip("double grids block at most 3 steps per pass")
    shape = (37, 45, 70)
    iters = 6
    init = synth.uniform(shape, 12).astype(dtype)
    ps.set_fma(True)
    ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, k, warps=warps, rows=rows, ns=ns)
    try:
        a, b = run_pingpong(ps.PS_KERNEL_DIFFUSION7, init, ps.full_domain(shape), DIFF_COEF,
                            iters, dtype)
        ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, 1)
        pa, pb = run_pingpong(ps.PS_KERNEL_DIFFUSION7, init, ps.full_domain(shape), DIFF_COEF,
                              iters, dtype)
    finally:
        ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, 1)
        ps.set_fma(False)
    nz, ny, nx = shape
    dom = (0, nx, 0, ny, 0, nz)
    r1, r2 = init.copy(), np.zeros_like(init)
    oracle.run7(oracle.V_DIFFUSION7, r1, r2, dom, DIFF_COEF, iter=iters)
    f1, f2 = init.astype(np.float64), np.zeros(shape)
    oracle.run7(oracle.V_DIFFUSION7, f1, f2, dom, DIFF_COEF, iter=iters)
    for got, ref, ref64 in ((a, r1, f1), (b, r2, f2)):
        assert np.allclose(got, ref, rtol=1e-5, atol=0)
        assert np.allclose(got, ref64, rtol=1e-5, atol=0)
    assert not np.array_equal(_bits(a), _bits(r1))
    assert np.array_equal(_bits(pa), _bits(r1))
    assert np.array_equal(_bits(pb), _bits(r2))


@pytest.mark.parametrize("k", [2, 3])
def test_temporal_blocking_double(rt, oracle, k):
    shape = (19, 33, 70)
    init = synth.uniform(shape, 9).astype(np.float64)
    ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, k, warps=8, rows=2, ns=3)
    try:
        a, b = run_pingpong(ps.PS_KERNEL_DIFFUSION7, init, ps.full_domain(shape),
                            DIFF_COEF, 4, np.float64)
    finally:
        ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, 1)
    r1, r2 = init.copy(), np.zeros_like(init)
    nz, ny, nx = shape
    oracle.run7(oracle.V_DIFFUSION7, r1, r2, (0, nx, 0, ny, 0, nz), DIFF_COEF, iter=4)
    assert np.array_equal(_bits(a), _bits(r1))
    assert np.array_equal(_bits(b), _bits(r2))


def test_temporal_blocking_not_used_for_subdomains(rt, oracle):
    # an interior domain keeps the plain path (cells outside stay untouched)
    shape = (21, 31, 41)
    init, other = synth.uniform(shape, 4), synth.uniform(shape, 5)
    dom = (1, 40, 2, 30, 3, 20)
    ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, 3, warps=8, rows=2, ns=3)
    try:
        a, b = run_pingpong(ps.PS_KERNEL_DIFFUSION7, init, ps.domain(*dom),
                            DIFF_COEF, 3, out0=other)
    finally:
        ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, 1)
    r1, r2 = init.copy(), other.copy()
    oracle.run7(oracle.V_DIFFUSION7, r1, r2, dom, DIFF_COEF, iter=3)
    assert np.array_equal(_bits(a), _bits(r1))
    assert np.array_equal(_bits(b), _bits(r2))


def test_temporal_blocking_rejects_bad_shapes(rt):
    with pytest.raises(ps.PSError):
        ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, 9)
    with pytest.raises(ps.PSError):
        ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, 5, warps=1, rows=4)  # tile too short
    with pytest.raises(ps.PSError):
        ps.set_temporal(ps.PS_KERNEL_SUM7, 2)
    assert ps.get_temporal(ps.PS_KERNEL_DIFFUSION7)[0] == 1


# ---- autotuner ---------------------------------------------------------------

def test_autotuner_trials_are_ordinary_iterations(rt, oracle, tmp_path):
    # Tuning spends the run's first iterations on candidate shapes/depths;
    # every candidate is bit-identical, so the run's result must equal the
    # oracle's, and the signature ends with a tuned plan saved to the cache.
    shape = (40, 70, 300)
    init = synth.uniform(shape, 12)
    cache = str(tmp_path / "tune.jsonl")
    ps.lib().PSClearTuning()
    ps.set_autotune(True, cache)
    try:
        g1, g2 = ps.Grid(shape), ps.Grid(shape)
        g1.copyin(init)
        dom = ps.full_domain(shape)
        m1 = ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, dom, [g1, g2], DIFF_COEF)
        m2 = ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, dom, [g2, g1], DIFF_COEF)
        ps.stencil_run([m1, m2], 30)   # tuning continues across runs
        ps.stencil_run([m1, m2], 40)
        a, b = g1.copyout(), g2.copyout()
        tuned, sh, k, tsh = ps.stencil_plan(m1)
        assert tuned
    finally:
        ps.set_autotune(False, "")
    r1, r2 = init.copy(), np.zeros_like(init)
    nz, ny, nx = shape
    oracle.run7(oracle.V_DIFFUSION7, r1, r2, (0, nx, 0, ny, 0, nz), DIFF_COEF,
                iter=70, nthreads=0)
    assert np.array_equal(_bits(a), _bits(r1))
    assert np.array_equal(_bits(b), _bits(r2))
    # the plan persists: a fresh tuning table loads it and applies it
    lines = open(cache).read().splitlines()
    assert len(lines) == 1 and '"key": "k2 t2 g300x70x40' in lines[0]
    ps.lib().PSClearTuning()
    assert ps.lib().PSLoadTuneCache(cache.encode()) == 1
    m3 = ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, dom, [g1, g2], DIFF_COEF)
    m4 = ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, dom, [g2, g1], DIFF_COEF)
    ps.stencil_run([m3, m4], 1)
    assert ps.stencil_plan(m3)[0]
    assert ps.stencil_plan(m3)[1:] == (sh, k, tsh)
    ps.lib().PSClearTuning()
    g1.free()
    g2.free()


def test_corrupt_tune_cache_is_skipped(rt, tmp_path):
    p = tmp_path / "bad.jsonl"
    good = ('{"key": "k2 t2 g8x8x8 d0:8,0:8,0:8;x/1sm", "warps": 4, "rows": 2, '
            '"ns": 3, "ns2": 0, "ctas": 0, "k": 1, "twarps": 8, "trows": 4, '
            '"tns": 3, "ms": 0.1}')
    p.write_text("garbage\n" + good + "\n{\"key\": \"x\", \"warps\": 99}\n")
    ps.clear_error()
    assert ps.lib().PSLoadTuneCache(str(p).encode()) == 1
    assert ps.last_error()[0] == ps.PS_ERR_IO
    ps.clear_error()
    ps.lib().PSClearTuning()


# ---- CUDA graph replay of launch-bound runs ----------------------------------

def test_graph_replay_matches_and_survives_reallocation(rt, oracle):
    # 37 iterations: one ordinary, two 16-iteration graph replays, 4 ordinary
    shape = (16, 24, 40)
    for seed in (30, 31):  # second round: new grids at possibly reused addresses
        init = synth.uniform(shape, seed)
        n0 = ps.launch_count()
        a, b = run_pingpong(ps.PS_KERNEL_DIFFUSION7, init, ps.full_domain(shape),
                            DIFF_COEF, 37)
        assert ps.launch_count() - n0 == 74
        r1, r2 = init.copy(), np.zeros_like(init)
        oracle.run7(oracle.V_DIFFUSION7, r1, r2, (0, 40, 0, 24, 0, 16), DIFF_COEF,
                    iter=37)
        assert np.array_equal(_bits(a), _bits(r1))
        assert np.array_equal(_bits(b), _bits(r2))


def test_run_with_freed_grid_is_rejected(rt):
    g1, g2 = ps.Grid((8, 8, 8)), ps.Grid((8, 8, 8))
    m = ps.stencil_map(ps.PS_KERNEL_COPY, ps.full_domain((8, 8, 8)), [g1, g2])
    g2.free()
    with pytest.raises(ps.PSError) as e:
        ps.stencil_run([m])
    assert e.value.code == ps.PS_ERR_BAD_HANDLE
    g1.free()


# ---- batches of independent runs --------------------------------------------

@pytest.mark.parametrize("iters", [3, 21])
def test_batch_of_uneven_runs_bit_exact(rt, oracle, iters):
    rng = np.random.default_rng(40)
    runs, refs, keep = [], [], []
    for i, shape in enumerate([(24, 40, 130), (9, 17, 33), (40, 8, 300)]):
        init = synth.uniform(shape, 50 + i)
        g1, g2 = ps.Grid(shape), ps.Grid(shape)
        g1.copyin(init)
        dom = ps.full_domain(shape)
        runs.append([ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, dom, [g1, g2], DIFF_COEF),
                     ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, dom, [g2, g1], DIFF_COEF)])
        r1, r2 = init.copy(), np.zeros_like(init)
        nz, ny, nx = shape
        oracle.run7(oracle.V_DIFFUSION7, r1, r2, (0, nx, 0, ny, 0, nz), DIFF_COEF,
                    iter=iters)
        refs.append((g1, g2, r1, r2))
    shape = (12, 19, 37)
    init = rng.random(shape).astype(np.float32)
    g1, g2 = ps.Grid(shape), ps.Grid(shape)
    g1.copyin(init)
    g2.copyin(init)
    domt = (1, 36, 1, 18, 1, 11)
    runs.append([ps.stencil_map(ps.PS_KERNEL_SUM7, ps.domain(*domt), [g1, g2]),
                 ps.stencil_map(ps.PS_KERNEL_SUM7, ps.domain(*domt), [g2, g1])])
    r1, r2 = init.copy(), init.copy()
    oracle.run7(oracle.V_SUM7, r1, r2, domt, iter=iters)
    refs.append((g1, g2, r1, r2))
    for shape in [(20, 33, 130), (9, 11, 13)]:
        arrays = _himeno_random(shape, 60 + shape[0])
        gs = himeno_grids(shape, arrays)
        keep.append(gs)
        nz, ny, nx = shape
        domt = (1, nx - 1, 1, ny - 1, 1, nz - 1)
        dom = ps.domain(*domt)
        runs.append([ps.stencil_map(ps.PS_KERNEL_HIMENO19, dom, gs, [0.8]),
                     ps.stencil_map(ps.PS_KERNEL_HIMENO19, dom, [gs[1], gs[0]] + gs[2:],
                                    [0.8])])
        g = [a.copy() for a in arrays]
        for _ in range(2 * iters):
            oracle.himeno19(g, domt, np.float32(0.8))
            g[0], g[1] = g[1], g[0]
        refs.append((gs[0], gs[1], g[0], g[1]))
    b = ps.batch_create(runs)
    n0 = ps.launch_count()
    ps.batch_run(b, iters)
    # one launch per kernel family (7-point, Himeno) per step for all runs
    assert ps.launch_count() - n0 == 2 * 2 * iters
    for ga, gb, ra, rb in refs:
        assert np.array_equal(_bits(ga.copyout()), _bits(ra))
        assert np.array_equal(_bits(gb.copyout()), _bits(rb))
    ps.batch_free(b)
    for ga, gb, _, _ in refs:
        ga.free()
        gb.free()
    for gs in keep:
        for g in gs[2:]:
            g.free()


def test_batch_rejects_unsupported(rt):
    g1, g2 = ps.Grid((8, 8, 8), np.float64), ps.Grid((8, 8, 8), np.float64)
    m = ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, ps.full_domain((8, 8, 8)), [g1, g2],
                       DIFF_COEF)
    with pytest.raises(ps.PSError) as e:
        ps.batch_create([[m]])
    assert e.value.code == ps.PS_ERR_UNSUPPORTED
    g1.free()
    g2.free()
