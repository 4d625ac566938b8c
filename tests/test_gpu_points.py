"""Point-list stencils and red/black maps on the GPU, against the oracle.

* the reference's point-list system tests (tests/system_cases.py): exact
  stdout text of their REF programs;
* seeded random stencils (offsets, weights, boundary rules, element types,
  ragged shapes, subdomains): bit-identical to oracle/ps_oracle.c;
* red/black maps (point stencils and the 7-point builtins): bit-identical to
  the oracle's sequential in-place REF order;
* a size-independent property at a large size: a periodic unit-weight sum
  of n points maps a grid of ones to n everywhere and multiplies the total
  of an integer grid by n exactly (mod 2^64);
* argument checking of the new entry points.
"""
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


@pytest.fixture(params=["compiled", "table"])
def kernel_form(request):
    """Runs a test with the per-stencil compiled kernel (the default) and
    with the run-time table kernel (PS_POINTS_JIT=0)."""
    import os
    old = os.environ.get("PS_POINTS_JIT")
    if request.param == "table":
        os.environ["PS_POINTS_JIT"] = "0"
    else:
        os.environ.pop("PS_POINTS_JIT", None)
    yield request.param
    if old is None:
        os.environ.pop("PS_POINTS_JIT", None)
    else:
        os.environ["PS_POINTS_JIT"] = old


def _bits(a):
    return a.view({1: np.uint8, 4: np.uint32, 8: np.uint64}[a.dtype.itemsize])


def _dom(d):
    return ps.domain(*d)


class _G:
    """A device grid standing for one of a system test's arrays."""

    def __init__(self, arr):
        self.g = ps.Grid(arr.shape, arr.dtype)
        self.g.copyin(arr)


@pytest.mark.parametrize("name", sorted(sc.CASES))
def test_point_system_tests(rt, kernel_form, name):
    case = dict(sc.CASES[name])
    dom = _dom(sc.domain(case))
    k = ps.point_stencil(case["points"], boundary=case["boundary"])
    a, b = sc.initial(case)
    case["grids"] = (_G(a), _G(b))

    def sweep(src, dst):
        ps.stencil_run([ps.stencil_map(k, dom, [src.g, dst.g])])

    def color_sweep(g, color):
        ps.stencil_run([ps.stencil_map_color(k, color, dom, [g.g])])

    text = sc.run(case, sweep, color_sweep,
                  lambda g: ps.reduce(g.g, ps.PS_SUM),
                  lambda g: gio.dump_text(g.g.copyout(), sc.fmt(case)))
    for g in case["grids"]:
        g.g.free()
    assert text == gio.stdout_text(name)


def test_point_system_tests_as_one_run(rt):
    # test_5-pt-periodic's two maps as one PSStencilRun(m1, m2) (its .c form).
    case = sc.CASES["test_5-pt-periodic"]
    k = ps.point_stencil(case["points"], boundary=1)
    a, b = sc.initial(case)
    g1, g2 = _G(a), _G(b)
    dom = _dom(sc.domain(case))
    ps.stencil_run([ps.stencil_map(k, dom, [g1.g, g2.g]),
                    ps.stencil_map(k, dom, [g2.g, g1.g])])
    assert gio.dump_text(g1.g.copyout()) == gio.stdout_text("test_5-pt-periodic")
    g1.g.free()
    g2.g.free()


def _random_stencil(rng, radius, npts, boundary, shape, weighted, integer):
    nz, ny, nx = shape
    pts = []
    for _ in range(npts):
        p = []
        for n in (nx, ny, nz):
            # none: the domain must keep reads inside; periodic: |d| <= n
            r = {0: min(radius, (n - 1) // 2), 1: min(radius, n), 2: radius}[boundary]
            p.append(int(rng.integers(-r, r + 1)) if n > 1 else 0)
        pts.append(tuple(p))
    if not weighted:
        return pts, None
    if integer:
        return pts, [float(v) for v in rng.integers(-3, 4, size=npts)]
    return pts, [float(np.float32(v)) for v in rng.uniform(-1.5, 1.5, size=npts)]


def _domain_for(rng, pts, boundary, shape, shrink):
    nz, ny, nx = shape
    dom = []
    for d, n in enumerate((nx, ny, nz)):
        lo = -min(0, min(p[d] for p in pts))
        hi = max(0, max(p[d] for p in pts))
        a, b = (lo, n - hi) if boundary == 0 else (0, n)
        if shrink and b - a > 4:
            a += int(rng.integers(0, 3))
            b -= int(rng.integers(0, 3))
        dom += [a, b]
    return tuple(dom)


def _fill(rng, shape, dtype):
    if np.issubdtype(dtype, np.integer):
        return rng.integers(-1000, 1000, size=shape).astype(dtype)
    return rng.uniform(-1.0, 1.0, size=shape).astype(dtype)


CASES = [
    # (seed, shape (nz, ny, nx), dtype, boundary, npts, radius, weighted, shrink)
    (1, (9, 17, 300), np.float32, 0, 27, 1, False, False),
    (2, (12, 33, 129), np.float32, 1, 9, 2, True, False),
    (3, (7, 40, 200), np.float64, 2, 13, 3, True, True),
    (4, (16, 16, 16), np.int32, 1, 27, 1, False, False),
    (5, (10, 21, 77), np.int64, 0, 5, 4, True, True),
    (6, (1, 64, 500), np.float32, 1, 9, 2, False, False),
    (7, (1, 1, 3000), np.float64, 0, 3, 4, True, False),
    (8, (33, 9, 140), np.float32, 2, 64, 4, True, True),
    (9, (20, 25, 130), np.int32, 2, 7, 2, True, False),
    (10, (6, 70, 260), np.float64, 1, 19, 4, False, True),
]


@pytest.mark.parametrize("seed,shape,dtype,boundary,npts,radius,weighted,shrink", CASES)
def test_random_point_stencils_bit_exact(rt, oracle, kernel_form, seed, shape, dtype,
                                         boundary, npts, radius, weighted, shrink):
    rng = np.random.default_rng(seed)
    integer = np.issubdtype(dtype, np.integer)
    pts, w = _random_stencil(rng, radius, npts, boundary, shape, weighted, integer)
    dom = _domain_for(rng, pts, boundary, shape, shrink)
    src = _fill(rng, shape, dtype)
    out0 = _fill(rng, shape, dtype)
    ref = out0.copy()
    oracle.points(src, ref, dom, pts, weights=w, boundary=boundary)
    k = ps.point_stencil(pts, weights=w, boundary=boundary)
    g1, g2 = ps.Grid(shape, dtype), ps.Grid(shape, dtype)
    g1.copyin(src)
    g2.copyin(out0)
    ps.stencil_run([ps.stencil_map(k, _dom(dom), [g1, g2])])
    got = g2.copyout()
    g1.free()
    g2.free()
    assert np.array_equal(_bits(got), _bits(ref))


@pytest.mark.parametrize("warps,rows", [(8, 2), (8, 1), (4, 2), (16, 1), (2, 2), (1, 1), (8, 4), (4, 4)])
def test_point_launch_shapes_do_not_change_results(rt, oracle, kernel_form, warps, rows):
    rng = np.random.default_rng(42)
    shape = (11, 45, 270)
    pts = sc.P27
    src = _fill(rng, shape, np.float32)
    ref = np.zeros(shape, np.float32)
    dom = (0, shape[2], 0, shape[1], 0, shape[0])
    oracle.points(src, ref, dom, pts, boundary=1)
    k = ps.point_stencil(pts, boundary=1)
    old = ps.get_launch_shape(k)
    ps.set_launch_shape(k, warps=warps, rows=rows)
    try:
        g1, g2 = ps.Grid(shape), ps.Grid(shape)
        g1.copyin(src)
        ps.stencil_run([ps.stencil_map(k, _dom(dom), [g1, g2])])
        got = g2.copyout()
        g1.free()
        g2.free()
    finally:
        ps.set_launch_shape(k, warps=old[0], rows=old[1])
    assert np.array_equal(_bits(got), _bits(ref))


RB_CASES = [
    # (seed, shape, dtype, boundary, points, weighted, halo)
    (1, (16, 20, 150), np.float32, 0, sc.P7_RB, False, 1),
    (2, (18, 24, 130), np.float64, 1, sc.P7_RB, True, 0),
    (3, (13, 15, 140), np.float32, 2, sc.P7_RB, True, 0),
    (4, (20, 22, 160), np.int32, 1,
     [(0, 0, 0), (1, 0, 0), (0, 2, 1), (-3, 0, 0), (1, 1, 1), (0, 0, -1)], True, 0),
    (5, (14, 19, 133), np.int64, 0,
     [(0, 0, 0), (2, 1, 0), (-1, 0, 0), (0, -2, -1), (0, 0, 3)], False, 3),
    (6, (1, 40, 300), np.float32, 1,
     [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0)], False, 0),
]


@pytest.mark.parametrize("seed,shape,dtype,boundary,pts,weighted,halo", RB_CASES)
@pytest.mark.parametrize("color", [0, 1, 2])
def test_red_black_bit_exact(rt, oracle, kernel_form, seed, shape, dtype, boundary, pts,
                             weighted, halo, color):
    rng = np.random.default_rng(seed)
    integer = np.issubdtype(dtype, np.integer)
    w = None
    if weighted:
        w = ([float(v) for v in rng.integers(-2, 3, size=len(pts))] if integer else
             [float(np.float32(v)) for v in rng.uniform(-0.5, 0.5, size=len(pts))])
    nz, ny, nx = shape
    dom = tuple(v for n in (nx, ny, nz) for v in
                ((halo, n - halo) if n > 2 * halo else (0, n)))
    g = _fill(rng, shape, dtype)
    ref = g.copy()
    for c in ((0, 1) if color == 2 else (color,)):
        oracle.points(ref, ref, dom, pts, weights=w, boundary=boundary, color=c)
    k = ps.point_stencil(pts, weights=w, boundary=boundary)
    dg = ps.Grid(shape, dtype)
    dg.copyin(g)
    ps.stencil_run([ps.stencil_map_color(k, color, _dom(dom), [dg])])
    got = dg.copyout()
    dg.free()
    assert np.array_equal(_bits(got), _bits(ref))


def test_red_black_builtins(rt, oracle):
    # PSStencilMapRedBlack(PS_KERNEL_SUM7 / DIFFUSION7, dom, g, scalars...):
    # the 7-point builtins run as their point-stencil equivalents.
    rng = np.random.default_rng(7)
    shape = (12, 18, 140)
    g = rng.uniform(0, 1, size=shape).astype(np.float32)
    nz, ny, nx = shape
    inner = (1, nx - 1, 1, ny - 1, 1, nz - 1)
    ref = g.copy()
    for c in (0, 1):
        oracle.points(ref, ref, inner, sc.P7_RB, color=c)
    dg = ps.Grid(shape)
    dg.copyin(g)
    ps.stencil_run([ps.stencil_map_color(ps.PS_KERNEL_SUM7, 2, _dom(inner), [dg])], 1)
    assert np.array_equal(_bits(dg.copyout()), _bits(ref))

    coef = (0.11, 0.12, 0.13, 0.14, 0.15, 0.16, 0.4)  # ce cw cn cs ct cb cc
    full = (0, nx, 0, ny, 0, nz)
    pts = [(0, 0, 0), (-1, 0, 0), (1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, -1), (0, 0, 1)]
    w = [coef[6], coef[1], coef[0], coef[3], coef[2], coef[5], coef[4]]
    ref = g.copy()
    for _ in range(3):
        for c in (0, 1):
            oracle.points(ref, ref, full, pts, weights=w, boundary=2, color=c)
    dg.copyin(g)
    s = ps.stencil_map_color(ps.PS_KERNEL_DIFFUSION7, 2, _dom(full), [dg], coef)
    ps.stencil_run([s], 3)
    assert np.array_equal(_bits(dg.copyout()), _bits(ref))
    dg.free()


def test_point_pingpong_graph_replay(rt, oracle):
    # 40 iterations of (g1 -> g2, g2 -> g1): the CUDA-graph path of plain runs.
    rng = np.random.default_rng(11)
    shape = (10, 30, 140)
    pts = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
    w = [0.4, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1]
    src = rng.uniform(0, 1, size=shape).astype(np.float32)
    a, b = src.copy(), src.copy()
    full = (0, shape[2], 0, shape[1], 0, shape[0])
    for _ in range(40):
        oracle.points(a, b, full, pts, weights=w, boundary=1)
        oracle.points(b, a, full, pts, weights=w, boundary=1)
    k = ps.point_stencil(pts, weights=w, boundary=1)
    g1, g2 = ps.Grid(shape), ps.Grid(shape)
    g1.copyin(src)
    g2.copyin(src)
    dom = _dom(full)
    before = ps.lib().PSGetLaunchCount()
    ps.stencil_run([ps.stencil_map(k, dom, [g1, g2]), ps.stencil_map(k, dom, [g2, g1])], 40)
    assert ps.lib().PSGetLaunchCount() - before == 80
    assert np.array_equal(_bits(g1.copyout()), _bits(a))
    assert np.array_equal(_bits(g2.copyout()), _bits(b))
    g1.free()
    g2.free()


def test_point_autotuner_keeps_results(rt, oracle, tmp_path):
    rng = np.random.default_rng(12)
    shape = (16, 40, 256)
    src = rng.uniform(0, 1, size=shape).astype(np.float32)
    a, b = src.copy(), src.copy()
    full = (0, shape[2], 0, shape[1], 0, shape[0])
    iters = 12
    for _ in range(iters):
        oracle.points(a, b, full, sc.P27, boundary=1)
        oracle.points(b, a, full, sc.P27, boundary=1)
    k = ps.point_stencil(sc.P27, boundary=1)
    g1, g2 = ps.Grid(shape), ps.Grid(shape)
    g1.copyin(src)
    g2.copyin(src)
    dom = _dom(full)
    ps.set_autotune(True, str(tmp_path / "tune.jsonl"))
    try:
        m1, m2 = ps.stencil_map(k, dom, [g1, g2]), ps.stencil_map(k, dom, [g2, g1])
        ps.stencil_run([m1, m2], iters)
        tuned = ps.stencil_plan(m1)[0]
    finally:
        ps.set_autotune(False)
        ps.lib().PSClearTuning()
    assert tuned
    assert np.array_equal(_bits(g1.copyout()), _bits(a))
    g1.free()
    g2.free()


def test_periodic_sum_property_at_size(rt):
    # 27-point periodic unit-weight sum over 512 x 512 x 256 (268 MB per
    # float grid): ones -> 27 exactly; a random int64 grid's total is
    # multiplied by 27 exactly (mod 2^64), whatever the tiling.
    shape = (256, 512, 512)
    k = ps.point_stencil(sc.P27, boundary=1)
    dom = _dom((0, 512, 0, 512, 0, 256))
    g1, g2 = ps.Grid(shape), ps.Grid(shape)
    g1.copyin(np.ones(shape, np.float32))
    ps.stencil_run([ps.stencil_map(k, dom, [g1, g2])])
    assert ps.reduce(g2, ps.PS_MIN) == 27.0 and ps.reduce(g2, ps.PS_MAX) == 27.0
    g1.free()
    g2.free()
    rng = np.random.default_rng(3)
    src = rng.integers(-2 ** 40, 2 ** 40, size=shape, dtype=np.int64)
    g1, g2 = ps.Grid(shape, np.int64), ps.Grid(shape, np.int64)
    g1.copyin(src)
    ps.stencil_run([ps.stencil_map(k, dom, [g1, g2])])
    total = int(ps.reduce(g2, ps.PS_SUM))
    expect = (27 * int(src.sum(dtype=np.int64))) % 2 ** 64
    assert total % 2 ** 64 == expect
    g1.free()
    g2.free()


def _err(fn):
    ps.clear_error()
    with pytest.raises(ps.PSError) as e:
        fn()
    return e.value.code


def test_point_stencil_argument_checks(rt):
    g = ps.Grid((8, 8, 8))
    h = ps.Grid((8, 8, 8))
    gi = ps.Grid((8, 8, 8), np.int32)
    gi2 = ps.Grid((8, 8, 8), np.int32)
    godd = ps.Grid((7, 8, 8))
    full = ps.full_domain((8, 8, 8))
    assert _err(lambda: ps.point_stencil([(5, 0, 0)])) == ps.PS_ERR_INVALID_ARGUMENT
    assert _err(lambda: ps.point_stencil([])) == ps.PS_ERR_INVALID_ARGUMENT
    assert _err(lambda: ps.point_stencil([(0, 0, 0)], boundary=7)) == \
        ps.PS_ERR_INVALID_ARGUMENT
    k = ps.point_stencil([(0, 0, 0), (1, 0, 0)])
    # boundary none: a full-grid domain reads x = 8
    assert _err(lambda: ps.stencil_map(k, full, [g, h])) == ps.PS_ERR_INVALID_ARGUMENT
    assert _err(lambda: ps.stencil_map(k, full, [g, g])) == ps.PS_ERR_INVALID_ARGUMENT
    kw = ps.point_stencil([(0, 0, 0)], weights=[0.5])
    assert _err(lambda: ps.stencil_map(kw, full, [gi, gi2])) == ps.PS_ERR_INVALID_ARGUMENT
    even = ps.point_stencil([(0, 0, 0), (1, 1, 0)], boundary=1)
    assert _err(lambda: ps.stencil_map_color(even, 0, full, [g])) == ps.PS_ERR_UNSUPPORTED
    odd = ps.point_stencil([(0, 0, 0), (0, 0, 1)], boundary=1)
    assert _err(lambda: ps.stencil_map_color(odd, 2, ps.full_domain((7, 8, 8)), [godd])) \
        == ps.PS_ERR_UNSUPPORTED
    assert _err(lambda: ps.stencil_map_color(ps.PS_KERNEL_HIMENO19, 0, full, [g], [0.8])) \
        == ps.PS_ERR_UNSUPPORTED
    assert _err(lambda: ps.stencil_map_color(odd, 0, full, [g, h])) == \
        ps.PS_ERR_INVALID_ARGUMENT
    # registering the same stencil again returns the same id
    assert ps.point_stencil([(0, 0, 0), (1, 0, 0)]) == k
    for x in (g, h, gi, gi2, godd):
        x.free()
