"""Pin the CPU oracle against the reference's own outputs (no GPU needed).

Every case here re-runs a reference program's computation through the oracle
restatement (oracle/ps_oracle.c) on the same inputs and compares with the
reference's own output captured in tests/golden/ -- exact text for the
system-test oracles (the reference's driver diffs stdout exactly,
tests/system_tests/run_system_tests.sh.cmake:874), exact bits for the
diffusion and Himeno benchmark harnesses.
"""
import numpy as np
import pytest

import golden_io as gio


def _iota(n, dtype):
    return np.arange(n ** 3, dtype=np.int64).astype(dtype).reshape(n, n, n)


@pytest.mark.parametrize("test,dtype,fmt", [
    ("test_7-pt", np.float32, "%f"),
    ("test_7-pt-double-type", np.float64, "%f"),
    ("test_7-pt-int-type", np.int32, "%d"),
])
def test_sum7_single_sweep(oracle, test, dtype, fmt):
    # test_7-pt.c:31-56: N=32, indata[i]=i in both grids, interior domain,
    # one PSStencilRun of the 7-point sum g1 -> g2, dump g2.
    n = 32
    g1, g2 = _iota(n, dtype), _iota(n, dtype)
    oracle.sweep7(oracle.V_SUM7, g1, g2, (1, n - 1, 1, n - 1, 1, n - 1))
    assert gio.dump_text(g2, fmt) == gio.stdout_text(test)


def test_sum7_multi_iterations(oracle):
    # test_7-pt-multi-iterations.c: N=32, ITER=5 of (g1->g2, g2->g1), dump g1.
    n = 32
    g1, g2 = _iota(n, np.float32), _iota(n, np.float32)
    oracle.run7(oracle.V_SUM7, g1, g2, (1, n - 1, 1, n - 1, 1, n - 1), iter=5)
    assert gio.dump_text(g1) == gio.stdout_text("test_7-pt-multi-iterations")


def test_neumann_clamped(oracle):
    # test_7-pt-neumann-cond.c: N=8, full domain, clamped faces,
    # c + w + e + s + n + b + t == DIFFUSION7 with unit weights.
    n = 8
    g1 = _iota(n, np.float32)
    g2 = np.zeros_like(g1)
    oracle.sweep7(oracle.V_DIFFUSION7, g1, g2, (0, n, 0, n, 0, n),
                  coef=[1.0] * 7)
    assert gio.dump_text(g2) == gio.stdout_text("test_7-pt-neumann-cond")


def test_sum7_periodic(oracle):
    # test_7-pt-periodic.c: N=32, full domain, periodic wrap.
    n = 32
    g1, g2 = _iota(n, np.float32), _iota(n, np.float32)
    oracle.sweep7(oracle.V_SUM7_PERIODIC, g1, g2, (0, n, 0, n, 0, n))
    assert gio.dump_text(g2) == gio.stdout_text("test_7-pt-periodic")


def test_reduce_sum(oracle):
    # test_reduction-3d-sum.c: N=16, indata[i]=i, PS_SUM, printf("%f").
    v = oracle.reduce_ref(np.arange(16 ** 3, dtype=np.float32), oracle.PS_SUM)
    assert "%f\n" % float(v) == gio.stdout_text("test_reduction-3d-sum")


@pytest.mark.parametrize("op,data,expect", [
    # Known answers restated from the reference tests that check themselves:
    # test_reduction-3d-max.c (N=4, i) -> 63; -min.c (N=8, i+10) -> 10;
    # -int.c / -long.c (N=8, i) -> sum 0..511 = 130816.
    ("max", np.arange(64, dtype=np.float32), 63.0),
    ("min", np.arange(512, dtype=np.float32) + 10, 10.0),
    ("sum", np.arange(512, dtype=np.int32), 130816),
    ("sum", np.arange(512, dtype=np.int64), 130816),
])
def test_reduce_known_answers(oracle, op, data, expect):
    opc = {"max": oracle.PS_MAX, "min": oracle.PS_MIN, "sum": oracle.PS_SUM}[op]
    assert oracle.reduce_ref(data, opc) == expect


def test_reduce_prod_matches_float_fold(oracle):
    # test_reduction-3d-prod.c: N=4, all 1.1f, PS_PROD; its own check is a
    # float fold, which the oracle must reproduce bit for bit.
    data = np.full(64, np.float32(1.1), dtype=np.float32)
    v = np.float32(1.1)
    for _ in range(63):
        v = np.float32(v * np.float32(1.1))
    assert oracle.reduce_ref(data, oracle.PS_PROD) == v


def test_diffusion_matches_reference_baseline(oracle):
    # The reference's own sequential diffusion (baseline.cc:22-49), 21^3,
    # 6 steps, its own initial field and coefficients: bit-exact.
    n, count = 21, 6
    init = gio.f32("diffusion_ref_n21_c6.init.f32.gz", (n, n, n))
    final = gio.f32("diffusion_ref_n21_c6.final.f32.gz", (n, n, n))
    coef = gio.hexfloats("diffusion_ref_n21_c6.coef.txt")  # ce cw cn cs ct cb cc
    g1, g2 = init.copy(), np.zeros_like(init)
    oracle.run7(oracle.V_DIFFUSION7, g1, g2, (0, n, 0, n, 0, n), coef,
                iter=count // 2)
    assert np.array_equal(g1.view(np.uint32), final.view(np.uint32))


def himeno_inputs(nx, ny, nz, dtype=np.float32):
    """Himeno set-up of himenobmtxpa_physis.c:126-141 / the original's 86-116:
    p = z^2/(nz-1)^2 in both p grids, a0=a1=a2=1, a3=1/6, b*=0, c*=1,
    bnd=1, wrk1=0.  Returns the 14 grids in map order."""
    shape = (nz, ny, nx)
    z = np.arange(nz, dtype=np.int64)
    pz = (np.float32(1.0) * (z * z).astype(np.float32) /
          np.float32((nz - 1) * (nz - 1))).astype(dtype)
    p0 = np.broadcast_to(pz[:, None, None], shape).astype(dtype).copy()
    ones = np.ones(shape, dtype)
    zeros = np.zeros(shape, dtype)
    g = [p0, p0.copy(), ones.copy(), ones.copy(), ones.copy(),
         np.full(shape, dtype(np.float32(1.0 / 6.0)), dtype),
         zeros.copy(), zeros.copy(), zeros.copy(),
         ones.copy(), ones.copy(), ones.copy(), ones.copy(), zeros.copy()]
    return g


def test_himeno_matches_original(oracle):
    # The original Himeno jacobi (himenobmtxpa_original.c:297-346) at
    # rows=33 (z), cols=17 (y), deps=19 (x), 3 sweeps: p bit-exact and the
    # last sweep's float gosa bit-exact against the REF-order fold.
    nz, ny, nx, nn = 33, 17, 19, 3
    g = himeno_inputs(nx, ny, nz)
    dom = (1, nx - 1, 1, ny - 1, 1, nz - 1)
    for s in range(nn):
        gr, g64 = oracle.himeno19(g, dom, np.float32(0.8))
        g[0], g[1] = g[1], g[0]
    ref_p = gio.f32("himeno_ref_33x17x19_nn3.p.f32.gz", (nz, ny, nx))
    ref_gosa = gio.hexfloats("himeno_ref_33x17x19_nn3.gosa.txt")[0]
    assert np.array_equal(g[0].view(np.uint32), ref_p.view(np.uint32))
    assert float(gr) == ref_gosa
    # The FP64 residual differs from the float fold only by the fold's own
    # rounding (about 2e-5 relative here, 17,000 terms).
    assert abs(g64 - ref_gosa) <= 1e-4 * abs(g64)


def test_fp64_reduce_is_accurate(oracle):
    rng = np.random.default_rng(0)
    data = rng.random(100_000).astype(np.float32)
    exact = float(np.sum(data.astype(np.float64)))
    assert abs(oracle.reduce_fp64(data, oracle.PS_SUM) - exact) <= 1e-9 * exact


def test_uniform_stream_matches_python(oracle):
    from physis_gb300 import synth
    a = oracle.fill_uniform((3, 5, 7), seed=1)
    b = synth.uniform((3, 5, 7), seed=1)
    assert np.array_equal(a, b)
    assert a.min() >= 0.0 and a.max() < 1.0


@pytest.mark.parametrize("name", sorted(__import__("system_cases").CASES))
def test_point_stencil_system_tests(oracle, name):
    # The point-list system tests (tests/system_cases.py) through the
    # oracle's point-stencil restatement, against the programs' stdout.
    import system_cases as sc
    case = dict(sc.CASES[name])
    dom = sc.domain(case)
    case["grids"] = sc.initial(case)
    text = sc.run(
        case,
        lambda a, b: oracle.points(a, b, dom, case["points"],
                                   boundary=case["boundary"]),
        lambda a, color: oracle.points(a, a, dom, case["points"],
                                       boundary=case["boundary"], color=color),
        lambda a: oracle.reduce_ref(a.reshape(-1), oracle.PS_SUM),
        lambda a: gio.dump_text(a, sc.fmt(case)))
    assert text == gio.stdout_text(name)


def test_point_stencil_matches_sweep7(oracle):
    # The point-list form of DIFFUSION7 (clamp, weights in expression order
    # cc cw ce cs cn cb ct) equals the dedicated 7-point restatement.
    g = oracle.fill_uniform((9, 10, 11), seed=5)
    ref, out = np.zeros_like(g), np.zeros_like(g)
    coef = [0.11, 0.12, 0.13, 0.14, 0.15, 0.16, 0.4]  # ce cw cn cs ct cb cc
    dom = (0, 11, 0, 10, 0, 9)
    oracle.sweep7(oracle.V_DIFFUSION7, g, ref, dom, coef=coef)
    pts = [(0, 0, 0), (-1, 0, 0), (1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, -1),
           (0, 0, 1)]
    w = [coef[6], coef[1], coef[0], coef[3], coef[2], coef[5], coef[4]]
    oracle.points(g, out, dom, pts, weights=w, boundary=2)
    assert np.array_equal(ref.view(np.uint32), out.view(np.uint32))


def test_point_stencil_rejects_out_of_grid_reads(oracle):
    g = np.zeros((4, 4, 4), np.float32)
    with pytest.raises(ValueError):
        oracle.points(g, g.copy(), (0, 4, 0, 4, 0, 4), [(1, 0, 0)], boundary=0)
