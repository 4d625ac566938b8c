"""Parity at the full benchmark sizes.  The oracle runs a few steps there
(seconds on the host cores); longer runs are checked through properties
that do not depend on the size.

* 7-point diffusion, 512^3 float (the bench's headline run):
  * 20 steps: bit-identical to the oracle;
  * 1000 steps: the sweep conserves the grid's sum up to the coefficients'
    float sum (every cell's value leaves with total weight cc + cw + ce + ...,
    because the clamped faces reuse the centre and cw = ce, cn = cs, ct = cb);
    values stay inside the initial range times that factor; the FP64
    reduction equals a host FP64 sum; temporal blocking (k = 2) gives the same
    bits as the plain sweeps;
  * contracted temporal passes stay within 1e-5 relative per cell of the
    plain (REF) result over 200 and 600 steps; over the whole 1000 steps
    they drift to about 1.2e-5 (checked to stay under 2e-5), which is why
    they are not reported as results of the 1000-step run.
* Himeno 19-point, 257 x 257 x 513 float (the bench's set-up), 12 sweeps:
  every fused residual equals the oracle's FP64 residual of the same sweep,
  the pressure is bit-identical to the oracle's, and the plain sweep writes
  the same bits as the fused one.  (In float32 this residual does not fall
  monotonically at this size: the oracle's sequence rises at sweeps 2, 3, 7
  and 9, by up to 1 %.)
This file runs last in the GPU suite (its name sorts last): it holds up to 2 GB
of device memory for a few seconds.
"""
import os

import numpy as np
import pytest

import physis_gb300 as ps
from physis_gb300 import synth

pytestmark = pytest.mark.gpu

COEF = (0.1, 0.1, 0.1, 0.1, 0.1, 0.1, 0.4)  # ce cw cn cs ct cb cc


@pytest.fixture(scope="module")
def rt():
    ps.build()
    ps.init()
    yield ps
    ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, 1)
    ps.set_fma(False)
    ps.clear_error()


def _bits(a):
    return a.view(np.uint32)


def _threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def test_diffusion_512_cubed(rt, oracle):
    n, steps = 512, 1000
    shape = (n, n, n)
    init = synth.uniform(shape, 1)
    g1, g2 = ps.Grid(shape), ps.Grid(shape)
    dom = ps.full_domain(shape)
    m1 = ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, dom, [g1, g2], COEF)
    m2 = ps.stencil_map(ps.PS_KERNEL_DIFFUSION7, dom, [g2, g1], COEF)

    def run(k=1, fma=False, n_steps=steps):
        ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, k, warps=8, rows=4, ns=3)
        ps.set_fma(fma)
        try:
            g1.copyin(init)
            g2.copyin(init)
            ps.stencil_run([m1, m2], n_steps // 2)
        finally:
            ps.set_temporal(ps.PS_KERNEL_DIFFUSION7, 1)
            ps.set_fma(False)
        return g1.copyout()

    # 20 steps against the oracle, bit for bit
    short = run(n_steps=20)
    r1, r2 = init.copy(), np.zeros_like(init)
    oracle.run7(oracle.V_DIFFUSION7, r1, r2, (0, n, 0, n, 0, n), COEF, iter=10,
                nthreads=_threads())
    assert np.array_equal(_bits(short), _bits(r1))
    del r1, r2, short

    plain = run()
    growth = float(np.sum([np.float64(np.float32(c)) for c in COEF])) ** steps
    sum0 = float(init.sum(dtype=np.float64))
    host = float(plain.sum(dtype=np.float64))
    dev = ps.reduce_f64(g1, ps.PS_SUM)
    assert abs(dev - host) <= 1e-6 * abs(host)
    # rounding drifts the sum by about -7.5e-6 over 1000 steps (measured with
    # the oracle at 64^3 and 128^3, independent of the size); a face that
    # lost its clamp would move it by ~2e-4 per step
    assert abs(host / (sum0 * growth) - 1.0) < 3e-5
    assert np.isfinite(plain).all()
    assert plain.min() >= float(init.min()) * growth - 1e-4
    assert plain.max() <= float(init.max()) * growth + 1e-4

    temporal = run(k=2)
    assert np.array_equal(_bits(temporal), _bits(plain))

    # contraction changes each step's rounding; the difference grows by about
    # 1.3e-8 relative per step (2.7e-6 after 200 steps in a numpy model at 64^3)
    fused = run(k=2, fma=True, n_steps=200)
    plain200 = run(n_steps=200)
    assert np.allclose(fused, plain200, rtol=1e-5, atol=0)
    # Longer runs: the plain sweeps are the REF sequence bit for bit (20
    # steps against the oracle above, and temporal = plain bits), so this is
    # the contracted pass against REF.  The drift keeps growing: within 1e-5
    # at 600 steps, but 1.2e-5 after the benchmark's 1000 steps, so
    # contracted passes are not reported as results of the 1000-step run.
    fused = run(k=2, fma=True, n_steps=600)
    plain600 = run(n_steps=600)
    rel = float(np.max(np.abs(fused.astype(np.float64) - plain600) / np.abs(plain600)))
    assert rel <= 1e-5, rel
    fused = run(k=2, fma=True)
    rel = float(np.max(np.abs(fused.astype(np.float64) - plain) / np.abs(plain)))
    assert 1e-6 < rel <= 2e-5, rel
    g1.free()
    g2.free()


def _himeno_setup(nx, ny, nz):
    import bench
    return bench.himeno_arrays(nx, ny, nz)


def _host_gosa(arrays):
    """Sum of ss^2 (FP64 of float32 ss) of one sweep from arrays[0], the REF
    expression order of himenobmtxpa_physis.c:331-361 with b = 0 (its three
    b-terms add exact zeros)."""
    p, a0, a1, a2, a3, c0, c1, c2, bnd, wrk1 = (arrays[0], arrays[2], arrays[3], arrays[4],
                                                arrays[5], arrays[9], arrays[10], arrays[11],
                                                arrays[12], arrays[13])
    assert not arrays[6].any() and not arrays[7].any() and not arrays[8].any()
    i = (slice(1, -1), slice(1, -1), slice(1, -1))
    zp = (slice(2, None), slice(1, -1), slice(1, -1))
    zm = (slice(None, -2), slice(1, -1), slice(1, -1))
    yp = (slice(1, -1), slice(2, None), slice(1, -1))
    ym = (slice(1, -1), slice(None, -2), slice(1, -1))
    xp = (slice(1, -1), slice(1, -1), slice(2, None))
    xm = (slice(1, -1), slice(1, -1), slice(None, -2))
    s0 = a0[i] * p[zp]
    s0 = s0 + a1[i] * p[yp]
    s0 = s0 + a2[i] * p[xp]
    s0 = s0 + c0[i] * p[zm]
    s0 = s0 + c1[i] * p[ym]
    s0 = s0 + c2[i] * p[xm]
    s0 = s0 + wrk1[i]
    ss = (s0 * a3[i] - p[i]) * bnd[i]
    assert ss.dtype == np.float32
    return float(np.square(ss.astype(np.float64)).sum())


def test_himeno_257x257x513(rt, oracle):
    nx, ny, nz = 257, 257, 513
    shape = (nz, ny, nx)
    arrays = _himeno_setup(nx, ny, nz)
    gs = [ps.Grid(shape) for _ in range(14)]
    for g, a in zip(gs, arrays):
        g.copyin(a)
    domt = (1, nx - 1, 1, ny - 1, 1, nz - 1)
    dom = ps.domain(*domt)
    omega = np.float32(0.8)
    host0 = _host_gosa(arrays)
    ref = [a.copy() for a in arrays]
    order = [gs, [gs[1], gs[0]] + gs[2:]]
    for s in range(12):
        gosa = float(ps.reduce_kernel(ps.PS_SUM, ps.PS_KERNEL_HIMENO19_GOSA, dom,
                                      order[s % 2], [omega]))
        _, g64 = oracle.himeno19(ref, domt, omega, nthreads=_threads())
        ref[0], ref[1] = ref[1], ref[0]
        if s == 0:
            assert abs(g64 - host0) <= 1e-12 * host0
        assert abs(gosa - g64) <= 1e-5 * g64, s
    fused = gs[0].copyout()  # 12 sweeps: the result is back in p0
    assert np.array_equal(_bits(fused), _bits(ref[0]))
    # the same 12 sweeps with the plain kernel from the initial state
    gs[0].copyin(arrays[0])
    gs[1].copyin(arrays[1])
    m1 = ps.stencil_map(ps.PS_KERNEL_HIMENO19, dom, gs, [omega])
    m2 = ps.stencil_map(ps.PS_KERNEL_HIMENO19, dom, [gs[1], gs[0]] + gs[2:], [omega])
    ps.stencil_run([m1, m2], 6)
    assert np.array_equal(_bits(gs[0].copyout()), _bits(fused))
    for g in gs:
        g.free()
