"""Float32 Jacobi near its fixed point, on the CPU.

The C oracle's REF-order Himeno sweep gives the same bits as the GPU kernel
(tests/test_gpu_parity.py), so its float32 behaviour is the GPU's.  Started
from zero, the iteration ends at an exact fixed point (computed residual 0).
Started a few ulps away from that point, it can lock into a 2-cycle whose
residual stays a little above 1e-6 -- which is where learned restarts leave
an iterate.  Pulling such a start back along the solution by a relative 1e-4
(what the warm start's `pullback` does) makes the last approach run like a
zero start's, and it ends at or below the tolerance.
"""
import numpy as np

from oracle import pyoracle
from physis_gb300 import warmstart as ws

SHAPE = (33, 17, 17)
OMEGA = np.float32(0.8)


def _grids(inst, p):
    return [p.copy(), p.copy()] + ws.himeno_arrays(inst)


def _dom():
    nz, ny, nx = SHAPE
    return (1, nx - 1, 1, ny - 1, 1, nz - 1)


def _sweep(g, n):
    for _ in range(n):
        pyoracle.himeno19(g, _dom(), OMEGA)
        g[0], g[1] = g[1], g[0]


def _residual(g, r0):
    h = [x.copy() for x in g]
    _, g64 = pyoracle.himeno19(h, _dom(), OMEGA)
    return float(np.sqrt(g64 / r0))


def test_close_starts_lock_into_two_cycles_and_pullback_avoids_them():
    rng = np.random.default_rng(0)
    inst = ws.make_instance(rng, SHAPE)
    inst["wrk1"] = (inst["wrk1"] * 8).astype(np.float32)  # |p| ~ 60: floor near 1e-6
    r0 = ws.residual0(inst)
    g = _grids(inst, np.zeros(SHAPE, np.float32))
    prev = None
    for _ in range(400):
        _sweep(g, 100)
        if prev is not None and np.array_equal(prev, g[0]):
            break
        prev = g[0].copy()
    fixed = g[0].copy()
    assert np.array_equal(fixed, g[1]) and _residual(g, r0) == 0.0  # a fixed point
    ulp = np.spacing(np.abs(fixed)).astype(np.float64)
    locked = 0
    for trial in range(2):
        pert = np.random.default_rng(100 + trial).integers(-4, 5, size=SHAPE) * ulp
        start = (fixed + pert * inst["bnd"]).astype(np.float32)
        h = _grids(inst, start)
        _sweep(h, 3000)
        a = h[0].copy()
        _sweep(h, 1)
        b = h[0].copy()
        _sweep(h, 1)
        if np.array_equal(a, h[0]) and not np.array_equal(a, b) and _residual(h, r0) > 1e-6:
            locked += 1
        # the same start pulled back by a relative 1e-4
        h = _grids(inst, (start * np.float32(1.0 - 1e-4)).astype(np.float32))
        _sweep(h, 3000)
        assert _residual(h, r0) <= 1e-6, trial
    assert locked >= 1
