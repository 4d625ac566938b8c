"""Pins the learned warm start's CPU oracle (oracle/nn_oracle.py) without a
GPU: analytic backprop against central finite differences in float64, BF16
rounding against known encodings, pooling and upsampling against their
definitions."""
import numpy as np
import pytest

from oracle import nn_oracle as nn


def _net(rng, cin=3, c=4, layers=3):
    ws, bs = [], []
    for l in range(layers):
        ci = cin if l == 0 else c
        co = 1 if l == layers - 1 else c
        ws.append(rng.normal(0, 0.3, size=(27, ci, co)))
        bs.append(rng.normal(0, 0.1, size=co))
    return ws, bs


def test_backprop_matches_finite_differences():
    rng = np.random.default_rng(0)
    x = rng.normal(size=(2, 3, 4, 5, 3))
    t = rng.normal(size=(2, 3, 4, 5))
    ws, bs = _net(rng)
    loss, dws, dbs = nn.network_grads(x, ws, bs, t)
    h = 1e-6
    for l in range(len(ws)):
        for idx in [(0, 0, 0), (13, 1, 0), (26, 2, -1), (5, -1, 0)]:
            w2 = [w.copy() for w in ws]
            w2[l][idx] += h
            lp = nn.network_grads(x, w2, bs, t)[0]
            w2[l][idx] -= 2 * h
            lm = nn.network_grads(x, w2, bs, t)[0]
            fd = (lp - lm) / (2 * h)
            assert abs(fd - dws[l][idx]) <= 1e-6 * max(1.0, abs(fd)), (l, idx)
        b2 = [b.copy() for b in bs]
        b2[l][0] += h
        lp = nn.network_grads(x, ws, b2, t)[0]
        b2[l][0] -= 2 * h
        lm = nn.network_grads(x, ws, b2, t)[0]
        assert abs((lp - lm) / (2 * h) - dbs[l][0]) <= 1e-6 * max(1.0, abs(dbs[l][0]))


def test_bwd_data_is_the_adjoint_of_fwd():
    rng = np.random.default_rng(1)
    x = rng.normal(size=(1, 4, 3, 5, 6))
    dy = rng.normal(size=(1, 4, 3, 5, 7))
    w = rng.normal(size=(27, 6, 7))
    lhs = (nn.conv_fwd(x, w) * dy).sum()
    rhs = (x * nn.conv_bwd_data(dy, w)).sum()
    assert abs(lhs - rhs) <= 1e-9 * abs(lhs)


def test_bf16_rounding():
    vals = np.array([1.0, -2.5, 3.14159265, 1e-3, 65504.0, 1.00390625, 1.01171875],
                    np.float32)
    b = nn.to_bf16(vals)
    assert list(b[:2]) == [0x3F80, 0xC020]
    assert nn.from_bf16(nn.to_bf16(np.float32(1.00390625)))[()] == 1.0   # tie -> even
    assert nn.from_bf16(nn.to_bf16(np.float32(1.01171875)))[()] == 1.015625
    back = nn.from_bf16(b)
    assert np.all(np.abs(back - vals) <= np.abs(vals) * 2 ** -8)


def test_pool_and_upsample():
    rng = np.random.default_rng(2)
    f = rng.normal(size=(9, 6, 5))
    p = nn.pool(f, 4)
    assert p.shape == (3, 2, 2)
    assert np.isclose(p[0, 0, 0], f[:4, :4, :4].mean())
    assert np.isclose(p[2, 1, 1], f[8:, 4:, 4:].mean())
    c = rng.normal(size=(3, 2, 2))
    u = nn.upsample(np.ones_like(c) * 2.5, (9, 6, 5), 4)
    assert np.allclose(u, 2.5)
    # the coarse values are reproduced at the coarse centres, and linear
    # fields between the second and the second-to-last centre (where all
    # four Catmull-Rom points lie inside)
    lin = np.fromfunction(lambda z, y, x: 0.5 * z - y + 2 * x, (5, 5, 5))
    up = nn.upsample(lin, (20, 20, 20), 4)
    zf, yf, xf = np.meshgrid(*([(np.arange(20) + 0.5) / 4 - 0.5] * 3), indexing="ij")
    inside = (zf >= 1) & (zf <= 3) & (yf >= 1) & (yf <= 3) & (xf >= 1) & (xf <= 3)
    assert np.allclose(up[inside], (0.5 * zf - yf + 2 * xf)[inside])
    w = nn.catmull_rom(np.linspace(0, 1, 7))
    assert np.allclose(sum(w), 1.0)
    f2 = np.arange(8 * 8 * 8, dtype=float).reshape(8, 8, 8)
    cs = nn.centre_sample(f2, 4)
    assert cs.shape == (2, 2, 2)
    assert np.isclose(cs[0, 0, 0], f2[1:3, 1:3, 1:3].mean())


def test_mirror_images_solve_the_mirrored_problem():
    # The 19-point operator with c_i = a_i and b = 0 weighs both neighbours
    # of a cell along an axis with that cell's a_i, and the Dirichlet faces
    # are symmetric: Jacobi sweeps of a mirrored instance give the mirrored
    # iterate (to rounding: the mirrored sum runs in another order).  This is
    # what lets one solve stand for 16 training pairs.
    from oracle import pyoracle as po
    from physis_gb300 import warmstart as ws
    rng = np.random.default_rng(11)
    shape = (10, 7, 7)
    inst = ws.make_instance(rng, shape)

    def jacobi(fields, sweeps=30):
        arr = [np.ascontiguousarray(a, np.float32) for a in ws.himeno_arrays(fields)]
        p0 = np.zeros(shape, np.float32)
        p1 = np.zeros(shape, np.float32)
        dom = (1, shape[2] - 1, 1, shape[1] - 1, 1, shape[0] - 1)
        for _ in range(sweeps):
            po.himeno19([p0, p1] + arr, dom, ws.OMEGA)
            p0, p1 = p1, p0
        return p0

    base = jacobi(inst)
    assert np.abs(base).max() > 0
    for flip in (1, 2, 4, 8, 15):
        got = jacobi(nn.mirror_instance(inst, flip))
        assert np.allclose(got, nn.mirror(base, flip), rtol=1e-5, atol=1e-6 * np.abs(base).max()), flip
    # a1 and a2 (y and x coefficients) must trade places under the swap:
    # without it the swap is not a symmetry
    wrong = nn.mirror_instance(inst, 8)
    wrong["a1"], wrong["a2"] = wrong["a2"], wrong["a1"]
    assert not np.allclose(jacobi(wrong), nn.mirror(base, 8), rtol=1e-3)


def test_pool_features_definition():
    rng = np.random.default_rng(12)
    inst = {k: np.exp(rng.uniform(-0.7, 0.7, size=(6, 5, 5))) for k in ("a0", "a1", "a2")}
    inst["wrk1"] = rng.normal(size=(6, 5, 5))
    inst["bnd"] = np.ones((6, 5, 5))
    feats = nn.pool_features(inst, 2, 0.5)
    assert feats.shape == (3, 3, 3, nn.POOL_CHANNELS)
    blk = (slice(0, 2), slice(0, 2), slice(2, 4))
    a = [inst[k][blk] for k in ("a0", "a1", "a2")]
    w = inst["wrk1"][blk]
    assert np.isclose(feats[0, 0, 1, 5], (w * 3 / (a[0] + a[1] + a[2])).mean() * 0.5)
    assert np.isclose(feats[0, 0, 1, 7], -np.log((1 / a[1]).mean()))
    # partial block at the far x edge (one column)
    assert np.isclose(feats[0, 0, 2, 0], np.log(inst["a0"][0:2, 0:2, 4:5]).mean())


def test_unmirror_inverts_mirror():
    a = np.arange(4 * 5 * 5).reshape(4, 5, 5)
    for flip in range(16):
        assert np.array_equal(nn.unmirror(nn.mirror(a, flip), flip), a), flip


def test_mirror_image_lists():
    # the warm start's host helpers: a square x-y section has 16 mirror
    # images (8 axis mirrors, then the same with x and y swapped), any other
    # shape 8; coarse grids round up
    from physis_gb300 import warmstart as ws
    assert ws.mirror_images((257, 129, 129), 16) == list(range(16))
    assert ws.mirror_images((65, 33, 31), 16) == list(range(8))
    assert ws.mirror_images((65, 33, 33), 1) == [0]
    assert ws.mirror_images((65, 33, 33), 0) == [0]
    assert ws.coarse_shape((257, 129, 129), 16) == (17, 9, 9)
    assert ws.coarse_shape((65, 33, 33), 4) == (17, 9, 9)


def test_residual_source_is_the_himeno_residual_over_a3():
    # The correction problem's source r = ss / a3 (nn.residual_source)
    # against the REF Himeno sweep of the C oracle: its gosa is sum ss^2, and
    # with omega = 1 its update is p1 = p0 + ss, so ss = p1 - p0.
    from oracle import pyoracle
    from physis_gb300 import warmstart as ws
    rng = np.random.default_rng(3)
    shape = (11, 9, 8)
    inst = ws.make_instance(rng, shape)
    p = rng.normal(size=shape).astype(np.float32)
    arrays = [p.copy(), np.zeros(shape, np.float32)] + ws.himeno_arrays(inst)
    nz, ny, nx = shape
    g_ref, g64 = pyoracle.himeno19(arrays, (1, nx - 1, 1, ny - 1, 1, nz - 1), np.float32(1.0))
    ss = (arrays[1].astype(np.float64) - p)[1:-1, 1:-1, 1:-1]
    a3 = arrays[5].astype(np.float64)[1:-1, 1:-1, 1:-1]
    r = nn.residual_source(inst, p)
    assert np.allclose(r[1:-1, 1:-1, 1:-1] * a3, ss, rtol=1e-5, atol=1e-5 * np.abs(ss).max())
    assert abs(float(((r[1:-1, 1:-1, 1:-1] * a3) ** 2).sum()) - g64) <= 1e-4 * g64
    assert not r[0].any() and not r[-1].any() and not r[:, 0].any() and not r[:, :, -1].any()
