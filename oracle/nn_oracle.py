"""CPU oracle of the learned warm start's arithmetic (numpy, FP64).

TEST INFRASTRUCTURE ONLY: imported by tests/ and by the smoke check in
__graft_entry__.py as the checker, never by the product.  The learned warm start has no counterpart in the reference, so
this oracle is pinned by its own consistency checks (the analytic gradients
below against central finite differences, tests/test_nn_oracle.py) and the
GPU kernels are checked against it.

Tensors are channels-last, [batch, z, y, x, 16], BF16 stored as uint16.
conv: Y[b,z,y,x,o] = bias[o] + sum_{t, i} X[b, (z,y,x) + d_t, i] * W[t, i, o]
with the 27 taps t = (dz+1)*9 + (dy+1)*3 + (dx+1), zero padding.
"""
import numpy as np

C = 16          # channels of every layer (inputs and the output padded)
TAPS = [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def to_bf16(a):
    """float -> bf16 bits (uint16), round to nearest even."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return r.astype(np.uint16)


def from_bf16(b):
    return (np.asarray(b, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def _shift(x, d):
    """x[b, z+dz, y+dy, x+dx, :] with zeros outside (x: [B,Z,Y,X,C])."""
    dz, dy, dx = d
    out = np.zeros_like(x)
    B, Z, Y, X, _ = x.shape
    zs = slice(max(0, -dz), min(Z, Z - dz))
    ys = slice(max(0, -dy), min(Y, Y - dy))
    xs = slice(max(0, -dx), min(X, X - dx))
    zt = slice(max(0, dz), min(Z, Z + dz))
    yt = slice(max(0, dy), min(Y, Y + dy))
    xt = slice(max(0, dx), min(X, X + dx))
    out[:, zs, ys, xs, :] = x[:, zt, yt, xt, :]
    return out


def conv_fwd(x, w, bias=None):
    """x [B,Z,Y,X,Ci], w [27,Ci,Co] -> [B,Z,Y,X,Co] in float64."""
    x = np.asarray(x, np.float64)
    w = np.asarray(w, np.float64)
    y = np.zeros(x.shape[:4] + (w.shape[2],))
    for t, d in enumerate(TAPS):
        y += _shift(x, d) @ w[t]
    if bias is not None:
        y += np.asarray(bias, np.float64)
    return y


def conv_bwd_data(dy, w):
    """dL/dx of conv_fwd given dL/dy: the conv of dy with w flipped in space
    and transposed in channels."""
    wt = np.asarray(w, np.float64)[::-1].transpose(0, 2, 1)
    return conv_fwd(dy, wt)


def conv_bwd_weight(x, dy):
    """dL/dw [27,Ci,Co] and dL/dbias [Co]."""
    x = np.asarray(x, np.float64)
    dy = np.asarray(dy, np.float64)
    ci, co = x.shape[-1], dy.shape[-1]
    dw = np.zeros((27, ci, co))
    for t, d in enumerate(TAPS):
        dw[t] = _shift(x, d).reshape(-1, ci).T @ dy.reshape(-1, co)
    return dw, dy.reshape(-1, co).sum(0)


def relu(a):
    return np.maximum(a, 0.0)


def _round_bf16(a):
    return from_bf16(to_bf16(a)).astype(np.float64)


def network_fwd(x, ws, bs, bf16=False):
    """The 6-layer net: conv+ReLU x5, conv; returns every layer's output in
    float64.  bf16=True rounds the hidden activations to BF16 where the GPU
    stores them (the last layer's output stays unrounded)."""
    acts = [np.asarray(x, np.float64)]
    for l, (w, b) in enumerate(zip(ws, bs)):
        y = conv_fwd(acts[-1], w, b)
        if l < len(ws) - 1:
            y = relu(y)
            if bf16:
                y = _round_bf16(y)
        acts.append(y)
    return acts


def mse_loss(pred, target):
    """Mean of (pred[..., 0] - target)^2 and its gradient wrt pred."""
    diff = np.asarray(pred[..., 0], np.float64) - np.asarray(target, np.float64)
    g = np.zeros(np.shape(pred))
    g[..., 0] = 2.0 * diff / diff.size
    return float((diff ** 2).mean()), g


def network_grads(x, ws, bs, target, bf16=False):
    """Loss and gradients of every weight and bias (float64 backprop).
    bf16=True also rounds the activations and the propagated gradients to
    BF16 at the points where the GPU stores them in BF16."""
    acts = network_fwd(x, ws, bs, bf16)
    loss, g = mse_loss(acts[-1], target)
    if bf16:
        g = _round_bf16(g)
    dws, dbs = [None] * len(ws), [None] * len(ws)
    for l in range(len(ws) - 1, -1, -1):
        dws[l], dbs[l] = conv_bwd_weight(acts[l], g)
        if l:
            g = conv_bwd_data(g, ws[l]) * (acts[l] > 0)
            if bf16:
                g = _round_bf16(g)
    return loss, dws, dbs


def adam(w, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba 2015), bias-corrected; returns new w, m, v."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return w - lr * mh / (np.sqrt(vh) + eps), m, v


def pool(fine, f):
    """Mean over f x f x f blocks (partial blocks at the far edges average
    what they hold): fine [Z,Y,X] -> [ceil(Z/f), ceil(Y/f), ceil(X/f)]."""
    Z, Y, X = fine.shape
    zc, yc, xc = -(-Z // f), -(-Y // f), -(-X // f)
    s = np.zeros((zc, yc, xc))
    n = np.zeros((zc, yc, xc))
    iz, iy, ix = np.meshgrid(np.arange(Z) // f, np.arange(Y) // f, np.arange(X) // f,
                             indexing="ij")
    np.add.at(s, (iz, iy, ix), fine)
    np.add.at(n, (iz, iy, ix), 1.0)
    return s / n


def centre_sample(fine, f):
    """Value at each f^3 block's centre (z_c + 0.5) f - 0.5: the mean of the
    fine cells nearest to it (2 per axis for even f, 1 for odd f), clamped to
    the grid."""
    out = np.asarray(fine, np.float64)
    for axis, n in enumerate(fine.shape):
        nc = -(-n // f)
        pos = (np.arange(nc) + 0.5) * f - 0.5
        i0 = np.minimum(np.floor(pos).astype(int), n - 1)
        i1 = np.minimum(np.ceil(pos).astype(int), n - 1)
        out = 0.5 * (np.take(out, i0, axis=axis) + np.take(out, i1, axis=axis))
    return out


def catmull_rom(t):
    """Weights of points -1, 0, 1, 2 for a position t in [0, 1] past point 0
    (Catmull & Rom 1974: the cubic through the four points with central-
    difference end slopes)."""
    t2, t3 = t * t, t * t * t
    return ((-t3 + 2 * t2 - t) / 2, (3 * t3 - 5 * t2 + 2) / 2,
            (-3 * t3 + 4 * t2 + t) / 2, (t3 - t2) / 2)


def upsample(coarse, shape, f):
    """Catmull-Rom cubic interpolation, axis by axis, from coarse cell
    centres (c + 0.5) f - 0.5 to every fine point; positions are clamped to
    [0, nc - 1] and neighbour indices to the coarse grid."""
    out = np.asarray(coarse, np.float64)
    for axis, n in enumerate(shape):
        nc = coarse.shape[axis]
        pos = np.clip((np.arange(n) + 0.5) / f - 0.5, 0, nc - 1)
        i0 = np.minimum(np.floor(pos).astype(int), nc - 1)
        t = pos - i0
        ws = catmull_rom(t)
        sh = [1] * out.ndim
        sh[axis] = n
        acc = 0.0
        for k, w in zip((-1, 0, 1, 2), ws):
            idx = np.clip(i0 + k, 0, nc - 1)
            acc = acc + np.take(out, idx, axis=axis) * w.reshape(sh)
        out = acc
    return out


def mirror(field, flip):
    """Mirror image of a [z, y, x] field: flip bits 0/1/2 mirror x/y/z and bit
    3 swaps x and y (the swap is applied to the stored field first, then the
    mirrors, so image(z', y', x') = field(z, y, x) with x1 = mirrored x',
    y1 = mirrored y' and (x, y) = (y1, x1) under the swap)."""
    a = np.asarray(field)
    if flip & 8:
        a = a.transpose(0, 2, 1)
    if flip & 1:
        a = a[:, :, ::-1]
    if flip & 2:
        a = a[:, ::-1, :]
    if flip & 4:
        a = a[::-1, :, :]
    return np.ascontiguousarray(a)


def unmirror(field, flip):
    """The inverse of mirror(): a field given in mirror-image coordinates,
    back in the stored instance's."""
    a = np.asarray(field)
    if flip & 4:
        a = a[::-1, :, :]
    if flip & 2:
        a = a[:, ::-1, :]
    if flip & 1:
        a = a[:, :, ::-1]
    if flip & 8:
        a = a.transpose(0, 2, 1)
    return np.ascontiguousarray(a)


def mirror_instance(inst, flip):
    """The mirrored instance: every field mirrored, a2 and a1 exchanged under
    the x/y swap (the 19-point sweep weighs the z neighbours with a0, the y
    neighbours with a1 and the x neighbours with a2)."""
    out = {k: mirror(v, flip) for k, v in inst.items()}
    if flip & 8:
        out["a1"], out["a2"] = out["a2"], out["a1"]
    return out


POOL_CHANNELS = 9


def pool_features(inst, f, wscale):
    """The network input of one instance, [zc, yc, xc, 9] float64: block means
    of ln a0, ln a1, ln a2, wrk1 * wscale, bnd, wrk1 * 3 / (a0 + a1 + a2) *
    wscale, and -ln of the block means of 1 / a0, 1 / a1, 1 / a2."""
    a0, a1, a2 = (np.asarray(inst[k], np.float64) for k in ("a0", "a1", "a2"))
    w = np.asarray(inst["wrk1"], np.float64)
    feats = [pool(np.log(a0), f), pool(np.log(a1), f), pool(np.log(a2), f),
             pool(w, f) * wscale, pool(np.asarray(inst["bnd"], np.float64), f),
             pool(w * 3.0 / (a0 + a1 + a2), f) * wscale,
             -np.log(pool(1.0 / a0, f)), -np.log(pool(1.0 / a1, f)), -np.log(pool(1.0 / a2, f))]
    return np.stack(feats, axis=-1)


def residual_source(inst, p):
    """Source of the correction problem for an iterate p of one instance
    (arrays [z, y, x]): with c_i = a_i and b = 0 the Himeno residual is
    ss = (s0 a3 - p) bnd, s0 = sum_i a_i (p(x + e_i) + p(x - e_i)) + wrk1,
    a3 = 1 / (2 (a0 + a1 + a2)) (examples/himeno/himenobmtxpa_original.c:
    331-334 with these coefficients), and r = ss / a3.  a0 weighs the z
    neighbours, a1 the y and a2 the x neighbours.  Zero on the faces."""
    a0, a1, a2 = (np.asarray(inst[k], np.float64) for k in ("a0", "a1", "a2"))
    w, bnd = np.asarray(inst["wrk1"], np.float64), np.asarray(inst["bnd"], np.float64)
    p = np.asarray(p, np.float64)
    r = np.zeros_like(p)
    i = (slice(1, -1),) * 3
    s0 = (a0[i] * (p[2:, 1:-1, 1:-1] + p[:-2, 1:-1, 1:-1]) +
          a1[i] * (p[1:-1, 2:, 1:-1] + p[1:-1, :-2, 1:-1]) +
          a2[i] * (p[1:-1, 1:-1, 2:] + p[1:-1, 1:-1, :-2]) + w[i])
    r[i] = (s0 - 2.0 * (a0[i] + a1[i] + a2[i]) * p[i]) * bnd[i]
    return r
