"""Learned warm start for the 19-point Jacobi (Himeno) pressure-Poisson solve.

No counterpart in the reference.  A small 3D convolutional network predicts
the solution of a variable-coefficient Jacobi solve from its coefficient and
source fields; Jacobi then iterates from that prediction to the same
residual tolerance, so the plain zero-start solve stays both the fallback
and the yardstick (a bad prediction costs sweeps, it cannot change the
answer).

Pieces, all on the GPU through libphysis_gb300's C ABI:
* instances (seeded, built on the host): coefficients a0, a1, a2 log-uniform
  in [0.5, 2] smoothed by a Gaussian of sigma 4 cells (then stretched back to
  [0.5, 2]); c_i = a_i; a3 = 1 / (2 (a0 + a1 + a2)); b = 0; source wrk1 = 8
  Gaussian blobs (centres uniform, widths U[3, 12] cells, amplitudes N(0, 1));
  bnd = 1 inside, 0 on the faces (Dirichlet zero); omega = 0.8;
* targets: the library's own Himeno sweeps (PS_KERNEL_HIMENO19) run to a
  relative residual of 1e-7, many instances at once in one stacked grid
  (instances side by side in x and z; their bnd = 0 faces keep them apart),
  the per-instance residual read with PSReduce's kernel form;
* the network: pool the fine fields to factor^3 blocks, 6 conv layers 3x3x3 x
  16 channels (ReLU between), BF16 weights and activations, FP32
  accumulation (PSWarmStartConv on tensor cores), trained with MSE and Adam
  (PSWarmStartWeightGrad, PSWarmStartLoss, PSWarmStartAdam); the coarse
  prediction is upsampled to the fine grid by Catmull-Rom cubic
  interpolation (PSWarmStartUpsample); targets are sampled at the block
  centres, so the upsampled target reproduces the solution to O(h^3);
* training pairs: each solved instance and its mirror images (axis mirrors
  and the x/y swap), which solve the mirrored problem exactly.

Relative residual: ||ss|| / ||ss(p = 0)|| with ss = (s0 a3 - p) bnd, the
Himeno residual (examples/himeno/himenobmtxpa_original.c:331-334).
PyTorch provides device buffers and copies only; every computation is one of
the library's kernels.
"""
import ctypes
import math
import time

import numpy as np

import physis_gb300 as ps

OMEGA = 0.8
C = 16
LAYERS = 6
CIN = 9  # input channels the pooling kernel fills (the rest are zeros)


# ---- instances ----------------------------------------------------------------

def _gaussian_smooth(u, sigma):
    """Separable Gaussian filter (truncated at 3 sigma, edges mirrored about
    the boundary half-sample, scipy.ndimage's "reflect")."""
    try:  # scipy's C implementation of the same filter, when present
        from scipy.ndimage import gaussian_filter
        return gaussian_filter(u, sigma, mode="reflect", truncate=3.0)
    except ImportError:
        pass
    r = int(math.ceil(3 * sigma))
    k = np.exp(-0.5 * (np.arange(-r, r + 1) / sigma) ** 2)
    k /= k.sum()
    out = u
    for axis in range(3):
        pad = [(0, 0)] * 3
        pad[axis] = (r, r)
        p = np.pad(out, pad, mode="symmetric")
        acc = np.zeros_like(out)
        for i, w in enumerate(k):
            sl = [slice(None)] * 3
            sl[axis] = slice(i, i + out.shape[axis])
            acc += w * p[tuple(sl)]
        out = acc
    return out


def make_instance(rng, shape):
    """One seeded instance: dict of float32 fields shaped (nz, ny, nx)."""
    lo, hi = math.log(0.5), math.log(2.0)
    f = {}
    for name in ("a0", "a1", "a2"):
        s = _gaussian_smooth(rng.uniform(lo, hi, size=shape), 4.0)
        s = (s - s.min()) / max(s.max() - s.min(), 1e-12) * (hi - lo) + lo
        f[name] = np.exp(s).astype(np.float32)
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    w = np.zeros(shape)
    for _ in range(8):
        cz, cy, cx = rng.uniform(0, nz), rng.uniform(0, ny), rng.uniform(0, nx)
        width = rng.uniform(3.0, 12.0)
        amp = rng.normal()
        w += amp * np.exp(-((z - cz) ** 2 + (y - cy) ** 2 + (x - cx) ** 2) / (2 * width ** 2))
    f["wrk1"] = w.astype(np.float32)
    bnd = np.zeros(shape, np.float32)
    bnd[1:-1, 1:-1, 1:-1] = 1.0
    f["bnd"] = bnd
    return f


def himeno_arrays(inst):
    """The 12 coefficient/source arrays of PS_KERNEL_HIMENO19, in map order
    (a0 a1 a2 a3 b0 b1 b2 c0 c1 c2 bnd wrk1)."""
    a0, a1, a2 = inst["a0"], inst["a1"], inst["a2"]
    a3 = (1.0 / (2.0 * (a0.astype(np.float64) + a1 + a2))).astype(np.float32)
    z = np.zeros_like(a0)
    return [a0, a1, a2, a3, z, z, z, a0, a1, a2, inst["bnd"], inst["wrk1"]]


def residual0(inst):
    """||ss(p = 0)||^2 = sum (wrk1 a3 bnd)^2 in FP64."""
    arr = himeno_arrays(inst)
    ss = arr[11].astype(np.float64) * arr[3] * arr[10]
    return float((ss * ss).sum())


# ---- stacked solves -------------------------------------------------------------

class Stack:
    """Up to nsx * nsz instances side by side in x and z of one set of
    Himeno grids; unused slots have bnd = 0 (nothing moves there)."""

    def __init__(self, instances, shape, nsx):
        self.shape = shape
        nz, ny, nx = shape
        self.count = len(instances)
        self.nsx = nsx
        self.nsz = -(-self.count // nsx)
        gshape = (self.nsz * nz, ny, nsx * nx)
        host = [np.zeros(gshape, np.float32) for _ in range(12)]
        ones = np.ones(shape, np.float32)
        self.r0 = []
        for b in range(self.nsx * self.nsz):
            sl = self.slot(b)
            if b < self.count:
                arrs = himeno_arrays(instances[b])
                self.r0.append(residual0(instances[b]))
            else:
                z = np.zeros(shape, np.float32)
                arrs = [ones, ones, ones, ones * 0.1, z, z, z, ones, ones, ones, z, z]
            for h, a in zip(host, arrs):
                h[sl] = a
        self.grids = [ps.Grid(gshape) for _ in range(14)]  # p0 p1 + 12
        zero = np.zeros(gshape, np.float32)
        self.grids[0].copyin(zero)
        self.grids[1].copyin(zero)
        for g, h in zip(self.grids[2:], host):
            g.copyin(h)
        self.scratch = ps.Grid(gshape)
        self.gshape = gshape
        self.inner = ps.domain(1, gshape[2] - 1, 1, gshape[1] - 1, 1, gshape[0] - 1)
        order = [0, 1] + list(range(2, 14))
        self.m1 = ps.stencil_map(ps.PS_KERNEL_HIMENO19, self.inner,
                                 [self.grids[i] for i in order], [OMEGA])
        order2 = [1, 0] + list(range(2, 14))
        self.m2 = ps.stencil_map(ps.PS_KERNEL_HIMENO19, self.inner,
                                 [self.grids[i] for i in order2], [OMEGA])

    def slot(self, b):
        nz, ny, nx = self.shape
        ix, iz = b % self.nsx, b // self.nsx
        return (slice(iz * nz, (iz + 1) * nz), slice(0, ny), slice(ix * nx, (ix + 1) * nx))

    def set_p(self, p=None):
        """p0 = p (a device grid's contents already written) or zeros."""
        if p is None:
            self.grids[0].copyin(np.zeros(self.gshape, np.float32))

    def sweeps(self, n):
        """n sweeps (n even: the result is back in p0)."""
        assert n % 2 == 0
        if n:
            ps.stencil_run([self.m1, self.m2], n // 2)

    def residuals(self):
        """Relative residual of every instance (p in p0): one kernel-form
        PSReduce over the instance's interior, into a scratch grid."""
        nz, ny, nx = self.shape
        out = []
        grids = [self.grids[0], self.scratch] + self.grids[2:]
        for b in range(self.count):
            ix, iz = b % self.nsx, b // self.nsx
            dom = ps.domain(ix * nx + 1, (ix + 1) * nx - 1, 1, ny - 1,
                            iz * nz + 1, (iz + 1) * nz - 1)
            g = ps.reduce_kernel(ps.PS_SUM, ps.PS_KERNEL_HIMENO19_GOSA, dom, grids, [OMEGA])
            out.append(math.sqrt(max(float(g), 0.0) / self.r0[b]))
        return np.array(out)

    def solve(self, tol, chunk, max_sweeps, snapshots=()):
        """Sweeps (a multiple of `chunk`) after which each instance first
        met `tol`; -1 if it did not within max_sweeps.  `snapshots` pairs
        (sweep count, grid): p is copied into the grid when the count is
        reached (even counts; iterates for training the restarts)."""
        done = np.full(self.count, -1)
        snaps = sorted(snapshots, key=lambda t: t[0])
        n = 0
        while n < max_sweeps and ((done < 0).any() or snaps):
            stop = (n // chunk + 1) * chunk
            if snaps and snaps[0][0] < stop:
                stop = snaps[0][0]
            self.sweeps(stop - n)
            n = stop
            while snaps and snaps[0][0] == n:
                self.copy_p(snaps.pop(0)[1])
            if n % chunk == 0 and (done < 0).any():
                r = self.residuals()
                done[(done < 0) & (r <= tol)] = n
        return done

    def copy_p(self, grid):
        """grid = p (p0), through the library's copy kernel."""
        full = ps.full_domain(self.gshape)
        ps.stencil_run([ps.stencil_map(ps.PS_KERNEL_COPY, full, [self.grids[0], grid])])

    def residual_source(self, target_rms, p=None):
        """Residual source r of p (default p0) for the correction problem
        into self.rgrid, and the per-instance scales that bring r to
        target_rms (a float32 tensor, one per instance)."""
        import torch
        if getattr(self, "rgrid", None) is None:
            self.rgrid = ps.Grid(self.gshape)
            self.rwork = torch.empty(self.count * 64, dtype=torch.float64, device="cuda")
            self.rscale = torch.empty(self.count, dtype=torch.float32, device="cuda")
        f = self.fields(1, with_p=True)
        if p is not None:
            f.p = p.dev_ptr
        _ok(ps.lib().PSWarmStartResidualSource(
            ctypes.byref(f), ctypes.c_void_p(self.rgrid.dev_ptr), _p(self.rscale),
            ctypes.c_float(target_rms), _p(self.rwork), self.rwork.numel(), None))
        return self.rscale

    def fields(self, factor, wscale=1.0, pscale=1.0, with_p=False, flip=0, wrk1=None,
               inst_scale=None, p=None, p_sub=None):
        """PSWarmStartFields describing this stack for the pooling kernels
        (of mirror image `flip` of every instance).  wrk1: another source
        grid (a residual source); inst_scale: per-instance scales (tensor);
        p / p_sub: the solution grid and an iterate to subtract from it."""
        f = ps.PSWarmStartFields()
        g = self.grids
        f.a0, f.a1, f.a2 = g[2].dev_ptr, g[3].dev_ptr, g[4].dev_ptr
        f.wrk1, f.bnd = (wrk1 or g[13]).dev_ptr, g[12].dev_ptr
        f.p = (p or g[0]).dev_ptr if (with_p or p is not None) else None
        f.inst_scale = None if inst_scale is None else inst_scale.data_ptr()
        f.p_sub = None if p_sub is None else p_sub.dev_ptr
        f.pitch = g[0].pitch
        f.ny = self.gshape[1]
        f.inz, f.iny, f.inx = self.shape
        f.nsx = self.nsx
        f.factor = factor
        f.batch = self.count
        f.wscale, f.pscale = wscale, pscale
        f.flip = flip
        return f

    def free(self):
        for g in self.grids + [self.scratch]:
            g.free()
        if getattr(self, "rgrid", None) is not None:
            self.rgrid.free()
            self.rgrid = None


def coarse_shape(shape, factor):
    return tuple(-(-n // factor) for n in shape)


# ---- the network --------------------------------------------------------------

class Net:
    """6 conv layers 3x3x3 x 16 channels, ReLU between, on the coarse grid.
    FP32 master weights and Adam moments; BF16 copies for the kernels."""

    def __init__(self, seed=0):
        import torch
        self.torch = torch
        dev = "cuda"
        rng = np.random.default_rng(seed)
        self.w, self.b = [], []
        for l in range(LAYERS):
            fan_in = 27 * (CIN if l == 0 else C)
            std = math.sqrt(2.0 / fan_in) if l < LAYERS - 1 else 0.1 * math.sqrt(1.0 / fan_in)
            w = rng.normal(0, std, size=(27, C, C)).astype(np.float32)
            if l == 0:
                w[:, CIN:, :] = 0.0
            self.w.append(torch.tensor(w, device=dev))
            self.b.append(torch.zeros(C, device=dev))
        self.params = self.w + self.b
        self.grads = [torch.zeros_like(p) for p in self.params]
        self.m = [torch.zeros_like(p) for p in self.params]
        self.v = [torch.zeros_like(p) for p in self.params]
        self.wf = [torch.empty(27 * C * C, dtype=torch.bfloat16, device=dev) for _ in range(LAYERS)]
        self.wb = [torch.empty(27 * C * C, dtype=torch.bfloat16, device=dev) for _ in range(LAYERS)]
        self.step = 0
        self._acts = None
        self.prepare()

    def stream(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def prepare(self):
        L = ps.lib()
        for l in range(LAYERS):
            _ok(L.PSWarmStartPrepareWeights(_p(self.w[l]), _p(self.wf[l]), _p(self.wb[l]),
                                            self.stream()))

    def forward(self, x, dims):
        """x: BF16 tensor [B*Z*Y*X*16]; returns the FP32 channel-0 output."""
        torch = self.torch
        B, Z, Y, X = dims
        n = B * Z * Y * X
        L = ps.lib()
        acts = [x]
        out0 = torch.empty(n, dtype=torch.float32, device="cuda")
        for l in range(LAYERS):
            y = torch.empty(n * C, dtype=torch.bfloat16, device="cuda")
            last = l == LAYERS - 1
            _ok(L.PSWarmStartConv(_p(acts[-1]), _p(self.wf[l]), _p(self.b[l]), None,
                                  0 if last else 1, _p(y), _p(out0) if last else None,
                                  B, Z, Y, X, self.stream()))
            acts.append(y)
        self._acts = acts
        return out0

    def backward(self, dy, dims, work):
        """Gradients of every parameter from dL/d(output) (BF16, [n*16])."""
        torch = self.torch
        B, Z, Y, X = dims
        n = B * Z * Y * X
        L = ps.lib()
        nsplit = work.numel() // (27 * C * C + C)
        g = dy
        for l in range(LAYERS - 1, -1, -1):
            _ok(L.PSWarmStartWeightGrad(_p(self._acts[l]), _p(g), _p(work), nsplit,
                                        _p(self.grads[l]), _p(self.grads[LAYERS + l]),
                                        B, Z, Y, X, self.stream()))
            if l:
                dx = torch.empty(n * C, dtype=torch.bfloat16, device="cuda")
                _ok(L.PSWarmStartConv(_p(g), _p(self.wb[l]), None, _p(self._acts[l]), 0,
                                      _p(dx), None, B, Z, Y, X, self.stream()))
                g = dx

    def adam(self, lr, b1=0.9, b2=0.999, eps=1e-8):
        self.step += 1
        L = ps.lib()
        for p, g, m, v in zip(self.params, self.grads, self.m, self.v):
            _ok(L.PSWarmStartAdam(_p(p), _p(g), _p(m), _p(v), p.numel(), ctypes.c_float(lr),
                                  ctypes.c_float(b1), ctypes.c_float(b2), ctypes.c_float(eps),
                                  self.step, self.stream()))
        self.prepare()


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _ok(code):
    if code != 0:
        ps.check()
        raise ps.PSError(code, "warm-start call failed")


def loss_grad(pred, target, work64):
    """MSE of pred vs target (both FP32 [n]) and dL/dpred as BF16 [n*16]."""
    import torch
    n = pred.numel()
    dy = torch.empty(n * C, dtype=torch.bfloat16, device="cuda")
    _ok(ps.lib().PSWarmStartLoss(_p(pred), _p(target), n, _p(dy), _p(work64),
                                 ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    nb = (n + 255) // 256
    return float(work64[:nb].cpu().numpy().sum()) / n, dy


# ---- data, training, evaluation -------------------------------------------------

def _instance_job(args):
    seed, shape = args
    return make_instance(np.random.default_rng(seed), shape)


def make_instances(rng, count, shape, workers=0):
    """count instances; with workers > 1 they are built in a spawned process
    pool (each from its own seed drawn from rng, so the result does not
    depend on the number of workers)."""
    seeds = [int(v) for v in rng.integers(0, 2 ** 63 - 1, size=count)]
    if workers <= 1 or count < 2:
        return [_instance_job((sd, shape)) for sd in seeds]
    import multiprocessing as mp
    with mp.get_context("spawn").Pool(workers) as pool:
        return pool.map(_instance_job, [(sd, shape) for sd in seeds])


def mirror_images(shape, count):
    """The first `count` of the 16 mirror images (flip codes) an instance of
    this shape has: the 8 axis mirrors, then with x and y swapped when
    nx == ny."""
    nz, ny, nx = shape
    codes = list(range(16)) if nx == ny else list(range(8))
    return codes[:max(1, min(count, len(codes)))]


class Dataset:
    """Pooled inputs and targets of many instances, resident on the GPU.

    Each solved instance gives `mirrors` training pairs (its mirror images,
    which solve the mirrored problem).  With `snapshots` (sweep counts), the
    iterates of the target solve at those counts give further pairs for the
    correction problem: input the residual source r of the iterate (scaled
    per instance to the source's RMS), target the iterate's error p* - p
    (scaled alike), which is what a learned restart predicts.  Samples are
    stored kind-major (the source pairs, then each snapshot's pairs), then
    mirror-major: sample (k * nm + m) * count + i is mirror image m of
    instance i, so contiguous minibatches hold different instances."""

    def __init__(self, rng, count, shape, factor, nsx=15, per_stack=300, tol=1e-7,
                 chunk=256, max_sweeps=40000, wscale=None, pscale=None, log=None, workers=0,
                 mirrors=1, snapshots=()):
        import torch
        self.shape, self.factor = shape, factor
        zc, yc, xc = coarse_shape(shape, factor)
        self.dims1 = (zc, yc, xc)
        self.flips = mirror_images(shape, mirrors)
        nm = len(self.flips)
        self.count = count
        self.snapshots = tuple(int(v) for v in snapshots)
        kinds = 1 + len(self.snapshots)
        self.x = torch.empty((kinds * nm * count, zc, yc, xc, C), dtype=torch.bfloat16,
                             device="cuda")
        self.t = torch.empty((kinds * nm * count, zc, yc, xc), dtype=torch.float32,
                             device="cuda")
        self.sweeps = np.zeros(count, int)
        self.wscale, self.pscale = wscale, pscale
        self.solve_seconds = 0.0
        L = ps.lib()
        done = 0
        while done < count:
            k = min(per_stack, count - done)
            insts = make_instances(rng, k, shape, workers)
            if self.wscale is None:
                self.wscale = 1.0 / float(np.std(np.concatenate([i["wrk1"].ravel() for i in insts])))
            st = Stack(insts, shape, nsx)
            snaps = [(n, ps.Grid(st.gshape)) for n in self.snapshots]
            ps.synchronize()
            t0 = time.perf_counter()
            self.sweeps[done:done + k] = st.solve(tol, chunk, max_sweeps, snaps)
            ps.synchronize()
            self.solve_seconds += time.perf_counter() - t0
            if self.pscale is None:
                tmp = torch.empty((k, zc, yc, xc), dtype=torch.float32, device="cuda")
                _ok(L.PSWarmStartPoolTarget(ctypes.byref(st.fields(factor, 1.0, 1.0, True)),
                                            _p(tmp), None))
                ps.synchronize()
                self.pscale = 1.0 / float(np.std(tmp.cpu().numpy().astype(np.float64)))
            for m, flip in enumerate(self.flips):
                f = st.fields(factor, self.wscale, self.pscale, True, flip)
                lo = m * count + done
                _ok(L.PSWarmStartPool(ctypes.byref(f), _p(self.x[lo:lo + k]), None))
                _ok(L.PSWarmStartPoolTarget(ctypes.byref(f), _p(self.t[lo:lo + k]), None))
            for j, (_, g) in enumerate(snaps):
                scale = st.residual_source(1.0 / self.wscale, p=g)
                for m, flip in enumerate(self.flips):
                    f = st.fields(factor, self.wscale, self.pscale, True, flip,
                                  wrk1=st.rgrid, inst_scale=scale, p_sub=g)
                    lo = ((1 + j) * nm + m) * count + done
                    _ok(L.PSWarmStartPool(ctypes.byref(f), _p(self.x[lo:lo + k]), None))
                    _ok(L.PSWarmStartPoolTarget(ctypes.byref(f), _p(self.t[lo:lo + k]), None))
            ps.synchronize()
            for _, g in snaps:
                g.free()
            st.free()
            done += k
            if log:
                log(f"solved {done}/{count} instances")


def train(net, data, epochs, batch, lr, log=None, seed=0):
    import torch
    count = data.x.shape[0]
    zc, yc, xc = data.dims1
    nvox = batch * zc * yc * xc
    nsplit = 64
    work = torch.empty(nsplit * (27 * C * C + C), dtype=torch.float32, device="cuda")
    work64 = torch.empty((nvox + 255) // 256, dtype=torch.float64, device="cuda")
    rng = np.random.default_rng(seed)
    history = []
    steps = epochs * (count // batch)
    s = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    nb = count // batch
    for e in range(epochs):
        # The instances are generated independently, so minibatches are
        # fixed contiguous slices (views: no copy) visited in a new random
        # order each epoch.
        order = rng.permutation(nb)
        tot = 0.0
        for i in range(nb):
            j = int(order[i])
            x = data.x[j * batch:(j + 1) * batch].reshape(-1)
            t = data.t[j * batch:(j + 1) * batch].reshape(-1)
            pred = net.forward(x, (batch, zc, yc, xc))
            loss, dy = loss_grad(pred, t, work64)
            net.backward(dy, (batch, zc, yc, xc), work)
            rate = lr * 0.5 * (1 + math.cos(math.pi * s / max(steps, 1)))
            net.adam(rate)
            tot += loss
            s += 1
        history.append(tot / max(nb, 1))
        if log:
            log(f"epoch {e}: loss {history[-1]:.5f}")
    torch.cuda.synchronize()
    return history, time.perf_counter() - t0


def predict_into(net, stack, data_scales, factor, mirrors=1, restarts=0, nu=0,
                 restart_mirrors=None, pullback=0.0):
    """Warm start: pool the stack's fields, run the network, upsample into
    the stack's p0 (p1 too, so the first sweep starts from it).  With
    mirrors > 1 the prediction is the mean of the network's predictions for
    that many mirror images of each instance, each mapped back to the
    instance (the network is not mirror-equivariant, so their errors partly
    cancel).

    With restarts > 0, that many learned restarts follow: nu Jacobi sweeps
    (nu even), then the network applied to the correction problem -- the
    same coefficients with the current iterate's residual source r, scaled
    per instance to the source's RMS -- and its prediction of the error
    added to p0.  The equation is linear in the source, so the same network
    predicts the solution and the correction; each restart divides the
    error the network can see by roughly its relative accuracy, and the
    sweeps between restarts remove the fine-scale part of the error that
    the coarse grid cannot represent.  The sweeps are real iterations:
    returns the number run (restarts * nu).

    pullback > 0 scales the restarted iterate by 1 - pullback at the end.
    Restarts can bring an iterate so close that float32 Jacobi then locks
    into a 2-cycle a little above 1e-6; pulled back along the solution
    itself, the last approach runs like a zero start's, which ends at a
    fixed point."""
    import torch
    wscale, pscale = data_scales
    zc, yc, xc = coarse_shape(stack.shape, factor)
    n = stack.count
    L = ps.lib()
    flips = mirror_images(stack.shape, mirrors)
    x = torch.empty(n * zc * yc * xc * C, dtype=torch.bfloat16, device="cuda")
    for i, flip in enumerate(flips):
        f = stack.fields(factor, wscale, pscale * len(flips), flip=flip)
        _ok(L.PSWarmStartPool(ctypes.byref(f), _p(x), net.stream()))
        pred = net.forward(x, (n, zc, yc, xc))
        up = L.PSWarmStartUpsample if i == 0 else L.PSWarmStartUpsampleAdd
        for g in (stack.grids[0], stack.grids[1]):
            _ok(up(ctypes.byref(f), _p(pred), ctypes.c_void_p(g.dev_ptr), net.stream()))
    used = 0
    rflips = flips if restart_mirrors is None else mirror_images(stack.shape, restart_mirrors)
    for _ in range(restarts):
        torch.cuda.synchronize()
        stack.sweeps(nu)
        used += nu
        scale = stack.residual_source(1.0 / wscale)
        ps.synchronize()
        # the mirror predictions summed into a scratch grid, then added to
        # the iterate with a single rounding
        for i, flip in enumerate(rflips):
            f = stack.fields(factor, wscale, pscale * len(rflips), flip=flip, wrk1=stack.rgrid,
                             inst_scale=scale)
            _ok(L.PSWarmStartPool(ctypes.byref(f), _p(x), net.stream()))
            pred = net.forward(x, (n, zc, yc, xc))
            up = L.PSWarmStartUpsample if i == 0 else L.PSWarmStartUpsampleAdd
            _ok(up(ctypes.byref(f), _p(pred), ctypes.c_void_p(stack.scratch.dev_ptr),
                   net.stream()))
        f = stack.fields(factor)
        _ok(L.PSWarmStartAddCorrection(ctypes.byref(f), ctypes.c_void_p(stack.scratch.dev_ptr),
                                       ctypes.c_float(1.0),
                                       ctypes.c_void_p(stack.grids[0].dev_ptr), net.stream()))
    if restarts and pullback > 0:
        f = stack.fields(factor)
        _ok(L.PSWarmStartAddCorrection(ctypes.byref(f), None, ctypes.c_float(1.0 - pullback),
                                       ctypes.c_void_p(stack.grids[0].dev_ptr), net.stream()))
    torch.cuda.synchronize()
    return used


def _time_forward(instances=1024, shape=(65, 33, 33), factor=4, reps=5):
    """Times the forward pass of a randomly initialised network over the
    coarse grids of `instances` instances (zeros: the arithmetic does not
    depend on the values); returns milliseconds per pass and TFLOP/s."""
    import torch
    ps.init()
    zc, yc, xc = coarse_shape(shape, factor)
    net = Net(seed=0)
    x = torch.zeros(instances * zc * yc * xc * C, dtype=torch.bfloat16, device="cuda")
    dims = (instances, zc, yc, xc)
    net.forward(x, dims)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        net.forward(x, dims)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) / reps * 1e3
    flops = 2.0 * 27 * C * C * instances * zc * yc * xc * LAYERS
    return ms, flops / (ms / 1e3) / 1e12


if __name__ == "__main__":
    import sys
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 1024
    ms, tf = _time_forward(n)
    print(f"network forward, {n} instances: {ms:.3f} ms, {tf:.1f} TFLOP/s")
