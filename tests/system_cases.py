"""The reference's point-list system tests, restated as data.

Each case is one program of tests/system_tests/test_cases/ whose stencil is a
weighted (here: unit-weight) sum over a fixed list of neighbour offsets.  The
offsets are listed in the order the program's expression adds them (the sum
is evaluated left to right, so the order is part of the result), with the
boundary rule of its index arithmetic and the maps its main() runs.  The
oracle tests run a case through oracle/ps_oracle.c, the GPU tests through the
library; both compare with the program's own stdout in tests/golden/.

Boundary: 0 none (the domain keeps every read inside the grid), 1 periodic
((i + n) % n), 2 clamp (`if (x == 0) w = c;` branches).
Steps: ("map", src, dst) = one sweep src -> dst over the domain;
("red", g) / ("black", g) = one in-place red / black sweep of g;
("dump", g) = print every element of g; ("reduce", g) = print the PS_SUM.
"""
import numpy as np

C = (0, 0, 0)

# The 3x3 planes of test_27-pt*.manual.ref.c, each in the order
# (x,y) (x+1,y) (x-1,y) (x,y+1) (x+1,y+1) (x-1,y+1) (x,y-1) (x+1,y-1) (x-1,y-1).
_PLANE9 = [(0, 0), (1, 0), (-1, 0), (0, 1), (1, 1), (-1, 1), (0, -1), (1, -1),
           (-1, -1)]
P27 = [(x, y, z) for z in (-1, 0, 1) for (x, y) in _PLANE9]

# test_9-pt-*: c, x-1, x+1, y-1, y+1, (x-1,y-1), (x+1,y-1), (x-1,y+1), (x+1,y+1)
P9_2D = [C, (-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (-1, -1, 0),
         (1, -1, 0), (-1, 1, 0), (1, 1, 0)]

# test_redblack.manual.ref.c: c + (x+1) + (x-1) + (y+1) + (y-1) + (z-1) + (z+1)
P7_RB = [C, (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, -1), (0, 0, 1)]


def _box(shape, h):
    """Domain [h, n-h) in every used dimension (x, y, z order)."""
    nz, ny, nx = shape
    out = []
    for n in (nx, ny, nz):
        out += [h, n - h] if n > 1 else [0, 1]
    return tuple(out)


def _full(shape):
    nz, ny, nx = shape
    return (0, nx, 0, ny, 0, nz)


CASES = {
    # tests/system_tests/test_cases/<name>.manual.ref.c
    "test_3-pt-1d": dict(
        shape=(1, 1, 1024), dtype=np.float32, halo=1, boundary=0,
        points=[(-1, 0, 0), C, (1, 0, 0)],
        steps=[("map", 1, 2), ("dump", 2)]),
    "test_3-pt-periodic": dict(
        shape=(32, 32, 32), dtype=np.float32, halo=0, boundary=1,
        points=[C, (0, 0, 1), (0, 0, -1)],
        steps=[("map", 1, 2), ("dump", 2)]),
    "test_5-pt-2d": dict(
        shape=(1, 32, 32), dtype=np.float32, halo=1, boundary=0,
        points=[C, (-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0)],
        steps=[("map", 1, 2), ("dump", 2)]),
    "test_5-pt-periodic": dict(
        shape=(1, 32, 32), dtype=np.float32, halo=0, boundary=1,
        points=[C, (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0)],
        steps=[("map", 1, 2), ("map", 2, 1), ("dump", 1)]),
    "test_9-pt-2d": dict(
        shape=(1, 32, 32), dtype=np.float32, halo=1, boundary=0,
        points=P9_2D, steps=[("map", 1, 2), ("dump", 2)]),
    "test_9-pt-reduction": dict(
        shape=(1, 32, 32), dtype=np.int32, halo=1, boundary=0,
        points=P9_2D, steps=[("map", 1, 2), ("map", 2, 1), ("reduce", 1)]),
    "test_9-pt-periodic-reduction": dict(
        shape=(1, 32, 32), dtype=np.int32, halo=0, boundary=1,
        points=P9_2D, steps=[("map", 1, 2), ("map", 2, 1), ("reduce", 1)]),
    "test_27-pt": dict(
        shape=(32, 32, 32), dtype=np.float32, halo=1, boundary=0,
        points=P27, steps=[("map", 1, 2), ("dump", 2)]),
    "test_27-pt-periodic": dict(
        shape=(32, 32, 32), dtype=np.float32, halo=0, boundary=1,
        points=P27, steps=[("map", 1, 2), ("dump", 2)]),
    "test_27-pt-reduction": dict(
        shape=(16, 16, 16), dtype=np.int32, halo=1, boundary=0,
        points=P27,
        steps=[("map", 1, 2), ("reduce", 2), ("map", 2, 1), ("reduce", 1)]),
    "test_asymmetric": dict(
        shape=(32, 32, 32), dtype=np.float32, halo=2, boundary=0,
        points=[C, (1, 1, 1), (-2, -2, -2)],
        steps=[("map", 1, 2), ("dump", 2)]),
    "test_asymmetric-periodic": dict(
        shape=(32, 32, 32), dtype=np.float32, halo=2, boundary=1,
        points=[C, (-1, 0, 0), (2, 0, 0)],
        steps=[("map", 1, 2), ("dump", 2)]),
    "test_stencil-hole": dict(
        shape=(32, 32, 32), dtype=np.float32, halo=2, boundary=0,
        points=[C, (2, 0, 0), (-2, 0, 0)],
        steps=[("map", 1, 2), ("dump", 2)]),
    "test_redblack": dict(
        shape=(32, 32, 32), dtype=np.float32, halo=1, boundary=0,
        points=P7_RB, steps=[("red", 1), ("black", 1), ("dump", 1)]),
    "test_redblack-periodic": dict(
        shape=(32, 32, 32), dtype=np.float32, halo=0, boundary=1,
        points=[C, (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1),
                (0, 0, -1)],
        steps=[("red", 1), ("black", 1), ("dump", 1)]),
    "test_16": dict(
        shape=(32, 32, 32), dtype=np.float32, halo=0, boundary=2,
        points=[C, (-1, 0, 0), (1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, -1),
                (0, 0, 1)],
        steps=[("map", 1, 2), ("dump", 2)]),
}


def domain(case):
    h = case["halo"]
    return _box(case["shape"], h) if h else _full(case["shape"])


def initial(case):
    """main(): g1[i] = g2[i] = i for every element (x fastest)."""
    n = int(np.prod(case["shape"]))
    a = np.arange(n, dtype=np.int64).astype(case["dtype"]).reshape(case["shape"])
    return a, a.copy()


def fmt(case):
    return "%d" if np.issubdtype(case["dtype"], np.integer) else "%f"


def run(case, sweep, color_sweep, reduce_sum, dump_text):
    """Runs a case's steps with the given executors; returns its stdout.

    sweep(src, dst) and color_sweep(g, color) act on the grids (whatever
    they are), reduce_sum(g) returns the PS_SUM value, dump_text(g) the
    printed elements.  Grids are numbered 1 and 2 as in main().
    """
    g = dict(zip((1, 2), case["grids"]))
    out = []
    for step in case["steps"]:
        if step[0] == "map":
            sweep(g[step[1]], g[step[2]])
        elif step[0] == "red":
            color_sweep(g[step[1]], 0)
        elif step[0] == "black":
            color_sweep(g[step[1]], 1)
        elif step[0] == "reduce":
            out.append("%d\n" % int(reduce_sum(g[step[1]])))
        else:
            out.append(dump_text(g[step[1]]))
    return "".join(out)
