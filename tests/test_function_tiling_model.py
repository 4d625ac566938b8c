"""CPU model of the tiled stencil-function entry's staging (jit.cpp,
tiled_entry_source / __ps_stage): tile and window geometry, the cp.async ring
schedule with its commit groups, and the cell-relative reads.  It checks, for
many shapes, halos, domains and z chunks, that every copy stays inside the
grid and the ring, that a plane is never refilled while a thread one step
behind can still read it, and that every read inside the window returns the
grid value at the read's (clamped or wrapped) coordinates."""
import numpy as np
import pytest

TX, TY, AHEAD = 64, 16, 3


def fit(v, n, periodic):
    if periodic:
        return v % n
    return min(max(v, 0), n - 1)


def ring_planes(rz):
    return 2 * rz + 2 + AHEAD


def simulate(shape, dom, r, periodic, esz=4, zlen=None):
    nz, ny, nx = shape
    rx, ry, rz = r
    v = 16 // esz
    rxw = (rx + v - 1) // v * v
    W, H, S = TX + 2 * rxw, TY + 2 * ry, ring_planes(rz)
    grid = np.arange(nz * ny * nx).reshape(shape)
    (x_lo, x_hi), (y_lo, y_hi), (z_lo, z_hi) = dom
    zlen = zlen or (z_hi - z_lo)
    for ty in range(0, y_hi - y_lo, TY):
        for tx in range(0, x_hi - x_lo, TX):
            x0, y0 = x_lo + tx, y_lo + ty
            for zs in range(z_lo, z_hi, zlen):
                ze = min(zs + zlen, z_hi)
                ring = np.full((S, H, W), -1)
                plane_in = np.full(S, None, dtype=object)   # plane a slot holds
                pending = []                                  # commit groups (planes)
                group = []

                def stage(zp):
                    slot = zp % S
                    gz = fit(zp, nz, periodic)
                    assert 0 <= gz < nz
                    for rr in range(H):
                        gy = fit(y0 - ry + rr, ny, periodic)
                        assert 0 <= gy < ny
                        for c in range(W):
                            gx = fit(x0 - rxw + c, nx, periodic)
                            assert 0 <= gx < nx
                            ring[slot, rr, c] = grid[gz, gy, gx]
                    plane_in[slot] = zp
                    group.append(zp)

                def commit():
                    pending.append(list(group))
                    group.clear()

                def wait(n):  # at most n pending groups
                    while len(pending) > n:
                        pending.pop(0)

                def in_flight():
                    return {p for g in pending for p in g}

                for d in range(-rz, rz + 1):
                    stage(zs + d)
                commit()
                for a in range(1, AHEAD):
                    if zs + a < ze:
                        stage(zs + rz + a)
                    commit()
                needed_prev = set()
                for z in range(zs, ze):
                    if z + AHEAD < ze:
                        q = z + rz + AHEAD
                        # the slot refilled must not hold a plane step z-1 reads
                        old = plane_in[q % S]
                        assert old is None or old not in needed_prev, (z, q, old)
                        stage(q)
                    commit()
                    wait(AHEAD)
                    needed = set(range(z - rz, z + rz + 1))
                    for p in needed:
                        assert plane_in[p % S] == p and p not in in_flight(), (z, p)
                    needed_prev = needed
                    for y in range(y0, min(y0 + TY, y_hi)):
                        for x in range(x0, min(x0 + TX, x_hi)):
                            for dz in (-rz, 0, rz):
                                for dy in (-ry, 0, ry):
                                    for dx in (-rxw, -rx, 0, rx, rxw):
                                        wy = y - y0 + ry + dy
                                        wx = x - x0 + rxw + dx
                                        assert 0 <= wy < H and 0 <= wx < W
                                        got = ring[(z + dz) % S, wy, wx]
                                        want = grid[fit(z + dz, nz, periodic),
                                                    fit(y + dy, ny, periodic),
                                                    fit(x + dx, nx, periodic)]
                                        assert got == want, (x, y, z, dx, dy, dz)


@pytest.mark.parametrize("shape,dom,r,periodic,zlen", [
    ((9, 20, 70), ((0, 70), (0, 20), (0, 9)), (1, 1, 1), False, None),
    ((9, 20, 70), ((0, 70), (0, 20), (0, 9)), (1, 1, 1), True, 4),
    ((12, 23, 150), ((5, 144), (3, 21), (1, 8)), (4, 3, 4), False, 3),
    ((12, 23, 150), ((0, 150), (0, 23), (0, 12)), (4, 3, 4), True, 5),
    ((7, 17, 40), ((1, 39), (1, 16), (1, 6)), (0, 2, 0), False, 2),
    ((6, 18, 66), ((0, 66), (0, 18), (0, 6)), (2, 0, 3), True, None),
])
def test_staging_model(shape, dom, r, periodic, zlen):
    simulate(shape, dom, r, periodic, zlen=zlen)


def test_staging_model_double_halo_rounding():
    # doubles: the x halo rounds up to 2 cells (16 bytes)
    simulate((5, 18, 70), ((0, 70), (0, 18), (0, 5)), (1, 1, 2), False, esz=8)
