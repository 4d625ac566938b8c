"""CPU model of the persistent chunk-major schedule of the z-marching kernels
(march.cpp choose_zchunk_overhead; the item loops of stencil7.cu,
himeno19.cu, points_body.cuh and temporal7.cu).  For many grid shapes,
domains, tile heights and resident-CTA counts it checks that the
(z-chunk, tile) items a persistent grid takes round-robin write every cell of
the domain exactly once and nothing outside it."""
import pytest


def choose_zchunk_overhead(tiles, nz, resident, overhead):
    """Restates march.cpp: the chunk length whose rounds of `resident` items
    waste the least, counting `overhead` start-up planes per item."""
    if nz <= 1 or tiles <= 0 or resident <= 0:
        return nz if nz > 0 else 1
    best_len, best = nz, -1.0
    for chunks in range(1, nz + 1):
        ln = -(-nz // chunks)
        if -(-nz // ln) != chunks:
            continue
        items = tiles * chunks
        rounds = -(-items // resident)
        eff = tiles * nz / (rounds * resident * (ln + overhead))
        if eff > best + 1e-9:
            best, best_len = eff, ln
        if ln <= 4:
            break
    return best_len


def written_cells(dom, tx_cells, ty, xbase, resident, overhead=1):
    """Cells the items write: tile (tx_cells wide from xbase, ty rows from
    dom's y0) x z-chunk, items in chunk-major order, clipped to the domain."""
    x0d, x1d, y0d, y1d, z0d, z1d = dom
    tiles_x = -(-(x1d - xbase) // tx_cells)
    tiles = tiles_x * -(-(y1d - y0d) // ty)
    nz = z1d - z0d
    zlen = choose_zchunk_overhead(tiles, nz, resident, overhead)
    items = tiles * -(-nz // zlen)
    grid = max(1, min(resident, items))
    seen = {}
    for b in range(grid):
        for item in range(b, items, grid):
            chunk, tile = divmod(item, tiles)
            zs = z0d + chunk * zlen
            ze = min(zs + zlen, z1d)
            assert z0d <= zs < ze <= z1d
            x0 = xbase + (tile % tiles_x) * tx_cells
            y0 = y0d + (tile // tiles_x) * ty
            for z in range(zs, ze):
                for y in range(y0, min(y0 + ty, y1d)):
                    for x in range(max(x0, x0d), min(x0 + tx_cells, x1d)):
                        seen[(x, y, z)] = seen.get((x, y, z), 0) + 1
    return seen


SHAPES = [(70, 45, 37), (7, 1, 1), (4, 130, 2), (150, 45, 23), (33, 17, 9), (129, 33, 16)]


@pytest.mark.parametrize("nx,ny,nz", SHAPES)
@pytest.mark.parametrize("vec,ty,resident", [(4, 16, 152), (4, 8, 608), (2, 4, 1216),
                                             (4, 32, 1), (4, 2, 304)])
def test_every_cell_once(nx, ny, nz, vec, ty, resident):
    for dom in [(0, nx, 0, ny, 0, nz),
                (1, max(nx - 1, 2), 1, max(ny - 1, 2), 1, max(nz - 1, 2)),
                (min(3, nx - 1), nx, 0, max(ny - 2, 1), min(2, nz - 1), nz)]:
        if dom[1] > nx or dom[3] > ny or dom[5] > nz or dom[0] >= dom[1]:
            continue
        if dom[2] >= dom[3] or dom[4] >= dom[5]:
            continue
        # 7-point / Himeno / point sweeps: 32 lanes x 16 bytes (or 128 cells)
        # per tile row, the tile's x origin rounded down to a 16-byte boundary
        xbase = (dom[0] // vec) * vec
        seen = written_cells(dom, 32 * vec, ty, xbase, resident)
        want = {(x, y, z) for z in range(dom[4], dom[5]) for y in range(dom[2], dom[3])
                for x in range(dom[0], dom[1])}
        assert set(seen) == want
        assert all(v == 1 for v in seen.values())


@pytest.mark.parametrize("k,tye", [(2, 32), (3, 16), (5, 16), (2, 8)])
@pytest.mark.parametrize("nx,ny,nz", [(70, 45, 37), (121, 130, 20), (9, 3, 1), (250, 17, 9)])
def test_temporal_output_tiles_cover_the_grid_once(k, tye, nx, ny, nz):
    # temporal7.cu: output tiles of 30 * VEC columns and tye - 2 (k - 1) rows
    # over the whole grid, items in chunk-major order with 2k - 1 start-up
    # planes per item
    vec = 4
    tyo = tye - 2 * (k - 1)
    seen = written_cells((0, nx, 0, ny, 0, nz), 30 * vec, tyo, 0, 304, 2 * k - 1)
    assert len(seen) == nx * ny * nz
    assert all(v == 1 for v in seen.values())


def test_batch_family_tables():
    # runtime.cpp batch_build: problems ordered by kernel family, each
    # family's item_begin counted from 0; batch.cu finds an item's problem by
    # binary search over item_begin (the last problem whose first item is <=
    # the item).  Every item of every problem is found exactly once.
    import random
    rnd = random.Random(3)
    kinds = [rnd.choice(["d7", "him"]) for _ in range(48)]
    items = [rnd.randint(1, 40) for _ in range(48)]
    for fam in ("d7", "him"):
        probs = [r for r in range(48) if kinds[r] == fam]
        begin, total = [], 0
        for r in probs:
            begin.append(total)
            total += items[r]
        found = []
        for item in range(total):
            lo, hi = 0, len(probs) - 1
            while lo < hi:
                mid = (lo + hi + 1) >> 1
                if begin[mid] <= item:
                    lo = mid
                else:
                    hi = mid - 1
            local = item - begin[lo]
            assert 0 <= local < items[probs[lo]]
            found.append((probs[lo], local))
        assert sorted(found) == sorted((r, i) for r in probs for i in range(items[r]))
