"""CPU model of the union-find labelling in ccl.cu against the oracle.

ccl_local labels each LT x LT tile on its own (unions with the left, up and,
for 8-connectivity, the two upper diagonal neighbours inside the tile);
ccl_border then unites only the neighbour pairs that cross a tile border.  It
runs one block per tile and one thread per pixel that can have such a pair:
the tile's top row (LT pixels), then its left column and its right column
below the top row (LT - 1 each), thread t mapped to (bx, by) as below.  This
model follows that index arithmetic exactly, with the union-find's rule (the
larger root hooks under the smaller, so roots are minimum raster indices, in
any order of unions), and compares the labels with the oracle's bwlabel2 on
ragged image sizes, for the kernel's tile size and for small tiles that put
most pairs on a border."""
import numpy as np
import pytest


def border_pixel(t, lt):
    """(bx, by) of border thread t, as ccl_border maps it."""
    if t < lt:
        return t, 0
    if t < 2 * lt - 1:
        return 0, t - (lt - 1)
    return lt - 1, t - (2 * lt - 2)


def find(parent, x):
    while parent[x] != x:
        x = parent[x]
    return x


def unite(parent, a, b):
    a, b = find(parent, a), find(parent, b)
    if a != b:
        parent[max(a, b)] = min(a, b)


def model_labels(img, conn, lt):
    rows, cols = img.shape
    fg = img.reshape(-1) != 0
    parent = np.where(fg, np.arange(rows * cols), -1)
    # ccl_local: pairs inside one tile
    for y in range(rows):
        for x in range(cols):
            i = y * cols + x
            if not fg[i]:
                continue
            bx, by = x % lt, y % lt
            if bx > 0 and fg[i - 1]:
                unite(parent, i, i - 1)
            if by > 0:
                u = i - cols
                if fg[u]:
                    unite(parent, i, u)
                if conn == 8:
                    if bx > 0 and fg[u - 1]:
                        unite(parent, i, u - 1)
                    if bx < lt - 1 and x < cols - 1 and fg[u + 1]:
                        unite(parent, i, u + 1)
    # ccl_border: one "block" per tile, one "thread" per border pixel
    covered = set()
    for ty in range((rows + lt - 1) // lt):
        for tx in range((cols + lt - 1) // lt):
            for t in range(lt + 2 * (lt - 1)):
                bx, by = border_pixel(t, lt)
                x, y = tx * lt + bx, ty * lt + by
                if x >= cols or y >= rows:
                    continue
                covered.add((y, x))
                i = y * cols + x
                if not fg[i]:
                    continue
                if x > 0 and bx == 0 and fg[i - 1]:
                    unite(parent, i, i - 1)
                if y > 0:
                    u = i - cols
                    if by == 0 and fg[u]:
                        unite(parent, i, u)
                    if conn == 8:
                        if x > 0 and (bx == 0 or by == 0) and fg[u - 1]:
                            unite(parent, i, u - 1)
                        if x < cols - 1 and (bx == lt - 1 or by == 0) and fg[u + 1]:
                            unite(parent, i, u + 1)
    lab = np.array([find(parent, i) if fg[i] else -1 for i in range(rows * cols)], np.int32)
    return lab.reshape(rows, cols), covered


@pytest.mark.parametrize("lt", [32, 4, 3])
def test_border_threads_cover_exactly_the_border_pixels(lt):
    got = {border_pixel(t, lt) for t in range(lt + 2 * (lt - 1))}
    want = {(bx, by) for by in range(lt) for bx in range(lt) if by == 0 or bx == 0 or bx == lt - 1}
    assert got == want and len(got) == lt + 2 * (lt - 1)


@pytest.mark.parametrize("shape,lt", [((70, 90), 32), ((33, 65), 32), ((23, 17), 4), ((19, 26), 3), ((1, 9), 4),
                                      ((9, 1), 4)])
@pytest.mark.parametrize("conn", [4, 8])
def test_tile_labelling_matches_oracle(orc, shape, lt, conn):
    rng = np.random.default_rng(shape[0] * 131 + shape[1] * 7 + lt + conn)
    for density in (0.35, 0.55, 0.75):
        img = ((rng.random(shape) < density) * 255).astype(np.uint8)
        lab, _ = model_labels(img, conn, lt)
        np.testing.assert_array_equal(lab, orc.bwlabel2(img, conn))
