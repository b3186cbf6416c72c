"""CPU model of the uint8 grey reconstruction's tile queue (recon_cta in
recon.cu) against the oracle.

The kernel stops a tile pass when a column phase changes nothing, rescans only
the lines a change can affect (a pixel changed along a row dirties its column
and the two beside it, and the other way round), and re-queues a neighbour
tile only when a changed edge pixel can raise one of its pixels, with that
neighbour's facing edge line dirty (diagonal neighbours too, for 8-connectivity).
Any of these rules stopping too early would leave a pixel below the least fixed
point.  This model applies exactly those rules, one line at a time (the
lane-per-line scan: raster then anti-raster step, neighbours read as they are)
and tiles in a random order, with small tiles so that propagation crosses many
of them, and compares with the oracle's reconstruction.

The worklist form (a tuning option, off by default) is modelled too: a whole-tile pass runs one
row + column phase pair and then a pixel worklist seeded with the pixels the
column phase changed; a pass for changed halo sides skips the phases and
seeds the worklist from the edge pixels those sides can raise.  Pixels are
popped in random order (the kernel's warps take them in any order).
"""
import random

import numpy as np
import pytest

D_N, D_S, D_W, D_E, D_ALL = 1, 2, 4, 8, 16


def clamp(x, lo, hi):
    return min(max(x, lo), hi)


def worklist(o, hm, seeds, TH, TW, conn8, rng):
    """Pop pixels (tile coordinates + 1) in random order; raise in-tile
    neighbours below min(popped value, their mask) and queue them."""
    queued = set(seeds)
    changed = False
    while queued:
        p = rng.choice(sorted(queued))
        queued.discard(p)
        y, x = p
        v = o[y, x]
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                if (dy == 0 and dx == 0) or (not conn8 and dy and dx):
                    continue
                qy, qx = y + dy, x + dx
                if not (1 <= qy <= TH and 1 <= qx <= TW):
                    continue
                cand = min(v, hm[qy, qx])
                if o[qy, qx] < cand:
                    o[qy, qx] = cand
                    queued.add((qy, qx))
                    changed = True
    return changed


def tile_pass(out, mask, ty, tx, TH, TW, conn8, dirty_in, rng, wl=False, wl_phases=1):
    """One pass over tile (ty, tx); returns the neighbours to queue as (dy, dx, edge line)."""
    H, W = out.shape
    y0, x0 = ty * TH, tx * TW
    # tile + one-pixel halo (0 outside the image), mask (0 outside the image)
    o = np.zeros((TH + 2, TW + 2), np.int64)
    m = np.zeros((TH + 2, TW + 2), np.int64)
    ys, xs = slice(max(y0 - 1, 0), min(y0 + TH + 1, H)), slice(max(x0 - 1, 0), min(x0 + TW + 1, W))
    o[ys.start - (y0 - 1):ys.stop - (y0 - 1), xs.start - (x0 - 1):xs.stop - (x0 - 1)] = out[ys, xs]
    m[ys.start - (y0 - 1):ys.stop - (y0 - 1), xs.start - (x0 - 1):xs.stop - (x0 - 1)] = mask[ys, xs]
    inside = np.zeros_like(m, bool)
    inside[1:TH + 1, 1:TW + 1] = True
    hm = np.where(inside, m, 0)  # the clamp's upper bound: the tile's own mask only
    loaded = o.copy()
    drow = set(range(TH)) if dirty_in & D_ALL else set()
    dcol = set(range(TW)) if dirty_in & D_ALL else set()
    if dirty_in & D_N:
        drow.add(0)
    if dirty_in & D_S:
        drow.add(TH - 1)
    if dirty_in & D_W:
        dcol.add(0)
    if dirty_in & D_E:
        dcol.add(TW - 1)
    anych = False
    phases = not wl or bool(dirty_in & D_ALL)
    it = 0
    need_wl = False
    while phases:
        it += 1
        cbm = set()  # pixels the column phase changes
        rows, drow = sorted(drow), set()
        rng.shuffle(rows)
        for r in rows:
            R = r + 1
            prev = o[R, 0]
            for x in range(1, TW + 1):
                w = max(o[R, x], o[R - 1, x], o[R + 1, x])
                if conn8:
                    w = max(w, o[R - 1, x - 1], o[R - 1, x + 1], o[R + 1, x - 1], o[R + 1, x + 1])
                v = clamp(prev, min(w, hm[R, x]), hm[R, x])
                if v != o[R, x]:
                    o[R, x] = v
                    dcol |= {x - 2, x - 1, x} & set(range(TW))
                    anych = True
                prev = v
            nxt = o[R, TW + 1]
            for x in range(TW, 0, -1):
                v = clamp(nxt, o[R, x], hm[R, x])
                if v != o[R, x]:
                    o[R, x] = v
                    dcol |= {x - 2, x - 1, x} & set(range(TW))
                    anych = True
                nxt = v
        cols, dcol = sorted(dcol), set()
        rng.shuffle(cols)
        chc = False
        for c in cols:
            C = c + 1
            prev = o[0, C]
            for y in range(1, TH + 1):
                w = max(o[y, C], o[y, C - 1], o[y, C + 1])
                if conn8:
                    w = max(w, o[y - 1, C - 1], o[y - 1, C + 1], o[y + 1, C - 1], o[y + 1, C + 1])
                v = clamp(prev, min(w, hm[y, C]), hm[y, C])
                if v != o[y, C]:
                    o[y, C] = v
                    drow |= {y - 2, y - 1, y} & set(range(TH))
                    chc = anych = True
                    cbm.add((y, C))
                prev = v
            nxt = o[TH + 1, C]
            for y in range(TH, 0, -1):
                v = clamp(nxt, o[y, C], hm[y, C])
                if v != o[y, C]:
                    o[y, C] = v
                    drow |= {y - 2, y - 1, y} & set(range(TH))
                    chc = anych = True
                    cbm.add((y, C))
                nxt = v
        if not chc:
            break
        if wl and it == wl_phases:
            need_wl = True
            break
    if wl:
        seeds = set()
        if need_wl:
            seeds = cbm
        elif not phases:
            c8 = 1 if conn8 else 0
            sides = []
            if dirty_in & D_N:
                sides += [((1, x), [(0, x + d) for d in range(-c8, c8 + 1)]) for x in range(1, TW + 1)]
            if dirty_in & D_S:
                sides += [((TH, x), [(TH + 1, x + d) for d in range(-c8, c8 + 1)]) for x in range(1, TW + 1)]
            if dirty_in & D_W:
                sides += [((y, 1), [(y + d, 0) for d in range(-c8, c8 + 1)]) for y in range(1, TH + 1)]
            if dirty_in & D_E:
                sides += [((y, TW), [(y + d, TW + 1) for d in range(-c8, c8 + 1)]) for y in range(1, TH + 1)]
            for (qy, qx), halo in sides:
                best = max(min(o[h], hm[qy, qx]) for h in halo)
                if o[qy, qx] < best:
                    o[qy, qx] = best
                    seeds.add((qy, qx))
                    anych = True
        if seeds and worklist(o, hm, seeds, TH, TW, conn8, rng):
            anych = True
    # neighbours to queue: a changed edge pixel above a halo pixel that is below its mask
    notes = []
    if anych:
        c8 = 1 if conn8 else 0

        def raises(py, px, hy, hx):
            return o[py, px] != loaded[py, px] and o[py, px] > o[hy, hx] and m[hy, hx] > o[hy, hx]

        for x in range(1, TW + 1):
            for d in range(-c8, c8 + 1):
                if 1 <= x + d <= TW:
                    if raises(1, x, 0, x + d):
                        notes.append((-1, 0, D_S))
                    if raises(TH, x, TH + 1, x + d):
                        notes.append((1, 0, D_N))
        for y in range(1, TH + 1):
            for d in range(-c8, c8 + 1):
                if 1 <= y + d <= TH:
                    if raises(y, 1, y + d, 0):
                        notes.append((0, -1, D_E))
                    if raises(y, TW, y + d, TW + 1):
                        notes.append((0, 1, D_W))
        if conn8:
            if raises(1, 1, 0, 0):
                notes.append((-1, -1, D_S))
            if raises(1, TW, 0, TW + 1):
                notes.append((-1, 1, D_S))
            if raises(TH, 1, TH + 1, 0):
                notes.append((1, -1, D_N))
            if raises(TH, TW, TH + 1, TW + 1):
                notes.append((1, 1, D_N))
        ys, xs = slice(y0, min(y0 + TH, H)), slice(x0, min(x0 + TW, W))
        out[ys, xs] = o[1:1 + ys.stop - y0, 1:1 + xs.stop - x0]
    return notes


def reconstruct_model(marker, mask, conn, TH, TW, rng, wl=False, wl_phases=1):
    H, W = mask.shape
    out = np.minimum(marker, mask).astype(np.int64)
    m = mask.astype(np.int64)
    ty_n, tx_n = (H + TH - 1) // TH, (W + TW - 1) // TW
    dirty = {(ty, tx): D_ALL for ty in range(ty_n) for tx in range(tx_n)}
    queue = list(dirty)
    rng.shuffle(queue)
    while queue:
        t = queue.pop(rng.randrange(len(queue)))  # any tile that is queued, in any order
        bits = dirty.pop(t)
        for dy, dx, edge in tile_pass(out, m, t[0], t[1], TH, TW, conn == 8, bits, rng, wl, wl_phases):
            nt = (t[0] + dy, t[1] + dx)
            if 0 <= nt[0] < ty_n and 0 <= nt[1] < tx_n:
                if nt not in dirty:
                    queue.append(nt)
                dirty[nt] = dirty.get(nt, 0) | edge
    return out.astype(np.uint8)


@pytest.mark.parametrize("form", ["phases", "worklist", "worklist2"])
@pytest.mark.parametrize("conn", [4, 8])
@pytest.mark.parametrize("shape,tile", [((37, 53), (8, 8)), ((64, 40), (16, 8)), ((29, 61), (8, 16))])
def test_tile_queue_reaches_the_fixed_point(orc, form, conn, shape, tile):
    from nscale_gb300 import synth
    rng = random.Random(0x5EED00C0 + conn + shape[0])
    for seed in range(4):
        g = np.random.default_rng(0x5EED0031 + seed)
        if seed % 2 == 0:  # smooth mask
            marker, mask = synth.recon_inputs(*shape, seed=0x5EED0031 + seed)
        else:  # rough mask: propagation follows single-pixel (often diagonal) paths
            mask = g.integers(0, 256, size=shape).astype(np.uint8)
            marker = mask.copy()
        # sparse seeds make long winding propagation across many tiles
        marker = np.where(g.random(shape) < 0.02, marker, 0).astype(np.uint8)
        got = reconstruct_model(marker, mask, conn, tile[0], tile[1], rng, wl=form != "phases",
                                wl_phases=2 if form == "worklist2" else 1)
        np.testing.assert_array_equal(got, orc.imreconstruct(marker, mask, conn))
