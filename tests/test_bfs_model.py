"""CPU model of the watershed's cluster BFS (k_bfs in watershed_pws.cu) against
a plain FIFO BFS.

The kernel orders region R's flood without global ranks: a frontier entry's
key is its slot (base + segment * capacity + position), claims are atomicMin of
4 * key + direction, each CTA reads the claims of its chunk right after one
cluster barrier and at once issues its winners' claims, and a balanced layer
keeps each CTA's own segment as its next chunk.  This model replays exactly
those steps, CTA after CTA (so that a CTA that runs ahead issues the next
layer's claims before another reads the current layer's, the interleaving
the single barrier allows), and checks that R's pop sequence and the order in
which R pushes its fg neighbours are those of the queue the reference runs.
"""
import random

import pytest

OFF = None  # set per grid: left, right, up, down
INF = 1 << 62


def fifo_reference(W, ucand, fgc, seed):
    """R's pops in FIFO order and the order in which R first touches each fg
    pixel (pop order, then direction), as the reference's queue produces them."""
    off = (-1, 1, -W, W)
    order, touched = [seed], []
    seen, seen_fg = {seed}, set()
    head = 0
    while head < len(order):
        p = order[head]
        head += 1
        for k in range(4):
            q = p + off[k]
            if q in ucand and q not in seen:
                seen.add(q)
                order.append(q)
            if q in fgc and q not in seen_fg:
                seen_fg.add(q)
                touched.append(q)
    return order, touched


def cluster_model(W, ucand, fgc, seed, C, cta_items, slack):
    off = (-1, 1, -W, W)

    def nbm(p):
        m = 0
        for k in range(4):
            if p + off[k] in ucand:
                m |= 1 << k
            if p + off[k] in fgc:
                m |= 16 << k
        return m

    claim, inj = {}, {}

    def amin(table, q, v):
        if v < table.get(q, INF):
            table[q] = v

    # the seed: key 0, its claims before the first barrier
    seg_items = [[(seed, nbm(seed))]] + [[] for _ in range(C - 1)]  # each CTA's segment, in order
    for k in range(4):
        if nbm(seed) & (1 << k):
            amin(claim, seed + off[k], k)
        if nbm(seed) & (16 << k):
            amin(inj, seed + off[k], k)
    base, prevcap = 0, 1
    pops = []  # R's pop sequence: the frontiers in order
    while True:
        tots = [len(x) for x in seg_items]
        s = sum(tots)
        if s == 0:
            break
        offs = [sum(tots[:c]) for c in range(C + 1)]
        per_cta = (s + C - 1) // C
        mx = max(tots)
        local = mx <= per_cta + per_cta // 4 + slack and mx <= cta_items
        segcap = 4 * (mx if local else per_cta)
        assert per_cta <= cta_items
        nbase = base + C * prevcap
        # the frontier in order, each entry with its slot key
        frontier = []
        for c in range(C):
            for i, e in enumerate(seg_items[c]):
                frontier.append((e, base + c * prevcap + i))
        pops.extend(e[0] for e, _ in frontier)
        new_items = [[] for _ in range(C)]
        for me in range(C):  # one CTA after another: the next layer's claims land before later CTAs read
            lo, hi = (offs[me], offs[me + 1]) if local else (min(s, me * per_cta), min(s, me * per_cta + per_cta))
            winners = []
            for (p, m), key in frontier[lo:hi]:
                for k in range(4):
                    if m & (1 << k) and claim.get(p + off[k]) == 4 * key + k:
                        winners.append(p + off[k])
            for pos, q in enumerate(winners):
                mq = nbm(q)
                key = nbase + me * segcap + pos
                for k in range(4):
                    if mq & (1 << k):
                        amin(claim, q + off[k], 4 * key + k)
                    if mq & (16 << k):
                        amin(inj, q + off[k], 4 * key + k)
                new_items[me].append((q, mq))
        seg_items = new_items
        base, prevcap = nbase, segcap
    touched = sorted(inj, key=lambda q: inj[q])
    return pops, touched, claim


def random_grid(rng, H, W, p_u, p_fg):
    ucand, fgc = set(), set()
    for y in range(1, H - 1):
        for x in range(1, W - 1):
            r = rng.random()
            if r < p_u:
                ucand.add(y * W + x)
            elif r < p_u + p_fg:
                fgc.add(y * W + x)
    seed = rng.choice(sorted(ucand))
    ucand.discard(seed)  # the seed is in R from the start (k_state marks it)
    return ucand, fgc, seed


@pytest.mark.parametrize("C", [1, 2, 3, 5, 16])
@pytest.mark.parametrize("slack", [0, 16])
def test_cluster_bfs_order_matches_fifo(C, slack):
    rng = random.Random(0x5EED00B0 + 7 * C + slack)
    for trial in range(12):
        H, W = rng.randint(6, 40), rng.randint(6, 40)
        ucand, fgc, seed = random_grid(rng, H, W, rng.uniform(0.45, 0.8), rng.uniform(0.05, 0.3))
        want_pops, want_touched = fifo_reference(W, ucand, fgc, seed)
        got_pops, got_touched, claim = cluster_model(W, ucand, fgc, seed, C, cta_items=64, slack=slack)
        assert got_pops == want_pops, (C, slack, trial)
        assert got_touched == want_touched, (C, slack, trial)
        # R = the seed and every claimed pixel
        assert {seed} | set(claim) == set(want_pops)


def test_cluster_bfs_snake_and_open_field():
    """A one-pixel snake (one entry per layer, local mode throughout) and an
    open field (a wide diamond frontier that restages when unbalanced)."""
    W = 30
    snake = {y * W + x for y in range(1, 29) for x in range(1, 29) if y % 4 == 1 or (y % 4 == 2 and x == 28)
             or (y % 4 == 3 and x in range(1, 29)) or (y % 4 == 0 and x == 1)}
    field = {y * W + x for y in range(1, 29) for x in range(1, 29)}
    fg = {y * W + x for y in (0, 29) for x in range(W)}
    for region in (snake, field):
        seed = min(region)
        u = set(region) - {seed}
        want = fifo_reference(W, u, fg, seed)
        for C in (1, 4, 16):
            got = cluster_model(W, u, fg, seed, C, cta_items=4096, slack=16)
            assert got[0] == want[0] and got[1] == want[1]
