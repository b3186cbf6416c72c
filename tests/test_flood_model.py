"""CPU model of two steps of the watershed's per-domain floods
(watershed_pws.cu) against the straightforward forms they replace:

* P1 pushes a black unknown pixel (U) at most once per domain.  The flood
  once kept, per U pixel, the sides it was pushed from and asked whether one
  of them belonged to the domain; it now asks whether a pixel of the domain
  beside it has popped with a label.  Both must give the same pushes.
* P3 starts a one-domain group from the domain's state at T_e.  It used to
  replay the flood up to the cut; it now rebuilds the queue from P1's records
  (initial entries in raster order, then the pushes of every pop before the
  cut that are still queued).  Both must give the same queue, level by level.

Both are modelled on random domains with random colours, markers, initial
entries and U pixels, for every cut.
"""
import random

import pytest

WSHED, IN_QUEUE = -1, -2


def cdiff(a, b):
    return max(abs(x - y) for x, y in zip(a, b))


def make_domain(rng, H, W):
    """A 4-connected fg domain grown from a centre, markers and U pixels around
    it, a border ring; colours per pixel."""
    cells = {(H // 2, W // 2)}
    target = rng.randint(4, max(4, (H - 2) * (W - 2) // 2))
    while len(cells) < target:
        y, x = rng.choice(sorted(cells))
        dy, dx = rng.choice(((0, 1), (0, -1), (1, 0), (-1, 0)))
        if 1 <= y + dy < H - 1 and 1 <= x + dx < W - 1:
            cells.add((y + dy, x + dx))
    kind, mk = {}, {}
    for y in range(H):
        for x in range(W):
            p = y * W + x
            if y in (0, H - 1) or x in (0, W - 1):
                kind[p] = "border"
            elif (y, x) in cells:
                kind[p] = "fg"
            else:
                r = rng.random()
                kind[p] = "marker" if r < 0.35 else "U"
                if kind[p] == "marker":
                    mk[p] = rng.randint(1, 3)
    col = {p: tuple(rng.randint(0, 255) for _ in range(3)) for p in kind}
    fg = [p for p in sorted(kind) if kind[p] == "fg"]
    # initial entries: fg pixels beside a marker, queued at a random level
    init = {p: rng.randint(0, 40) for p in fg
            if any(kind.get(p + o) == "marker" for o in (-1, 1, -W, W)) and rng.random() < 0.8}
    if not init:
        init[fg[0]] = 0
    return kind, mk, col, fg, init


def flood(kind, mk, col, init, W, dedupe, shells=None, cut=None):
    """The domain's flood in the reference's queue order.  shells is None: P1
    (every U push is a dummy, deduplicated by `dedupe`); otherwise the replay
    of P3 up to `cut` pops, pushing only the U pixels in `shells` (as real
    entries).  Returns the records and, for a replay, the queue per level."""
    off = (-1, 1, -W, W)
    q = [[] for _ in range(256)]
    lab = {p: 0 for p in kind if kind[p] == "fg"}
    rparent, rlocal, level = {}, {}, {}
    pops, dummies = [], []  # dummies: (U pixel, pusher, direction, level, pops before it popped)
    sides = {}  # U pixel -> pushers (the side-flag form)
    for p in sorted(init):
        q[init[p]].append(("px", p))
        lab[p] = IN_QUEUE
        rparent[p] = -1
        level[p] = init[p]
    while True:
        if shells is not None and len(pops) == cut:
            return None, q
        lv = next((i for i in range(256) if q[i]), None)
        if lv is None:
            break
        what, e = q[lv].pop(0)
        if what == "dummy":
            dummies[e] = dummies[e][:4] + (len(pops),)
            continue
        if what == "shell":
            return "U pop before the cut", q
        p = e
        rlocal[p] = len(pops)
        pops.append(p)
        lb = 0
        for o in off:
            t = mk.get(p + o, 0) if kind[p + o] == "marker" else (lab[p + o] if kind[p + o] == "fg" else 0)
            if t > 0:
                lb = t if lb == 0 else (lb if t == lb else WSHED)
        lab[p] = lb
        assert lb != 0, "a pop with no labelled neighbour"
        if lb == WSHED:
            continue
        for k, o in enumerate(off):
            qq = p + o
            if kind[qq] == "U":
                l2 = cdiff(col[p], col[qq])
                if shells is not None:
                    if qq in shells and lab.get(qq, 0) == 0:
                        lab[qq] = IN_QUEUE
                        q[l2].append(("shell", qq))
                    continue
                if dedupe == "sides":
                    mine = bool(sides.get(qq))
                    if mine:
                        continue
                    sides.setdefault(qq, []).append(p)
                else:  # a pixel of the domain beside qq has popped with a label
                    if any(n != p and kind.get(n) == "fg" and lab[n] > 0 for n in (qq - 1, qq + 1, qq - W, qq + W)):
                        continue
                dummies.append((qq, p, k, l2, None))
                q[l2].append(("dummy", len(dummies) - 1))
            elif kind[qq] == "fg" and lab[qq] == 0:
                l2 = cdiff(col[p], col[qq])
                lab[qq] = IN_QUEUE
                rparent[qq], level[qq] = p, l2
                q[l2].append(("px", qq))
    return dict(pops=pops, rparent=rparent, rlocal=rlocal, level=level, dummies=dummies, lab=lab), None


def queue_from_records(rec, init, kind, W, shells, cut):
    """queue_at_te: the queue at the cut rebuilt from P1's records."""
    off = (-1, 1, -W, W)
    rl, rp = rec["rlocal"], rec["rparent"]

    def queued(p):  # k_state: not popped before the cut, pushed before it (-1: never popped, -2: never pushed)
        lc, par = rl.get(p, -1), rp.get(p, -2)
        popped = 0 <= lc < cut
        return not popped and (par == -1 or (par >= 0 and 0 <= rl[par] < cut))

    dummy_of = {d[0]: d for d in rec["dummies"] if d[0] in shells}  # the domain's dummy of each shell
    q = [[] for _ in range(256)]
    for p in sorted(init):
        if queued(p):
            q[init[p]].append(("px", p))
    for i in range(cut):
        p = rec["pops"][i]
        for k, o in enumerate(off):
            qq = p + o
            if kind[qq] == "fg" and queued(qq) and rp[qq] == p:
                q[rec["level"][qq]].append(("px", qq))
            elif kind[qq] == "U" and qq in dummy_of and dummy_of[qq][1] == p:
                q[dummy_of[qq][3]].append(("shell", qq))
    return q


@pytest.mark.parametrize("seed", range(40))
def test_push_dedupe_and_queue_at_te(seed):
    rng = random.Random(0x5EED00F0 + seed)
    H, W = rng.randint(6, 14), rng.randint(6, 14)
    kind, mk, col, fg, init = make_domain(rng, H, W)
    try:
        rec_sides, _ = flood(kind, mk, col, init, W, "sides")
    except AssertionError:
        pytest.skip("a pop with no labelled neighbour: the serial flood handles this domain")
    rec, _ = flood(kind, mk, col, init, W, "neighbours")
    assert rec["pops"] == rec_sides["pops"]
    assert [d[:4] for d in rec["dummies"]] == [d[:4] for d in rec_sides["dummies"]]
    # k_udom_count's reservation holds: one dummy slot per distinct U pixel beside the domain
    beside = {p + o for p in fg for o in (-1, 1, -W, W) if kind[p + o] == "U"}
    assert len(rec["dummies"]) <= len(beside)
    assert len({d[0] for d in rec["dummies"]}) == len(rec["dummies"])
    # P3's start, for every cut and a random set of active shells owned by the domain
    shells = {d[0] for d in rec["dummies"] if rng.random() < 0.6}
    for cut in range(len(rec["pops"]) + 1):
        bad, want = flood(kind, mk, col, init, W, "neighbours", shells=shells, cut=cut)
        # the replay fails exactly when a shell's dummy popped before the cut (k_p3_state's check)
        early = any(d[0] in shells and d[4] < cut for d in rec["dummies"])
        assert (bad is not None) == early
        if bad is None:
            assert queue_from_records(rec, init, kind, W, shells, cut) == want
