"""The batched form (nsg_segment_nuclei_batch) and the in-process server
(nsg_server_*) must give every tile exactly what a plain per-tile call gives,
whatever else is in flight (alone-vs-mix equality), and the per-tile call is
itself pinned to the oracle by test_gpu_pipeline."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(512, 512), (700, 1100), (1024, 768), (333, 1500), (900, 900)]


def _tiles():
    from nscale_gb300 import synth
    out = [synth.he_tile(r, c, seed=0x5EED7000 + i) for i, (r, c) in enumerate(SHAPES)]
    out.append(synth.white_tile(400, 600, seed=0x5EED7100))  # BACKGROUND early exit
    return out


def _single(img):
    import torch
    from nscale_gb300.histological_entities import HistologicalEntities as HE
    st, lab, n, bb = HE.segmentNuclei(torch.from_numpy(img).cuda())
    torch.cuda.synchronize()
    return st, lab.cpu().numpy(), n, bb


def test_batch_matches_per_tile_device_and_host(cuda):
    import torch
    from nscale_gb300.serving import TilePool
    tiles = _tiles()
    want = [_single(t) for t in tiles]
    pool = TilePool(1024, 1500, workers=3)
    try:
        dev = pool.segment([torch.from_numpy(t).cuda() for t in tiles])
        host = pool.segment(tiles)
        for got in (dev, host):
            for (ws, wl, wn, wb), (gs, gl, gn, gb) in zip(want, got):
                gl = gl.cpu().numpy() if hasattr(gl, "cpu") else gl
                assert gs == ws and gn == wn
                assert np.array_equal(gl, wl)
                assert np.array_equal(gb, wb)
    finally:
        pool.close()
    assert {w[0] for w in want} >= {0, 1}  # the mix holds a SUCCESS and a BACKGROUND tile


def test_server_alone_vs_mix(cuda):
    from nscale_gb300 import _lib
    from nscale_gb300.serving import TileServer
    tiles = _tiles()
    per = _lib.load().nsg_pool_context_bytes(1024, 1500)
    # alone: a one-worker server, one tile at a time
    alone = []
    srv = TileServer(1024, 1500, per, queue_cap=4)
    assert srv.workers == 1
    try:
        for t in tiles:
            lab = np.empty(t.shape[:2], np.int32)
            k = srv.submit(t, lab, want_bbox=True)
            (r,) = srv.poll(1, 60000)
            assert r["ticket"] == k
            alone.append((r["status"], lab, r["compcount"], r["bbox"]))
    finally:
        srv.close()
    # mix: three workers, every tile submitted twice, interleaved
    srv = TileServer(1024, 1500, 3 * per + per // 2, queue_cap=64)
    assert srv.workers == 3
    try:
        order = list(range(len(tiles))) * 2
        tick = {}
        for i in order:
            lab = np.empty(tiles[i].shape[:2], np.int32)
            tick[srv.submit(tiles[i], lab, want_bbox=True)] = (i, lab)
        got = []
        while len(got) < len(order):
            got += srv.poll(16, 60000)
        for r in got:
            i, lab = tick[r["ticket"]]
            assert r["labels"] is lab
            st, wl, wn, wb = alone[i]
            assert r["status"] == st and r["compcount"] == wn
            assert np.array_equal(lab, wl) and np.array_equal(r["bbox"], wb)
            assert r["latency_ms"] > 0
    finally:
        srv.close()


def test_server_queue_bound(cuda):
    from nscale_gb300 import _lib, synth
    from nscale_gb300.serving import TileServer
    per = _lib.load().nsg_pool_context_bytes(2048, 2048)
    srv = TileServer(2048, 2048, per, queue_cap=1)
    big = synth.he_tile(2048, 2048, seed=0x5EED7200)
    try:
        accepted, refused = 0, 0
        for _ in range(40):
            try:
                srv.submit(big, None)
                accepted += 1
            except _lib.NsgError as e:
                assert e.code == _lib.ERR_QUEUE_FULL
                refused += 1
        assert refused > 0 and accepted >= 1
        got = []
        while len(got) < accepted:
            got += srv.poll(8, 60000)
        assert all(r["status"] == 0 for r in got)
    finally:
        srv.close()


def test_server_features_match_feature_entry(cuda):
    """A tile served with want_features gets the features nsg_nucleus_features
    computes from its labels and the H channel of nsg_color_deconv."""
    import torch
    from nscale_gb300 import _lib, synth
    from nscale_gb300.features import ObjFeatures
    from nscale_gb300.histological_entities import PixelOperations as PO
    from nscale_gb300.serving import TilePool, TileServer
    img = synth.he_tile(700, 900, seed=0x5EED7300)
    per = _lib.load().nsg_pool_context_bytes(700, 900)
    srv = TileServer(700, 900, 2 * per, queue_cap=4)
    try:
        lab = np.empty(img.shape[:2], np.int32)
        srv.submit(img, lab, want_features=True)
        (r,) = srv.poll(1, 60000)
    finally:
        srv.close()
    assert r["status"] == 0 and r["compcount"] > 0
    H, _ = PO.ColorDeconv(torch.from_numpy(img).cuda())
    want = ObjFeatures.nucleusFeatures(torch.from_numpy(lab).cuda(), H).cpu().numpy()
    assert np.array_equal(r["features"], want)
    pool = TilePool(700, 900, workers=2)
    try:
        (st, lab2, n, bb, feats), = pool.segment([torch.from_numpy(img).cuda()], want_features=True)
    finally:
        pool.close()
    assert st == 0 and np.array_equal(lab2.cpu().numpy(), lab) and np.array_equal(feats, want)


def test_tuning_changes_no_result(cuda):
    """Launch shapes (reconstruction grid, BFS cluster) change speed only."""
    import torch
    from nscale_gb300.serving import TilePool
    tiles = [torch.from_numpy(t).cuda() for t in _tiles()[:3]]
    pool = TilePool(1024, 1500, workers=2)
    try:
        base = pool.segment(tiles)
        pool.set_tuning(recon_max_ctas=7, bfs_max_cluster=2)
        pool.set_timing(True)
        tuned = pool.segment(tiles)
        stages, timed = pool.stage_times()
        pool.set_timing(False)
        # the reconstruction's scan-to-queue switchover, another tuning knob
        pool.set_tuning(recon_max_ctas=5, bfs_max_cluster=16, recon_wl_phases=2)
        queued = pool.segment(tiles)
    finally:
        pool.close()
    for (s0, l0, n0, b0), (s1, l1, n1, b1), (s2, l2, n2, b2) in zip(base, tuned, queued):
        assert s0 == s1 == s2 and n0 == n1 == n2
        assert torch.equal(l0, l1) and np.array_equal(b0, b1)
        assert torch.equal(l0, l2) and np.array_equal(b0, b2)
    # per-stage timing of the pool's workers: every tile timed, the heavy stages seen
    assert timed == len(tiles)
    assert stages["reconToNuclei"] > 0 and stages["watershed"] > 0


def test_server_size_classes_route_and_match(cuda):
    """A server with workers in size classes: every tile runs on a context
    that holds it (small tiles do not need a large context), results equal
    the per-tile call's, and a tile no class holds is refused up front."""
    from nscale_gb300 import _lib
    from nscale_gb300.serving import TileServer
    tiles = _tiles()
    want = [_single(t) for t in tiles]
    L = _lib.load()
    small, big = (640, 640), (1024, 1500)
    budget = 2 * L.nsg_pool_context_bytes(*small) + 2 * L.nsg_pool_context_bytes(*big)
    srv = TileServer(0, 0, budget, queue_cap=64, classes=[small, big], weights=[1.0, 1.0])
    try:
        cw = srv.class_workers()
        assert cw[small] >= 1 and cw[big] >= 1, cw
        with pytest.raises(_lib.NsgError) as e:
            srv.submit(np.zeros((2000, 2000, 3), np.uint8))
        assert e.value.code == _lib.ERR_OOM
        tick = {}
        for i, t in enumerate(tiles * 2):
            lab = np.empty(t.shape[:2], np.int32)
            tick[srv.submit(t, lab, want_bbox=True)] = (i % len(tiles), lab)
        got = []
        while len(got) < len(tick):
            got += srv.poll(16, 60000)
        for r in got:
            i, lab = tick[r["ticket"]]
            ws, wl, wn, wb = want[i]
            assert r["status"] == ws and r["compcount"] == wn
            assert np.array_equal(lab, wl) and np.array_equal(r["bbox"], wb)
    finally:
        srv.close()


def test_server_budget_split_over_classes(cuda):
    """The budget buys workers in proportion to weight x context bytes, and
    the largest class always gets one."""
    from nscale_gb300 import _lib
    from nscale_gb300.serving import TileServer
    L = _lib.load()
    a, b = (512, 512), (1024, 1024)
    pa, pb = L.nsg_pool_context_bytes(*a), L.nsg_pool_context_bytes(*b)
    srv = TileServer(0, 0, 4 * pa + 2 * pb, queue_cap=8, classes=[a, b], weights=[1.0, 1.0])
    try:
        cw = srv.class_workers()
        assert cw[b] >= 1 and cw[a] >= 1
        assert cw[a] * pa + cw[b] * pb <= 4 * pa + 2 * pb
    finally:
        srv.close()
    # a budget that holds only one large context: one large worker
    srv = TileServer(0, 0, pb + pa // 2, queue_cap=8, classes=[a, b], weights=[10.0, 1.0])
    try:
        cw = srv.class_workers()
        assert cw[b] == 1
    finally:
        srv.close()


def test_pool_mixed_staging_widths_stress(cuda):
    """Tiles whose width is a multiple of 16 take the TMA-staged
    reconstruction (larger dynamic shared memory); the others take plain
    loads.  Many workers launching both forms at once must never fail a
    launch or change a label (the kernel's shared-memory limit is process-wide
    and set by every caller)."""
    import torch
    from nscale_gb300 import synth_torch
    from nscale_gb300.serving import TilePool
    shapes = [(384, 512), (384, 500), (256, 768), (256, 771)] * 6
    tiles = [synth_torch.he_tile(r, c, 0x5EED7200 + i, device="cuda") for i, (r, c) in enumerate(shapes)]
    want = [_single(t.cpu().numpy()) for t in tiles]
    pool = TilePool(384, 771, workers=12)
    try:
        for _ in range(3):
            got = pool.segment(tiles)
            for (ws, wl, wn, _wb), (gs, gl, gn, _gb) in zip(want, got):
                assert gs == ws and gn == wn
                assert np.array_equal(gl.cpu().numpy(), wl)
    finally:
        pool.close()
    torch.cuda.synchronize()
