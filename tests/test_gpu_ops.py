"""GPU parity tests: every operation on the segmentNuclei path, called through
libnsg.so (the C ABI), against the oracle on the same seeded inputs.
Integer, byte and label outputs must be bit-exact; float32 outputs must be
equal as values (IEEE ==, so +0 and -0 compare equal)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1), (1, 37), (41, 1), (64, 64), (97, 131), (256, 300)]


def T(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def N(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def masks(rows, cols, seed):
    from nscale_gb300 import synth
    yield "discs", synth.disc_mask(rows, cols, seed=seed)
    yield "zeros", np.zeros((rows, cols), np.uint8)
    yield "ones", np.full((rows, cols), 255, np.uint8)
    rng = np.random.default_rng(seed)
    yield "noise", ((rng.random((rows, cols)) < 0.5) * 255).astype(np.uint8)


@pytest.mark.parametrize("shape", SHAPES)
def test_background_and_rbc(cuda, orc, shape):
    from nscale_gb300 import synth
    from nscale_gb300.histological_entities import HistologicalEntities as HE
    img = synth.he_tile(*shape, seed=0x5EED2000 + shape[0])
    m, n = HE.getBackground(T(img))
    om, on = orc.get_background(img)
    assert n == on
    np.testing.assert_array_equal(N(m), om)
    np.testing.assert_array_equal(N(HE.getRBC(T(img))), orc.get_rbc(img))


def test_rbc_on_threshold_colour(cuda, orc):
    """RBC colour (200, 40, 40) puts R/G exactly at T1 = 5; a T1 ramp around it."""
    from nscale_gb300.histological_entities import HistologicalEntities as HE
    img = np.zeros((16, 256, 3), np.uint8)
    img[..., 0] = np.arange(256)[None, :]          # B ramp
    img[..., 1] = np.arange(16)[:, None] * 4 + 38  # G around 40
    img[..., 2] = 200
    for t1, t2 in ((5.0, 4.0), (2.5, 2.0), (5.1, 4.9)):
        np.testing.assert_array_equal(N(HE.getRBC(T(img), t1, t2)), orc.get_rbc(img, t1, t2))


@pytest.mark.parametrize("shape", SHAPES)
def test_morph_open(cuda, orc, shape):
    from nscale_gb300 import morphologic_operations as MO
    rng = np.random.default_rng(shape[0] * 7 + shape[1])
    img = rng.integers(0, 256, size=shape).astype(np.uint8)
    for se in (MO.disk19().numpy(), MO.cross3().numpy(), np.ones((5, 5), np.uint8),
               np.array([[1, 0, 0], [0, 1, 0], [1, 0, 1]], np.uint8)):
        np.testing.assert_array_equal(N(MO.erode(T(img), se)), orc.erode(img, se))
        np.testing.assert_array_equal(N(MO.dilate(T(img), se)), orc.dilate(img, se))
        np.testing.assert_array_equal(N(MO.morphOpen(T(img), se)), orc.morph_open(img, se))


@pytest.mark.parametrize("shape", SHAPES + [(1024, 1024), (513, 1999)])
@pytest.mark.parametrize("conn", [4, 8])
def test_imreconstruct_u8(cuda, orc, shape, conn):
    from nscale_gb300 import morphologic_operations as MO
    from nscale_gb300 import synth
    marker, mask = synth.recon_inputs(*shape, seed=0x5EED0001 + shape[1])
    np.testing.assert_array_equal(N(MO.imreconstruct(T(marker), T(mask), conn)),
                                  orc.imreconstruct(marker, mask, conn))


@pytest.mark.parametrize("wl", ["0", "1"])
@pytest.mark.parametrize("shape", [(300, 517), (1024, 777)])
@pytest.mark.parametrize("conn", [4, 8])
def test_imreconstruct_u8_rough(cuda, orc, shape, conn, wl, monkeypatch):
    """Per-pixel random mask and sparse seeds: propagation follows single-pixel
    (often diagonal) paths across many tiles, the case that exercises the
    dirty-line and neighbour-notification rules (smooth masks rarely do)."""
    from nscale_gb300 import morphologic_operations as MO
    monkeypatch.setenv("NSG_RECON_WL", wl)
    g = np.random.default_rng(0x5EED0041 + shape[0] + conn)
    mask = g.integers(0, 256, size=shape).astype(np.uint8)
    marker = np.where(g.random(shape) < 0.01, mask, 0).astype(np.uint8)
    np.testing.assert_array_equal(N(MO.imreconstruct(T(marker), T(mask), conn)),
                                  orc.imreconstruct(marker, mask, conn))


# every launch form of the uint8 reconstruction (tuning knobs, read at each
# call): lane-per-line scans at several thresholds, shuffle scans at each warp
# count and register budget, the packed strip pass; one result for all
@pytest.mark.parametrize("knobs", [
    {"NSG_RECON_SEQMIN": "1"}, {"NSG_RECON_SEQMIN": "33"}, {"NSG_RECON_CTAS_PER_SM": "1"},
    {"NSG_RECON_HYB": "0"}, {"NSG_RECON_HYB": "0", "NSG_RECON_MINB": "2"}, {"NSG_RECON_WARPS": "16"},
    {"NSG_RECON_WARPS": "32"}, {"NSG_RECON_PACKED": "1", "NSG_RECON_HYB": "0"}, {"NSG_RECON_MAX_CTAS": "3"},
    {"NSG_RECON_WL": "1"}, {"NSG_RECON_WL": "1", "NSG_RECON_WLPH": "3"}, {"NSG_RECON_WL": "1", "NSG_RECON_MAX_CTAS": "2"},
    {"NSG_RECON_TMA": "0"}, {"NSG_RECON_TMA": "0", "NSG_RECON_WL": "1"},
])
@pytest.mark.parametrize("conn", [4, 8])
def test_imreconstruct_u8_launch_forms(cuda, orc, conn, knobs, monkeypatch):
    from nscale_gb300 import morphologic_operations as MO
    from nscale_gb300 import synth
    for k, v in knobs.items():
        monkeypatch.setenv(k, v)
    # 704 x 896: a width the tensor maps accept (TMA-fed tile loads), and
    # 700 x 901: one they do not (plain loads)
    for shape in ((704, 896), (700, 901)):
        marker, mask = synth.recon_inputs(*shape, seed=0x5EED0021 + conn)
        np.testing.assert_array_equal(N(MO.imreconstruct(T(marker), T(mask), conn)),
                                      orc.imreconstruct(marker, mask, conn))


@pytest.mark.parametrize("wl", ["0", "1"])
@pytest.mark.parametrize("shape", [(1, 1), (37, 1), (64, 64), (97, 131), (600, 700)])
@pytest.mark.parametrize("conn", [4, 8])
def test_imreconstruct_f32(cuda, orc, shape, conn, wl, monkeypatch):
    from nscale_gb300 import morphologic_operations as MO
    from nscale_gb300 import synth
    monkeypatch.setenv("NSG_RECON_WL", wl)
    marker, mask = synth.recon_inputs_f32(*shape, seed=0x5EED0011 + shape[0])
    # signed values exercise the zero ring
    marker = marker - np.float32(100.0)
    mask = mask - np.float32(50.0)
    got = N(MO.imreconstruct(T(marker), T(mask), conn))
    ref = orc.imreconstruct(marker, mask, conn)
    assert (got == ref).all()


def test_imreconstruct_timeout_is_reported(cuda):
    """A spin budget of one iteration makes the persistent kernel give up: the
    call returns NSG_ERR_TIMEOUT and the context stays usable."""
    from nscale_gb300 import _lib, morphologic_operations as MO
    from nscale_gb300 import synth
    from nscale_gb300.context import get_context
    marker, mask = synth.recon_inputs(512, 512, seed=3)
    ctx = get_context(512, 512)
    ctx.set_spin_budget(1)
    try:
        with pytest.raises(_lib.NsgError) as e:
            for _ in range(50):
                MO.imreconstruct(T(marker), T(mask), 8)
        assert e.value.code == _lib.ERR_TIMEOUT
    finally:
        ctx.set_spin_budget(0)
    out = MO.imreconstruct(T(marker), T(mask), 8)
    assert N(out).shape == (512, 512)


def test_union_find_timeout_is_reported(cuda):
    """The union-find's bounded retries report too: with a budget of one step,
    every cross-tile union on an all-foreground image runs out (its first find
    walks from a pixel to its tile's root), so bwlabel2 returns NSG_ERR_TIMEOUT
    instead of partial labels; with the budget restored the same context gives
    the full answer."""
    from nscale_gb300 import _lib, morphologic_operations as MO
    from nscale_gb300.context import get_context
    img = np.full((256, 256), 255, np.uint8)
    ctx = get_context(256, 256)
    ctx.set_spin_budget(1)
    try:
        with pytest.raises(_lib.NsgError) as e:
            MO.bwlabel2(T(img), 8)
        assert e.value.code == _lib.ERR_TIMEOUT
        with pytest.raises(_lib.NsgError) as e:
            MO.imfillHoles(T(255 - img), True, 4)
        assert e.value.code == _lib.ERR_TIMEOUT
    finally:
        ctx.set_spin_budget(0)
    np.testing.assert_array_equal(N(MO.bwlabel2(T(img), 8)), np.zeros((256, 256), np.int32))


@pytest.mark.parametrize("shape", SHAPES + [(1024, 1024)])
@pytest.mark.parametrize("conn", [4, 8])
def test_binary_ops(cuda, orc, shape, conn):
    from nscale_gb300 import morphologic_operations as MO
    for name, m in masks(*shape, seed=0x5EED3000 + shape[0]):
        np.testing.assert_array_equal(N(MO.imfillHoles(T(m), True, conn)), orc.imfill_holes(m, conn), err_msg=name)
        seeds = np.zeros_like(m)
        seeds[::7, ::5] = 255
        np.testing.assert_array_equal(N(MO.bwselect(T(m), T(seeds), conn)), orc.bwselect(m, seeds, conn),
                                      err_msg=name)
        marker = (m & seeds)
        np.testing.assert_array_equal(N(MO.imreconstructBinary(T(marker), T(m), conn)),
                                      orc.imreconstruct_binary(marker, m, conn), err_msg=name)


@pytest.mark.parametrize("shape", SHAPES + [(1024, 1024), (2048, 777)])
@pytest.mark.parametrize("conn", [4, 8])
def test_bwlabel_and_areaopen(cuda, orc, shape, conn):
    from nscale_gb300 import morphologic_operations as MO
    for name, m in masks(*shape, seed=0x5EED4000 + shape[1]):
        np.testing.assert_array_equal(N(MO.bwlabel2(T(m), conn)), orc.bwlabel2(m, conn), err_msg=name)
        for lo, hi in ((11, 1000), (21, 1000), (30, 2 ** 31 - 1), (1, 3)):
            out, n = MO.bwareaopen2(T(m), False, True, lo, hi, conn)
            oout, on = orc.bwareaopen2(m, lo, hi, conn)
            assert n == on, (name, lo, hi)
            np.testing.assert_array_equal(N(out), oout, err_msg=name)
    rng = np.random.default_rng(5)
    mv = (rng.integers(0, 4, size=shape) * 60).astype(np.uint8)  # equal-value components
    np.testing.assert_array_equal(N(MO.bwlabel2(T(mv), conn)), orc.bwlabel2(mv, conn))


def test_bwlabel_matches_reference_golden(cuda):
    """GPU labels against the reference's own ConnComponents outputs."""
    import os
    from nscale_gb300 import morphologic_operations as MO
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "cc_golden.npz"))
    for name in sorted({k.split("/")[0] for k in g.files}):
        img = g[f"{name}/img"]
        for conn in (4, 8):
            np.testing.assert_array_equal(N(MO.bwlabel2(T(img), conn)), g[f"{name}/label{conn}"], err_msg=name)


@pytest.mark.parametrize("shape", SHAPES + [(1024, 1024)])
def test_bounding_box(cuda, orc, shape):
    import ctypes as C
    from nscale_gb300 import morphologic_operations as MO
    from nscale_gb300.context import get_context, ptr, stream_handle
    for name, m in masks(*shape, seed=0x5EED5000 + shape[0]):
        lab = MO.bwlabel2(T(m), 8)
        ctx = get_context(*shape)
        cap = shape[0] * shape[1]
        buf = np.zeros(5 * cap + 5, np.int32)
        cnt = C.c_int(0)
        ctx.check(ctx.L.nsg_bounding_box(ctx.h, ptr(lab), shape[0], shape[1], buf.ctypes.data, cap, C.byref(cnt),
                                         stream_handle()))
        n = cnt.value
        np.testing.assert_array_equal(buf[:5 * n].reshape(5, n), orc.bounding_box(N(lab)), err_msg=name)


@pytest.mark.parametrize("shape", SHAPES + [(1024, 1024), (700, 1500)])
def test_dist_transform(cuda, orc, shape):
    from nscale_gb300 import morphologic_operations as MO
    from nscale_gb300 import synth
    for m in (synth.disc_pairs_mask(*shape, seed=0x5EED0002), np.full(shape, 255, np.uint8),
              np.zeros(shape, np.uint8)):
        np.testing.assert_array_equal(N(MO.distTransform(T(m))), orc.dist_transform(m))


def _distance2_inputs(shape, seed):
    from nscale_gb300 import synth
    m = synth.disc_pairs_mask(*shape, seed=seed)
    d = np.asarray(__import__("oracle").dist_transform(m))
    distance = np.where(m > 0, -d, -np.finfo(np.float32).max).astype(np.float32)
    return m, distance


@pytest.mark.parametrize("shape", [(1, 1), (64, 64), (97, 131), (512, 512)])
def test_imhmin_and_minima(cuda, orc, shape):
    from nscale_gb300 import morphologic_operations as MO
    m, distance = _distance2_inputs(shape, 0x5EED0002 + shape[0])
    d2 = N(MO.imhmin(T(distance), 1.0, 8))
    od2 = orc.imhmin(distance, 1.0, 8)
    assert (d2 == od2).all()
    for conn in (4, 8):
        np.testing.assert_array_equal(N(MO.localMinima(T(od2), conn)), orc.local_minima(od2, conn))
        np.testing.assert_array_equal(N(MO.localMaxima(T(-od2), conn)), orc.local_maxima(-od2, conn))


@pytest.mark.parametrize("shape", [(3, 3), (64, 64), (97, 131), (256, 300)])
@pytest.mark.parametrize("conn", [4, 8])
def test_watershed2(cuda, orc, shape, conn):
    from nscale_gb300 import morphologic_operations as MO
    from nscale_gb300 import synth
    m, distance = _distance2_inputs(shape, 0x5EED0022 + shape[1])
    d2 = orc.imhmin(distance, 1.0, 8)
    bgr = synth.colorize_mask(m, seed=0x5EED0000)
    got = N(MO.watershed2(T(bgr), T(d2), conn))
    np.testing.assert_array_equal(got, orc.watershed2(bgr, d2, conn))


def _ws_diag():
    import ctypes as C
    from nscale_gb300.context import get_context, stream_handle
    ctx = get_context(1, 1)
    out = (C.c_int * 16)()
    ctx.check(ctx.L.nsg_watershed_diagnostics(ctx.h, out, stream_handle()))
    return list(out)


def _pipeline_ws_inputs(orc, rows, cols, seed):
    from nscale_gb300 import synth
    img = synth.he_tile(rows, cols, seed)
    _, _, _, _, d = orc.segment_nuclei(img, dump_stages=("seg_big", "distance2"))
    nuclei = img.copy()
    nuclei[d["seg_big"] == 0] = 0
    return nuclei, d["distance2"]


@pytest.mark.parametrize("shape,seed", [((512, 512), 0x5EED0000), ((1024, 1024), 0x5EED0001),
                                        ((2048, 2048), 0x5EED0000), ((777, 1313), 0x5EED0003)])
def test_watershed_domain_parallel_on_tiles(cuda, orc, shape, seed):
    """The domain-parallel flood (no serial fallback) is bit-exact on the
    watershed inputs segmentNuclei produces."""
    from nscale_gb300 import morphologic_operations as MO
    nuclei, d2 = _pipeline_ws_inputs(orc, *shape, seed)
    got = N(MO.watershed2(T(nuclei), T(d2), 8))
    diag = _ws_diag()
    np.testing.assert_array_equal(got, orc.watershed2(nuclei, d2, 8))
    assert diag[0] == 0, f"fast path not taken (fallback code {diag[0]})"
    assert diag[9] == 1  # a background flood event was resolved


@pytest.mark.parametrize("conn", [4, 8])
@pytest.mark.parametrize("const_colour", [False, True])
def test_watershed_disc_pairs(cuda, orc, conn, const_colour):
    from nscale_gb300 import morphologic_operations as MO
    from nscale_gb300 import synth
    m = synth.disc_pairs_mask(1024, 1024, seed=0x5EED0002)
    d = orc.dist_transform(m)
    distance = np.where(m > 0, -d, -np.finfo(np.float32).max).astype(np.float32)
    d2 = orc.imhmin(distance, 1.0, 8)
    bgr = synth.colorize_mask(m, seed=0x5EED0000)
    if const_colour:
        bgr = np.repeat(np.where(m[..., None] > 0, 128, 0).astype(np.uint8), 3, axis=2)
    got = N(MO.watershed2(T(bgr), T(d2), conn))
    np.testing.assert_array_equal(got, orc.watershed2(bgr, d2, conn))
    assert _ws_diag()[0] == 0


def test_watershed_serial_entry(cuda, orc):
    import ctypes as C
    import torch
    from nscale_gb300.context import get_context, ptr, stream_handle
    nuclei, d2 = _pipeline_ws_inputs(orc, 256, 300, 0x5EED0004)
    ctx = get_context(256, 300)
    out = torch.empty((256, 300), dtype=torch.int32, device="cuda")
    tn, td = T(nuclei), T(d2)  # keep the device buffers alive across the call
    ctx.check(ctx.L.nsg_watershed_serial(ctx.h, ptr(tn), ptr(td), ptr(out), 256, 300, 8, stream_handle()))
    np.testing.assert_array_equal(N(out), orc.watershed2(nuclei, d2, 8))


def test_watershed_adversarial_small(cuda, orc):
    """Random colours (many black pixels) and random minima: whichever path the
    flood takes (domain-parallel or its serial fallback), labels are exact."""
    from nscale_gb300 import morphologic_operations as MO
    rng = np.random.default_rng(7)
    paths = {}
    for it in range(150):
        h, w = (int(v) for v in rng.integers(3, 48, size=2))
        d2 = rng.integers(0, 6, size=(h, w)).astype(np.float32)
        bgr = rng.integers(0, int(rng.integers(2, 256)), size=(h, w, 3)).astype(np.uint8)
        bgr[rng.random((h, w)) < rng.random()] = 0
        got = N(MO.watershed2(T(bgr), T(d2), 8 if it % 2 else 4))
        paths[_ws_diag()[0]] = paths.get(_ws_diag()[0], 0) + 1
        np.testing.assert_array_equal(got, orc.watershed2(bgr, d2, 8 if it % 2 else 4), err_msg=f"case {it}")
    assert paths.get(0, 0) > 0


@pytest.mark.parametrize("shape", [(1, 1), (97, 131), (512, 700)])
def test_color_deconv(cuda, orc, shape):
    """ColorDeconv (PixelOperations.cpp:170-274) against the FP32 oracle.  The
    optical-density table, the stain matrix and the double-summed products
    are bit-exact; expf may differ from the host's in the last bit, so a grey
    level may flip at a rounding boundary: tolerance 1 level on at most 0.01 %
    of pixels."""
    from nscale_gb300 import synth
    from nscale_gb300.histological_entities import PixelOperations as PO
    img = synth.he_tile(*shape, seed=0x5EED0A00 + shape[0])
    q = PO.ComputeInverseStainMatrix()
    assert np.array_equal(q, orc.stain_matrix().astype(np.float32))
    H, E = PO.ColorDeconv(T(img))
    oH, oE = orc.color_deconv(img)
    for g, o in ((N(H), oH), (N(E), oE)):
        d = np.abs(g.astype(int) - o.astype(int))
        assert d.max() <= 1
        assert (d > 0).sum() <= max(0, int(1e-4 * d.size))


@pytest.mark.parametrize("shape", [(64, 80), (300, 411)])
def test_gradient_and_nucleus_features(cuda, orc, shape):
    """Operators::gradient bit-exact; per-nucleus area exact, the histogram
    statistics exact as float, perimeter (counted cell classes against the
    reference's ordered sum) within 1e-6 relative."""
    from nscale_gb300 import synth
    from nscale_gb300.features import ObjFeatures, Operators
    from nscale_gb300.histological_entities import PixelOperations as PO
    img = synth.he_tile(*shape, seed=0x5EEDF000 + shape[0])
    H, _ = PO.ColorDeconv(T(img))
    Hn = N(H)
    assert np.array_equal(N(Operators.gradient(H)), orc.gradient(Hn))
    lab = orc.bwlabel2(synth.disc_mask(*shape, seed=shape[1]), 8)
    got = N(ObjFeatures.nucleusFeatures(T(lab), H))
    want = orc.nucleus_features(lab, Hn)
    assert got.shape == want.shape and len(want) > 0
    assert np.array_equal(got[:, 0], want[:, 0])
    assert np.allclose(got[:, 1], want[:, 1], rtol=1e-6, atol=0)
    assert np.array_equal(got[:, 2:], want[:, 2:])


@pytest.mark.parametrize("n", [1, 15, 16, 17, 4099, 1 << 20])
def test_invert_all_types(cuda, n):
    """PixelOperations::invert<T> for the three instantiations, on lengths
    around the 16-byte vector width and on views that start off a 16-byte
    boundary (element tail path)."""
    import torch
    from nscale_gb300.histological_entities import PixelOperations as PO
    g = np.random.default_rng(n)
    u8 = g.integers(0, 256, size=n + 3).astype(np.uint8)
    i32 = g.integers(-2 ** 31, 2 ** 31, size=n + 3, dtype=np.int64).astype(np.int32)
    i32[0] = np.iinfo(np.int32).min  # ~x + 1 wraps there, as the reference's int arithmetic
    f32 = g.standard_normal(n + 3).astype(np.float32)
    f32[:2] = (0.0, -0.0)
    for a, want in ((u8, (255 - u8).astype(np.uint8)), (i32, (~i32 + np.int32(1)).astype(np.int32)),
                    (f32, (-f32 + np.float32(0)).astype(np.float32))):
        t = torch.from_numpy(a).cuda()
        for off in (0, 1):
            got = N(PO.invert(t[off:off + n]))
            assert got.dtype == a.dtype
            np.testing.assert_array_equal(got, want[off:off + n])
    with pytest.raises(TypeError):
        PO.invert(torch.zeros(4, dtype=torch.float64, device="cuda"))


def test_segment_nuclei_host_entry(cuda, orc):
    """nsg_segment_nuclei_host (host buffers in and out, the entry a C++
    caller without device memory uses) against the oracle."""
    import ctypes as C
    from nscale_gb300 import _lib, synth
    from nscale_gb300.context import get_context, stream_handle
    img = np.ascontiguousarray(synth.he_tile(300, 517, seed=0x5EED0003))
    rows, cols = img.shape[:2]
    ctx = get_context(rows, cols)
    lab = np.empty((rows, cols), np.int32)
    mask = np.empty((rows, cols), np.uint8)
    cc = C.c_int(0)
    bbox = C.POINTER(C.c_int32)()
    st = ctx.L.nsg_segment_nuclei_host(ctx.h, img.ctypes.data, rows, cols, None, lab.ctypes.data, mask.ctypes.data,
                                       C.byref(cc), C.byref(bbox), stream_handle())
    ost, olab, omask, obox, _ = orc.segment_nuclei(img)
    assert st == ost == 0
    np.testing.assert_array_equal(lab, olab)
    np.testing.assert_array_equal(mask, omask)
    boxes = np.ctypeslib.as_array(bbox, shape=(5 * cc.value,)).reshape(5, cc.value).copy()
    ctx.L.nsg_free(bbox)
    np.testing.assert_array_equal(boxes, obox)
    # a tile larger than the context is refused, nothing is written
    big = get_context(rows, cols)
    st = big.L.nsg_segment_nuclei_host(big.h, img.ctypes.data, big.max_rows + 1, big.max_cols + 1, None, None,
                                       None, None, None, stream_handle())
    assert st == _lib.ERR_OOM


@pytest.mark.parametrize("shape", [(1, 7), (97, 131), (512, 700), (4096, 4096)])
def test_color_normalization(cuda, orc, shape):
    """Normalization::targetParameters / normalization on the GPU against the
    oracle: statistics within 1e-5 relative; output levels within one, on at
    most 0.1 % of the values (log10f / powf last bits on a rounding boundary),
    and a tile normalised to its own statistics comes back unchanged."""
    import torch
    from nscale_gb300 import synth_torch
    from nscale_gb300.normalization import Normalization
    img_t = synth_torch.he_tile(*shape, 0x5EED0500 + shape[0], device="cuda")
    tgt_t = synth_torch.he_tile(256, 256, 0x5EED0501, device="cuda")
    img, tgt = img_t.cpu().numpy(), tgt_t.cpu().numpy()
    m, s = Normalization.targetParameters(img_t)
    om, os_ = orc.target_parameters(img)
    if np.isfinite(om).all():
        np.testing.assert_allclose(m, om, rtol=1e-5, atol=1e-7)
        np.testing.assert_allclose(s, os_, rtol=1e-5, atol=1e-7)
    mt, st = orc.target_parameters(tgt)
    got = N(Normalization.normalization(img_t, mt, st))
    want = orc.normalization(img, mt, st)
    d = np.abs(got.astype(np.int16) - want.astype(np.int16))
    assert d.max() <= 1, d.max()
    assert (d > 0).mean() <= 1e-3, (d > 0).mean()
    if shape[0] > 1:
        same = N(Normalization.normalization(img_t, m, s))
        dd = np.abs(same.astype(np.int16) - img.astype(np.int16))
        assert dd.max() <= 1 and (dd > 0).mean() <= 1e-3
    torch.cuda.synchronize()
