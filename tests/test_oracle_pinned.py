"""The oracle pinned to nscale's OWN code for every nscale-authored stage of
segmentNuclei.

tests/golden/nscale_ref_golden.npz holds outputs of nscale's functions
(MorphologicOperations.cpp, NeighborOperations.cpp, PixelOperations.cpp and
HistologicalEntities.cpp:33-664, taken from the nscale sources at build time
and compiled against the OpenCV stand-in in oracle/cvstandin; generator
tests/golden/make_golden.py).  The oracle must reproduce them bit for bit.
When the nscale sources are present, the same library (oracle/_ref) is also
run live on more shapes, connectivities and parameter sets.  OpenCV's own
calls stay restated and unpinned: erode/dilate, getStructuringElement and
floodFill are the stand-in's, distanceTransform and watershed the oracle's."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")
FLT_MAX = np.finfo(np.float32).max
ALT_PARAMS = dict(T1=2.5, T2=2.0, G1=60, G2=30, minSize=5, maxSize=2000, minSizeSeg=15,
                  fillHolesConnectivity=8, reconConnectivity=4, watershedConnectivity=4)


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(GOLD, "nscale_ref_golden.npz"))


@pytest.fixture(scope="module")
def refn(orc):
    R = orc.refn_lib()
    if R is None:
        pytest.skip("nscale sources not present here (oracle/_ref not built)")
    return R


@pytest.mark.parametrize("conn", [4, 8])
def test_recon_matches_nscale(orc, g, conn):
    np.testing.assert_array_equal(orc.imreconstruct(g["recon/marker"], g["recon/mask"], conn), g[f"recon/u8_{conn}"])
    got = orc.imreconstruct(g["recon/markerf"], g["recon/maskf"], conn)
    assert np.array_equal(got, g[f"recon/f32_{conn}"])


@pytest.mark.parametrize("conn", [4, 8])
def test_binary_ops_match_nscale(orc, g, conn):
    bw, seeds = g["bin/bw"], g["bin/seeds"]
    marker = np.where(seeds > 0, bw, 0).astype(np.uint8)
    np.testing.assert_array_equal(orc.imfill_holes(bw, conn), g[f"bin/fill_{conn}"])
    np.testing.assert_array_equal(orc.bwselect(bw, seeds, conn), g[f"bin/bwselect_{conn}"])
    np.testing.assert_array_equal(orc.imreconstruct_binary(marker, bw, conn), g[f"bin/reconbin_{conn}"])
    np.testing.assert_array_equal(orc.bwlabel2(bw, conn), g[f"bin/bwlabel2_{conn}"])
    o, n = orc.bwareaopen2(bw, 30, 400, conn)
    np.testing.assert_array_equal(o, g[f"bin/areaopen_{conn}"])
    assert n == int(g[f"bin/areaopen_{conn}_n"])


def test_distance_chain_matches_nscale(orc, g):
    d2 = orc.imhmin(g["ws/distance"], 1.0, 8)
    assert np.array_equal(d2, g["ws/distance2"])
    for conn in (4, 8):
        np.testing.assert_array_equal(orc.local_minima(d2, conn), g[f"ws/minima_{conn}"])
        np.testing.assert_array_equal(orc.watershed2(g["ws/bgr"], d2, conn), g[f"ws/watershed2_{conn}"])


def test_open_border_pixel_ops_match_nscale(orc, g):
    img = g["open/img"]
    np.testing.assert_array_equal(orc.morph_open(img, orc.se_disk19()), g["open/disk19"])
    np.testing.assert_array_equal(orc.morph_open(img, orc.se_cross3()), g["open/cross3"])
    # border() leaves row 0 and the first / last column unwritten (padding)
    got = orc.border_fix(g["border/img"], -1)
    np.testing.assert_array_equal(got[1:, 1:-1], g["border/out"][1:, 1:-1])
    bgr = g["pixel/bgr"]
    np.testing.assert_array_equal(orc.get_rbc(bgr, 5.0, 4.0), g["pixel/rbc_5.0"])
    np.testing.assert_array_equal(orc.get_rbc(bgr, 2.5, 2.0), g["pixel/rbc_2.5"])
    np.testing.assert_array_equal(orc.get_background(bgr)[0], g["pixel/background"])


@pytest.mark.parametrize("key", ["seg_a", "seg_b", "seg_alt", "seg_white", "seg_empty", "seg_likely"])
def test_segment_nuclei_matches_nscale(orc, g, key):
    kw = ALT_PARAMS if key == "seg_alt" else {}
    st, lab, mask, _, _ = orc.segment_nuclei(g[f"{key}/img"], orc.Params(**kw))
    assert st == int(g[f"{key}/status"])
    if st == 0:
        np.testing.assert_array_equal(lab, g[f"{key}/labels"])
        np.testing.assert_array_equal(mask, g[f"{key}/mask"])
        # the reference's own box output: boundingBox(bgval 0) on a -1
        # background (HistologicalEntities.cpp:591), kept by the oracle's
        # bug-compatible variant
        np.testing.assert_array_equal(orc.bounding_box_refbug(lab, 0), g[f"{key}/ref_bbox"])


# ---- live, when the nscale sources are present ------------------------------

@pytest.mark.parametrize("shape", [(1, 1), (1, 37), (41, 1), (64, 64), (300, 517)])
@pytest.mark.parametrize("conn", [4, 8])
def test_live_recon_and_binary(orc, refn, shape, conn):
    from nscale_gb300 import synth
    r, c = shape
    mk, ms = synth.recon_inputs(r, c, seed=r * 7 + c)
    o = np.empty_like(ms)
    assert refn.ref_imreconstruct_u8(mk, ms, r, c, conn, o) == 0
    np.testing.assert_array_equal(o, orc.imreconstruct(mk, ms, conn))
    mkf, msf = synth.recon_inputs_f32(r, c, seed=r + c)
    o = np.empty_like(msf)
    assert refn.ref_imreconstruct_f32(mkf, msf, r, c, conn, o) == 0
    assert np.array_equal(o, orc.imreconstruct(mkf, msf, conn))
    rng = np.random.default_rng(r * c + conn)
    for m in (synth.disc_mask(r, c, seed=r), ((rng.random((r, c)) < 0.5) * 255).astype(np.uint8),
              np.zeros((r, c), np.uint8), np.full((r, c), 255, np.uint8)):
        o = np.empty_like(m)
        refn.ref_imfill_holes_u8(m, r, c, conn, o)
        np.testing.assert_array_equal(o, orc.imfill_holes(m, conn))
        seeds = ((rng.random((r, c)) < 0.02) * 255).astype(np.uint8)
        refn.ref_bwselect_u8(m, seeds, r, c, conn, o)
        np.testing.assert_array_equal(o, orc.bwselect(m, seeds, conn))


@pytest.mark.parametrize("shape,seed", [((512, 512), 0x5EED0000), ((300, 517), 0x5EED0003),
                                        ((384, 320), 0x5EED0006)])
@pytest.mark.parametrize("alt", [False, True])
def test_live_segment_nuclei(orc, refn, shape, seed, alt):
    from nscale_gb300 import synth
    img = synth.he_tile(*shape, seed=seed)
    p = orc.Params(**(ALT_PARAMS if alt else {}))
    st, lab, mask, box, mst = orc.ref_segment_nuclei(img, p)
    ost, olab, omask, _, _ = orc.segment_nuclei(img, p)
    assert st == ost == mst
    if st == 0:
        np.testing.assert_array_equal(lab, olab)
        np.testing.assert_array_equal(mask, omask)
        np.testing.assert_array_equal(box, orc.bounding_box_refbug(olab, 0))
