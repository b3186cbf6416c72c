"""CPU tests of the oracle: pinned against the reference's own
ConnComponents outputs (tests/golden/cc_golden.npz, generated by
tests/golden/make_golden.py from src/segment/ConnComponents.cpp), against
independent scipy implementations, and on known-answer cases."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")
INT_MAX = 2 ** 31 - 1


@pytest.fixture(scope="module")
def cc_gold():
    return np.load(os.path.join(GOLD, "cc_golden.npz"))


def _names(g):
    return sorted({k.split("/")[0] for k in g.files})


def test_cc_label_matches_reference(orc, cc_gold):
    for name in _names(cc_gold):
        img = cc_gold[f"{name}/img"]
        for conn in (4, 8):
            got = orc.cc_label(img, conn)
            np.testing.assert_array_equal(got, cc_gold[f"{name}/label{conn}"], err_msg=f"{name} conn {conn}")


def test_area_threshold_matches_reference(orc, cc_gold):
    for name in _names(cc_gold):
        for conn in (4, 8):
            lab = cc_gold[f"{name}/label{conn}"]
            for lo, hi in ((11, 1000), (21, 1000), (30, INT_MAX), (1, 5)):
                got, n = orc.area_threshold_labeled(lab, lo, hi)
                np.testing.assert_array_equal(got, cc_gold[f"{name}/athr{conn}_{lo}_{hi}"])
                assert n == int(cc_gold[f"{name}/athr{conn}_{lo}_{hi}_n"]), (name, conn, lo, hi)


def test_bwareaopen_matches_reference_area_threshold(orc, cc_gold):
    """ConnComponents::areaThreshold (one-pass form) and bwareaopen2 agree."""
    for name in _names(cc_gold):
        img = cc_gold[f"{name}/img"]
        for conn in (4, 8):
            ref = cc_gold[f"{name}/areathr{conn}"]
            out, n = orc.bwareaopen2(img, 11, 1000, conn)
            np.testing.assert_array_equal(out, np.where(ref > -1, 255, 0).astype(np.uint8), err_msg=name)
            assert n == int(cc_gold[f"{name}/areathr{conn}_n"])


def test_bounding_box_matches_reference(orc, cc_gold):
    for name in _names(cc_gold):
        for conn in (4, 8):
            lab = cc_gold[f"{name}/label{conn}"]
            # bug-compatible restatement: the reference stops at a 0 or -1 label
            np.testing.assert_array_equal(orc.bounding_box_refbug(lab, -1), cc_gold[f"{name}/bbox{conn}"])
            np.testing.assert_array_equal(orc.bounding_box_refbug(lab, 0), cc_gold[f"{name}/bbox{conn}_bg0"])
            # where the reference's scan is not cut short, the correct boxes agree with it
            if not (lab == 0).any():
                np.testing.assert_array_equal(orc.bounding_box(lab), cc_gold[f"{name}/bbox{conn}"])


def _canon(lab):
    """relabel any labelling to min-raster-index labels (-1 background)."""
    flat = lab.ravel()
    out = np.full(flat.shape, -1, np.int64)
    fg = flat > 0 if lab.min() >= 0 else flat >= 0
    ids = flat[fg]
    idx = np.nonzero(fg)[0]
    first = {}
    for l, i in zip(ids.tolist(), idx.tolist()):
        if l not in first:
            first[l] = i
    out[fg] = [first[l] for l in ids.tolist()]
    return out.reshape(lab.shape)


def test_cc_label_matches_scipy(orc):
    ndi = pytest.importorskip("scipy.ndimage")
    from nscale_gb300 import synth
    m = synth.disc_mask(200, 173, seed=0x5EED0201)
    for conn, st in ((4, ndi.generate_binary_structure(2, 1)), (8, ndi.generate_binary_structure(2, 2))):
        lab, _ = ndi.label(m > 0, structure=st)
        np.testing.assert_array_equal(orc.bwlabel2(m, conn), _canon(lab))


def test_edt_matches_scipy(orc):
    ndi = pytest.importorskip("scipy.ndimage")
    from nscale_gb300 import synth
    m = synth.disc_pairs_mask(300, 277, seed=0x5EED0202)
    ref = ndi.distance_transform_edt(m > 0).astype(np.float32)
    np.testing.assert_array_equal(orc.dist_transform(m), ref)


def test_edt_no_zero_pixel(orc):
    m = np.full((7, 9), 255, np.uint8)
    np.testing.assert_array_equal(orc.dist_transform(m), np.full((7, 9), np.sqrt(np.float32(1e15)), np.float32))


def test_fill_holes_matches_scipy(orc):
    ndi = pytest.importorskip("scipy.ndimage")
    from nscale_gb300 import synth
    m = synth.disc_mask(211, 190, seed=0x5EED0203)
    for conn, st in ((4, ndi.generate_binary_structure(2, 1)), (8, ndi.generate_binary_structure(2, 2))):
        ref = ndi.binary_fill_holes(m > 0, structure=st)
        np.testing.assert_array_equal(orc.imfill_holes(m, conn), np.where(ref, 255, 0).astype(np.uint8))


def test_recon_known_answer(orc):
    # 1-D profile: a marker spike reconstructs the whole plateau under the mask
    mask = np.array([[0, 5, 9, 9, 3, 7, 7, 7, 2, 8]], np.uint8)
    marker = np.array([[0, 0, 0, 9, 0, 0, 0, 0, 0, 0]], np.uint8)
    out = orc.imreconstruct(marker, mask, 4)
    np.testing.assert_array_equal(out, [[0, 5, 9, 9, 3, 3, 3, 3, 2, 2]])
    # float with a negative marker next to the zero ring: the ring propagates 0
    maskf = np.array([[2.0, 2.0, 2.0]], np.float32)
    markerf = np.array([[-1.0, -1.0, -1.0]], np.float32)
    np.testing.assert_array_equal(orc.imreconstruct(markerf, maskf, 4), [[0.0, 0.0, 0.0]])


def test_recon_matches_naive_fixed_point(orc):
    """reconstruction == iterated geodesic dilation on the 0-padded image."""
    from nscale_gb300 import synth
    marker, mask = synth.recon_inputs(40, 37, seed=0x5EED0204)
    for conn in (4, 8):
        got = orc.imreconstruct(marker, mask, conn)
        cur = np.minimum(marker, mask).astype(np.int32)
        while True:
            p = np.pad(cur, 1)
            nb = [p[1:-1, 1:-1], p[:-2, 1:-1], p[2:, 1:-1], p[1:-1, :-2], p[1:-1, 2:]]
            if conn == 8:
                nb += [p[:-2, :-2], p[:-2, 2:], p[2:, :-2], p[2:, 2:]]
            nxt = np.maximum(cur, np.minimum(np.max(nb, axis=0), mask))
            if (nxt == cur).all():
                break
            cur = nxt
        np.testing.assert_array_equal(got, cur.astype(np.uint8))


def test_local_maxima_plateaus(orc):
    img = np.array([[1, 1, 1, 0],
                    [1, 3, 3, 0],
                    [1, 3, 2, 0],
                    [0, 1, 1, 5]], np.float32)
    out = orc.local_maxima(img, 8)
    exp = np.zeros((4, 4), np.uint8)
    exp[1, 1] = exp[1, 2] = exp[2, 1] = 255  # the 3-plateau
    exp[3, 3] = 255                           # the 5 peak
    np.testing.assert_array_equal(out, exp)


def test_watershed_two_markers_line(orc):
    """Two flat basins split by a line where their floods meet."""
    rows, cols = 5, 9
    img = np.zeros((rows, cols, 3), np.uint8)
    img[:, :, :] = 100
    markers = np.zeros((rows, cols), np.int32)
    markers[2, 1] = 1
    markers[2, 7] = 2
    out = orc.cv_watershed(img, markers)
    assert (out[0, :] == -1).all() and (out[-1, :] == -1).all()
    assert (out[1:-1, 1:4] == 1).all() and (out[1:-1, 5:8] == 2).all()
    assert (out[1:-1, 4] == -1).all()


def test_segment_small_regression(orc):
    g = np.load(os.path.join(GOLD, "seg_small.npz"))
    for key in ("tile_a", "tile_b"):
        st, lab, _, bbox, _ = orc.segment_nuclei(g[f"{key}/img"])
        assert st == int(g[f"{key}/status"])
        np.testing.assert_array_equal(lab, g[f"{key}/labels"])
        np.testing.assert_array_equal(bbox, g[f"{key}/bbox"])


def test_segment_background_status(orc):
    from nscale_gb300 import synth
    st, lab, _, bbox, _ = orc.segment_nuclei(synth.white_tile(64, 80, seed=1))
    assert st == 1 and (lab == -1).all() and bbox.shape == (5, 0)


def test_color_lut_and_stain_matrix(orc):
    """ComputeLookupTable / ComputeInverseStainMatrix (PixelOperations.cpp:94-168)
    against a numpy restatement in double."""
    k = np.float32(-255.0 / np.log(255.0))
    want = (np.float64(k) * np.log(np.arange(256, dtype=np.float32).astype(np.float64) + 1.0) + 255.0)
    assert np.array_equal(orc.color_lut(), want.astype(np.float32))
    M = orc.STAINS_M.copy()
    N = M / np.maximum(np.linalg.norm(M, axis=0), 1e-300)
    N[:, 2] = 0
    rn = np.linalg.norm(N, axis=1)
    N[:, 2] = np.where(rn > 1, 0, np.sqrt(np.maximum(0, 1 - rn * rn)))
    N[:, 2] /= np.linalg.norm(N[:, 2])
    Q = np.linalg.inv(N)[:2]
    assert np.allclose(orc.stain_matrix(), Q, rtol=1e-12, atol=1e-14)


def test_color_deconv_fp32_vs_fp64(orc):
    """FP oracle: the FP32 path (the reference CPU's) against the FP64 one:
    at most one grey level apart, on a small fraction of pixels."""
    from nscale_gb300 import synth
    img = synth.he_tile(256, 320, seed=0x5EED0A22)
    H32, E32 = orc.color_deconv(img)
    H64, E64 = orc.color_deconv(img, f64=True)
    for a, b in ((H32, H64), (E32, E64)):
        d = np.abs(a.astype(int) - b.astype(int))
        assert d.max() <= 1
        assert (d > 0).mean() < 0.01
    assert H32.std() > 5  # the channel carries the nuclei


def test_perimeter_known_answers(orc):
    """ObjFeatures::perimeter (ObjFeatures.cpp:143-270) restated: a lone pixel
    is four one-corner cells (4 / sqrt 2); a 2 x 2 block adds four edge cells."""
    lab = np.full((6, 7), -1, np.int32)
    lab[1, 1] = 8
    lab[3:5, 3:5] = 24
    f = orc.nucleus_features(lab, np.full(lab.shape, 100, np.uint8))
    assert f.shape == (2, 5)
    assert np.allclose(f[:, 0], [1, 4])
    assert np.allclose(f[:, 1], [4 * 0.70710678118, 4 * 0.70710678118 + 4], rtol=1e-7)
    assert np.allclose(f[:, 2], [100, 100]) and np.allclose(f[:, 3], [0, 0])


def test_gradient_matches_numpy(orc):
    """Operators::gradient: central differences, one-sided at the edges,
    float magnitude rounded half up."""
    rng = np.random.default_rng(5)
    img = rng.integers(0, 256, (37, 53)).astype(np.uint8)
    f = img.astype(np.float32)
    dx = np.empty_like(f)
    dy = np.empty_like(f)
    dx[:, 1:-1] = (f[:, 2:] - f[:, :-2]) * np.float32(0.5)
    dx[:, 0], dx[:, -1] = f[:, 1] - f[:, 0], f[:, -1] - f[:, -2]
    dy[1:-1] = (f[2:] - f[:-2]) * np.float32(0.5)
    dy[0], dy[-1] = f[1] - f[0], f[-1] - f[-2]
    m = np.sqrt(dx * dx + dy * dy, dtype=np.float32)
    want = np.clip(np.floor(m) + ((m - np.floor(m)) >= 0.5), 0, 255).astype(np.uint8)
    assert np.array_equal(orc.gradient(img), want)


def test_features_count_form_matches_reference_order(orc):
    """The GPU sums perimeter cell classes as counts; on random discs that
    equals the reference's ordered double sum to within float rounding."""
    from nscale_gb300 import synth
    m = synth.disc_mask(200, 240, seed=77)
    lab = orc.bwlabel2(m, 8)
    gray = synth.he_tile(200, 240, seed=78)[:, :, 0]
    f = orc.nucleus_features(lab, gray)
    assert len(f) >= 2
    # count form over the whole image, per component
    cls = np.zeros(16, int)
    cls[[1, 2, 4, 8, 7, 11, 13, 14]] = 1
    cls[[3, 6, 9, 12]] = 2
    cls[[5, 10]] = 3
    pad = np.pad(lab, 1, constant_values=-1)
    roots = np.unique(lab[lab >= 0])
    for k, L in enumerate(roots):
        b = (pad == L).astype(int)
        mk = (b[:-1, :-1] << 3) | (b[:-1, 1:] << 2) | (b[1:, 1:] << 1) | b[1:, :-1]
        c = cls[mk]
        per = (c == 1).sum() * 0.70710678118 + (c == 2).sum() * 1.0 + (c == 3).sum() * 1.41421356237
        assert abs(per - f[k, 1]) <= 1e-5 * max(1.0, per)
        assert f[k, 0] == (lab == L).sum()


def test_normalization_to_own_statistics_is_identity(orc):
    """Colour normalisation towards a tile's own foreground statistics maps the
    tile onto itself (the lab round trip and rndint give back every level),
    and towards another tile's statistics moves the foreground only."""
    from nscale_gb300 import synth
    img = synth.he_tile(300, 400, seed=5)
    m, s = orc.target_parameters(img)
    assert np.all(np.isfinite(m)) and np.all(s > 0)
    np.testing.assert_array_equal(orc.normalization(img, m, s), img)
    mt, st = orc.target_parameters(synth.he_tile(200, 200, seed=77))
    out = orc.normalization(img, mt, st)
    assert out.shape == img.shape and out.dtype == np.uint8
    assert (out != img).any()
