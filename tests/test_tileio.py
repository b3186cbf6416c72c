"""Tile I/O of the segmentation driver (nscale_gb300/tileio.py): output names
as nu-segment.cpp:123-160 derives them, the label PNG as imwrite stores an
int32 label image (saturated to uint8), the bounds CSV, raw tile reading;
and, on a GPU, a directory of tiles segmented through the batched form with
outputs equal to the oracle's."""
import os

import numpy as np
import pytest


def test_output_names_mirror_the_input_tree(tmp_path):
    from nscale_gb300 import tileio
    src = tmp_path / "in"
    (src / "slide1").mkdir(parents=True)
    a = src / "slide1" / "t_0_0.npy"
    b = src / "t_1.512x256.bgr"
    np.save(a, np.zeros((4, 5, 3), np.uint8))
    np.zeros(512 * 256 * 3, np.uint8).tofile(b)
    (src / "notes.txt").write_text("x")
    tiles = tileio.list_tiles(str(src))
    assert tiles == sorted([str(a), str(b)])
    out = str(tmp_path / "out")
    assert tileio.output_names(str(a), str(src), out) == (os.path.join(out, "slide1", "t_0_0.mask.png"),
                                                          os.path.join(out, "slide1", "t_0_0.bounds.csv"))
    assert tileio.output_names(str(b), str(src), out)[0] == os.path.join(out, "t_1.mask.png")
    assert tileio.read_tile(str(b)).shape == (512, 256, 3)
    assert tileio.read_tile(str(a)).shape == (4, 5, 3)
    bad = src / "t_2.10x10.bgr"
    np.zeros(7, np.uint8).tofile(bad)
    with pytest.raises(ValueError):
        tileio.read_tile(str(bad))


def test_label_png_saturates_like_imwrite_and_reads_back(tmp_path):
    from nscale_gb300 import tileio
    lab = np.array([[-1, 0, 1], [254, 255, 70000]], np.int32)
    p = tmp_path / "m.mask.png"
    bbox = np.array([[1, 254], [2, 0], [2, 0], [0, 1], [0, 1]], np.int32)
    tileio.write_outputs(str(p), str(tmp_path / "m.bounds.csv"), lab, bbox)
    np.testing.assert_array_equal(tileio.read_mask_png(str(p)), [[0, 0, 1], [254, 255, 255]])
    assert (tmp_path / "m.bounds.csv").read_text().splitlines() == ["label,minx,maxx,miny,maxy", "1,2,2,0,0",
                                                                       "254,0,0,1,1"]


@pytest.mark.gpu
def test_segment_directory_matches_oracle(cuda, orc, tmp_path):
    from nscale_gb300 import synth, tileio
    src = tmp_path / "tiles"
    src.mkdir()
    imgs = {"a": synth.he_tile(192, 256, 0x5EED1000), "b": synth.he_tile(257, 203, 0x5EED1001),
            "w": synth.white_tile(64, 80, 7)}
    np.save(src / "a.npy", imgs["a"])
    imgs["b"].tofile(src / "b.257x203.bgr")
    np.save(src / "w.npy", imgs["w"])
    out = tmp_path / "out"
    res = tileio.segment_directory(str(src), str(out), workers=2)
    for k, img in imgs.items():
        path = [p for p in res if os.path.basename(p).startswith(k + ".")][0]
        ost, olab, _, obox, _ = orc.segment_nuclei(img)
        assert res[path] == ost
        mp, bp = tileio.output_names(path, str(src), str(out))
        if ost != 0:
            assert not os.path.exists(mp)
            continue
        np.testing.assert_array_equal(tileio.read_mask_png(mp), np.clip(olab, 0, 255).astype(np.uint8))
        rows = open(bp).read().splitlines()[1:]
        np.testing.assert_array_equal(np.array([[int(v) for v in r.split(",")] for r in rows]).T.reshape(5, -1),
                                      obox)
