"""Generates the committed golden fixtures under tests/golden/.

cc_golden.npz — outputs of the REFERENCE's own union-find code
(src/segment/ConnComponents.cpp, compiled from the nscale sources into
oracle/_ref/ by oracle/Makefile) on small seeded inputs:
  label()                 ConnComponents.cpp:52-86   (bgval -1, conn 4 / 8)
  areaThresholdLabeled()  ConnComponents.cpp:205-239 (bwareaopen2's bounds)
  areaThreshold()         ConnComponents.cpp:150-202
  boundingBox()           ConnComponents.cpp:241-284 (bgval -1, and the
                          bgval 0 call of HistologicalEntities.cpp:591)
These pin the oracle's CCL / area / bounding-box restatement.

seg_small.npz — the oracle's segmentNuclei on two small synthetic tiles
(a regression fixture for the oracle itself; not a reference output).

nscale_ref_golden.npz — outputs of nscale's OWN functions on the
segmentNuclei path (oracle/_ref/libnsg_refnscale.so: the definitions taken
from the nscale sources at build time and compiled against the OpenCV
stand-in, whose distanceTransform and watershed are the oracle's) on seeded
inputs:
  imreconstruct<uchar/float>   MorphologicOperations.cpp:1730-1903
  imreconstructBinary, imfillHoles, bwselect   :2768-3031
  bwlabel2, bwareaopen2        :3092-3117, 3281-3314
  imhmin, localMinima, watershed2, morphOpen   :3342-3364, 3717-3882
  NeighborOperations::border   NeighborOperations.cpp:17-44
  getRBC, getBackground        HistologicalEntities.cpp:33-109
  invert<uchar/int/float>      PixelOperations.cpp:21-43
  segmentNuclei (both overloads, default and non-default parameters, and the
  BACKGROUND / BACKGROUND_LIKELY / NO_CANDIDATES_LEFT exits)
                               HistologicalEntities.cpp:115-664
These pin the oracle's restatement of every nscale-authored stage.

Run from the repository root:  python tests/golden/make_golden.py
(needs the nscale sources, for oracle/_ref).
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402
from nscale_gb300 import synth  # noqa: E402

INT_MAX = 2 ** 31 - 1


def inputs() -> dict[str, np.ndarray]:
    rng = np.random.default_rng(0x5EED0009)
    d = {}
    d["zeros_17x23"] = np.zeros((17, 23), np.uint8)
    d["ones_32x32"] = np.full((32, 32), 255, np.uint8)
    cb = (np.indices((16, 16)).sum(axis=0) % 2 * 255).astype(np.uint8)
    d["checker_16x16"] = cb
    d["single_1x1"] = np.full((1, 1), 255, np.uint8)
    d["row_1x40"] = ((rng.random((1, 40)) < 0.5) * 255).astype(np.uint8)
    d["col_40x1"] = ((rng.random((40, 1)) < 0.5) * 255).astype(np.uint8)
    d["noise_97x131"] = ((rng.random((97, 131)) < 0.45) * 255).astype(np.uint8)
    d["multival_64x64"] = rng.integers(0, 4, size=(64, 64)).astype(np.uint8) * 60
    d["discs_256x256"] = synth.disc_mask(256, 256, seed=0x5EED0101)
    # nested-disc phantom in the manner of src/segment/test/sizePhantom.m, at 256x256
    z = np.zeros((256, 256), np.uint8)
    rmax = 64
    r = rmax - 1
    start = 0
    while r >= 0:
        dd = 2 * r + 1
        yy, xx = np.mgrid[-r:r + 1, -r:r + 1]
        w = (yy * yy + xx * xx) <= r * r
        if start + dd > 256:
            break
        z[start:start + dd, start:start + dd][w] = 255
        start += dd + 1
        r = (r + 1) // 2 - 1
    d["phantom_256x256"] = z
    return d


def main() -> None:
    oracle.build(ref=True)
    R = oracle.ref_lib()
    assert R is not None, "oracle/_ref was not built (nscale sources missing?)"
    out = {}
    for name, img in inputs().items():
        h, w = img.shape
        out[f"{name}/img"] = img
        for conn in (4, 8):
            lab = np.empty((h, w), np.int32)
            R.ref_cc_label(np.ascontiguousarray(img), w, h, lab, -1, conn)
            out[f"{name}/label{conn}"] = lab
            for lo, hi in ((11, 1000), (21, 1000), (30, INT_MAX), (1, 5)):
                th = np.empty((h, w), np.int32)
                n = R.ref_cc_area_threshold_labeled(lab, w, h, th, -1, lo, hi)
                out[f"{name}/athr{conn}_{lo}_{hi}"] = th
                out[f"{name}/athr{conn}_{lo}_{hi}_n"] = np.int32(n)
            th2 = np.empty((h, w), np.int32)
            n2 = R.ref_cc_area_threshold(np.ascontiguousarray(img), w, h, th2, -1, 11, 1000, conn)
            out[f"{name}/areathr{conn}"] = th2
            out[f"{name}/areathr{conn}_n"] = np.int32(n2)
            buf = np.zeros(5 * h * w + 5, np.int32)
            n = R.ref_cc_bounding_box(lab, w, h, -1, buf.ctypes.data)
            out[f"{name}/bbox{conn}"] = buf[:5 * n].reshape(5, n).copy()
            buf[:] = 0
            n = R.ref_cc_bounding_box(lab, w, h, 0, buf.ctypes.data)
            out[f"{name}/bbox{conn}_bg0"] = buf[:5 * n].reshape(5, n).copy()
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "cc_golden.npz"), **out)

    seg = {}
    for key, (rows, cols, seed) in {"tile_a": (192, 256, 0x5EED1000), "tile_b": (257, 203, 0x5EED1001)}.items():
        img = synth.he_tile(rows, cols, seed)
        st, lab, mask, bbox, _ = oracle.segment_nuclei(img)
        seg[f"{key}/img"] = img
        seg[f"{key}/status"] = np.int32(st)
        seg[f"{key}/labels"] = lab
        seg[f"{key}/bbox"] = bbox
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "seg_small.npz"), **seg)
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "nscale_ref_golden.npz"), **nscale_ref_cases())
    print("wrote cc_golden.npz, seg_small.npz and nscale_ref_golden.npz")


FLT_MAX = np.finfo(np.float32).max
# non-default segmentNuclei parameters (every connectivity switched)
ALT_PARAMS = dict(T1=2.5, T2=2.0, G1=60, G2=30, minSize=5, maxSize=2000, minSizeSeg=15,
                  fillHolesConnectivity=8, reconConnectivity=4, watershedConnectivity=4)


def nscale_ref_cases() -> dict[str, np.ndarray]:
    """Inputs and nscale's own outputs, keyed "<case>/<name>"."""
    R = oracle.refn_lib()
    assert R is not None, "oracle/_ref/libnsg_refnscale.so was not built (nscale sources missing?)"
    out: dict[str, np.ndarray] = {}
    r, c = 97, 131
    mk, ms = synth.recon_inputs(r, c, seed=0x5EED0201)
    mkf, msf = synth.recon_inputs_f32(r, c, seed=0x5EED0202)
    mkf, msf = mkf - np.float32(100.0), msf - np.float32(50.0)
    out["recon/marker"], out["recon/mask"], out["recon/markerf"], out["recon/maskf"] = mk, ms, mkf, msf
    rng = np.random.default_rng(0x5EED0203)
    bw = synth.disc_mask(r, c, seed=0x5EED0204)
    seeds = ((rng.random((r, c)) < 0.02) * 255).astype(np.uint8)
    out["bin/bw"], out["bin/seeds"] = bw, seeds
    marker = np.where(seeds > 0, bw, 0).astype(np.uint8)
    for conn in (4, 8):
        o = np.empty_like(ms)
        R.ref_imreconstruct_u8(mk, ms, r, c, conn, o)
        out[f"recon/u8_{conn}"] = o
        o = np.empty_like(msf)
        R.ref_imreconstruct_f32(mkf, msf, r, c, conn, o)
        out[f"recon/f32_{conn}"] = o
        o = np.empty_like(bw)
        R.ref_imfill_holes_u8(bw, r, c, conn, o)
        out[f"bin/fill_{conn}"] = o
        o = np.empty_like(bw)
        R.ref_bwselect_u8(bw, seeds, r, c, conn, o)
        out[f"bin/bwselect_{conn}"] = o
        o = np.empty_like(bw)
        R.ref_imreconstruct_binary_u8(marker, bw, r, c, conn, o)
        out[f"bin/reconbin_{conn}"] = o
        o = np.empty((r, c), np.int32)
        R.ref_bwlabel2(bw, r, c, conn, o)
        out[f"bin/bwlabel2_{conn}"] = o
        o = np.empty_like(bw)
        n = C.c_int(0)
        R.ref_bwareaopen2(bw, r, c, 30, 400, conn, o, C.byref(n))
        out[f"bin/areaopen_{conn}"], out[f"bin/areaopen_{conn}_n"] = o, np.int32(n.value)
    # distance chain on disc pairs
    m = synth.disc_pairs_mask(128, 160, seed=0x5EED0205)
    d = oracle.dist_transform(m)
    distance = np.where(m > 0, -d, -FLT_MAX).astype(np.float32)
    o = np.empty_like(distance)
    R.ref_imhmin_f32(distance, 128, 160, 1.0, 8, o)
    out["ws/distance"], out["ws/distance2"] = distance, o
    bgr = synth.colorize_mask(m, seed=0x5EED0206)
    out["ws/bgr"] = bgr
    for conn in (4, 8):
        mn = np.empty((128, 160), np.uint8)
        R.ref_local_minima_f32(o, 128, 160, conn, mn)
        out[f"ws/minima_{conn}"] = mn
        w = np.empty((128, 160), np.int32)
        R.ref_watershed2(bgr, o, 128, 160, conn, w)
        out[f"ws/watershed2_{conn}"] = w
    img = np.random.default_rng(0x5EED0207).integers(0, 256, size=(64, 80)).astype(np.uint8)
    out["open/img"] = img
    for name, se in (("disk19", oracle.se_disk19()), ("cross3", oracle.se_cross3())):
        o2 = np.empty_like(img)
        R.ref_morph_open_u8(img, 64, 80, np.ascontiguousarray(se), se.shape[0], o2)
        out[f"open/{name}"] = o2
    lab = rng.integers(-1, 4, size=(40, 50)).astype(np.int32)
    o3 = np.zeros_like(lab)
    R.ref_border_i32(lab, 40, 50, -1, o3)
    out["border/img"], out["border/out"] = lab, o3
    tile = synth.he_tile(64, 96, seed=0x5EED0208)
    out["pixel/bgr"] = tile
    for t1, t2 in ((5.0, 4.0), (2.5, 2.0)):
        o4 = np.empty((64, 96), np.uint8)
        R.ref_get_rbc(tile, 64, 96, t1, t2, o4)
        out[f"pixel/rbc_{t1}"] = o4
    o5 = np.empty((64, 96), np.uint8)
    R.ref_get_background(tile, 64, 96, 220, 220, 220, o5)
    out["pixel/background"] = o5
    # segmentNuclei
    tiles = {
        "seg_a": (synth.he_tile(192, 256, 0x5EED1000), {}),
        "seg_b": (synth.he_tile(257, 203, 0x5EED1001), {}),
        "seg_alt": (synth.he_tile(160, 200, 0x5EED0006), ALT_PARAMS),
        "seg_white": (synth.white_tile(64, 48, seed=7), {}),
        "seg_empty": (synth.he_tile(96, 96, seed=11, n_nuclei=0, n_rbc=0), {}),
    }
    likely = synth.white_tile(100, 100, seed=8)
    likely[:8, :] = synth.he_tile(8, 100, seed=9)
    tiles["seg_likely"] = (likely, {})
    for key, (img, kw) in tiles.items():
        st, lab2, mask, box, mst = oracle.ref_segment_nuclei(img, oracle.Params(**kw))
        assert st == mst
        out[f"{key}/img"], out[f"{key}/status"] = img, np.int32(st)
        out[f"{key}/labels"], out[f"{key}/mask"] = lab2, mask
        out[f"{key}/ref_bbox"] = box
    return out


if __name__ == "__main__":
    main()
