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
    print("wrote cc_golden.npz and seg_small.npz")


if __name__ == "__main__":
    main()
