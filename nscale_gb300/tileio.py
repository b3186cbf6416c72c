"""Tile input / output of the segmentation driver, without an image library.

The reference's driver (src/segment/nu-segment.cpp) walks an image directory,
names each tile's outputs by replacing the extension and the directory
(getFiles, nu-segment.cpp:123-160: `<name>.mask.png` and `<name>.bounds.csv`
under the output directory, mirroring the input tree), segments every tile
with HistologicalEntities::segmentNuclei(in, out, ...) and writes the label
image with imwrite (HistologicalEntities.cpp:453-470).  OpenCV's PNG writer
stores 8-bit images only, so imwrite turns the int32 labels into uint8 with
saturation (background -1 -> 0, labels from 255 up -> 255); `mask_png_bytes`
does the same.  The reference names the bounds file but does not write it;
here it receives the bounding boxes as CSV (label, minx, maxx, miny, maxy).

Tiles are read from raw buffers: `.npy` arrays (rows x cols x 3, BGR uint8)
or `.bgr` files named `<name>.<rows>x<cols>.bgr` (raw BGR bytes), the form a
slide tiler hands over; PNG/TIFF decoding is out of scope (no image library
on this path).

    python -m nscale_gb300.tileio <image_dir> <output_dir> [--workers N]
"""
from __future__ import annotations

import argparse
import os
import re
import struct
import sys
import zlib

import numpy as np

TILE_EXTS = (".npy", ".bgr")
_RAW = re.compile(r"\.(\d+)x(\d+)\.bgr$")


def list_tiles(image_dir: str) -> list[str]:
    """Tile files under image_dir (recursive, sorted), or image_dir itself
    when it is one file."""
    if os.path.isfile(image_dir):
        return [image_dir]
    out = []
    for root, _dirs, files in os.walk(image_dir):
        for f in files:
            if f.endswith(TILE_EXTS):
                out.append(os.path.join(root, f))
    return sorted(out)


def output_names(tile_path: str, image_dir: str, out_dir: str) -> tuple[str, str]:
    """(<out>/<rel>.mask.png, <out>/<rel>.bounds.csv): the input's extension
    replaced and its directory moved under out_dir (getFiles,
    nu-segment.cpp:123-160)."""
    base = image_dir if os.path.isdir(image_dir) else os.path.dirname(image_dir)
    rel = os.path.relpath(tile_path, base)
    m = _RAW.search(rel)
    stem = rel[: m.start()] if m else os.path.splitext(rel)[0]
    return os.path.join(out_dir, stem + ".mask.png"), os.path.join(out_dir, stem + ".bounds.csv")


def read_tile(path: str) -> np.ndarray:
    """BGR uint8 (rows, cols, 3) from a .npy array or a <name>.<rows>x<cols>.bgr raw file."""
    if path.endswith(".npy"):
        a = np.load(path)
    else:
        m = _RAW.search(path)
        if not m:
            raise ValueError(f"{path}: raw tiles are named <name>.<rows>x<cols>.bgr")
        rows, cols = int(m.group(1)), int(m.group(2))
        a = np.fromfile(path, dtype=np.uint8)
        if a.size != rows * cols * 3:
            raise ValueError(f"{path}: {a.size} bytes, expected {rows * cols * 3}")
        a = a.reshape(rows, cols, 3)
    if a.dtype != np.uint8 or a.ndim != 3 or a.shape[2] != 3:
        raise ValueError(f"{path}: expected a rows x cols x 3 uint8 BGR array")
    return np.ascontiguousarray(a)


def _chunk(kind: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)


def mask_png_bytes(labels: np.ndarray) -> bytes:
    """An 8-bit greyscale PNG of the labels saturated to uint8, as imwrite
    stores an int32 label image (values below 0 -> 0, above 255 -> 255)."""
    img = np.clip(np.asarray(labels), 0, 255).astype(np.uint8)
    rows, cols = img.shape
    raw = np.zeros((rows, cols + 1), np.uint8)  # filter byte 0 (None) per row
    raw[:, 1:] = img
    ihdr = struct.pack(">IIBBBBB", cols, rows, 8, 0, 0, 0, 0)
    return (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", ihdr) + _chunk(b"IDAT", zlib.compress(raw.tobytes(), 6)) +
            _chunk(b"IEND", b""))


def read_mask_png(path: str) -> np.ndarray:
    """Reads back the PNGs mask_png_bytes writes (8-bit grey, filter 0)."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, hdr = 8, b"", None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat += body
    if hdr is None:
        raise ValueError("no IHDR chunk")
    cols, rows, depth, ctype = hdr[0], hdr[1], hdr[2], hdr[3]
    if depth != 8 or ctype != 0:
        raise ValueError("only 8-bit greyscale PNGs")
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(rows, cols + 1)
    if (raw[:, 0] != 0).any():
        raise ValueError("only unfiltered rows")
    return raw[:, 1:].copy()


def bounds_csv(bbox: np.ndarray) -> str:
    """label,minx,maxx,miny,maxy per component (bbox as 5 x n arrays)."""
    lines = ["label,minx,maxx,miny,maxy"]
    for k in range(bbox.shape[1]):
        lines.append(",".join(str(int(v)) for v in bbox[:, k]))
    return "\n".join(lines) + "\n"


def write_outputs(mask_path: str, bounds_path: str, labels: np.ndarray, bbox: np.ndarray) -> None:
    for p in (mask_path, bounds_path):
        os.makedirs(os.path.dirname(p) or ".", exist_ok=True)
    with open(mask_path, "wb") as f:
        f.write(mask_png_bytes(labels))
    with open(bounds_path, "w") as f:
        f.write(bounds_csv(bbox))


def segment_directory(image_dir: str, out_dir: str, workers: int = 8, device: int = 0) -> dict[str, int]:
    """Every tile under image_dir through the batched form; the outputs of
    each tile that ends in SUCCESS are written (the reference writes only
    then, HistologicalEntities.cpp:465-466).  Returns {tile path: status}."""
    from .serving import TilePool
    paths = list_tiles(image_dir)
    if not paths:
        return {}
    tiles = [read_tile(p) for p in paths]
    pool = TilePool(max(t.shape[0] for t in tiles), max(t.shape[1] for t in tiles),
                    workers=max(1, min(workers, len(tiles))), device=device)
    try:
        res = pool.segment(tiles, want_bbox=True)
    finally:
        pool.close()
    out = {}
    for p, (status, labels, _n, bbox) in zip(paths, res):
        out[p] = status
        if status == 0:
            mp, bp = output_names(p, image_dir, out_dir)
            write_outputs(mp, bp, labels, bbox)
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="segmentNuclei over a directory of raw BGR tiles")
    ap.add_argument("image_dir")
    ap.add_argument("output_dir")
    ap.add_argument("--workers", type=int, default=8)
    a = ap.parse_args(argv)
    res = segment_directory(a.image_dir, a.output_dir, a.workers)
    for p, st in res.items():
        print(f"{p}: status {st}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
