"""Deterministic synthetic H&E-like tiles and morphology test inputs.

The reference's validation tiles (TCGA / astroII / oligoIII slides) are not
available, so seeded synthetic inputs with the same shapes, sizes and value
distributions stand in for them:

* ``he_tile`` — a BGR-interleaved uint8 tile: background RGB uniform 215-240
  per pixel and channel, value-noise eosin stroma around RGB (230,170,200)
  with amplitude 25, ~6000 hematoxylin ellipses per 4096x4096 (semi-axes
  4-12 px, random orientation, 30 % in overlapping pairs, RGB (70,40,120)
  +-15), ~200 red-blood-cell discs (radius 3-5, RGB (200,40,40)) and additive
  Gaussian-like noise (sigma 8), clipped to [0, 255].
* ``white_tile`` — a tissue-free near-white tile (RGB >= 230) that the
  background test classifies as BACKGROUND.
* ``recon_inputs`` — grey marker/mask pair for imreconstruct: mask = smoothed
  uniform noise rescaled to [0,255], marker = max(mask-30, 0).
* ``disc_mask`` — binary masks of random discs (radius 2-40) at ~40 %
  foreground with 5 % single-pixel holes (imfillHoles / CCL inputs).
* ``disc_pairs_mask`` — overlapping disc pairs + isolated discs (distance
  transform + watershed inputs).

All randomness comes from a counter-based hash (splitmix64) of
(seed, stream, index), so any pixel can be regenerated independently and
results do not depend on generation order.  Integer arithmetic is used
wherever pixels are decided; the few floating-point steps (ellipse rotation,
interpolation) use plain IEEE float64.
"""
from __future__ import annotations

import math

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def _key(seed: int, stream: int) -> np.uint64:
    s = _splitmix64(np.array([(seed * 1000003 + stream) & 0xFFFFFFFFFFFFFFFF], dtype=np.uint64))
    return s[0]


def _hash(seed: int, stream: int, idx: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        return _splitmix64(idx.astype(np.uint64) * np.uint64(0xD1B54A32D192ED03) + _key(seed, stream))


def _uniform(seed: int, stream: int, idx: np.ndarray) -> np.ndarray:
    """float64 uniforms in [0, 1)."""
    return (_hash(seed, stream, idx) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _randint(seed: int, stream: int, idx: np.ndarray, lo: int, hi: int) -> np.ndarray:
    """integers uniform in [lo, hi] (inclusive)."""
    span = np.uint64(hi - lo + 1)
    return (_hash(seed, stream, idx) % span).astype(np.int64) + lo


class _Scalars:
    """Sequential scalar draws from one stream (for object parameters)."""

    def __init__(self, seed: int, stream: int):
        self.seed, self.stream, self.i = seed, stream, 0

    def u(self) -> float:
        v = float(_uniform(self.seed, self.stream, np.array([self.i]))[0])
        self.i += 1
        return v

    def ri(self, lo: int, hi: int) -> int:
        v = int(_randint(self.seed, self.stream, np.array([self.i]), lo, hi)[0])
        self.i += 1
        return v


def _value_noise(rows: int, cols: int, seed: int, stream: int, cell: int) -> np.ndarray:
    """Smooth value noise in [0,1]: random lattice every `cell` px, smoothstep-
    interpolated (a Perlin-style texture)."""
    gr = rows // cell + 2
    gc = cols // cell + 2
    lat = _uniform(seed, stream, np.arange(gr * gc)).reshape(gr, gc)
    y = np.arange(rows, dtype=np.float64) / cell
    x = np.arange(cols, dtype=np.float64) / cell
    y0 = np.floor(y).astype(np.int64)
    x0 = np.floor(x).astype(np.int64)
    fy = y - y0
    fx = x - x0
    sy = fy * fy * (3 - 2 * fy)
    sx = fx * fx * (3 - 2 * fx)
    a = lat[y0][:, x0]
    b = lat[y0][:, x0 + 1]
    c = lat[y0 + 1][:, x0]
    d = lat[y0 + 1][:, x0 + 1]
    top = a + (b - a) * sx[None, :]
    bot = c + (d - c) * sx[None, :]
    return top + (bot - top) * sy[:, None]


def _fill_ellipse(mask_rgb: np.ndarray, cy: float, cx: float, a: float, b: float, th: float, color) -> None:
    rows, cols = mask_rgb.shape[:2]
    r = int(math.ceil(max(a, b))) + 1
    y0, y1 = max(0, int(cy) - r), min(rows, int(cy) + r + 1)
    x0, x1 = max(0, int(cx) - r), min(cols, int(cx) + r + 1)
    if y0 >= y1 or x0 >= x1:
        return
    yy, xx = np.mgrid[y0:y1, x0:x1]
    dy = yy - cy
    dx = xx - cx
    c, s = math.cos(th), math.sin(th)
    u = (dx * c + dy * s) / a
    v = (-dx * s + dy * c) / b
    inside = (u * u + v * v) <= 1.0
    sub = mask_rgb[y0:y1, x0:x1]
    sub[inside] = color


def he_tile(rows: int = 4096, cols: int = 4096, seed: int = 0x5EED0000,
            n_nuclei: int | None = None, n_rbc: int | None = None) -> np.ndarray:
    """H&E-like BGR uint8 tile of shape (rows, cols, 3)."""
    area = rows * cols
    scale = area / float(4096 * 4096)
    if n_nuclei is None:
        n_nuclei = int(round(6000 * scale))
    if n_rbc is None:
        n_rbc = int(round(200 * scale))
    idx = np.arange(area, dtype=np.uint64).reshape(rows, cols)
    rgb = np.empty((rows, cols, 3), dtype=np.float64)
    for ch in range(3):
        rgb[..., ch] = _randint(seed, 1 + ch, idx, 215, 240)
    # eosin stroma: value noise mask and colour modulation
    v = 0.65 * _value_noise(rows, cols, seed, 10, 96) + 0.35 * _value_noise(rows, cols, seed, 11, 24)
    s = np.clip((v - 0.5) * 3.0, 0.0, 1.0)
    stroma_base = (230.0, 170.0, 200.0)
    for ch in range(3):
        mod = 25.0 * (2.0 * _value_noise(rows, cols, seed, 12 + ch, 32) - 1.0)
        rgb[..., ch] = rgb[..., ch] * (1.0 - s) + (stroma_base[ch] + mod) * s
    del v, s
    # nuclei: 70 % single, 30 % in overlapping pairs
    sc = _Scalars(seed, 100)
    n_pairs = int(round(n_nuclei * 0.15))
    n_single = max(0, n_nuclei - 2 * n_pairs)
    objs = []
    for _ in range(n_single + n_pairs):
        cy, cx = sc.u() * rows, sc.u() * cols
        a, b = 4.0 + 8.0 * sc.u(), 4.0 + 8.0 * sc.u()
        th = math.pi * sc.u()
        objs.append((cy, cx, a, b, th))
    for k in range(n_pairs):
        cy, cx, a, b, th = objs[n_single + k]
        a2, b2 = 4.0 + 8.0 * sc.u(), 4.0 + 8.0 * sc.u()
        ang = 2.0 * math.pi * sc.u()
        dist = (0.5 * (a + b) + 0.5 * (a2 + b2)) * (0.45 + 0.35 * sc.u())
        objs.append((cy + dist * math.sin(ang), cx + dist * math.cos(ang), a2, b2, math.pi * sc.u()))
    for (cy, cx, a, b, th) in objs:
        color = (70 + sc.ri(-15, 15), 40 + sc.ri(-15, 15), 120 + sc.ri(-15, 15))
        _fill_ellipse(rgb, cy, cx, a, b, th, color)
    for _ in range(n_rbc):
        cy, cx = sc.u() * rows, sc.u() * cols
        r = 3.0 + 2.0 * sc.u()
        _fill_ellipse(rgb, cy, cx, r, r, 0.0, (200.0, 40.0, 40.0))
    # noise ~ N(0, 8^2): Irwin-Hall of 4 uniforms (16-bit each) from one hash
    for ch in range(3):
        h = _hash(seed, 20 + ch, idx)
        acc = np.zeros((rows, cols), dtype=np.float64)
        for k in range(4):
            acc += ((h >> np.uint64(16 * k)) & np.uint64(0xFFFF)).astype(np.float64)
        acc = (acc / 65536.0 - 2.0) * (8.0 * math.sqrt(3.0))
        rgb[..., ch] += acc
    out = np.clip(np.floor(rgb + 0.5), 0, 255).astype(np.uint8)
    return np.ascontiguousarray(out[..., ::-1])  # RGB -> BGR


def white_tile(rows: int, cols: int, seed: int) -> np.ndarray:
    """Tissue-free near-white BGR tile (every channel in 230..250)."""
    idx = np.arange(rows * cols, dtype=np.uint64).reshape(rows, cols)
    out = np.empty((rows, cols, 3), dtype=np.uint8)
    for ch in range(3):
        out[..., ch] = _randint(seed, 40 + ch, idx, 230, 250).astype(np.uint8)
    return out


def recon_inputs(rows: int = 4096, cols: int = 4096, seed: int = 0x5EED0001):
    """(marker, mask) uint8 pair: mask = smoothed uniform noise rescaled to
    [0,255] (sigma ~4: two passes of a 9-tap box filter along each axis),
    marker = max(mask - 30, 0)."""
    idx = np.arange(rows * cols, dtype=np.uint64).reshape(rows, cols)
    u = _uniform(seed, 1, idx)
    for _ in range(2):
        u = _box_rows(u, 4)
        u = _box_rows(u.T, 4).T
    lo, hi = u.min(), u.max()
    mask = np.floor((u - lo) / max(hi - lo, 1e-12) * 255.0 + 0.5).clip(0, 255).astype(np.uint8)
    marker = np.maximum(mask.astype(np.int16) - 30, 0).astype(np.uint8)
    return marker, mask


def _box_rows(a: np.ndarray, r: int) -> np.ndarray:
    """Box filter of radius r along axis 1 with zero padding (cumsum)."""
    c = np.cumsum(np.pad(a, ((0, 0), (r + 1, r)), mode="constant"), axis=1)
    return (c[:, 2 * r + 1:] - c[:, :-2 * r - 1]) / (2 * r + 1)


def recon_inputs_f32(rows: int = 4096, cols: int = 4096, seed: int = 0x5EED0001):
    """float32 (marker, mask): the uint8 pair plus a deterministic fractional
    part, so that float reconstruction sees non-integer values."""
    marker, mask = recon_inputs(rows, cols, seed)
    idx = np.arange(rows * cols, dtype=np.uint64).reshape(rows, cols)
    frac = (_randint(seed, 7, idx, 0, 1023).astype(np.float32) / np.float32(1024.0))
    maskf = mask.astype(np.float32) + frac
    markerf = np.maximum(maskf - np.float32(30.0), np.float32(0.0)).astype(np.float32)
    return markerf, maskf


def disc_mask(rows: int = 4096, cols: int = 4096, seed: int = 0x5EED0001, coverage: float = 0.40,
              hole_frac: float = 0.05) -> np.ndarray:
    """uint8 0/255 mask of random discs (radius 2-40) at ~`coverage`
    foreground, then `hole_frac` of the foreground pixels punched out as
    single-pixel holes."""
    m = np.zeros((rows, cols), dtype=np.uint8)
    sc = _Scalars(seed, 200)
    target = coverage * rows * cols
    # expected disc area E[pi r^2] with r ~ U(2,40): pi*(40^3-2^3)/(3*38)
    mean_area = math.pi * (40 ** 3 - 2 ** 3) / (3 * 38.0)
    n = int(-math.log(max(1e-9, 1.0 - coverage)) * rows * cols / mean_area)
    for _ in range(max(1, n)):
        cy, cx, r = sc.u() * rows, sc.u() * cols, 2.0 + 38.0 * sc.u()
        _fill_disc(m, cy, cx, r)
    idx = np.arange(rows * cols, dtype=np.uint64).reshape(rows, cols)
    holes = (_uniform(seed, 201, idx) < hole_frac) & (m > 0)
    m[holes] = 0
    del target
    return m


def _fill_disc(m: np.ndarray, cy: float, cx: float, r: float, val: int = 255) -> None:
    rows, cols = m.shape
    ri = int(math.ceil(r)) + 1
    y0, y1 = max(0, int(cy) - ri), min(rows, int(cy) + ri + 1)
    x0, x1 = max(0, int(cx) - ri), min(cols, int(cx) + ri + 1)
    if y0 >= y1 or x0 >= x1:
        return
    yy, xx = np.mgrid[y0:y1, x0:x1]
    inside = (yy - cy) ** 2 + (xx - cx) ** 2 <= r * r
    m[y0:y1, x0:x1][inside] = val


def disc_pairs_mask(rows: int = 4096, cols: int = 4096, seed: int = 0x5EED0002,
                    n_pairs: int | None = None, n_single: int | None = None) -> np.ndarray:
    """uint8 0/255 mask: overlapping disc pairs (radii 6-14, centre distance
    0.6-1.4 x the radius sum) plus isolated discs."""
    scale = rows * cols / float(4096 * 4096)
    if n_pairs is None:
        n_pairs = int(round(3000 * scale))
    if n_single is None:
        n_single = int(round(2000 * scale))
    m = np.zeros((rows, cols), dtype=np.uint8)
    sc = _Scalars(seed, 300)
    for _ in range(n_pairs):
        cy, cx = sc.u() * rows, sc.u() * cols
        r1, r2 = 6.0 + 8.0 * sc.u(), 6.0 + 8.0 * sc.u()
        ang = 2.0 * math.pi * sc.u()
        d = (r1 + r2) * (0.6 + 0.8 * sc.u())
        _fill_disc(m, cy, cx, r1)
        _fill_disc(m, cy + d * math.sin(ang), cx + d * math.cos(ang), r2)
    for _ in range(n_single):
        cy, cx, r = sc.u() * rows, sc.u() * cols, 6.0 + 8.0 * sc.u()
        _fill_disc(m, cy, cx, r)
    return m


def colorize_mask(mask: np.ndarray, seed: int) -> np.ndarray:
    """BGR image for watershed inputs: an H&E tile of the same shape masked by
    `mask` (0 outside)."""
    img = he_tile(mask.shape[0], mask.shape[1], seed)
    img[mask == 0] = 0
    return img


def tile_hash(a: np.ndarray) -> str:
    """Content hash recorded next to generated inputs."""
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:16]
