"""On-device (torch) version of synth.he_tile for large workloads.

Same recipe and parameters as nscale_gb300.synth.he_tile (background RGB
uniform 215-240, value-noise eosin stroma around (230,170,200) +-25,
hematoxylin ellipses with semi-axes 4-12 px, 30 % in overlapping pairs, colour
(70,40,120) +-15, red-blood-cell discs r 3-5 of (200,40,40), additive
Gaussian-like noise sigma 8, BGR interleaved), vectorised so a 4096x4096 tile
takes milliseconds on the GPU.  The random streams are the same counter hash,
but float rounding on the device may differ from numpy in the last bit, so
tiles are statistically identical, not byte-identical, to synth.he_tile.
Used for throughput workloads; parity tests use synth.he_tile.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import synth

_MASK64 = (1 << 64) - 1


def _i64(v: int) -> int:
    v &= _MASK64
    return v - (1 << 64) if v >= 1 << 63 else v


def _lsr(x: torch.Tensor, k: int) -> torch.Tensor:
    return (x >> k) & ((1 << (64 - k)) - 1)


def _splitmix(x: torch.Tensor) -> torch.Tensor:
    z = x + _i64(0x9E3779B97F4A7C15)
    z = (z ^ _lsr(z, 30)) * _i64(0xBF58476D1CE4E5B9)
    z = (z ^ _lsr(z, 27)) * _i64(0x94D049BB133111EB)
    return z ^ _lsr(z, 31)


def _hash(seed: int, stream: int, idx: torch.Tensor) -> torch.Tensor:
    key = int(synth._key(seed, stream))
    return _splitmix(idx * _i64(0xD1B54A32D192ED03) + _i64(key))


def _uniform(seed: int, stream: int, idx: torch.Tensor) -> torch.Tensor:
    return _lsr(_hash(seed, stream, idx), 11).to(torch.float64) * (1.0 / 9007199254740992.0)


def _randint(seed: int, stream: int, idx: torch.Tensor, lo: int, hi: int) -> torch.Tensor:
    # unsigned 64-bit hash modulo span, as numpy computes it on uint64
    h = _hash(seed, stream, idx)
    span = hi - lo + 1
    hi32, lo32 = _lsr(h, 32), h & 0xFFFFFFFF
    r = (torch.remainder(hi32, span) * ((1 << 32) % span) + lo32) % span
    return r + lo


def _value_noise(rows, cols, seed, stream, cell, device):
    gr, gc = rows // cell + 2, cols // cell + 2
    lat = _uniform(seed, stream, torch.arange(gr * gc, device=device, dtype=torch.int64)).view(gr, gc)
    y = torch.arange(rows, device=device, dtype=torch.float64) / cell
    x = torch.arange(cols, device=device, dtype=torch.float64) / cell
    y0, x0 = y.floor().long(), x.floor().long()
    fy, fx = y - y0, x - x0
    sy, sx = fy * fy * (3 - 2 * fy), fx * fx * (3 - 2 * fx)
    a = lat[y0][:, x0]
    b = lat[y0][:, x0 + 1]
    c = lat[y0 + 1][:, x0]
    d = lat[y0 + 1][:, x0 + 1]
    top = a + (b - a) * sx[None, :]
    bot = c + (d - c) * sx[None, :]
    return top + (bot - top) * sy[:, None]


def _objects(rows, cols, seed, n_nuclei, n_rbc):
    """Object list with the same draws as synth.he_tile (numpy, small)."""
    sc = synth._Scalars(seed, 100)
    n_pairs = int(round(n_nuclei * 0.15))
    n_single = max(0, n_nuclei - 2 * n_pairs)
    objs = []
    for _ in range(n_single + n_pairs):
        cy, cx = sc.u() * rows, sc.u() * cols
        a, b = 4.0 + 8.0 * sc.u(), 4.0 + 8.0 * sc.u()
        objs.append([cy, cx, a, b, math.pi * sc.u()])
    for k in range(n_pairs):
        cy, cx, a, b, _ = objs[n_single + k]
        a2, b2 = 4.0 + 8.0 * sc.u(), 4.0 + 8.0 * sc.u()
        ang = 2.0 * math.pi * sc.u()
        dist = (0.5 * (a + b) + 0.5 * (a2 + b2)) * (0.45 + 0.35 * sc.u())
        objs.append([cy + dist * math.sin(ang), cx + dist * math.cos(ang), a2, b2, math.pi * sc.u()])
    cols_ = [(70 + sc.ri(-15, 15), 40 + sc.ri(-15, 15), 120 + sc.ri(-15, 15)) for _ in objs]
    for _ in range(n_rbc):
        cy, cx = sc.u() * rows, sc.u() * cols
        r = 3.0 + 2.0 * sc.u()
        objs.append([cy, cx, r, r, 0.0])
        cols_.append((200, 40, 40))
    return np.array(objs, np.float64).reshape(-1, 5), np.array(cols_, np.float64).reshape(-1, 3)


def he_tile(rows: int, cols: int, seed: int, device="cuda", n_nuclei=None, n_rbc=None) -> torch.Tensor:
    """(rows, cols, 3) uint8 BGR tile on `device`."""
    scale = rows * cols / float(4096 * 4096)
    n_nuclei = int(round(6000 * scale)) if n_nuclei is None else n_nuclei
    n_rbc = int(round(200 * scale)) if n_rbc is None else n_rbc
    dev = torch.device(device)
    idx = torch.arange(rows * cols, device=dev, dtype=torch.int64).view(rows, cols)
    rgb = torch.empty((rows, cols, 3), device=dev, dtype=torch.float64)
    for ch in range(3):
        rgb[..., ch] = _randint(seed, 1 + ch, idx, 215, 240).to(torch.float64)
    v = 0.65 * _value_noise(rows, cols, seed, 10, 96, dev) + 0.35 * _value_noise(rows, cols, seed, 11, 24, dev)
    s = torch.clamp((v - 0.5) * 3.0, 0.0, 1.0)
    base = (230.0, 170.0, 200.0)
    for ch in range(3):
        mod = 25.0 * (2.0 * _value_noise(rows, cols, seed, 12 + ch, 32, dev) - 1.0)
        rgb[..., ch] = rgb[..., ch] * (1.0 - s) + (base[ch] + mod) * s
    del v, s
    objs, colors = _objects(rows, cols, seed, n_nuclei, n_rbc)
    if len(objs):
        o = torch.from_numpy(objs).to(dev)
        cl = torch.from_numpy(colors).to(dev)
        R = 14
        off = torch.arange(-R, R + 1, device=dev, dtype=torch.float64)
        cy, cx = o[:, 0:1, None], o[:, 1:2, None]
        yy = (cy.floor() + off[None, :, None])  # (n, 2R+1, 1)
        xx = (cx.floor() + off[None, None, :])  # (n, 1, 2R+1)
        dy, dx = yy - cy, xx - cx
        c, s_ = torch.cos(o[:, 4])[:, None, None], torch.sin(o[:, 4])[:, None, None]
        u = (dx * c + dy * s_) / o[:, 2, None, None]
        w = (-dx * s_ + dy * c) / o[:, 3, None, None]
        inside = (u * u + w * w) <= 1.0
        yi = yy.expand_as(inside).long()
        xi = xx.expand_as(inside).long()
        ok = inside & (yi >= 0) & (yi < rows) & (xi >= 0) & (xi < cols)
        obj_id = torch.arange(len(objs), device=dev).view(-1, 1, 1).expand_as(inside)
        lin = (yi * cols + xi)[ok]
        top = torch.full((rows * cols,), -1, device=dev, dtype=torch.int64)
        top.scatter_reduce_(0, lin, obj_id[ok], reduce="amax")
        hit = top >= 0
        flat = rgb.view(-1, 3)
        flat[hit] = cl[top[hit]]
    for ch in range(3):
        h = _hash(seed, 20 + ch, idx)
        acc = torch.zeros((rows, cols), device=dev, dtype=torch.float64)
        for k in range(4):
            acc += (_lsr(h, 16 * k) & 0xFFFF).to(torch.float64)
        rgb[..., ch] += (acc / 65536.0 - 2.0) * (8.0 * math.sqrt(3.0))
    out = torch.clamp(torch.floor(rgb + 0.5), 0, 255).to(torch.uint8)
    return out.flip(-1).contiguous()


def batch_shapes(n: int = 256, seed: int = 0x5EED0003) -> list[tuple[int, int]]:
    """Uneven tile shapes of a slide batch: squares 512-4096 px plus ragged
    slide-edge tiles (4096 x r and r x 4096)."""
    sc = synth._Scalars(seed, 400)
    shapes = []
    n_ragged = n // 5
    for _ in range(n - n_ragged):
        side = 512 + 256 * sc.ri(0, 14)
        shapes.append((side, side))
    for k in range(n_ragged):
        r = sc.ri(200, 4095)
        shapes.append((4096, r) if k % 2 == 0 else (r, 4096))
    return shapes
