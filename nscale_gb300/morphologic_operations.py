"""nscale::MorphologicOperations (MorphologicOperations.h:29-212) on the GPU.

Each function keeps the reference's name, argument order and meaning, takes
CUDA tensors (uint8 / float32 / int32, 2-D, contiguous) and returns new CUDA
tensors.  Every call goes through libnsg.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import torch

from .context import get_context, ptr, stream_handle

# MATLAB strel('disk', 10) (HistologicalEntities.cpp:169-188) by chord half-width
_DISK19_HW = (5, 6, 7, 8, 9, 9, 9, 9, 9, 9, 9, 9, 9, 9, 9, 8, 7, 6, 5)


def disk19() -> torch.Tensor:
    se = torch.zeros(19, 19, dtype=torch.uint8)
    for r, w in enumerate(_DISK19_HW):
        se[r, 9 - w:9 + w + 1] = 1
    return se


def cross3() -> torch.Tensor:
    """getStructuringElement(MORPH_ELLIPSE, Size(3,3)) (HistologicalEntities.cpp:498)."""
    return torch.tensor([[0, 1, 0], [1, 1, 1], [0, 1, 0]], dtype=torch.uint8)


def _2d(t: torch.Tensor, dtype) -> torch.Tensor:
    if t.dim() != 2:
        raise ValueError("expected a 2-D image")
    if t.dtype != dtype:
        raise TypeError(f"expected {dtype}, got {t.dtype}")
    return t.contiguous()


def _se_bytes(kernel) -> tuple[C.Array, int]:
    k = torch.as_tensor(kernel).to(torch.uint8).cpu().contiguous()
    if k.dim() != 2 or k.shape[0] != k.shape[1] or k.shape[0] % 2 == 0:
        raise ValueError("structuring element must be square with odd size")
    buf = (C.c_uint8 * k.numel()).from_buffer_copy(bytes(k.numpy().tobytes()))
    return buf, int(k.shape[0])


def imreconstruct(seeds: torch.Tensor, image: torch.Tensor, connectivity: int = 4) -> torch.Tensor:
    """MorphologicOperations.cpp:1731-1903 (uint8 or float32)."""
    if image.dtype == torch.float32:
        seeds, image = _2d(seeds, torch.float32), _2d(image, torch.float32)
        fn = "nsg_imreconstruct_f32"
    else:
        seeds, image = _2d(seeds, torch.uint8), _2d(image, torch.uint8)
        fn = "nsg_imreconstruct_u8"
    rows, cols = image.shape
    ctx = get_context(rows, cols)
    out = torch.empty_like(image)
    ctx.check(getattr(ctx.L, fn)(ctx.h, ptr(seeds), ptr(image), ptr(out), rows, cols, connectivity,
                                 stream_handle()))
    return out


def imreconstructBinary(seeds: torch.Tensor, binaryImage: torch.Tensor, connectivity: int = 4) -> torch.Tensor:
    """MorphologicOperations.cpp:2769-2909."""
    seeds, binaryImage = _2d(seeds, torch.uint8), _2d(binaryImage, torch.uint8)
    rows, cols = binaryImage.shape
    ctx = get_context(rows, cols)
    out = torch.empty_like(binaryImage)
    ctx.check(ctx.L.nsg_imreconstruct_binary_u8(ctx.h, ptr(seeds), ptr(binaryImage), ptr(out), rows, cols,
                                                connectivity, stream_handle()))
    return out


def imfillHoles(image: torch.Tensor, binary: bool = True, connectivity: int = 4) -> torch.Tensor:
    """MorphologicOperations.cpp:2940-3006 (the binary form used on the path)."""
    if not binary:
        raise NotImplementedError("only the binary imfillHoles is on the segmentNuclei path")
    image = _2d(image, torch.uint8)
    rows, cols = image.shape
    ctx = get_context(rows, cols)
    out = torch.empty_like(image)
    ctx.check(ctx.L.nsg_imfill_holes_u8(ctx.h, ptr(image), ptr(out), rows, cols, connectivity, stream_handle()))
    return out


def bwselect(binaryImage: torch.Tensor, seeds: torch.Tensor, connectivity: int = 8) -> torch.Tensor:
    """MorphologicOperations.cpp:3010-3031."""
    binaryImage, seeds = _2d(binaryImage, torch.uint8), _2d(seeds, torch.uint8)
    rows, cols = binaryImage.shape
    ctx = get_context(rows, cols)
    out = torch.empty_like(binaryImage)
    ctx.check(ctx.L.nsg_bwselect_u8(ctx.h, ptr(binaryImage), ptr(seeds), ptr(out), rows, cols, connectivity,
                                    stream_handle()))
    return out


def bwlabel2(binaryImage: torch.Tensor, connectivity: int = 8, relab: bool = True) -> torch.Tensor:
    """MorphologicOperations.cpp:3092-3117: int32, background -1, label = min
    raster index (the reference's relabel step is disabled)."""
    del relab
    binaryImage = _2d(binaryImage, torch.uint8)
    rows, cols = binaryImage.shape
    ctx = get_context(rows, cols)
    out = torch.empty((rows, cols), dtype=torch.int32, device=binaryImage.device)
    ctx.check(ctx.L.nsg_bwlabel(ctx.h, ptr(binaryImage), ptr(out), rows, cols, connectivity, stream_handle()))
    return out


def bwareaopen2(image: torch.Tensor, labeled: bool = False, flatten: bool = True, minSize: int = 11,
                maxSize: int = 1000, connectivity: int = 8) -> tuple[torch.Tensor, int]:
    """MorphologicOperations.cpp:3281-3314 (labeled=False, flatten=True):
    returns (uint8 mask, count)."""
    if labeled or not flatten:
        raise NotImplementedError("only bwareaopen2(img, false, true, ...) is on the segmentNuclei path")
    image = _2d(image, torch.uint8)
    rows, cols = image.shape
    ctx = get_context(rows, cols)
    out = torch.empty_like(image)
    cnt = C.c_int(0)
    ctx.check(ctx.L.nsg_bwareaopen(ctx.h, ptr(image), ptr(out), rows, cols, minSize, maxSize, connectivity,
                                   C.byref(cnt), stream_handle()))
    return out, cnt.value


def distTransform(mask: torch.Tensor) -> torch.Tensor:
    """cv::distanceTransform(mask, dist, CV_DIST_L2, CV_DIST_MASK_PRECISE) as
    HistologicalEntities.cpp:359 calls it."""
    mask = _2d(mask, torch.uint8)
    rows, cols = mask.shape
    ctx = get_context(rows, cols)
    out = torch.empty((rows, cols), dtype=torch.float32, device=mask.device)
    ctx.check(ctx.L.nsg_dist_transform(ctx.h, ptr(mask), ptr(out), rows, cols, stream_handle()))
    return out


def imhmin(image: torch.Tensor, h: float = 1.0, connectivity: int = 8) -> torch.Tensor:
    """MorphologicOperations.cpp:3343-3364 (float32)."""
    image = _2d(image, torch.float32)
    rows, cols = image.shape
    ctx = get_context(rows, cols)
    out = torch.empty_like(image)
    ctx.check(ctx.L.nsg_imhmin_f32(ctx.h, ptr(image), ptr(out), rows, cols, h, connectivity, stream_handle()))
    return out


def localMaxima(image: torch.Tensor, connectivity: int = 8) -> torch.Tensor:
    """MorphologicOperations.cpp:3764-3836 (float32)."""
    image = _2d(image, torch.float32)
    rows, cols = image.shape
    ctx = get_context(rows, cols)
    out = torch.empty((rows, cols), dtype=torch.uint8, device=image.device)
    ctx.check(ctx.L.nsg_local_maxima_f32(ctx.h, ptr(image), ptr(out), rows, cols, connectivity, stream_handle()))
    return out


def localMinima(image: torch.Tensor, connectivity: int = 8) -> torch.Tensor:
    """MorphologicOperations.cpp:3839-3845 (float32)."""
    image = _2d(image, torch.float32)
    rows, cols = image.shape
    ctx = get_context(rows, cols)
    out = torch.empty((rows, cols), dtype=torch.uint8, device=image.device)
    ctx.check(ctx.L.nsg_local_minima_f32(ctx.h, ptr(image), ptr(out), rows, cols, connectivity, stream_handle()))
    return out


def watershed2(origImage: torch.Tensor, image: torch.Tensor, connectivity: int = 8) -> torch.Tensor:
    """MorphologicOperations.cpp:3717-3760: origImage is BGR uint8 (rows, cols, 3)."""
    if origImage.dim() != 3 or origImage.shape[2] != 3 or origImage.dtype != torch.uint8:
        raise ValueError("origImage must be a (rows, cols, 3) uint8 BGR image")
    origImage = origImage.contiguous()
    image = _2d(image, torch.float32)
    rows, cols = image.shape
    ctx = get_context(rows, cols)
    out = torch.empty((rows, cols), dtype=torch.int32, device=image.device)
    ctx.check(ctx.L.nsg_watershed(ctx.h, ptr(origImage), ptr(image), ptr(out), rows, cols, connectivity,
                                  stream_handle()))
    return out


def erode(image: torch.Tensor, kernel) -> torch.Tensor:
    image = _2d(image, torch.uint8)
    rows, cols = image.shape
    ctx = get_context(rows, cols)
    buf, k = _se_bytes(kernel)
    out = torch.empty_like(image)
    ctx.check(ctx.L.nsg_morph_erode_u8(ctx.h, ptr(image), ptr(out), rows, cols, buf, k, stream_handle()))
    return out


def dilate(image: torch.Tensor, kernel) -> torch.Tensor:
    image = _2d(image, torch.uint8)
    rows, cols = image.shape
    ctx = get_context(rows, cols)
    buf, k = _se_bytes(kernel)
    out = torch.empty_like(image)
    ctx.check(ctx.L.nsg_morph_dilate_u8(ctx.h, ptr(image), ptr(out), rows, cols, buf, k, stream_handle()))
    return out


def morphOpen(image: torch.Tensor, kernel) -> torch.Tensor:
    """MorphologicOperations.cpp:3849-3882."""
    image = _2d(image, torch.uint8)
    rows, cols = image.shape
    ctx = get_context(rows, cols)
    buf, k = _se_bytes(kernel)
    out = torch.empty_like(image)
    ctx.check(ctx.L.nsg_morph_open_u8(ctx.h, ptr(image), ptr(out), rows, cols, buf, k, stream_handle()))
    return out
