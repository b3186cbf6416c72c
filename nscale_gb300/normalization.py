"""nscale::Normalization on the GPU (src/normalization/Normalization.h:30-47),
through libnsg.so: colour normalisation of a BGR tile towards a target's lab
statistics, the pre-pass the reference's test driver runs before
segmentNuclei (nu-segmentTest.cpp:200)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from .context import get_context, ptr, stream_handle


def _bgr(img: torch.Tensor) -> torch.Tensor:
    if img.dim() != 3 or img.shape[2] != 3 or img.dtype != torch.uint8 or not img.is_cuda:
        raise ValueError("expected a (rows, cols, 3) uint8 BGR CUDA tensor")
    return img.contiguous()


class Normalization:
    @staticmethod
    def targetParameters(img: torch.Tensor) -> tuple[np.ndarray, np.ndarray]:
        """Normalization.cpp:520-577: (targetMean[3], targetStd[3]) float32."""
        img = _bgr(img)
        rows, cols = img.shape[:2]
        ctx = get_context(rows, cols)
        m, s = (C.c_float * 3)(), (C.c_float * 3)()
        ctx.check(ctx.L.nsg_color_target_parameters(ctx.h, ptr(img), rows, cols, 0, m, s, stream_handle()))
        return np.array(m[:], np.float32), np.array(s[:], np.float32)

    @staticmethod
    def normalization(img: torch.Tensor, targetMean, targetStd) -> torch.Tensor:
        """Normalization.cpp:487-517: the tile moved to the target's lab
        mean / std (foreground only), as uint8 BGR."""
        img = _bgr(img)
        rows, cols = img.shape[:2]
        ctx = get_context(rows, cols)
        m = (C.c_float * 3)(*[float(v) for v in targetMean])
        s = (C.c_float * 3)(*[float(v) for v in targetStd])
        out = torch.empty_like(img)
        ctx.check(ctx.L.nsg_color_normalization(ctx.h, ptr(img), rows, cols, 0, m, s, ptr(out), stream_handle()))
        return out
