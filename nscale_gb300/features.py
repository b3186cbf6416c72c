"""Per-nucleus features of the serving output, mirroring nscale's feature
classes (src/features): Operators::gradient and the ObjFeatures area,
perimeter and histogram statistics, over torch CUDA tensors."""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .context import get_context, ptr, stream_handle

N_FEATURES = 5  # area, perimeter, mean gray, std gray, mean gradient
FEATURE_NAMES = ("area", "perimeter", "mean_intensity", "std_intensity", "mean_gradient")


class Operators:
    @staticmethod
    def gradient(img: torch.Tensor) -> torch.Tensor:
        """Operators.cpp:568-640: uint8 gradient magnitude."""
        img = img.contiguous()
        rows, cols = img.shape
        ctx = get_context(rows, cols)
        out = torch.empty_like(img)
        ctx.check(ctx.L.nsg_gradient_u8(ctx.h, ptr(img), ptr(out), rows, cols, stream_handle()))
        return out


class ObjFeatures:
    @staticmethod
    def nucleusFeatures(labels: torch.Tensor, gray: torch.Tensor, capacity: int | None = None) -> torch.Tensor:
        """(n, 5) float32 CUDA tensor, one row per component in bounding-box
        order: area (ObjFeatures.cpp:15-43), perimeter (:143-270), mean and std
        of `gray` and mean of its gradient (:342-418)."""
        labels, gray = labels.contiguous(), gray.contiguous()
        rows, cols = labels.shape
        cap = capacity if capacity is not None else max(1, rows * cols // 4)
        out = torch.empty((cap, N_FEATURES), dtype=torch.float32, device=labels.device)
        ctx = get_context(rows, cols)
        n = C.c_int(0)
        ctx.check(ctx.L.nsg_nucleus_features(ctx.h, ptr(labels), ptr(gray), rows, cols, ptr(out), cap, C.byref(n),
                                             stream_handle()))
        return out[: n.value]
