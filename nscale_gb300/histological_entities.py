"""nscale::HistologicalEntities (HistologicalEntities.h:29-68) and
nscale::PixelOperations::invert on the GPU, through libnsg.so."""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .context import Context, get_context, ptr, stream_handle


class HistologicalEntities:
    BACKGROUND = 1
    BACKGROUND_LIKELY = 2
    NO_CANDIDATES_LEFT = 3
    INVALID_IMAGE = -1
    SUCCESS = 0
    CONTINUE = 4
    RUNTIME_FAILED = -2

    @staticmethod
    def getBackground(img: torch.Tensor, blue: int = 220, green: int = 220, red: int = 220):
        """HistologicalEntities.cpp:84-109; returns (mask, count)."""
        img = _bgr(img)
        rows, cols = img.shape[:2]
        ctx = get_context(rows, cols)
        out = torch.empty((rows, cols), dtype=torch.uint8, device=img.device)
        cnt = C.c_int64(0)
        ctx.check(ctx.L.nsg_get_background(ctx.h, ptr(img), rows, cols, blue, green, red, ptr(out), C.byref(cnt),
                                           stream_handle()))
        return out, cnt.value

    @staticmethod
    def getRBC(img: torch.Tensor, T1: float = 5.0, T2: float = 4.0) -> torch.Tensor:
        """HistologicalEntities.cpp:24-82."""
        img = _bgr(img)
        rows, cols = img.shape[:2]
        ctx = get_context(rows, cols)
        out = torch.empty((rows, cols), dtype=torch.uint8, device=img.device)
        ctx.check(ctx.L.nsg_get_rbc(ctx.h, ptr(img), rows, cols, T1, T2, ptr(out), stream_handle()))
        return out

    @staticmethod
    def segmentNuclei(img, blue=220, green=220, red=220, T1=5.0, T2=4.0, G1=80, minSize=11, maxSize=1000, G2=45,
                      minSizePl=30, minSizeSeg=21, maxSizeSeg=1000, fillHolesConnectivity=4, reconConnectivity=8,
                      watershedConnectivity=8, *, return_mask: bool = False, context: Context | None = None):
        """HistologicalEntities.cpp:473-598.

        `img` is a BGR uint8 (rows, cols, 3) CUDA tensor (or a numpy array,
        copied to the device).  Returns (status, labels int32 CUDA tensor
        [bg -1, label = min raster index], compcount, bbox int32 (5, n) numpy
        array [label, minx, maxx, miny, maxy]) and, with return_mask=True, the
        filled uint8 mask as a fifth element.
        """
        if isinstance(img, np.ndarray):
            img = torch.from_numpy(np.ascontiguousarray(img)).cuda()
        img = _bgr(img)
        rows, cols = img.shape[:2]
        ctx = context if context is not None else get_context(rows, cols)
        p = _lib.SegParams(blue=blue, green=green, red=red, T1=T1, T2=T2, G1=G1, minSize=minSize, maxSize=maxSize,
                           G2=G2, minSizePl=minSizePl, minSizeSeg=minSizeSeg, maxSizeSeg=maxSizeSeg,
                           fillHolesConnectivity=fillHolesConnectivity, reconConnectivity=reconConnectivity,
                           watershedConnectivity=watershedConnectivity)
        labels = torch.empty((rows, cols), dtype=torch.int32, device=img.device)
        mask = torch.empty((rows, cols), dtype=torch.uint8, device=img.device) if return_mask else None
        cc = C.c_int(0)
        bb = C.POINTER(C.c_int32)()
        st = ctx.L.nsg_segment_nuclei(ctx.h, ptr(img), rows, cols, cols * 3, C.byref(p), ptr(labels),
                                      ptr(mask) if mask is not None else None, C.byref(cc), C.byref(bb),
                                      stream_handle())
        ctx.check(st)
        n = cc.value
        if bb:
            bbox = np.ctypeslib.as_array(bb, shape=(5 * n,)).copy().reshape(5, n) if n else np.zeros((5, 0), np.int32)
            ctx.L.nsg_free(bb)
        else:
            bbox = np.zeros((5, 0), np.int32)
        if return_mask:
            return st, labels, n, bbox, mask
        return st, labels, n, bbox


class PixelOperations:
    @staticmethod
    def ComputeInverseStainMatrix(M=None, b=None) -> np.ndarray:
        """PixelOperations.cpp:94-156: float32 (2, 3), columns R, G, B.  None =
        the feature pipeline's stains (nu-features.cpp:691-692)."""
        L = _lib.load()
        q = (C.c_float * 6)()
        Mp = np.ascontiguousarray(M, np.float64).ravel() if M is not None else None
        bp = np.ascontiguousarray(b, np.uint8).ravel() if b is not None else None
        rc = L.nsg_stain_matrix(Mp.ctypes.data if Mp is not None else None,
                                bp.ctypes.data if bp is not None else None, q)
        if rc < 0:
            raise _lib.NsgError(rc, "stain matrix")
        return np.array(q[:], np.float32).reshape(2, 3)

    @staticmethod
    def ColorDeconv(image, Q=None):
        """PixelOperations::ColorDeconv(image, Q, lut, H, E, BGR2RGB = true)
        (PixelOperations.cpp:170-274): uint8 H and E CUDA tensors."""
        if isinstance(image, np.ndarray):
            image = torch.from_numpy(np.ascontiguousarray(image)).cuda()
        image = _bgr(image)
        rows, cols = image.shape[:2]
        q = np.ascontiguousarray(PixelOperations.ComputeInverseStainMatrix() if Q is None else Q, np.float32)
        ctx = get_context(rows, cols)
        H = torch.empty((rows, cols), dtype=torch.uint8, device=image.device)
        E = torch.empty_like(H)
        qp = q.ravel().ctypes.data_as(C.POINTER(C.c_float))
        ctx.check(ctx.L.nsg_color_deconv(ctx.h, ptr(image), rows, cols, cols * 3, qp, ptr(H), ptr(E),
                                         stream_handle()))
        return H, E

    @staticmethod
    def invert(img: torch.Tensor) -> torch.Tensor:
        """PixelOperations::invert<T> (PixelOperations.cpp:22-43): uint8
        255 - x, int32 ~x + 1, float32 -x."""
        fn = {torch.uint8: "nsg_invert_u8", torch.int32: "nsg_invert_i32", torch.float32: "nsg_invert_f32"}
        if img.dtype not in fn:
            raise TypeError("invert takes uint8, int32 or float32 (the reference's instantiations on the path)")
        img = img.contiguous()
        ctx = get_context(1, 1)
        out = torch.empty_like(img)
        ctx.check(getattr(ctx.L, fn[img.dtype])(ctx.h, ptr(img), ptr(out), img.numel(), stream_handle()))
        return out


def _bgr(img: torch.Tensor) -> torch.Tensor:
    if img.dim() != 3 or img.shape[2] != 3 or img.dtype != torch.uint8:
        raise ValueError("expected a (rows, cols, 3) uint8 BGR image")
    if not img.is_cuda:
        raise ValueError("expected a CUDA tensor")
    return img.contiguous()
