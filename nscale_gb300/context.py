"""Workspace context: one nsg_context (device arena) per device, grown on demand.

All device memory the library works in is allocated here once; the
operations below allocate nothing else on the device except their outputs.
"""
from __future__ import annotations

import ctypes as C
import threading

import torch

from . import _lib


class Context:
    def __init__(self, max_rows: int, max_cols: int, device: int = 0):
        self.L = _lib.load()
        self.device = device
        self.max_rows, self.max_cols = max_rows, max_cols
        h = C.c_void_p()
        with torch.cuda.device(device):
            rc = self.L.nsg_context_create(C.byref(h), max_rows, max_cols, device)
        if rc != 0:
            raise _lib.NsgError(rc, "nsg_context_create failed")
        self.h = h

    def fits(self, rows: int, cols: int) -> bool:
        return rows * cols <= self.max_rows * self.max_cols and \
            (rows + 2) * (cols + 2) <= (self.max_rows + 2) * (self.max_cols + 2)

    def last_error(self) -> str:
        return self.L.nsg_context_last_error(self.h).decode()

    def check(self, rc: int, ok=(0,)) -> int:
        if rc not in ok and rc < 0:
            raise _lib.NsgError(rc, self.last_error())
        return rc

    def bytes(self) -> int:
        return int(self.L.nsg_context_bytes(self.h))

    def set_spin_budget(self, iters: int) -> None:
        self.check(self.L.nsg_context_set_spin_budget(self.h, iters))

    def close(self) -> None:
        if getattr(self, "h", None):
            self.L.nsg_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_lock = threading.Lock()
_default: dict[int, Context] = {}


def get_context(rows: int, cols: int, device: int | None = None) -> Context:
    """The per-device default context, recreated larger when an image does
    not fit."""
    dev = torch.cuda.current_device() if device is None else device
    with _lock:
        ctx = _default.get(dev)
        if ctx is None or not ctx.fits(rows, cols):
            r = max(rows, ctx.max_rows if ctx else 0)
            c = max(cols, ctx.max_cols if ctx else 0)
            if ctx is not None:
                torch.cuda.synchronize(dev)
                ctx.close()
            ctx = Context(r, c, dev)
            _default[dev] = ctx
        return ctx


def stream_handle(stream: torch.cuda.Stream | None = None) -> C.c_void_p:
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def ptr(t: torch.Tensor) -> C.c_void_p:
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return C.c_void_p(t.data_ptr())
