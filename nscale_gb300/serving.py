"""Many tiles on one GPU: the batched form and the in-process server.

The reference segments one tile per process and farms tiles over MPI
(nu-segment.cpp:274-430).  `TilePool` keeps several tiles in flight on one
GPU (nsg_pool / nsg_segment_nuclei_batch: one host thread, context and CUDA
stream per worker, all inside libnsg.so); `TileServer` takes tiles one at a
time from host memory with a bounded queue and a memory budget
(nsg_server_*), for serving-style arrivals.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib


def _check(rc: int, what: str) -> None:
    if rc < 0:
        raise _lib.NsgError(rc, what)


def _feature_array(L, ptr, n: int) -> np.ndarray | None:
    if not ptr:
        return None
    arr = np.ctypeslib.as_array(ptr, shape=(5 * n,)).copy().reshape(n, 5) if n else np.zeros((0, 5), np.float32)
    L.nsg_free(ptr)
    return arr


def _bbox_array(L, ptr, n: int) -> np.ndarray:
    if not ptr:
        return np.zeros((5, 0), np.int32)
    arr = np.ctypeslib.as_array(ptr, shape=(5 * n,)).copy().reshape(5, n) if n else np.zeros((5, 0), np.int32)
    L.nsg_free(ptr)
    return arr


class TilePool:
    """`workers` tiles in flight on `device`, each worker a context sized for
    max_rows x max_cols (nsg_pool_create).  32 workers is the measured best for
    4096 x 4096 tiles on GB300 (4 GiB of device memory each);
    `nscale_gb300.autotune` picks the count and launch shapes for a batch."""

    def __init__(self, max_rows: int, max_cols: int, workers: int = 8, device: int = 0):
        self.L = _lib.load()
        self.h = C.c_void_p()
        _check(self.L.nsg_pool_create(C.byref(self.h), max_rows, max_cols, workers, device), "nsg_pool_create")
        self.max_rows, self.max_cols, self.device = max_rows, max_cols, device

    @property
    def workers(self) -> int:
        return self.L.nsg_pool_workers(self.h)

    def set_tuning(self, recon_max_ctas: int = 0, bfs_max_cluster: int = 0, recon_wl_phases: int = -1) -> None:
        """nsg_pool_set_tuning: launch shapes of every worker and the
        reconstruction's scan-to-queue switchover (results do not change)."""
        t = _lib.Tuning(recon_max_ctas, bfs_max_cluster, recon_wl_phases)
        _check(self.L.nsg_pool_set_tuning(self.h, C.byref(t)), "nsg_pool_set_tuning")

    def set_timing(self, on: bool = True) -> None:
        """nsg_pool_set_timing: per-stage CUDA-event timing on every worker (resets the sums)."""
        _check(self.L.nsg_pool_set_timing(self.h, 1 if on else 0), "nsg_pool_set_timing")

    def stage_times(self) -> tuple[dict, int]:
        """nsg_pool_stage_times: ({stage name: ms summed over workers}, tiles timed)."""
        ms = (C.c_double * 32)()
        calls = C.c_longlong(0)
        n = self.L.nsg_pool_stage_times(self.h, ms, 32, C.byref(calls))
        _check(n, "nsg_pool_stage_times")
        return {self.L.nsg_stage_name(i).decode(): ms[i] for i in range(n)}, calls.value

    def run(self, tiles: "C.Array", params: _lib.SegParams | None = None, host: bool = False) -> int:
        """nsg_segment_nuclei_batch over a prepared ctypes array of Tile."""
        rc = self.L.nsg_segment_nuclei_batch(self.h, tiles, len(tiles), C.byref(params) if params else None,
                                             _lib.TILE_HOST if host else 0)
        _check(rc, "nsg_segment_nuclei_batch")
        return rc

    def segment(self, images, params: _lib.SegParams | None = None, want_bbox: bool = True,
                want_features: bool = False):
        """segmentNuclei on every image (BGR uint8 (rows, cols, 3) CUDA tensors,
        or host numpy arrays).  Returns [(status, labels, compcount, bbox)], with
        a fifth element, the (n, 5) per-nucleus features of the H channel
        (area, perimeter, mean H, std H, mean gradient), when want_features."""
        host = not isinstance(images[0], torch.Tensor) or not images[0].is_cuda
        arr = (_lib.Tile * len(images))()
        keep = []
        for i, im in enumerate(images):
            if host:
                im = np.ascontiguousarray(im, dtype=np.uint8)
                lab = np.empty(im.shape[:2], np.int32)
                bgr_p, lab_p = im.ctypes.data, lab.ctypes.data
            else:
                im = im.contiguous()
                lab = torch.empty(im.shape[:2], dtype=torch.int32, device=im.device)
                bgr_p, lab_p = im.data_ptr(), lab.data_ptr()
            keep.append((im, lab))
            arr[i].bgr, arr[i].rows, arr[i].cols = bgr_p, im.shape[0], im.shape[1]
            arr[i].row_stride_bytes = 0
            arr[i].labels, arr[i].mask, arr[i].want_bbox = lab_p, None, 1 if want_bbox else 0
            arr[i].want_features = 1 if want_features else 0
        self.run(arr, params, host)
        out = []
        for i, (im, lab) in enumerate(keep):
            t = arr[i]
            r = (t.status, lab, t.compcount, _bbox_array(self.L, t.bbox, t.compcount))
            if want_features:
                r = r + (_feature_array(self.L, t.features, t.compcount),)
            out.append(r)
        return out

    def close(self) -> None:
        if self.h:
            self.L.nsg_pool_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass


class TileServer:
    """Serving form (nsg_server_*): submit host tiles one at a time, poll results.

    Workers = memory_budget_bytes // nsg_pool_context_bytes(max_rows, max_cols)
    (at most 64); submit raises NSG_ERR_QUEUE_FULL when `queue_cap` tiles wait."""

    def __init__(self, max_rows: int, max_cols: int, memory_budget_bytes: int, queue_cap: int = 64,
                 device: int = 0, classes: list[tuple[int, int]] | None = None,
                 weights: list[float] | None = None):
        """classes: [(rows, cols), ...] size classes of the workers' contexts
        (nsg_server_create_classes: the budget is split in proportion to
        weight x context bytes); None = every worker max_rows x max_cols."""
        self.L = _lib.load()
        self.h = C.c_void_p()
        if classes:
            n = len(classes)
            rows = (C.c_int * n)(*[r for r, _ in classes])
            cols = (C.c_int * n)(*[c for _, c in classes])
            w = (C.c_double * n)(*(weights or [1.0] * n))
            _check(self.L.nsg_server_create_classes(C.byref(self.h), rows, cols, w, n, memory_budget_bytes,
                                                    queue_cap, device), "nsg_server_create_classes")
        else:
            _check(self.L.nsg_server_create(C.byref(self.h), max_rows, max_cols, memory_budget_bytes, queue_cap,
                                            device), "nsg_server_create")
        self.classes = list(classes) if classes else [(max_rows, max_cols)]
        self._live = {}

    def class_workers(self) -> dict[tuple[int, int], int]:
        return {c: self.L.nsg_server_class_workers(self.h, c[0], c[1]) for c in self.classes}

    @property
    def workers(self) -> int:
        return self.L.nsg_server_workers(self.h)

    def submit(self, image: np.ndarray, labels: np.ndarray | None = None, want_bbox: bool = False,
               params: _lib.SegParams | None = None, want_features: bool = False) -> int:
        """Queue one host BGR tile; `labels` (int32, rows x cols) receives the
        label image.  Both arrays stay referenced until the result is polled."""
        image = np.ascontiguousarray(image, dtype=np.uint8)
        t = _lib.Tile()
        t.bgr, t.rows, t.cols, t.row_stride_bytes = image.ctypes.data, image.shape[0], image.shape[1], 0
        t.labels = labels.ctypes.data if labels is not None else None
        t.mask, t.want_bbox, t.want_features = None, 1 if want_bbox else 0, 1 if want_features else 0
        ticket = C.c_longlong(-1)
        _check(self.L.nsg_server_submit(self.h, C.byref(t), C.byref(params) if params else None, C.byref(ticket)),
               "nsg_server_submit")  # NSG_ERR_QUEUE_FULL when queue_cap tiles wait: the caller sheds
        self._live[ticket.value] = (image, labels)
        return ticket.value

    def poll(self, max_results: int = 64, wait_ms: int = 0) -> list[dict]:
        buf = (_lib.Result * max_results)()
        n = self.L.nsg_server_poll(self.h, buf, max_results, wait_ms)
        _check(n, "nsg_server_poll")
        out = []
        for i in range(n):
            r = buf[i]
            _, labels = self._live.pop(r.ticket, (None, None))
            out.append({"ticket": r.ticket, "status": r.status, "compcount": r.compcount,
                        "bbox": _bbox_array(self.L, r.bbox, r.compcount), "labels": labels,
                        "features": _feature_array(self.L, r.features, r.compcount),
                        "latency_ms": r.latency_ms})
        return out

    def close(self) -> None:
        if self.h:
            self.L.nsg_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass
