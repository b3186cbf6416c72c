"""Autotuner for the batched form: measures nsg_segment_nuclei_batch on a
calibration batch for a small grid of launch shapes — tiles in flight
(workers), the reconstruction's persistent grid (as a fraction of the SMs)
and the largest BFS cluster — and returns the fastest.  Results do not
depend on these shapes, only the throughput does.

    python -m nscale_gb300.autotune [--tiles 32] [--out tuning.json]
"""
from __future__ import annotations

import argparse
import itertools
import json
import time

import torch

from . import _lib
from .serving import TilePool

WORKERS = (24, 32, 40)
RECON_FRACTIONS = (1 / 32, 1 / 16, 1 / 8)
BFS_CLUSTERS = (16,)


def _tile_array(tiles):
    arr = (_lib.Tile * len(tiles))()
    labels = []
    for i, t in enumerate(tiles):
        lab = torch.empty(t.shape[0] * t.shape[1], dtype=torch.int32, device=t.device)
        labels.append(lab)
        arr[i].bgr, arr[i].rows, arr[i].cols, arr[i].row_stride_bytes = t.data_ptr(), t.shape[0], t.shape[1], 0
        arr[i].labels, arr[i].mask, arr[i].want_bbox = lab.data_ptr(), None, 0
    return arr, labels


def max_workers(max_rows: int, max_cols: int, device: int = 0, reserve: float = 0.25) -> int:
    """Pool workers whose contexts fit in the device's free memory, keeping
    `reserve` of it (and at least 8 GiB) for the tiles and the caller."""
    free, _total = torch.cuda.mem_get_info(device)
    per = _lib.load().nsg_pool_context_bytes(max_rows, max_cols)
    usable = free - max(int(free * reserve), 8 << 30)
    return max(1, int(usable // per)) if per > 0 else 1


def autotune(tiles, workers=WORKERS, recon_fractions=RECON_FRACTIONS, bfs_clusters=BFS_CLUSTERS, reps: int = 1,
             device: int = 0) -> dict:
    """Best {"workers", "recon_max_ctas", "bfs_max_cluster", "mpx_s"} over the
    grid, and every measurement under "trials"."""
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    maxr = max(t.shape[0] for t in tiles)
    maxc = max(t.shape[1] for t in tiles)
    fit = max_workers(maxr, maxc, device)
    workers = tuple(sorted({min(w, fit) for w in workers}))
    px = sum(t.shape[0] * t.shape[1] for t in tiles)
    arr, _labels = _tile_array(tiles)
    params = _lib.SegParams()
    trials = []
    for w in workers:
        pool = TilePool(maxr, maxc, workers=w, device=device)
        try:
            for frac, bfs in itertools.product(recon_fractions, bfs_clusters):
                rc = max(1, int(sms * frac))
                pool.set_tuning(rc, bfs)
                pool.run(arr, params)  # warm-up
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for _ in range(reps):
                    pool.run(arr, params)
                torch.cuda.synchronize()
                mpx = px * reps / (time.perf_counter() - t0) / 1e6
                trials.append({"workers": w, "recon_max_ctas": rc, "bfs_max_cluster": bfs, "mpx_s": round(mpx, 2)})
        finally:
            pool.close()
    best = max(trials, key=lambda t: t["mpx_s"])
    return dict(best, trials=trials, calibration_tiles=len(tiles), calibration_mpx=round(px / 1e6, 1))


def main(argv=None) -> int:
    from . import synth_torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--tiles", type=int, default=96)
    ap.add_argument("--out", default="")
    a = ap.parse_args(argv)
    shapes = synth_torch.batch_shapes(256)[: a.tiles]
    tiles = [synth_torch.he_tile(r, c, 0x5EED0003 + i, device="cuda") for i, (r, c) in enumerate(shapes)]
    res = autotune(tiles)
    text = json.dumps(res, indent=1)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text)
    print(text)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
