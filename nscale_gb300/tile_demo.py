"""Segment one synthetic H&E tile on cuda:0 and print its status, nucleus
count and wall time:

    python -m nscale_gb300.tile_demo [ROWS [COLS [SEED]]]

The tile comes from the on-device generator (synth_torch.he_tile, default
seed 0x5EED0000); it is the small driver behind the ncu captures of single
kernels of the segmentNuclei path.
"""
from __future__ import annotations

import sys
import time


def main(argv: list[str]) -> int:
    import torch
    from . import synth_torch
    from .histological_entities import HistologicalEntities as HE
    rows = int(argv[0]) if len(argv) > 0 else 2048
    cols = int(argv[1]) if len(argv) > 1 else rows
    seed = int(argv[2], 0) if len(argv) > 2 else 0x5EED0000
    tile = synth_torch.he_tile(rows, cols, seed, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    status, _labels, n, _bbox = HE.segmentNuclei(tile)
    torch.cuda.synchronize()
    print(f"tile {rows}x{cols} status {status} nuclei {n} wall {1e3 * (time.perf_counter() - t0):.1f} ms")
    return 0 if status >= 0 else 1


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
