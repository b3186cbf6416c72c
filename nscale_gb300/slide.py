"""Synthetic whole-slide source for the serving form: a rows x cols slide
(default 80000 x 100000, the size the serving benchmark names) cut into tile x
tile requests (default 4096) with ragged tiles on the right and bottom edges,
the way a slide tiler hands tiles to nu-segment (nu-segment.cpp:123-163 reads
one tile image per task).  Nothing is stored: tile (i, j) is generated when it
is asked for, from the slide seed and its grid position, so the 2.4 TB slide
never exists in memory.  A fixed fraction of tiles (20 % by default) is
tissue-free (near-white BGR 230-250 in every channel: the BACKGROUND exit of
segmentNuclei); the rest follow the H&E statistics of synth_torch.he_tile.
"""
from __future__ import annotations

import numpy as np
import torch

from . import synth, synth_torch


class SyntheticSlide:
    def __init__(self, rows: int = 80000, cols: int = 100000, tile: int = 4096, seed: int = 0x5EED0004,
                 tissue_free: float = 0.2):
        if rows <= 0 or cols <= 0 or tile <= 0:
            raise ValueError("slide and tile sizes must be positive")
        self.rows, self.cols, self.tile_size, self.seed = rows, cols, tile, seed
        self.tissue_free = tissue_free
        self.grid = ((rows + tile - 1) // tile, (cols + tile - 1) // tile)

    def __len__(self) -> int:
        return self.grid[0] * self.grid[1]

    def position(self, k: int) -> tuple[int, int]:
        """Grid position of the k-th tile in raster order."""
        if not 0 <= k < len(self):
            raise IndexError(k)
        return divmod(k, self.grid[1])

    def shape(self, i: int, j: int) -> tuple[int, int]:
        """(rows, cols) of tile (i, j): ragged on the last row / column."""
        t = self.tile_size
        return min(t, self.rows - i * t), min(t, self.cols - j * t)

    def _tile_seed(self, i: int, j: int) -> int:
        return (self.seed * 1000003 + i * 65537 + j) & 0x7FFFFFFF

    def is_tissue_free(self, i: int, j: int) -> bool:
        u = synth._uniform(self.seed, 900, np.array([i * self.grid[1] + j], dtype=np.uint64))[0]
        return bool(u < self.tissue_free)

    def tile(self, i: int, j: int, device="cuda") -> torch.Tensor:
        """Tile (i, j) as a (rows, cols, 3) uint8 BGR tensor on `device`."""
        r, c = self.shape(i, j)
        s = self._tile_seed(i, j)
        if self.is_tissue_free(i, j):
            dev = torch.device(device)
            idx = torch.arange(r * c, device=dev, dtype=torch.int64).view(r, c)
            out = torch.empty((r, c, 3), device=dev, dtype=torch.uint8)
            for ch in range(3):
                out[..., ch] = synth_torch._randint(s, 40 + ch, idx, 230, 250).to(torch.uint8)
            return out
        return synth_torch.he_tile(r, c, s, device=device)
