"""Multi-process host logic.

Back-projection partitions by image region with no data exchange: each rank
images its own strip of rows (or, for weak scaling, its own replica of the
scene).  Only the timing needs a collective (max over ranks); the data path
has none.
"""
from __future__ import annotations

import numpy as np

from .scenes import Grid


def strip_bounds(ny: int, rank: int, world: int, align: int = 64):
    """Rows [y0, y1) of rank's strip; strips are multiples of `align` rows
    (the back-projection tile height) except the last."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    blocks = (ny + align - 1) // align
    b0 = blocks * rank // world
    b1 = blocks * (rank + 1) // world
    return min(ny, b0 * align), min(ny, b1 * align)


def grid_strip(grid: Grid, rank: int, world: int, align: int = 64) -> Grid:
    """Sub-grid of rows [y0, y1) with the same pixel positions as in `grid`."""
    y0, y1 = strip_bounds(grid.ny, rank, world, align)
    return Grid(origin=grid.origin + y0 * grid.uy, ux=grid.ux.copy(), uy=grid.uy.copy(), nx=grid.nx, ny=y1 - y0)


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """Max of a scalar over the default process group (identity without one)."""
    if dist is None or not dist.is_initialized():
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def assemble(strips, ny: int, nx: int, world: int, align: int = 64) -> np.ndarray:
    """Stack per-rank strips back into the full image."""
    out = np.zeros((ny, nx), dtype=strips[0].dtype)
    for r, s in enumerate(strips):
        y0, y1 = strip_bounds(ny, r, world, align)
        out[y0:y1] = s
    return out
