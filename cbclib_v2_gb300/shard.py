"""Frame sharding for one process per GPU.

Frames are independent: every line belongs to exactly one frame, and its pixels, its
adjoint and its parameter update touch only that frame.  A run over several GPUs
therefore gives each rank a contiguous range of frames whose work adds up to about
1/world of the total, taken from the prefix sums of the CSR line offsets, and every
rank renders, differentiates and updates only its own frames.  The data path has no
collective; the only cross-rank values are scalars for reporting (a loss), reduced on
the host side.
"""
from dataclasses import dataclass
from typing import Optional

import numpy as np

__all__ = ['partition_frames', 'Shard', 'shard_of']


def partition_frames(frame_offsets, world: int, frame_cost: Optional[float] = None) -> np.ndarray:
    """Frame boundaries (world + 1,) that split the stack into contiguous ranges of
    about equal cost.  A frame costs its line count plus `frame_cost` (default 5 % of
    the mean line count, at least 1) for the pixels every frame carries even when it
    holds few lines.  Rank r owns frames [bounds[r], bounds[r + 1])."""
    offs = np.asarray(frame_offsets, dtype=np.int64).reshape(-1)
    if offs.size < 1 or offs[0] != 0 or np.any(np.diff(offs) < 0):
        raise ValueError("frame_offsets must start at 0 and be non-decreasing")
    if world < 1:
        raise ValueError(f"world must be positive ({world})")
    n_frames = offs.size - 1
    counts = np.diff(offs).astype(np.float64)
    if frame_cost is None:
        frame_cost = max(1.0, 0.05 * counts.mean()) if n_frames else 1.0
    csum = np.concatenate([[0.0], np.cumsum(counts + frame_cost)])
    bounds = np.empty(world + 1, dtype=np.int64)
    bounds[0], bounds[-1] = 0, n_frames
    for r in range(1, world):
        target = csum[-1] * r / world
        i = int(np.searchsorted(csum, target))          # csum[i - 1] < target <= csum[i]
        if i > 0 and target - csum[i - 1] < csum[min(i, n_frames)] - target:
            i -= 1
        bounds[r] = min(max(i, bounds[r - 1]), n_frames)
    return bounds


@dataclass(frozen=True)
class Shard:
    """The frames [f0, f1) and lines [l0, l1) of one rank."""
    rank: int
    world: int
    f0: int
    f1: int
    l0: int
    l1: int

    @property
    def n_frames(self) -> int:
        return self.f1 - self.f0

    @property
    def n_lines(self) -> int:
        return self.l1 - self.l0

    def local_offsets(self, frame_offsets) -> np.ndarray:
        """CSR offsets of this rank's frames, rebased to its first line."""
        offs = np.asarray(frame_offsets, dtype=np.int64).reshape(-1)
        return offs[self.f0:self.f1 + 1] - offs[self.f0]


def shard_of(frame_offsets, rank: int, world: int, frame_cost: Optional[float] = None) -> Shard:
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside of [0, {world})")
    offs = np.asarray(frame_offsets, dtype=np.int64).reshape(-1)
    b = partition_frames(offs, world, frame_cost)
    f0, f1 = int(b[rank]), int(b[rank + 1])
    return Shard(rank, world, f0, f1, int(offs[f0]), int(offs[f1]))
