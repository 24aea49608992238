"""Sharding of a batch of independent structures over ranks (one process per GPU).

The reference distributes whole structures over MPI ranks with a contiguous block rule
(thread::Dist, src/thread/dist.hpp:21-53; nnpce.cpp:228) and, in nnptefr3, balances by atom count
(README.md:354-358). Structures never interact, so a rank's shard needs no data exchange; the
only collectives are a barrier and a max of the step time around the timed region (and, for
training, one sum of the parameter gradient, the reference's MPI_Reduce at nnptefr2.cpp:984).
"""
from __future__ import annotations

import numpy as np


def dist_block(n: int, rank: int, world: int) -> tuple[int, int]:
    """thread::Dist block rule: contiguous blocks, the first n % world blocks one longer."""
    q, r = divmod(n, world)
    lo = rank * q + min(rank, r)
    return lo, lo + q + (1 if rank < r else 0)


def shard_by_atoms(offsets, rank: int, world: int) -> tuple[int, int]:
    """Contiguous structure range [lo, hi) of `rank` whose atom count is as close as possible to
    1/world of the batch (cut points at the atom-count quantiles)."""
    offsets = np.asarray(offsets, dtype=np.int64)
    S = len(offsets) - 1
    total = int(offsets[-1])
    if world <= 1:
        return 0, S
    cuts = [0]
    for k in range(1, world):
        target = total * k / world
        s = int(np.searchsorted(offsets, target, side="left"))
        s = min(max(s, cuts[-1]), S)
        cuts.append(s)
    cuts.append(S)
    return cuts[rank], cuts[rank + 1]


def subset(offsets, posn, types, cell, lo: int, hi: int):
    """The packed arrays of structures [lo, hi)."""
    offsets = np.asarray(offsets, dtype=np.int64)
    a0, a1 = int(offsets[lo]), int(offsets[hi])
    return offsets[lo:hi + 1] - a0, posn[a0:a1], types[a0:a1], cell[lo:hi]
