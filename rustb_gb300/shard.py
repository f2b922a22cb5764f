"""k-range sharding of one uniform mesh over ranks.

The Direct Hall sum is a sum over independent k-points
(src/response/linear/mod.rs:198-223), so ranks take disjoint contiguous
ranges of the flat mesh index (gen_kmesh order) of a replicated model, and the
only exchange is a sum of n_mu doubles at the end.
"""

from __future__ import annotations

import math


def step_range(nk: int, batch: int, world: int, rank: int, step: int) -> tuple[int, int]:
    """Flat k-range (begin, count) that `rank` processes at `step` when every
    step hands one batch to each rank (the bench's weak-scaling layout)."""
    k0 = ((step * world + rank) * batch) % nk
    return k0, min(batch, nk - k0)


def rank_ranges(nk: int, world: int, rank: int, batch: int) -> list[tuple[int, int]]:
    """All ranges of `rank` when the whole mesh is split round-robin in batches."""
    out = []
    nbatches = math.ceil(nk / batch)
    for b in range(rank, nbatches, world):
        k0 = b * batch
        out.append((k0, min(batch, nk - k0)))
    return out


def combine(partials, nk: int, det: float):
    """sigma_j = (sum over ranks and ranges of the partial sums) / nk / det."""
    ncol = len(partials[0])
    return [math.fsum(p[j] for p in partials) / nk / det for j in range(ncol)]
