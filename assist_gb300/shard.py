"""Partitioning independent particles across ranks (one process per GPU).

Particles are independent given the read-only ephemeris, so a multi-GPU run
needs no data-path collective: each rank integrates its shard and the end
states are gathered once.  Shards balance the integration length (the cost
proxy) greedily, longest first.
"""
from __future__ import annotations

import heapq

import numpy as np


def shard_indices(lengths, rank: int, world: int) -> np.ndarray:
    """Indices of the particles rank `rank` of `world` integrates (sorted).
    Greedy longest-processing-time partition of |t_end - t0|."""
    lengths = np.abs(np.asarray(lengths, dtype=np.float64))
    if world <= 1:
        return np.arange(lengths.size)
    order = np.argsort(-lengths, kind="stable")
    heap = [(0.0, r) for r in range(world)]
    owner = np.empty(lengths.size, dtype=np.int64)
    for i in order:
        load, r = heapq.heappop(heap)
        owner[i] = r
        heapq.heappush(heap, (load + lengths[i], r))
    return np.nonzero(owner == rank)[0]


def gather_states(shards, n: int) -> np.ndarray:
    """Reassemble per-rank (indices, states) pairs into one (n, 6) array."""
    out = np.full((n, 6), np.nan)
    for idx, st in shards:
        out[np.asarray(idx)] = st
    return out
