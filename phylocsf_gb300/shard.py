"""Spreading independent regions over several GPUs (one engine per rank).

Regions are independent, so the path shards with no data-path collective:
each rank scores its own share with its own engine and the per-region results
are gathered on the host at the end.  The share is a longest-first greedy
partition by codon columns, the order the reference uses before forking
workers (src/PhyloCSF.ml:303-308).
"""
from __future__ import annotations

from typing import Callable, List, Sequence

import numpy as np


def partition_longest_first(lengths: Sequence[int], world: int) -> List[np.ndarray]:
    """Region indices per rank: longest region first, each to the least-loaded rank."""
    lengths = np.asarray(lengths, np.int64)
    order = np.argsort(-lengths, kind="stable")
    load = np.zeros(world, np.int64)
    parts: List[list] = [[] for _ in range(world)]
    for r in order:
        k = int(np.argmin(load))
        parts[k].append(int(r))
        load[k] += int(lengths[r])
    return [np.array(sorted(p), np.int64) for p in parts]


def subset(col_offsets: np.ndarray, leaves: np.ndarray, idx: np.ndarray):
    """(col_offsets, leaves) of the regions idx, in that order."""
    parts = [leaves[col_offsets[i]:col_offsets[i + 1]] for i in idx]
    offs = np.zeros(len(idx) + 1, np.int64)
    offs[1:] = np.cumsum([p.shape[0] for p in parts]) if len(parts) else []
    lv = np.concatenate(parts) if parts else leaves[:0]
    return offs, lv


def score_sharded(col_offsets: np.ndarray, leaves: np.ndarray, score_fn: Callable, rank: int, world: int,
                  group=None) -> np.ndarray:
    """Score this rank's share with score_fn(offs, leaves) -> structured array, then
    all-gather the results (host objects, gloo or NCCL) back into region order."""
    import torch.distributed as dist
    lengths = np.diff(col_offsets)
    parts = partition_longest_first(lengths, world)
    mine = parts[rank]
    offs, lv = subset(col_offsets, leaves, mine)
    res = score_fn(offs, lv)
    gathered = [None] * world
    if world > 1:
        dist.all_gather_object(gathered, (mine, res), group=group)
    else:
        gathered = [(mine, res)]
    out = np.zeros(len(lengths), res.dtype)
    for idx, r in gathered:
        out[idx] = r
    return out
