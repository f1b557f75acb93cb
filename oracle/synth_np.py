"""numpy restatement of the engine library's column simulator -- TEST INFRASTRUCTURE ONLY.

Only ``tests/`` and ``bench.py``'s reference (CPU) arm use it.  It lets the CPU arm
build the benchmark's regions without loading the product library: given the same
workload description (column offsets, per-region model, per (region, species) gap
probability, seed) it produces, for any subset of regions, exactly the leaf codes the
native ``pcsf_simulate`` writes for those columns.

What it restates (the native simulator follows PhyloModel.simulate,
lib/CamlPaml/PhyloModel.ml:38-54, and testSim's stop-codon rejection,
src/testSim.ml:52-65):
  * one counter-based SplitMix64 stream per global column c, seeded with
    mix64(seed * 0x9E3779B97F4A7C15 + c + 1);
  * root state drawn from the prior's cumulative sums, then every node from the
    cumulative row of its parent's state on its branch, nodes n-2 .. 0;
  * a column whose leaf 0 is a stop codon (TAA, TAG, TGA) is drawn again from the
    same stream, at most 1000 times;
  * then, leaf by leaf, one more draw below the gap probability marginalises it.
Draws use u * cum[63] against the cumulative sums and take the smallest index j with
u * cum[63] < cum[j] (63 at most).
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
STOPS = (48, 50, 56)          # TAA, TAG, TGA as 16 n1 + 4 n2 + n3
MARGINALIZE = 64


def _mix64(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


class _Streams:
    """One SplitMix64 stream per column."""

    def __init__(self, seed: int, cols: np.ndarray):
        with np.errstate(over="ignore"):
            self.s = _mix64(np.uint64(seed) * GOLDEN + cols.astype(np.uint64) + np.uint64(1))

    def next(self, idx: Optional[np.ndarray] = None) -> np.ndarray:
        with np.errstate(over="ignore"):
            if idx is None:
                self.s = self.s + GOLDEN
                z = self.s
            else:
                self.s[idx] = self.s[idx] + GOLDEN
                z = self.s[idx]
            return (_mix64(z) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _draw(cum_rows: np.ndarray, u: np.ndarray) -> np.ndarray:
    """Smallest j with u * cum[63] < cum[j] (63 at most), row by row."""
    thr = u * cum_rows[:, 63]
    return np.minimum((cum_rows <= thr[:, None]).sum(axis=1), 63)


def simulate_regions(parent: np.ndarray, P: np.ndarray, prior: np.ndarray, col_offsets: np.ndarray,
                     region_model: np.ndarray, gap_frac: Optional[np.ndarray], seed: int,
                     regions: Sequence[int], reject_stop_leaf0: bool = True) -> np.ndarray:
    """Leaf codes uint8 [sum of the regions' lengths][n_leaves] of `regions` (in that order),
    identical to the rows pcsf_simulate writes for their columns.

    parent: [n] (T order, root last); P: [models][nbr][64][64] row-stochastic;
    prior: [models][64]; col_offsets: [R+1] of the whole workload."""
    parent = np.asarray(parent, np.int64)
    n = len(parent)
    nl = (n + 1) // 2
    # cumulative sums in the same sequential order as the native simulator
    cum = np.cumsum(np.asarray(P, np.float64), axis=-1)
    cpr = np.cumsum(np.asarray(prior, np.float64), axis=-1)
    out = []
    for r in regions:
        c0, c1 = int(col_offsets[r]), int(col_offsets[r + 1])
        m = int(region_model[r])
        cols = np.arange(c0, c1, dtype=np.int64)
        nc = len(cols)
        st = np.zeros((nc, n), np.int64)
        if nc:
            rng = _Streams(seed, cols)
            todo = np.arange(nc)
            for _ in range(1000):
                u = rng.next(todo)
                st[todo, n - 1] = _draw(np.broadcast_to(cpr[m], (len(todo), 64)), u)
                for i in range(n - 2, -1, -1):
                    u = rng.next(todo)
                    st[todo, i] = _draw(cum[m, i][st[todo, parent[i]]], u)
                if not reject_stop_leaf0:
                    break
                todo = todo[np.isin(st[todo, 0], STOPS)]
                if len(todo) == 0:
                    break
            codes = st[:, :nl].astype(np.uint8)
            if gap_frac is not None:
                g = np.asarray(gap_frac, np.float64)[r]
                for leaf in range(nl):
                    u = rng.next()
                    codes[u < g[leaf], leaf] = MARGINALIZE
        else:
            codes = np.zeros((0, nl), np.uint8)
        out.append(codes)
    return np.concatenate(out) if out else np.zeros((0, nl), np.uint8)
