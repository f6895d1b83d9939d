"""Sharding a block scan across ranks (one GPU per rank), host side only.

The outer indices of a block are independent, so a scan shards into contiguous outer-index
ranges with no data exchange; the only reduction is on the host: the union of the ranks'
survivor indices, the sum of their per-stage pass counts, and the least good n.  There is no
collective on the data path (the reference scales the same way, by running separate processes
over separate ranges: harness/grind.py:58-79, harness/run_k_masks.py --start-block).
"""
from __future__ import annotations


def shard_range(o_begin: int, o_end: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous slice of [o_begin, o_end) for `rank` of `world`; slices tile the range."""
    if not (0 <= rank < world) or o_end < o_begin:
        raise ValueError("bad shard request")
    n = o_end - o_begin
    return o_begin + n * rank // world, o_begin + n * (rank + 1) // world


def merge(parts) -> tuple[list[int], list[int]]:
    """Union of per-shard (survivor indices, stage counts) -> (sorted survivors, summed counts)."""
    surv: list[int] = []
    counts: list[int] | None = None
    for s, c in parts:
        surv.extend(int(x) for x in s)
        counts = [int(x) for x in c] if counts is None else [a + int(b) for a, b in zip(counts, c)]
    return sorted(surv), counts or []


def least_good(plan, t: int, survivors, is_good) -> int | None:
    """The least survivor n = idx_to_n(idx, t) with n > k+1 that passes the exact test."""
    ns = sorted(plan.idx_to_n(int(i), t) for i in survivors)
    for n in ns:
        if n > plan.k + 1 and is_good(n, plan.k):
            return n
    return None
