"""Splitting a case range across ranks (one GPU per rank / per box).

The path shards by independent units with no data-path collective: rank r
counts cases [start + r*q + min(r, rem), ...) of the emission order and the
partial sums (uint128, as decimal strings) are added on the host -- the same
aggregation modal_sym.py performs over JSONL rows (modal_sym.py:36-77).
"""
from __future__ import annotations

from typing import Callable, Iterable


def shard_range(start: int, count: int, rank: int, world: int) -> tuple[int, int]:
    """(first case, number of cases) of `rank`'s contiguous share."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    q, rem = divmod(count, world)
    first = start + rank * q + min(rank, rem)
    return first, q + (1 if rank < rem else 0)


def combine(partials: Iterable[str | int]) -> int:
    """Exact sum of per-rank partial counts."""
    return sum(int(p) for p in partials)


def run_rank(count_chunk: Callable[[int, int], int], start: int, count: int, rank: int,
             world: int, gather: Callable[[str], list]) -> int:
    """Count this rank's share with `count_chunk(first, n)` and combine all
    ranks' partials through `gather` (e.g. torch.distributed.all_gather_object
    over gloo/NCCL); returns the total."""
    first, n = shard_range(start, count, rank, world)
    part = count_chunk(first, n) if n else 0
    return combine(gather(str(part)))
