"""Seeded workloads with the shapes of the benchmark configurations.

uneven_instances(seed, count)
    maps for the batched uneven launch: shape class uniform over
    {p x q with 2 <= p, q <= 6; 1-D strip of 2..20 stamps; 2 x 2 x k with
    k <= 5}, parameters uniform within the class.
serving_stream(seed, ...)
    8x8 chunk requests (MF_EXPANDED_N = 36, 50,000 consecutive cases, start
    uniform over [0, 240192829)) arriving as a Poisson process, interleaved
    with small whole-map requests (p x q <= 5 x 6).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

TOTAL_8X8_D36 = 240_192_829


def uneven_instances(seed: int, count: int = 64) -> list[tuple[int, ...]]:
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(count):
        cls = int(rng.integers(0, 3))
        if cls == 0:
            out.append((int(rng.integers(2, 7)), int(rng.integers(2, 7))))
        elif cls == 1:
            out.append((1, int(rng.integers(2, 21))))
        else:
            out.append((2, 2, int(rng.integers(1, 6))))
    return out


@dataclass
class Request:
    rid: int
    arrival_s: float
    kind: str               # "chunk" or "map"
    start_case: int = 0     # chunk requests
    max_cases: int = 0
    dims: tuple = ()        # map requests


def serving_stream(seed: int, requests: int, rate_per_s: float, chunk_cases: int = 50_000,
                   map_fraction: float = 0.25, total_cases: int = TOTAL_8X8_D36) -> list[Request]:
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    for rid in range(requests):
        t += float(rng.exponential(1.0 / rate_per_s))
        if rng.random() < map_fraction:
            p = int(rng.integers(2, 6))
            q = int(rng.integers(2, 7))
            out.append(Request(rid, t, "map", dims=(p, q)))
        else:
            start = int(rng.integers(0, total_cases))
            start = min(start, total_cases - chunk_cases)
            out.append(Request(rid, t, "chunk", start_case=start, max_cases=chunk_cases))
    return out
