"""Autotuner for the batched kernels.

Picks, per workload and GPU, the partition depth of each Lunnon map (how many
prefix states the host hands the device), the CTA size, the bookkeeping
period between split checks (`node_budget`) and the split-ring size, by
timing short replays of recorded CUDA graphs.  Results are cached in a JSON
file (MF_AUTOTUNE_CACHE, default ~/.cache/map_folding_gb300/autotune.json)
keyed by the workload signature and the GPU name, so a tuned workload
starts from its best configuration on the next run.
"""
from __future__ import annotations

import hashlib
import itertools
import json
import os
import time
from pathlib import Path
from typing import Sequence

from . import api
from ._native import BatchConfig


def _cache_path() -> Path:
    env = os.environ.get("MF_AUTOTUNE_CACHE")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "map_folding_gb300" / "autotune.json"


def _gpu_name() -> str:
    try:
        import torch

        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:
        pass
    return "unknown-gpu"


def _load_cache() -> dict:
    p = _cache_path()
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return {}
    return {}


def _store(key: str, value: dict) -> None:
    p = _cache_path()
    p.parent.mkdir(parents=True, exist_ok=True)
    cache = _load_cache()
    cache[key] = value
    tmp = p.with_suffix(".tmp")
    tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
    os.replace(tmp, p)


def signature(shapes: Sequence[Sequence[int]]) -> str:
    text = ";".join("x".join(map(str, s)) for s in shapes)
    return hashlib.sha1(text.encode()).hexdigest()[:16]


def default_depth(dims: Sequence[int]) -> int:
    n = 1
    for d in dims:
        n *= d
    d = n // 2 + 3 if n < 30 else n // 2
    return min(d, n)


def _config(tpb: int, period: int, cap: int) -> BatchConfig:
    c = BatchConfig()
    c.block_threads = tpb
    c.node_budget = period
    c.queue_capacity = cap
    return c


def tune_lunnon_batch(shapes: Sequence[Sequence[int]], depth_offsets=(-2, 0, 2),
                      block_threads=(128, 256), periods=(32, 64, 128),
                      capacities=(1 << 16,), repeats: int = 2, use_cache: bool = True) -> dict:
    """Best configuration for counting all `shapes` in one batched launch.

    Returns {"depths": [...], "block_threads", "node_budget", "queue_capacity",
    "seconds", "counts"}; every candidate's counts must agree (they are
    exact), which the tuner checks as it goes."""
    shapes = [tuple(s) for s in shapes]
    key = f"lunnon:{signature(shapes)}:{_gpu_name()}"
    if use_cache:
        hit = _load_cache().get(key)
        if hit:
            return hit
    best = None
    reference_counts = None
    for off in depth_offsets:
        depths = []
        for s in shapes:
            n = 1
            for d in s:
                n *= d
            depths.append(max(0, min(n, default_depth(s) + off)))
        for tpb, period, cap in itertools.product(block_threads, periods, capacities):
            batch = api.LunnonBatch(shapes, depths, _config(tpb, period, cap))
            try:
                times = []
                counts = None
                for _ in range(repeats + 1):  # the first replay warms up
                    counts, st = batch.run()
                    times.append(st.kernel_s)
                secs = min(times[1:]) if repeats else times[0]
            finally:
                batch.close()
            if reference_counts is None:
                reference_counts = counts
            elif counts != reference_counts:
                raise RuntimeError(f"counts changed under tuning: {depths} {tpb} {period}")
            cand = {"depths": depths, "block_threads": tpb, "node_budget": period,
                    "queue_capacity": cap, "seconds": secs, "counts": counts}
            if best is None or secs < best["seconds"]:
                best = cand
    best["tuned_at"] = time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())
    _store(key, best)
    return best


def tune_sym(n: int, expanded_n: int, block_threads=(128, 256), periods=(32, 64, 128),
             repeats: int = 1, max_cases: int = 0, use_cache: bool = True) -> dict:
    """Best CTA size and bookkeeping period for a sym case set, timed with
    graph replays on the device-resident cases."""
    import numpy as np
    import torch

    key = f"sym:{n}:{expanded_n}:{max_cases}:{_gpu_name()}"
    if use_cache:
        hit = _load_cache().get(key)
        if hit:
            return hit
    plan = api.SymPlan(n, expanded_n)
    cycles, mults = plan.cases(0, max_cases)
    d_cyc = torch.from_numpy(np.ascontiguousarray(cycles)).cuda()
    d_counts = torch.zeros(len(cycles), dtype=torch.int64, device="cuda")
    best = None
    want = None
    for tpb, period in itertools.product(block_threads, periods):
        cfg = _config(tpb, period, 1 << 16)
        ws = torch.empty(api.sym_workspace_bytes(cfg), dtype=torch.uint8, device="cuda")
        g = api.SymGraph(n, plan.start_i, n * n, d_cyc.data_ptr(), len(cycles), d_counts.data_ptr(),
                         ws.data_ptr(), ws.numel(), cfg=cfg)
        times = []
        for _ in range(repeats + 1):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            g.launch(torch.cuda.current_stream().cuda_stream)
            b.record()
            torch.cuda.synchronize()
            times.append(a.elapsed_time(b) * 1e-3)
        g.close()
        counts = d_counts.cpu().numpy().view(np.uint64).copy()
        if want is None:
            want = counts
        elif not (counts == want).all():
            raise RuntimeError("counts changed under tuning")
        secs = min(times[1:]) if repeats else times[0]
        if best is None or secs < best["seconds"]:
            best = {"block_threads": tpb, "node_budget": period, "seconds": secs}
    best["tuned_at"] = time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())
    _store(key, best)
    return best


def as_config(tuned: dict) -> BatchConfig:
    return _config(int(tuned["block_threads"]), int(tuned["node_budget"]),
                   int(tuned.get("queue_capacity", 1 << 16)))
